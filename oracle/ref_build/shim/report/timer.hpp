// Stand-in for the reference's report/timer.hpp: the devices start and stop named
// timers; the harness keeps no statistics (the reference's Timer needs
// Boost.Accumulators).
#pragma once
#include <string>
class Timer {
public:
    void start(std::string) {}
    void stop(std::string) {}
};
