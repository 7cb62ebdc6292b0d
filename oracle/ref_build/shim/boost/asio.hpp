// Stand-in for boost/asio.hpp: the devices take TCP endpoints of the writer and monitor
// services as constructor arguments; one process needs no transport.
#pragma once
namespace boost { namespace asio { namespace ip {
struct tcp {
    struct endpoint {};
};
} } }
