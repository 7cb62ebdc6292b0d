// Stand-in for boost/mpi.hpp: one process, one rank. The devices branch on the
// partition size; with one rank they never exchange frames or reduce across ranks,
// so the collectives only have to exist (they throw if a one-rank run reached them).
#pragma once
#include <stdexcept>

namespace boost {
namespace mpi {

class communicator {
public:
    int size() const { return 1; }
    int rank() const { return 0; }
    void barrier() const {}
};

template <class T, class N>
void all_to_all(const communicator&, const T*, N, T*) {
    throw std::logic_error("all_to_all reached in a one-rank run");
}

template <class T, class N, class Op>
void reduce(const communicator&, const T*, N, T*, Op, int) {
    throw std::logic_error("reduce reached in a one-rank run");
}

}  // namespace mpi
}  // namespace boost
