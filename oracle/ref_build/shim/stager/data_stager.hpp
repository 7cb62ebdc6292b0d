// Stand-in for the reference's data stagers with one rank. DataStagerByFrame returns
// the target selection's coordinates frame-major, float32 [NF][NA][3]
// (data_stager.cpp:102-118); DataStagerByAtom returns them atom-major [NA][NF][3]
// (data_stager.cpp:214-338 with one rank). Both buffers come from malloc: the devices
// free them.
#pragma once
#include <cstdlib>
#include <cstring>

#include <boost/mpi.hpp>

#include "common.hpp"
#include "report/timer.hpp"
#include "sample.hpp"

class DataStagerByFrame {
    Sample& m_sample;

public:
    DataStagerByFrame(Sample& sample, boost::mpi::communicator&, boost::mpi::communicator&, Timer&)
        : m_sample(sample) {}
    coor_t* stage() {
        const size_t nf = m_sample.coordinate_sets.size();
        const size_t na = m_sample.atoms.selections.begin()->second->size();
        coor_t* p = (coor_t*)malloc(nf * na * 3 * sizeof(coor_t));
        std::memcpy(p, m_sample.target_frames, nf * na * 3 * sizeof(coor_t));
        return p;
    }
};

class DataStagerByAtom {
    Sample& m_sample;

public:
    DataStagerByAtom(Sample& sample, boost::mpi::communicator&, boost::mpi::communicator&, Timer&)
        : m_sample(sample) {}
    coor_t* stage() {
        const size_t nf = m_sample.coordinate_sets.size();
        const size_t na = m_sample.atoms.selections.begin()->second->size();
        coor_t* p = (coor_t*)malloc(nf * na * 3 * sizeof(coor_t));
        for (size_t a = 0; a < na; ++a)
            for (size_t f = 0; f < nf; ++f)
                for (int c = 0; c < 3; ++c) p[(a * nf + f) * 3 + c] = m_sample.target_frames[(f * na + a) * 3 + c];
        return p;
    }
};
