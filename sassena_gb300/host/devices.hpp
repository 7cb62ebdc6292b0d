// GPU scatter devices: the IScatterDevice contract on top of the C ABI.
//
// Mirrors AbstractScatterDevice::run / runner / write
// (src/scatter_devices/abstract_scatter_device.cpp:105-244), the vectors-averaging
// sub-vector construction (abstract_vectors_scatter_device.cpp:112-175) and
// ScatterFactors (scatter_factors.cpp:34-123). Device selection follows
// ScatterDeviceFactory::create (scatter_device_factory.cpp:145-201):
// scattering.type all|self x average.orientation.type vectors|none.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "config.hpp"
#include "sample.hpp"
#include "signal_file.hpp"

namespace sassgpu {

// Atoms of the target selection grouped by (database ID, kappa): b depends only on
// the class and |q| (ScatterFactors::update, scatter_factors.cpp:56-78).
struct ScatterClasses {
    std::vector<int32_t> atom_class;  // [NA] class per target atom
    std::vector<size_t> id;           // [nclass] database ID
    std::vector<double> kappa;        // [nclass]
    // b_class(|q|) for one q (sf - background * efactor(kappa * volume))
    std::vector<double> factors(const Database& db, double background, double ql) const;
};

ScatterClasses build_classes(const Params& p, const Database& db, const Sample& s);

// Sub-vectors of q (init_subvectors): |q| u_i for file/sphere orientations, the
// cylinder construction around the axis, or {q} without averaging.
std::vector<Vec3> subvectors_for(const Params& p, const Vec3& q);

struct RunStats {
    size_t nq_total = 0, nq_computed = 0, na = 0, nf = 0, nsub = 0;
    double stage_s = 0, compute_s = 0, write_s = 0;
    double terms = 0;
};

// IScatterDevice::run for the configuration: stage, compute every q not already in
// the signal file, write rows. Returns false if nothing was left to compute.
bool run_scatter_device(const Params& p, Database& db, const Sample& s, RunStats& stats);

}  // namespace sassgpu
