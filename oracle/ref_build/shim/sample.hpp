// Stand-in for the reference's Sample: the parts the scatter devices and ScatterFactors
// read. The harness fills it: atom database IDs, one selection per name (the device's
// stager.target and the kappa selections), the frame count and the staged coordinates
// of the target selection as float32 [NF][NA][3].
#pragma once
#include <cstddef>
#include <map>
#include <string>
#include <vector>

#include "math/coor3d.hpp"  // the reference's sample.hpp brings the coordinate types

enum CoordinateRepresentation { CARTESIAN, SPHERICAL, CYLINDRICAL };

class IAtomselection {
public:
    std::vector<size_t> indexes;
    size_t size() { return indexes.size(); }
    size_t operator[](size_t i) { return indexes[i]; }
};

class SampleAtomsStandIn {
public:
    std::vector<size_t> ids;  // database ID of every atom of the system
    std::map<std::string, IAtomselection*> selections;
    size_t operator[](size_t i) { return ids[i]; }
    size_t size() { return ids.size(); }
};

class SampleCoordinateSetsStandIn {
public:
    size_t nframes = 0;
    size_t size() { return nframes; }
    void set_representation(CoordinateRepresentation) {}
    void set_selection(IAtomselection*) {}
};

class Sample {
public:
    SampleAtomsStandIn atoms;
    SampleCoordinateSetsStandIn coordinate_sets;
    const float* target_frames = nullptr;  // [NF][NA][3] of the target selection
};
