// Sample structure, selections, DCD trajectories and frame-major staging.
//
// Reference counterparts:
//   Atoms::add (PDB "ATOM  " names -> database IDs)   src/sample/atoms.cpp:64-86
//   selections "system", index, range, lexical        src/sample/sample.cpp:30-101,
//                                                     src/sample/atomselection.cpp:55-73
//   DCDFrameset::init/detect/read_frame, trim_index   src/sample/frames.cpp:232-436
//   Frames::add_frameset (clones)                     src/sample/frames.cpp:39-69
//   DataStagerByFrame::stage_firstpartition           src/stager/data_stager.cpp:102-118
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "config.hpp"

namespace sassgpu {

struct DcdFile {
    std::string path;
    size_t natoms = 0;
    size_t nframes_header = 0;
    bool ext_block1 = false, ext_block2 = false;
    uint64_t first_frame_pos = 0, frame_bytes = 0, x_off = 0, y_off = 0, z_off = 0;
    std::vector<uint64_t> frame_pos;  // byte position of every selected frame

    void open(const std::string& path);  // DCDFrameset::init + detect
    static bool detect(const std::string& path);
    // trim_index(first, last, last_set, stride) on the full frame index
    void select(size_t first, size_t last, bool last_set, size_t stride);
    // x, y, z (natoms floats each) of the i-th selected frame
    void read_frame(size_t i, float* x, float* y, float* z) const;
};

// Staged coordinates [nf][na][3] written as a CHARMM DCD in the layout of the reference's
// DCDCoordinateWriter (src/stager/coordinate_writer.cpp:27-137): 84-byte header with the
// unit-cell flag set, an empty title, the atom count, then per frame a zero unit cell and the
// X, Y, Z records (stager.dump, data_stager.cpp:91-94, 131-162).
void write_dcd(const std::string& path, const float* frames, size_t nf, size_t na);

// File selections (selection type "file"): the groups of an ndx index file whose names match
// `expression`, and the ATOM records of a PDB whose beta or segid field matches it.
std::map<std::string, std::vector<size_t>> read_ndx_groups(const std::string& path, const std::string& selector,
                                                          const std::string& expression);
std::vector<size_t> read_pdb_selection(const std::string& path, const std::string& selector,
                                       const std::string& expression);

class Sample {
public:
    std::vector<size_t> atom_ids;                          // database ID per atom (structure order)
    std::map<std::string, std::vector<size_t>> selections;  // name -> atom indices
    std::vector<DcdFile> framesets;                         // clones repeat a file
    size_t nframes = 0;

    void init(const Params& p, Database& db);
    const std::vector<size_t>& selection(const std::string& name) const;
    // frame-major float32 [nf][na][3] of the atoms in `target`
    // (CoordinateSets::load without motions/alignments reduces to the selection)
    std::vector<float> stage(const std::string& target) const;
    // The same frames written to `out` ([nframes][na][3]), e.g. page-locked host memory.
    void stage_into(const std::string& target, float* out) const;
};

}  // namespace sassgpu
