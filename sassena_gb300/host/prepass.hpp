// Staging pre-pass setup: the alignments and translation motions of the sample.
//
// Reference counterparts:
//   CoordinateSets::init (references, walkers, pre/post lists)  src/sample/coordinate_sets.cpp:54-232
//   CoordinateSets::load (the per-frame steps)                  src/sample/coordinate_sets.cpp:244-368
//   CenterOfMass, Fit (selection walks)                         src/sample/center_of_mass.cpp:53-264
//   Linear/Fixed/Oscillation motion walkers                     src/sample/motion_walker.cpp:340-400
//   PDBFrameset::generate_index / read_frame                    src/sample/frames.cpp:497-586
//
// The host resolves every selection walk of the reference into explicit atom lists and
// computes the walkers' per-frame translations; the device applies the steps
// (sass_stage_frames_prepass).
#pragma once

#include <cstddef>
#include <string>
#include <utility>
#include <vector>

#include "config.hpp"
#include "sample.hpp"

namespace sassgpu {

struct PrepassStep {
    int type = 0;                          // SASS_STEP_*
    std::vector<size_t> selection;         // atoms translated / centred
    std::vector<size_t> reference_selection;
    std::vector<double> reference;         // [nref][3]; empty: the current frame
    std::vector<size_t> fit_target, fit_source;
    std::vector<double> translations;      // motions: [nf][3]
    std::string label;                     // "pre center", "motion linear", ...
};

struct Prepass {
    std::vector<PrepassStep> steps;
    std::vector<double> masses;  // [nsys] database mass of every atom
};

// The reference's merge of a coordinate-set selection with a sub-selection: pairs
// (csel_iter, ssel_iter) with csel[csel_iter] == ssel[ssel_iter] (coordinate_set.cpp:48-64).
std::vector<std::pair<size_t, size_t>> merge_walk(const std::vector<size_t>& csel, const std::vector<size_t>& ssel);

// x, y, z of the ATOM records of frame `frame` of a PDB file (frames split at "END" lines);
// a frame number past the end takes the last frame, as the reference does with a warning.
std::vector<double> read_pdb_frame(const std::string& path, size_t frame);

// Steps for the configuration: pre-alignments, motions, post-alignments. `frames` holds the
// whole system's raw frames [nf][nsys][3] (references of type "frame"). Empty when the
// configuration has no alignments and no motions.
Prepass build_prepass(const Params& p, const Database& db, const Sample& s, const float* frames);

}  // namespace sassgpu
