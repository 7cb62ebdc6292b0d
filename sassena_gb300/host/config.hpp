// Scattering configuration (scatter.xml) and atom database (db.xml).
//
// Mirrors the subset of the reference's Params (src/control/parameters.cpp:64-792)
// and Database (src/control/database.cpp) that the scattering-amplitude path reads:
// sample structure/framesets/selections, stager.target, database file, the whole
// scattering section, limits.computation.threads and limits.signal.chunksize, plus a
// new <gpu> element for this build's own knobs. Defaults are the reference's.
#pragma once

#include <array>
#include <map>
#include <string>
#include <vector>

#include "xml.hpp"

namespace sassgpu {

typedef std::array<double, 3> Vec3;

struct FramesetParams {
    std::string file, filepath, format = "dcd";
    size_t first = 0, last = 0, stride = 1, clones = 1;
    bool last_set = false;
};

struct SelectionParams {
    std::string name, type = "index";
    std::vector<size_t> ids;
    size_t from = 0, to = 0;
    std::string expression;
    // type "file" (parameters.cpp:148-176): a PDB (beta or segid column) or an ndx index file
    std::string file, filepath, format, selector;
};

// sample.alignments.alignment (parameters.cpp:298-340)
struct AlignmentParams {
    std::string type = "center", selection = "system", order = "pre";
    std::string ref_type = "frame", ref_file, ref_filepath, ref_format, ref_selection;
    size_t ref_frame = 0;
};

// sample.motions.motion (parameters.cpp:234-296)
struct MotionParams {
    std::string type = "linear", selection = "system";
    double displace = 0.0, frequency = 0.001, radius = 0.0;
    Vec3 direction{1.0, 0.0, 0.0};
    unsigned long seed = 0;
    long sampling = 1;
    std::string ref_type = "instant", ref_file, ref_filepath, ref_format, ref_selection;
    size_t ref_frame = 0;
};

struct ScanParams {
    Vec3 base{1.0, 0.0, 0.0};
    double from = 0.0, to = 1.0;
    size_t points = 100;
    double exponent = 1.0;
};

struct Params {
    std::string config_path, config_dir;
    std::string rawconfig;  // the configuration file's bytes (stored in signal.h5 /meta)

    // sample
    std::string structure_file = "sample.pdb", structure_filepath, structure_format = "pdb";
    std::vector<SelectionParams> selections;
    std::vector<FramesetParams> framesets;
    std::vector<MotionParams> motions;
    std::vector<AlignmentParams> alignments;
    // stager (parameters.cpp:340-369): target selection; dump of the staged coordinates
    std::string target = "system";
    bool stager_dump = false;
    std::string stager_file = "dump.dcd", stager_filepath, stager_format = "dcd", stager_mode = "frames";
    // database
    std::string db_file = "db.xml", db_filepath;
    // scattering
    std::string scattering_type = "all";
    double background_factor = 0.0;
    std::vector<std::pair<std::string, double>> kappas;  // (selection, value)
    std::vector<Vec3> qvectors;
    std::vector<ScanParams> scans;
    std::string dsp_type = "autocorrelate", dsp_method = "fftw";
    std::string orientation_type = "none";
    Vec3 axis{0.0, 0.0, 1.0};
    std::string vectors_type = "sphere", vectors_algorithm = "boost_uniform_on_sphere";
    long resolution = 100;
    unsigned long seed = 0;
    std::string vectors_file = "qvector-orientations.txt", vectors_filepath;
    std::vector<Vec3> orientations;  // unit vectors (file, sphere) or 2-D (cylinder)
    // orientation type "multipole" (parameters.cpp:386-389, 552-576)
    std::string multipole_type = "sphere", moments_type;
    long moments_resolution = 20;
    std::string moments_file = "moments.txt", moments_filepath;
    std::vector<std::pair<long, long>> moments;  // (major, minor)
    std::string signal_file = "signal.h5", signal_filepath;
    bool signal_fqt = true, signal_fq0 = true, signal_fq = true, signal_fq2 = true;
    // limits
    size_t chunksize = 10000, threads = 1;
    size_t serverflush_s = 600;
    // gpu (new)
    std::string precision = "fp64";
    std::string boost_random = "1.56";  // Boost.Random release whose sphere draws are reproduced
    int device = 0;
    size_t batch_q = 0;            // q-vectors per sass_compute call (0 = all)
    size_t amplitude_budget = 0;   // bytes (0 = library default)

    std::string get_filepath(const std::string& fname) const;
    void read_xml(const std::string& path);
    // command-line overrides "key=value" for the keys the reference accepts
    // (parameters.cpp:795-882) that touch this path
    void overwrite(const std::string& key, const std::string& value);
};

// ScatteringVectorsParameters::create_from_scans, parameters.cpp:1125-1189.
std::vector<Vec3> create_from_scans(const std::vector<ScanParams>& scans);
// ScatteringAverageOrientationVectorsParameters::create, parameters.cpp:930-1034 (file,
// cylinder raster_linear as the reference; sphere/cylinder random draws use this
// project's seeded generator, not Boost's mt19937 stream).
std::vector<Vec3> create_orientations(const Params& p);
// ScatteringAverageOrientationMultipoleMomentsParameters::create, parameters.cpp:1037-1122
// (file or resolution, then the validity checks).
std::vector<std::pair<long, long>> create_moments(const Params& p);

struct FunctionEntry {
    size_t type = 0;
    std::vector<double> v;
};

class Database {
public:
    std::string rawconfig;
    std::map<std::string, std::string> pdb_regex;  // label -> regex (names/pdb)
    std::map<std::string, size_t> ids;             // label -> ID (registration order)
    std::vector<std::string> labels;               // ID -> label
    std::map<size_t, double> masses;
    std::map<size_t, FunctionEntry> volumes, exclusion, sfactors;

    void read_xml(const std::string& path);
    size_t id(const std::string& label);           // registers on first use
    std::string label_for_pdb_name(const std::string& pdbname) const;

    // DatabaseSFactorsParameters::get (database.cpp:469-528), types 0 and 2
    double sfactor(size_t id, double q) const;
    // DatabaseVolumesParameters::get (database.cpp:391-411)
    double volume(size_t id) const;
    // DatabaseExlusionParameters::get (database.cpp:430-450)
    double exclusion_factor(size_t id, double effvolume, double q) const;
};

}  // namespace sassgpu
