#include "config.hpp"

#include <random>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <regex>
#include <sstream>
#include <stdexcept>

namespace sassgpu {

namespace {

std::string read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error(path + " does not exist!");
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::string dirname_of(const std::string& p) {
    size_t k = p.find_last_of('/');
    if (k == std::string::npos) return ".";
    if (k == 0) return "/";
    return p.substr(0, k);
}

Vec3 read_vec(const XmlDoc& x, const std::string& base, const XmlNode* ctx, Vec3 v) {
    if (x.exists(base + "/x", ctx)) v[0] = x.get_double(base + "/x", ctx);
    if (x.exists(base + "/y", ctx)) v[1] = x.get_double(base + "/y", ctx);
    if (x.exists(base + "/z", ctx)) v[2] = x.get_double(base + "/z", ctx);
    return v;
}

double length(const Vec3& v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

// Orientation draws of vectors.type = sphere / cylinder with algorithm
// boost_uniform_on_sphere (parameters.cpp:945-959 and :1001-1012): a boost::mt19937 seeded
// with the configured seed, copied into a variate_generator with uniform_on_sphere<double>(3)
// or (2), one call per orientation. Restated from Boost.Random's published algorithms:
// - boost::mt19937 is the standard 32-bit Mersenne Twister (std::mt19937 gives the same
//   stream for the same seed, truncated to 32 bits as mt19937::seed truncates it);
// - uniform_01<double> maps a draw x to x * 2^-32 (exact);
// - Boost 1.56 and later (BoostRandom::Marsaglia, the default): uniform_on_sphere takes
//   Marsaglia's method for two and three dimensions: x, y = 2u - 1 until x^2 + y^2 <= 1
//   (and > 0 in two dimensions); three dimensions give (2x sqrt(1-s), 2y sqrt(1-s), 2s - 1),
//   two give (x, y) / sqrt(s);
// - Boost 1.47 to 1.55 (BoostRandom::BoxMuller, gpu/boost_random = 1.47): the distribution
//   holds a normal_distribution that draws Box-Muller pairs (rho = sqrt(-2 log(1 - u2)),
//   cos(2 pi u1) first, sin(2 pi u1) kept for the next variate, across orientations) and
//   divides the normal vector by its length.
// The host build has no FP contraction, so x*x + y*y rounds as on an x86-64 build.
struct BoostSphere {
    std::mt19937 eng;
    bool legacy;
    bool valid = false;  // Box-Muller: a cached second variate exists
    double r1 = 0, cached_rho = 0;
    BoostSphere(unsigned long seed, bool legacy_box_muller)
        : eng((std::mt19937::result_type)(uint32_t)seed), legacy(legacy_box_muller) {}
    double uniform01() { return (double)eng() * (1.0 / 4294967296.0); }
    double normal() {
        if (!valid) {
            r1 = uniform01();
            const double r2 = uniform01();
            cached_rho = std::sqrt(-2.0 * std::log(1.0 - r2));
            valid = true;
        } else {
            valid = false;
        }
        const double pi = 3.14159265358979323846;
        return cached_rho * (valid ? std::cos(2.0 * pi * r1) : std::sin(2.0 * pi * r1)) * 1.0 + 0.0;
    }
    std::vector<double> draw(int dim) {
        std::vector<double> v(dim);
        if (legacy) {
            double sq = 0;
            for (int k = 0; k < dim; ++k) {
                v[k] = normal();
                sq += v[k] * v[k];
            }
            const double l = std::sqrt(sq);
            for (int k = 0; k < dim; ++k) v[k] = v[k] / l;
            return v;
        }
        double x, y, sq;
        do {
            x = uniform01() * 2 - 1;
            y = uniform01() * 2 - 1;
            sq = x * x + y * y;
        } while ((dim == 2 && sq == 0) || sq > 1);
        if (dim == 3) {
            const double mult = 2 * std::sqrt(1 - sq);
            v[0] = x * mult;
            v[1] = y * mult;
            v[2] = 2 * sq - 1;
        } else {
            const double mult = 1 / std::sqrt(sq);
            v[0] = x * mult;
            v[1] = y * mult;
        }
        return v;
    }
};

}  // namespace

std::string Params::get_filepath(const std::string& fname) const {
    // Params::get_filepath, parameters.cpp:41-53: relative paths are taken from the
    // directory of the main configuration file.
    if (!fname.empty() && fname[0] == '/') return fname;
    std::string root = config_dir.empty() ? "." : config_dir;
    return root + "/" + fname;
}

void Params::read_xml(const std::string& path) {
    config_path = path;
    config_dir = dirname_of(path);
    rawconfig = read_file(path);
    XmlDoc x = XmlDoc::parse(rawconfig);

    // ---- sample (parameters.cpp:84-230) --------------------------------------------------
    structure_filepath = get_filepath(structure_file);
    if (x.exists("//sample/structure/file")) {
        structure_file = x.get_string("//sample/structure/file");
        structure_filepath = get_filepath(structure_file);
    }
    if (x.exists("//sample/structure/format")) structure_format = x.get_string("//sample/structure/format");
    if (x.exists("//sample/selections")) {
        auto sels = x.query("//sample/selections/selection");
        for (size_t i = 0; i < sels.size(); ++i) {
            const XmlNode* s = sels[i];
            SelectionParams sp;
            sp.name = "_" + std::to_string(i);
            if (x.exists("./type", s)) sp.type = x.get_string("./type", s);
            if (x.exists("./name", s)) sp.name = x.get_string("./name", s);
            if (sp.type == "index") {
                for (const XmlNode* n : x.query("./index", s)) sp.ids.push_back(x.get_size(".", n));
            } else if (sp.type == "range") {
                if (x.exists("./from", s)) sp.from = x.get_size("./from", s);
                if (x.exists("./to", s)) sp.to = x.get_size("./to", s);
            } else if (sp.type == "lexical") {
                if (x.exists("./expression", s)) sp.expression = x.get_string("./expression", s);
            } else if (sp.type == "file") {
                // defaults as the reference sets them; for ndx it switches selector and expression
                // (its default file name stays selection.pdb: the ndx branch assigns another variable)
                sp.file = "selection.pdb";
                sp.format = "pdb";
                sp.selector = "beta";
                sp.expression = "1|1\\.0|1\\.00";
                if (x.exists("./format", s)) sp.format = x.get_string("./format", s);
                if (sp.format == "ndx") {
                    sp.selector = "name";
                    sp.expression = ".*";
                }
                if (x.exists("./file", s)) sp.file = x.get_string("./file", s);
                sp.filepath = get_filepath(sp.file);
                if (x.exists("./selector", s)) sp.selector = x.get_string("./selector", s);
                if (x.exists("./expression", s)) sp.expression = x.get_string("./expression", s);
            } else {
                throw std::runtime_error("Selection type not supported by this build: " + sp.type);
            }
            selections.push_back(sp);
        }
    }
    if (x.exists("//sample/framesets")) {
        FramesetParams def;
        def.file = "sample.dcd";
        if (x.exists("//sample/framesets/first")) def.first = x.get_size("//sample/framesets/first");
        if (x.exists("//sample/framesets/last")) {
            def.last = x.get_size("//sample/framesets/last");
            def.last_set = true;
        }
        if (x.exists("//sample/framesets/stride")) def.stride = x.get_size("//sample/framesets/stride");
        if (x.exists("//sample/framesets/clones")) def.clones = x.get_size("//sample/framesets/clones");
        for (const XmlNode* f : x.query("//sample/framesets/frameset")) {
            FramesetParams fs = def;
            if (x.exists("./file", f)) fs.file = x.get_string("./file", f);
            fs.filepath = get_filepath(fs.file);
            if (x.exists("./format", f)) fs.format = x.get_string("./format", f);
            if (x.exists("./first", f)) fs.first = x.get_size("./first", f);
            if (x.exists("./last", f)) {
                fs.last = x.get_size("./last", f);
                fs.last_set = true;
            }
            if (x.exists("./stride", f)) fs.stride = x.get_size("./stride", f);
            if (x.exists("./clones", f)) fs.clones = x.get_size("./clones", f);
            if (fs.stride == 0) throw std::runtime_error("frameset stride must be > 0");
            framesets.push_back(fs);
        }
    }
    for (const XmlNode* e : x.query("//sample/motions/motion")) {
        MotionParams m;
        m.ref_file = structure_file;
        m.ref_filepath = structure_filepath;
        m.ref_format = structure_format;
        if (x.exists("./type", e)) m.type = x.get_string("./type", e);
        if (x.exists("./displace", e)) m.displace = x.get_double("./displace", e);
        if (x.exists("./frequency", e)) m.frequency = x.get_double("./frequency", e);
        if (x.exists("./seed", e)) m.seed = (unsigned long)x.get_size("./seed", e);
        if (x.exists("./sampling", e)) m.sampling = (long)x.get_long("./sampling", e);
        if (x.exists("./selection", e)) m.selection = x.get_string("./selection", e);
        if (x.exists("./direction/x", e)) m.direction[0] = x.get_double("./direction/x", e);
        if (x.exists("./direction/y", e)) m.direction[1] = x.get_double("./direction/y", e);
        if (x.exists("./direction/z", e)) m.direction[2] = x.get_double("./direction/z", e);
        m.radius = m.displace * 10;
        if (x.exists("./radius", e)) m.radius = x.get_double("./radius", e);
        m.ref_selection = m.selection;
        if (x.exists("./reference/type", e)) m.ref_type = x.get_string("./reference/type", e);
        if (x.exists("./reference/frame", e)) m.ref_frame = x.get_size("./reference/frame", e);
        if (x.exists("./reference/file", e)) {
            m.ref_file = x.get_string("./reference/file", e);
            m.ref_filepath = get_filepath(m.ref_file);
        }
        if (x.exists("./reference/format", e)) m.ref_format = x.get_string("./reference/format", e);
        if (x.exists("./reference/selection", e)) m.ref_selection = x.get_string("./reference/selection", e);
        motions.push_back(m);
    }
    for (const XmlNode* e : x.query("//sample/alignments/alignment")) {
        AlignmentParams a;
        if (x.exists("./type", e)) a.type = x.get_string("./type", e);
        if (x.exists("./selection", e)) a.selection = x.get_string("./selection", e);
        if (x.exists("./order", e)) a.order = x.get_string("./order", e);
        a.ref_file = structure_file;
        a.ref_filepath = structure_filepath;
        a.ref_format = structure_format;
        a.ref_selection = a.selection;
        if (x.exists("./reference/type", e)) a.ref_type = x.get_string("./reference/type", e);
        if (x.exists("./reference/frame", e)) a.ref_frame = x.get_size("./reference/frame", e);
        if (x.exists("./reference/file", e)) {
            a.ref_file = x.get_string("./reference/file", e);
            a.ref_filepath = get_filepath(a.ref_file);
        }
        if (x.exists("./reference/format", e)) a.ref_format = x.get_string("./reference/format", e);
        if (x.exists("./reference/selection", e)) a.ref_selection = x.get_string("./reference/selection", e);
        if (a.order != "pre" && a.order != "post")
            throw std::runtime_error("Ordering of alignment not understood. Must be pre or post.");
        alignments.push_back(a);
    }

    // ---- stager (parameters.cpp:340-369) ---------------------------------------------------
    if (x.exists("//stager/target")) target = x.get_string("//stager/target");
    stager_filepath = get_filepath(stager_file);
    if (x.exists("//stager/dump")) stager_dump = x.get_bool("//stager/dump");
    if (x.exists("//stager/file")) {
        stager_file = x.get_string("//stager/file");
        stager_filepath = get_filepath(stager_file);
    }
    if (x.exists("//stager/format")) stager_format = x.get_string("//stager/format");
    if (x.exists("//stager/mode")) stager_mode = x.get_string("//stager/mode");
    if (stager_mode != "frames" && stager_mode != "atoms")  // both map to the device's own layout
        throw std::runtime_error("stager.mode not understood: " + stager_mode);

    // ---- scattering (parameters.cpp:372-607) -------------------------------------------------
    if (x.exists("//scattering")) {
        if (x.exists("//scattering/type")) scattering_type = x.get_string("//scattering/type");
        if (x.exists("//scattering/target"))
            throw std::runtime_error("scattering.target is obsolete. Use stager.target instead.");
        if (x.exists("//scattering/background/factor"))
            background_factor = x.get_double("//scattering/background/factor");
        for (const XmlNode* k : x.query("//scattering/background/kappas/kappa")) {
            std::string sel = "system";
            double val = 1.0;
            if (x.exists("./selection", k)) sel = x.get_string("./selection", k);
            if (x.exists("./value", k)) val = x.get_double("./value", k);
            kappas.emplace_back(sel, val);
        }
        if (x.exists("//scattering/vectors")) {
            std::string vt = "single";
            if (x.exists("//scattering/vectors/type")) vt = x.get_string("//scattering/vectors/type");
            if (vt == "single") {
                Vec3 q{1.0, 0.0, 0.0};
                if (x.exists("//scattering/vectors/single/x")) q = read_vec(x, "//scattering/vectors/single", nullptr, Vec3{1.0, 0.0, 0.0});
                qvectors.push_back(q);
            } else if (vt == "scans") {
                for (const XmlNode* s : x.query("//scattering/vectors/scans/scan")) {
                    ScanParams sc;
                    if (x.exists("./base", s)) sc.base = read_vec(x, "./base", s, sc.base);
                    if (x.exists("./from", s)) sc.from = x.get_double("./from", s);
                    if (x.exists("./to", s)) sc.to = x.get_double("./to", s);
                    if (x.exists("./points", s)) sc.points = x.get_size("./points", s);
                    if (x.exists("./exponent", s)) sc.exponent = x.get_double("./exponent", s);
                    scans.push_back(sc);
                }
                qvectors = create_from_scans(scans);
            } else if (vt == "file") {
                std::string fn = "qvectors.txt";
                if (x.exists("//scattering/vectors/file")) fn = get_filepath(x.get_string("//scattering/vectors/file"));
                std::ifstream qf(fn);
                double a, b, c;
                while (qf >> a >> b >> c) qvectors.push_back(Vec3{a, b, c});
            } else {
                throw std::runtime_error("scattering.vectors.type not understood: " + vt);
            }
        }
        if (qvectors.empty())
            throw std::runtime_error("No q vectors generated. Check the scattering.vectors section for errors.");
        if (x.exists("//scattering/dsp/type")) dsp_type = x.get_string("//scattering/dsp/type");
        if (x.exists("//scattering/dsp/method")) dsp_method = x.get_string("//scattering/dsp/method");
        if (x.exists("//scattering/average/orientation/axis"))
            axis = Vec3{x.get_double("//scattering/average/orientation/axis/x"),
                        x.get_double("//scattering/average/orientation/axis/y"),
                        x.get_double("//scattering/average/orientation/axis/z")};
        if (x.exists("//scattering/average/orientation/type"))
            orientation_type = x.get_string("//scattering/average/orientation/type");
        if (orientation_type == "vectors") {
            const std::string b = "//scattering/average/orientation/vectors/";
            if (x.exists(b + "type")) vectors_type = x.get_string(b + "type");
            if (x.exists(b + "algorithm")) vectors_algorithm = x.get_string(b + "algorithm");
            if (x.exists(b + "resolution")) resolution = (long)x.get_long(b + "resolution");
            if (x.exists(b + "seed")) seed = (unsigned long)x.get_long(b + "seed");
            if (x.exists(b + "file")) vectors_file = x.get_string(b + "file");
            vectors_filepath = get_filepath(vectors_file);
            // the Boost.Random release whose draws are reproduced (an option of this build)
            if (x.exists("//gpu/boost_random")) boost_random = x.get_string("//gpu/boost_random");
            if (boost_random != "1.56" && boost_random != "1.47")
                throw std::runtime_error("gpu.boost_random must be 1.56 (Boost 1.56 and later) or 1.47 (1.47 to "
                                         "1.55): " + boost_random);
            orientations = create_orientations(*this);
        } else if (orientation_type == "multipole") {
            const std::string b = "//scattering/average/orientation/multipole/";
            if (x.exists(b + "type")) multipole_type = x.get_string(b + "type");
            if (x.exists(b + "moments/type")) moments_type = x.get_string(b + "moments/type");
            if (x.exists(b + "moments/resolution")) moments_resolution = (long)x.get_long(b + "moments/resolution");
            if (x.exists(b + "moments/file")) moments_file = x.get_string(b + "moments/file");
            moments_filepath = get_filepath(moments_file);
            moments = create_moments(*this);
        } else if (orientation_type != "none") {
            throw std::runtime_error("Orientation averaging type not understood: " + orientation_type);
        }
        if (x.exists("//scattering/signal/file")) signal_file = x.get_string("//scattering/signal/file");
        if (x.exists("//scattering/signal/fqt")) signal_fqt = x.get_bool("//scattering/signal/fqt");
        if (x.exists("//scattering/signal/fq0")) signal_fq0 = x.get_bool("//scattering/signal/fq0");
        if (x.exists("//scattering/signal/fq")) signal_fq = x.get_bool("//scattering/signal/fq");
        if (x.exists("//scattering/signal/fq2")) signal_fq2 = x.get_bool("//scattering/signal/fq2");
    } else {
        throw std::runtime_error("No q vectors generated. Check the scattering.vectors section for errors.");
    }
    signal_filepath = get_filepath(signal_file);
    if (scattering_type != "all" && scattering_type != "self")
        throw std::runtime_error("scattering.type not understood: " + scattering_type);
    if (dsp_type != "autocorrelate" && dsp_type != "square" && dsp_type != "plain")
        throw std::runtime_error("DSP type not understood: " + dsp_type);
    if (dsp_method != "fftw" && dsp_method != "direct")
        throw std::runtime_error("Correlation method not understood: " + dsp_method);

    // ---- limits (parameters.cpp:611-736) -------------------------------------------------------
    if (x.exists("//limits/signal/chunksize")) chunksize = x.get_size("//limits/signal/chunksize");
    if (x.exists("//limits/computation/threads")) threads = x.get_size("//limits/computation/threads");
    if (x.exists("//limits/services/signal/times/serverflush"))
        serverflush_s = x.get_size("//limits/services/signal/times/serverflush");

    // ---- database (parameters.cpp:776-792) -------------------------------------------------
    db_filepath = get_filepath(db_file);
    if (x.exists("//database/file")) {
        db_file = x.get_string("//database/file");
        db_filepath = get_filepath(db_file);
    }

    // ---- gpu (this build) ---------------------------------------------------------------------
    if (x.exists("//gpu/precision")) precision = x.get_string("//gpu/precision");
    if (x.exists("//gpu/device")) device = (int)x.get_long("//gpu/device");
    if (x.exists("//gpu/batch")) batch_q = x.get_size("//gpu/batch");
    if (x.exists("//gpu/memory")) amplitude_budget = x.get_size("//gpu/memory");
    if (precision != "fp64" && precision != "fp32")
        throw std::runtime_error("gpu.precision must be fp64 or fp32: " + precision);
}

void Params::overwrite(const std::string& key, const std::string& value) {
    if (key == "sample.structure.file") {
        structure_file = value;
        structure_filepath = get_filepath(value);
    } else if (key == "sample.structure.format") {
        structure_format = value;
    } else if (key == "stager.target") {
        target = value;
    } else if (key == "stager.dump") {
        stager_dump = value == "true" || value == "1" || value == "yes";
    } else if (key == "stager.file") {
        stager_file = value;
        stager_filepath = get_filepath(value);
    } else if (key == "stager.format") {
        stager_format = value;
    } else if (key == "scattering.signal.file") {
        signal_file = value;
        signal_filepath = get_filepath(value);
    } else if (key == "limits.computation.threads") {
        threads = std::stoul(value);
    } else if (key == "database.file") {
        db_file = value;
        db_filepath = get_filepath(value);
    } else if (key == "gpu.precision") {
        if (value != "fp64" && value != "fp32") throw std::runtime_error("gpu.precision must be fp64 or fp32");
        precision = value;
    } else if (key == "gpu.device") {
        device = std::stoi(value);
    } else {
        throw std::runtime_error("unknown option --" + key);
    }
}

std::vector<Vec3> create_from_scans(const std::vector<ScanParams>& scans) {
    if (scans.size() > 3) throw std::runtime_error("More than 3 scan definitions are not supported.");
    std::vector<std::vector<Vec3>> q(scans.size());
    auto mul = [](double s, const Vec3& b) { return Vec3{s * b[0], s * b[1], s * b[2]}; };
    for (size_t i = 0; i < scans.size(); ++i) {
        const ScanParams& sc = scans[i];
        if (sc.points == 0) continue;
        if (sc.points == 1) {
            q[i].push_back(mul((sc.from + sc.to) / 2, sc.base));
            continue;
        }
        if (sc.points == 2) {
            q[i].push_back(mul(sc.from, sc.base));
            q[i].push_back(mul(sc.to, sc.base));
            continue;
        }
        q[i].push_back(mul(sc.from, sc.base));
        for (size_t j = 1; j < sc.points - 1; ++j) {
            // the reference evaluates the exponent with single-precision powf
            double scal = sc.from + powf((float)(j * 1.0 / (sc.points - 1)), (float)sc.exponent) * (sc.to - sc.from);
            q[i].push_back(mul(scal, sc.base));
        }
        q[i].push_back(mul(sc.to, sc.base));
    }
    std::vector<Vec3> out;
    auto add = [](const Vec3& a, const Vec3& b) { return Vec3{a[0] + b[0], a[1] + b[1], a[2] + b[2]}; };
    if (scans.size() == 1) return q[0];
    if (scans.size() == 2)
        for (auto& a : q[0])
            for (auto& b : q[1]) out.push_back(add(a, b));
    if (scans.size() == 3)
        for (auto& a : q[0])
            for (auto& b : q[1])
                for (auto& c : q[2]) out.push_back(add(add(a, b), c));
    return out;
}

std::vector<std::pair<long, long>> create_moments(const Params& p) {
    std::vector<std::pair<long, long>> m;
    if (p.moments_type == "file") {
        std::ifstream f(p.moments_filepath);
        if (!f) throw std::runtime_error("cannot open multipole moments file " + p.moments_filepath);
        long major, minor;
        while (f >> major >> minor) m.emplace_back(major, minor);
    } else if (p.moments_type == "resolution") {
        if (p.multipole_type == "sphere") {
            m.emplace_back(0, 0);
            for (long l = 1; l <= p.moments_resolution; ++l)
                for (long k = -l; k <= l; ++k) m.emplace_back(l, k);
        } else if (p.multipole_type == "cylinder") {
            m.emplace_back(0, 0);
            for (long l = 1; l <= p.moments_resolution; ++l)
                for (long k = 0; k < 4; ++k) m.emplace_back(l, k);
        } else {
            throw std::runtime_error("Type not understood: scattering.average.orientation.multipole.moments.type=" +
                                     p.moments_type);
        }
    } else {
        throw std::runtime_error("Type not understood: scattering.average.orientation.multipole.type=" +
                                 p.multipole_type);
    }
    for (const auto& mm : m) {
        if (mm.first < 0) throw std::runtime_error("Major multipole moment must be >= 0!");
        if (p.multipole_type == "cylinder") {
            if (mm.second < 0 || mm.second > 3) throw std::runtime_error("Minor multipole moment must be between 0 and 3!");
            if (mm.first == 0 && mm.second != 0) throw std::runtime_error("Minor multipole moment must be 0 for Major 0!");
        } else if (p.multipole_type == "sphere") {
            if (std::labs(mm.second) > mm.first)
                throw std::runtime_error("Minor multipole moment must be between -Major and +Major!");
        }
    }
    return m;
}

std::vector<Vec3> create_orientations(const Params& p) {
    std::vector<Vec3> out;
    if (p.vectors_type == "file") {
        std::ifstream f(p.vectors_filepath);
        if (!f) throw std::runtime_error("cannot open orientation file " + p.vectors_filepath);
        double x, y, z;
        while (f >> x >> y >> z) {
            Vec3 q{x, y, z};
            double l = length(q);
            if (l != 0) q = Vec3{(1.0 / l) * x, (1.0 / l) * y, (1.0 / l) * z};
            out.push_back(q);
        }
    } else if (p.vectors_type == "sphere") {
        if (p.vectors_algorithm != "boost_uniform_on_sphere")
            throw std::runtime_error("Vectors algorithm not understood: " + p.vectors_algorithm);
        BoostSphere sphere(p.seed, p.boost_random == "1.47");
        for (long i = 0; i < p.resolution; ++i) {
            std::vector<double> r = sphere.draw(3);
            out.push_back(Vec3{r[0], r[1], r[2]});
        }
    } else if (p.vectors_type == "cylinder") {
        if (p.vectors_algorithm == "boost_uniform_on_sphere") {
            BoostSphere circle(p.seed, p.boost_random == "1.47");
            for (long i = 0; i < p.resolution; ++i) {
                std::vector<double> r = circle.draw(2);
                out.push_back(Vec3{r[0], r[1], 0.0});
            }
        } else if (p.vectors_algorithm == "raster_linear") {
            const double two_pi = 2 * M_PI;
            const double incr = two_pi / (360 * p.resolution);
            for (double phi = 0; phi < two_pi; phi += incr) out.push_back(Vec3{std::cos(phi), std::sin(phi), 0});
        } else {
            throw std::runtime_error("Vectors algorithm not understood: " + p.vectors_algorithm);
        }
    } else {
        throw std::runtime_error("Vectors orientation averaging type not understood: " + p.vectors_type);
    }
    return out;
}

// ---------------------------------------------------------------------------------------------
// Database (database.cpp:31-145 read_xml, :293-528 lookups)
// ---------------------------------------------------------------------------------------------
size_t Database::id(const std::string& label) {
    auto it = ids.find(label);
    if (it != ids.end()) return it->second;
    size_t n = labels.size();
    ids[label] = n;
    labels.push_back(label);
    return n;
}

void Database::read_xml(const std::string& path) {
    rawconfig = read_file(path);
    XmlDoc x = XmlDoc::parse(rawconfig);
    for (const XmlNode* e : x.query("//names/pdb/element"))
        pdb_regex[x.get_string("./name", e)] = x.get_string("./param", e);
    for (const XmlNode* e : x.query("//masses/element"))
        masses[id(x.get_string("./name", e))] = x.get_double("./param", e);
    auto functions = [&](const std::string& path, std::map<size_t, FunctionEntry>& dst) {
        for (const XmlNode* e : x.query(path)) {
            FunctionEntry f;
            f.type = x.get_size("./type", e);
            for (const XmlNode* p : x.query("./param", e)) f.v.push_back(x.get_double(".", p));
            dst[id(x.get_string("./name", e))] = f;
        }
    };
    functions("//sizes/element", volumes);
    functions("//exclusionfactors/element", exclusion);
    if (!x.exists("//scatterfactors")) throw std::runtime_error("Need scattering factors.");
    functions("//scatterfactors/element", sfactors);
}

std::string Database::label_for_pdb_name(const std::string& pdbname) const {
    // DatabaseNamesPDBParameters::get (database.cpp:308-340): exactly one label's
    // regular expression must match the whole name.
    std::string label;
    int matches = 0;
    for (const auto& kv : pdb_regex) {
        if (std::regex_match(pdbname, std::regex(kv.second))) {
            if (matches > 0)
                throw std::runtime_error("PDB atom name matches " + label + " and " + kv.first + ": " + pdbname);
            label = kv.first;
            ++matches;
        }
    }
    if (matches == 0) throw std::runtime_error("PDB atom name not recognized: " + pdbname);
    return label;
}

double Database::sfactor(size_t id, double q) const {
    auto it = sfactors.find(id);
    if (it == sfactors.end())
        throw std::runtime_error("Atom with label '" + labels.at(id) + "' is missing a scattering factor entry");
    const std::vector<double>& v = it->second.v;
    if (it->second.type == 0) {
        if (v.empty()) throw std::runtime_error("scattering factor type 0 needs one parameter");
        return v[0];
    }
    if (it->second.type == 2) {
        if (v.size() < 9) throw std::runtime_error("scattering factor type 2 needs nine parameters");
        double den = 0.0;
        den += v[0] * std::exp(-v[1] * q * q);
        den += v[2] * std::exp(-v[3] * q * q);
        den += v[4] * std::exp(-v[5] * q * q);
        den += v[6] * std::exp(-v[7] * q * q);
        den += v[8];
        return den;
    }
    throw std::runtime_error("ScatterFactor-type not implemented by this build: type=" +
                             std::to_string(it->second.type));
}

double Database::volume(size_t id) const {
    auto it = volumes.find(id);
    if (it == volumes.end() || it->second.v.empty())
        throw std::runtime_error("Atom with label '" + labels.at(id) + "' is missing a volume entry");
    const std::vector<double>& v = it->second.v;
    switch (it->second.type) {
        case 0: return v[0];
        case 1: return (4.0 / 3.0) * M_PI * powf((float)v[0], 3);
        case 2: return (double)(std::sqrt(powf((float)M_PI, 3)) * powf((float)v[0], 3));  // float, as the reference
    }
    throw std::runtime_error("Size-type not implemented: type=" + std::to_string(it->second.type));
}

double Database::exclusion_factor(size_t id, double effvolume, double q) const {
    auto it = exclusion.find(id);
    if (it == exclusion.end() || it->second.v.empty())
        throw std::runtime_error("Atom with label '" + labels.at(id) + "' is missing an exclusion factor entry");
    const std::vector<double>& v = it->second.v;
    switch (it->second.type) {
        case 0: return v[0];
        case 1: return effvolume * v[0];
        case 2:
            return effvolume * std::exp(-1.0 * powf((float)effvolume, 2.0f / 3.0f) * powf((float)q, 2) / (4 * M_PI)) * v[0];
    }
    throw std::runtime_error("ExclusionParameter-type not implemented: type=" + std::to_string(it->second.type));
}

}  // namespace sassgpu
