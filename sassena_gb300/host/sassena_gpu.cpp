// sassena-gpu: command-line driver of the GB300 scattering path.
//
// Same entry sequence as the reference's `sassena` (src/main/sassena.cpp:132-417) for
// one process: read the configuration (--config, default scatter.xml) and the
// database, initialise the sample, skip q-vectors already in the signal file, run the
// scatter device, write signal.h5. Command-line overrides use the reference's keys
// (parameters.cpp:795-882): --sample.structure.file=..., --stager.target=...,
// --scattering.signal.file=..., --limits.computation.threads=..., plus --gpu.precision
// and --gpu.device.
//
//   --dry-run FILE   parse and stage only (no GPU): write the parsed q-vectors,
//                    sub-vectors of the first q, classes, class factors and frame count
//                    as JSON to FILE (used by the CPU tests).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>

#include "config.hpp"
#include "devices.hpp"
#include "prepass.hpp"
#include "sample.hpp"

using namespace sassgpu;

namespace {

void json_vecs(std::ofstream& o, const std::vector<Vec3>& v) {
    o << "[";
    for (size_t i = 0; i < v.size(); ++i) {
        char b[128];
        snprintf(b, sizeof(b), "%s[%.17g,%.17g,%.17g]", i ? "," : "", v[i][0], v[i][1], v[i][2]);
        o << b;
    }
    o << "]";
}

void dry_run(const Params& p, Database& db, const Sample& s, const std::string& path) {
    ScatterClasses c = build_classes(p, db, s);
    std::ofstream o(path);
    o << "{\"nf\":" << s.nframes << ",\"na\":" << s.selection(p.target).size();
    o << ",\"qvectors\":";
    json_vecs(o, p.qvectors);
    o << ",\"orientations\":";
    json_vecs(o, p.orientations);
    o << ",\"subvectors_q0\":";
    json_vecs(o, p.orientation_type == "multipole" ? std::vector<Vec3>() : subvectors_for(p, p.qvectors.at(0)));
    o << ",\"atom_class\":[";
    for (size_t i = 0; i < c.atom_class.size(); ++i) o << (i ? "," : "") << c.atom_class[i];
    o << "],\"class_labels\":[";
    for (size_t i = 0; i < c.id.size(); ++i) o << (i ? "," : "") << "\"" << db.labels[c.id[i]] << "\"";
    o << "],\"class_factors\":[";
    for (size_t i = 0; i < p.qvectors.size(); ++i) {
        const Vec3& q = p.qvectors[i];
        std::vector<double> f = c.factors(db, p.background_factor, std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]));
        o << (i ? "," : "") << "[";
        for (size_t k = 0; k < f.size(); ++k) {
            char b[64];
            snprintf(b, sizeof(b), "%s%.17g", k ? "," : "", f[k]);
            o << b;
        }
        o << "]";
    }
    std::vector<float> coords = s.stage(p.target);
    // without alignments or motions the staged frames are the host's: the dry run dumps them
    if (p.stager_dump && p.alignments.empty() && p.motions.empty())
        write_dcd(p.stager_filepath, coords.data(), s.nframes, s.selection(p.target).size());
    double sum = 0;
    for (float v : coords) sum += v;
    char b[64];
    snprintf(b, sizeof(b), "%.17g", sum);
    o << "],\"coord_sum\":" << b;
    o << ",\"orientation\":\"" << p.orientation_type << "\",\"multipole\":\"" << p.multipole_type
      << "\",\"moments\":[";
    for (size_t i = 0; i < p.moments.size(); ++i)
        o << (i ? "," : "") << "[" << p.moments[i].first << "," << p.moments[i].second << "]";
    o << "]";
    // staging pre-pass steps (alignments, motions) as the device receives them
    o << ",\"prepass\":[";
    if (!p.alignments.empty() || !p.motions.empty()) {
        std::vector<float> sys = s.stage("system");
        Prepass pp = build_prepass(p, db, s, sys.data());
        auto ints = [&](const char* key, const std::vector<size_t>& v) {
            o << ",\"" << key << "\":[";
            for (size_t i = 0; i < v.size(); ++i) o << (i ? "," : "") << v[i];
            o << "]";
        };
        auto dbls = [&](const char* key, const std::vector<double>& v) {
            o << ",\"" << key << "\":[";
            for (size_t i = 0; i < v.size(); ++i) {
                char b[64];
                snprintf(b, sizeof(b), "%s%.17g", i ? "," : "", v[i]);
                o << b;
            }
            o << "]";
        };
        for (size_t i = 0; i < pp.steps.size(); ++i) {
            const PrepassStep& q = pp.steps[i];
            o << (i ? "," : "") << "{\"type\":" << q.type << ",\"label\":\"" << q.label << "\"";
            ints("selection", q.selection);
            ints("reference_selection", q.reference_selection);
            dbls("reference", q.reference);
            ints("fit_target", q.fit_target);
            ints("fit_source", q.fit_source);
            dbls("translations", q.translations);
            o << "}";
        }
        o << "],\"masses\":[";
        for (size_t i = 0; i < pp.masses.size(); ++i) {
            char b[64];
            snprintf(b, sizeof(b), "%s%.17g", i ? "," : "", pp.masses[i]);
            o << b;
        }
    }
    o << "]";
    o << ",\"scattering\":\"" << p.scattering_type << "\",\"dsp\":\"" << p.dsp_type << "\",\"method\":\""
      << p.dsp_method << "\",\"precision\":\"" << p.precision << "\",\"signal\":\"" << p.signal_filepath
      << "\"}\n";
}

}  // namespace

int main(int argc, char** argv) {
    std::string config = "scatter.xml", dry;
    std::vector<std::pair<std::string, std::string>> overrides;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "--help" || a == "-h") {
            printf("usage: sassena-gpu [--config scatter.xml] [--key=value ...] [--dry-run out.json]\n");
            return 0;
        }
        if (a.rfind("--", 0) != 0) {
            fprintf(stderr, "ERROR>> unexpected argument %s\n", a.c_str());
            return 2;
        }
        std::string key = a.substr(2), val;
        size_t eq = key.find('=');
        if (eq != std::string::npos) {
            val = key.substr(eq + 1);
            key = key.substr(0, eq);
        } else if (i + 1 < argc) {
            val = argv[++i];
        } else {
            fprintf(stderr, "ERROR>> option --%s needs a value\n", key.c_str());
            return 2;
        }
        if (key == "config") config = val;
        else if (key == "dry-run") dry = val;
        else overrides.emplace_back(key, val);
    }
    try {
        Params p;
        p.read_xml(config);
        for (auto& kv : overrides) p.overwrite(kv.first, kv.second);
        Database db;
        db.read_xml(p.db_filepath);
        Sample s;
        s.init(p, db);
        if (!dry.empty()) {
            dry_run(p, db, s, dry);
            return 0;
        }
        RunStats st;
        run_scatter_device(p, db, s, st);
        return 0;
    } catch (const std::exception& e) {
        fprintf(stderr, "ERROR>> %s\n", e.what());
        return 1;
    }
}
