#include "prepass.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <stdexcept>

#include "sassena_gb300.h"

namespace sassgpu {

namespace {

void warn(const std::string& m) { fprintf(stderr, "WARNING>> %s\n", m.c_str()); }

std::vector<size_t> system_list(size_t n) {
    std::vector<size_t> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = i;
    return v;
}

// values of csel reached by the walk (the atoms a translate or a centre of mass touches)
std::vector<size_t> walked(const std::vector<size_t>& csel, const std::vector<size_t>& ssel) {
    std::vector<size_t> out;
    for (const auto& pr : merge_walk(csel, ssel)) out.push_back(csel[pr.first]);
    return out;
}

// The reference structure of an alignment or motion (CoordinateSets::init,
// coordinate_sets.cpp:80-112 and 168-199): coordinates of `sel` in a raw trajectory frame
// or a PDB frame, or empty for "instant".
std::vector<double> reference_coords(const std::string& type, size_t frame, const std::string& filepath,
                                     const std::string& format, const std::vector<size_t>& sel, const float* frames,
                                     size_t nf, size_t nsys) {
    std::vector<double> out;
    if (type == "frame") {
        if (frame >= nf) {
            warn("reference frame number in alignment larger than size of frameset. Setting to last frame!");
            frame = nf - 1;
        }
        const float* fr = frames + frame * nsys * 3;
        for (size_t a : sel)
            for (int k = 0; k < 3; ++k) out.push_back((double)fr[3 * a + k]);
    } else if (type == "file") {
        if (format != "pdb") throw std::runtime_error("File format for alignment reference not understood, format=" + format);
        std::vector<double> xyz = read_pdb_frame(filepath, frame);
        const size_t n = xyz.size() / 3;
        if (sel.size() > n)  // CartesianCoordinateSet(Frame&, selection), coordinate_set.cpp:81-84
            throw std::runtime_error("Atom Index out of bounds for frame! Does the structure file match the frames?");
        for (size_t a : sel) {
            if (a >= n) throw std::runtime_error("reference selection refers to atom " + std::to_string(a) + " beyond " + filepath);
            for (int k = 0; k < 3; ++k) out.push_back(xyz[3 * a + k]);
        }
    } else if (type != "instant") {
        throw std::runtime_error("Reference type not understood:" + type);
    }
    return out;
}

double length(const Vec3& v) { return std::sqrt(std::pow(v[0], 2) + std::pow(v[1], 2) + std::pow(v[2], 2)); }

// translation(timepos) of the deterministic walkers, motion_walker.cpp:340-400
std::vector<double> motion_translations(const MotionParams& m, size_t nf) {
    std::vector<double> t(nf * 3);
    const double len = length(m.direction);
    Vec3 tr;
    if (m.type == "linear") {
        const double s = m.displace * (double)m.sampling;
        for (int k = 0; k < 3; ++k) tr[k] = (s * m.direction[k]) / len;
        for (size_t f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k) t[3 * f + k] = (double)f * tr[k];
    } else if (m.type == "fixed") {
        for (int k = 0; k < 3; ++k) tr[k] = (m.displace * m.direction[k]) / len;
        for (size_t f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k) t[3 * f + k] = tr[k];
    } else {  // oscillation
        for (int k = 0; k < 3; ++k) tr[k] = (m.displace * m.direction[k]) / len;
        for (size_t f = 0; f < nf; ++f) {
            const double w = std::sin(2 * M_PI * (double)f * m.frequency * (double)m.sampling);
            for (int k = 0; k < 3; ++k) t[3 * f + k] = w * tr[k];
        }
    }
    return t;
}

PrepassStep alignment_step(const AlignmentParams& a, const Sample& s, const float* frames) {
    const size_t nsys = s.atom_ids.size(), nf = s.nframes;
    const std::vector<size_t> system = system_list(nsys);
    const std::vector<size_t>& sel = s.selection(a.selection);
    const std::vector<size_t>& rsel = s.selection(a.ref_selection);
    std::vector<double> ref = reference_coords(a.ref_type, a.ref_frame, a.ref_filepath, a.ref_format, rsel, frames, nf, nsys);
    const bool instant = a.ref_type == "instant";
    PrepassStep st;
    st.label = a.order + " " + a.type;
    if (a.type == "center") {
        // CenterOfMass(cset, system, reference selection); translate(selection)
        st.type = SASS_STEP_CENTER;
        st.selection = walked(system, sel);
        st.reference_selection = walked(system, rsel);
    } else if (a.type == "fittrans") {
        st.type = SASS_STEP_FITTRANS;
        st.selection = walked(system, sel);
        st.reference_selection = instant ? system : rsel;
        st.reference = ref;
    } else if (a.type == "fitrottrans" || a.type == "fitrot") {
        st.type = a.type == "fitrot" ? SASS_STEP_FITROT : SASS_STEP_FITROTTRANS;
        const std::vector<size_t>& fsel = instant ? system : rsel;
        // the fit's reduced copy must hold every reference atom (center_of_mass.cpp:69-73)
        if (merge_walk(system, fsel).size() != fsel.size())
            throw std::runtime_error("Fitting requires the reference and the target to contain the same number of atoms");
        st.reference_selection = fsel;
        st.reference = ref;
        // write-back walk (center_of_mass.cpp:130-156): atom a takes the copy's entry at
        // index a (the reference indexes the reduced copy by the atom's system index)
        for (const auto& pr : merge_walk(sel, fsel)) {
            const size_t atom = sel[pr.first], src = fsel[pr.second];
            if (src >= fsel.size())
                throw std::runtime_error("fit alignment of selection '" + a.selection + "' on '" + a.ref_selection +
                                         "': the reference would read its reduced copy at index " + std::to_string(src) +
                                         " of " + std::to_string(fsel.size()) + " (undefined); not supported");
            st.fit_target.push_back(atom);
            st.fit_source.push_back(src);
        }
        if (st.type == SASS_STEP_FITROT) st.selection = walked(system, sel);
    } else {
        throw std::runtime_error("Fitting routine not understood: " + a.type +
                                 " (use either of: center , fittrans , fitrottrans, fitrot)");
    }
    return st;
}

}  // namespace

std::vector<std::pair<size_t, size_t>> merge_walk(const std::vector<size_t>& csel, const std::vector<size_t>& ssel) {
    std::vector<std::pair<size_t, size_t>> out;
    size_t i = 0, k = 0;
    while (i < csel.size() && k < ssel.size()) {
        if (csel[i] == ssel[k]) {
            out.emplace_back(i, k);
            ++i;
            ++k;
        } else if (csel[i] > ssel[k]) {
            ++k;
        } else {
            ++i;
        }
    }
    return out;
}

std::vector<double> read_pdb_frame(const std::string& path, size_t frame) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Couldn't open reference file: " + path);
    // generate_index: a frame ends at every line starting with "END"; an unterminated tail
    // is one more frame
    std::vector<std::vector<double>> frames(1);
    std::string line;
    bool last_end = false;
    while (std::getline(in, line)) {
        if (line.compare(0, 3, "END") == 0) {
            frames.emplace_back();
            last_end = true;
            continue;
        }
        last_end = false;
        if (line.compare(0, 6, "ATOM  ") == 0) {
            auto field = [&](size_t pos) { return std::atof(line.size() > pos ? line.substr(pos, 8).c_str() : ""); };
            frames.back().push_back(field(30));
            frames.back().push_back(field(38));
            frames.back().push_back(field(46));
        }
    }
    if (last_end) frames.pop_back();  // no tail after the last END
    if (frames.empty()) frames.emplace_back();
    if (frame >= frames.size()) {
        warn("reference frame number in alignment larger than size of frameset. Setting to last frame!");
        frame = frames.size() - 1;
    }
    return frames[frame];
}

Prepass build_prepass(const Params& p, const Database& db, const Sample& s, const float* frames) {
    Prepass pp;
    if (p.alignments.empty() && p.motions.empty()) return pp;
    const size_t nsys = s.atom_ids.size(), nf = s.nframes;
    const std::vector<size_t> system = system_list(nsys);
    pp.masses.resize(nsys);
    for (size_t i = 0; i < nsys; ++i) {
        auto it = db.masses.find(s.atom_ids[i]);
        if (it == db.masses.end())
            throw std::runtime_error("database has no mass for atom type " + db.labels.at(s.atom_ids[i]));
        pp.masses[i] = it->second;
    }
    for (const AlignmentParams& a : p.alignments)
        if (a.order == "pre") pp.steps.push_back(alignment_step(a, s, frames));
    for (const MotionParams& m : p.motions) {
        if (m.type == "none") continue;
        if (m.type == "randomwalk" || m.type == "brownian" || m.type == "localbrownian" || m.type == "rotationalbrownian")
            throw std::runtime_error("motion type " + m.type +
                                     " draws from Boost's mt19937 / normal / uniform_on_sphere streams, which this "
                                     "build does not reproduce");
        if (m.type != "linear" && m.type != "fixed" && m.type != "oscillation")
            throw std::runtime_error("Motion type not understood");
        const std::vector<size_t>& sel = s.selection(m.selection);
        const std::vector<size_t>& rsel = s.selection(m.ref_selection);
        PrepassStep st;
        st.type = SASS_STEP_MOTION;
        st.label = "motion " + m.type;
        st.selection = walked(system, sel);
        st.reference = reference_coords(m.ref_type, m.ref_frame, m.ref_filepath, m.ref_format, rsel, frames, nf, nsys);
        // instant: CenterOfMass(cset, system, reference selection); else the reference's own list
        st.reference_selection = m.ref_type == "instant" ? walked(system, rsel) : rsel;
        st.translations = motion_translations(m, nf);
        pp.steps.push_back(st);
    }
    for (const AlignmentParams& a : p.alignments)
        if (a.order == "post") pp.steps.push_back(alignment_step(a, s, frames));
    return pp;
}

}  // namespace sassgpu
