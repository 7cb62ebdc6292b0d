#include "devices.hpp"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <map>
#include <set>
#include <stdexcept>

#include "prepass.hpp"
#include "sassena_gb300.h"

namespace sassgpu {

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

double len(const Vec3& v) { return std::sqrt(std::pow(v[0], 2) + std::pow(v[1], 2) + std::pow(v[2], 2)); }

Vec3 cross(const Vec3& a, const Vec3& b) {
    return Vec3{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}

Vec3 scale(const Vec3& a, double s) { return Vec3{a[0] * s, a[1] * s, a[2] * s}; }
double dot(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// The reference's CartesianCoor3D ordering (coor3d.cpp:23-43), used for resume.
struct VecLess {
    bool operator()(const Vec3& a, const Vec3& b) const {
        if (a[0] != b[0]) return a[0] < b[0];
        if (a[1] != b[1]) return a[1] < b[1];
        return a[2] < b[2];
    }
};

void info(const std::string& m) { fprintf(stderr, "INFO>> %s\n", m.c_str()); }

void check(sass_plan* plan, int rc, const char* what) {
    if (rc != SASS_OK)
        throw std::runtime_error(std::string(what) + ": " + sass_status_name(rc) + ": " + sass_plan_error(plan));
}

}  // namespace

std::vector<double> ScatterClasses::factors(const Database& db, double background, double ql) const {
    std::vector<double> out(id.size());
    for (size_t c = 0; c < id.size(); ++c) {
        double sf = db.sfactor(id[c], ql);
        if (background != 0.0) {
            // sf - background * efactor(ID, kappa * volume, |q|), scatter_factors.cpp:66-73;
            // with background 0 the reference subtracts 0 * efactor, which leaves sf
            double v = db.volume(id[c]);
            sf = sf - background * db.exclusion_factor(id[c], kappa[c] * v, ql);
        }
        out[c] = sf;
    }
    return out;
}

ScatterClasses build_classes(const Params& p, const Database& db, const Sample& s) {
    // kappas map every atom of the sample (ScatterFactors::update_kappas, :34-54)
    std::vector<double> kappa(s.atom_ids.size(), 1.0);
    for (const auto& k : p.kappas)
        for (size_t a : s.selection(k.first)) kappa[a] = k.second;
    const std::vector<size_t>& target = s.selection(p.target);
    ScatterClasses c;
    std::map<std::pair<size_t, double>, int32_t> index;
    for (size_t a : target) {
        auto key = std::make_pair(s.atom_ids[a], kappa[a]);
        auto it = index.find(key);
        if (it == index.end()) {
            it = index.emplace(key, (int32_t)c.id.size()).first;
            c.id.push_back(key.first);
            c.kappa.push_back(key.second);
        }
        c.atom_class.push_back(it->second);
    }
    (void)db;
    return c;
}

std::vector<Vec3> subvectors_for(const Params& p, const Vec3& q) {
    std::vector<Vec3> out;
    if (p.orientation_type == "vectors" && !p.orientations.empty()) {
        if (p.vectors_type == "file" || p.vectors_type == "sphere") {
            double ql = len(q);
            for (const Vec3& u : p.orientations) out.push_back(scale(u, ql));
        } else if (p.vectors_type == "cylinder") {
            // CartesianVectorBase(axis) (coor3d.cpp:278-295), then the projection of q and
            // qnew = z*e_z + r*(u.x*e_r + u.y*e_phi) (abstract_vectors_scatter_device.cpp:130-149)
            Vec3 ek{0, 0, 1}, ej{0, 1, 0};
            Vec3 ez = scale(p.axis, 1.0 / len(p.axis));
            Vec3 ekez = cross(ek, ez);
            if (len(ekez) == 0) ekez = cross(ej, ez);
            Vec3 er = scale(ekez, 1.0 / len(ekez));
            Vec3 ezer = cross(ez, er);
            Vec3 ephi = scale(ezer, 1.0 / len(ezer));
            Vec3 qp{dot(q, er), dot(q, ephi), dot(q, ez)};
            double r = std::sqrt(std::pow(qp[0], 2) + std::pow(qp[1], 2));
            if (r == 0) {
                out.push_back(qp);  // the projected vector, as the reference pushes it
            } else {
                for (const Vec3& u : p.orientations) {
                    Vec3 a = scale(ez, qp[2]);
                    Vec3 b{u[0] * er[0] + u[1] * ephi[0], u[0] * er[1] + u[1] * ephi[1],
                           u[0] * er[2] + u[1] * ephi[2]};
                    out.push_back(Vec3{a[0] + r * b[0], a[1] + r * b[1], a[2] + r * b[2]});
                }
            }
        } else {
            throw std::runtime_error("Vectors orientation averaging type not understood: " + p.vectors_type);
        }
    } else {
        out.push_back(q);
    }
    return out;
}

bool run_scatter_device(const Params& p, Database& db, const Sample& s, RunStats& st) {
    const double t0 = now_s();
    const std::vector<size_t>& target = s.selection(p.target);
    const size_t na = target.size(), nf = s.nframes;
    st.na = na;
    st.nf = nf;
    st.nq_total = p.qvectors.size();

    // ---- resume: compute only q-vectors not yet in the signal file (sassena.cpp:270-308) ----
    SignalData out;
    bool existing = false;
    {
        FILE* f = fopen(p.signal_filepath.c_str(), "rb");
        if (f) {
            fclose(f);
            if (!is_hdf5_file(p.signal_filepath))
                throw std::runtime_error(p.signal_filepath + " does not to be a HDF5 data file. aborting...");
            out = read_signal_file(p.signal_filepath);
            existing = true;
            if (out.has_fqt && out.nf != nf)
                throw std::runtime_error("signal file " + p.signal_filepath + " holds fqt with NF=" +
                                         std::to_string(out.nf) + ", this run has NF=" + std::to_string(nf));
        }
    }
    std::set<Vec3, VecLess> done(out.qvectors.begin(), out.qvectors.end());
    std::vector<Vec3> todo;
    for (const Vec3& q : p.qvectors)
        if (!done.count(q)) todo.push_back(q);
    if (todo.size() != p.qvectors.size())
        info("Found " + std::to_string(p.qvectors.size() - todo.size()) + " old qvectors.");
    if (todo.empty()) {
        info("Very good. No qvectors left to compute.");
        return false;
    }
    if (!existing) {
        out.has_fqt = p.signal_fqt;
        out.has_fq0 = p.signal_fq0;
        out.has_fq = p.signal_fq;
        out.has_fq2 = p.signal_fq2;
    }
    out.nf = nf;
    out.chunksize = p.chunksize;
    out.rawconfig = p.rawconfig;
    out.config = p.rawconfig;
    out.database = db.rawconfig;

    // ---- device -------------------------------------------------------------------------------
    // ScatterDeviceFactory::create, scatter_device_factory.cpp:145-201
    const bool multipole = p.scattering_type == "all" && p.orientation_type == "multipole";
    if (multipole && p.multipole_type != "sphere" && p.multipole_type != "cylinder")
        throw std::runtime_error("scattering.average.orientation.multipole.type not understood: " + p.multipole_type);
    if (multipole && p.precision != "fp64") info("The multipole devices run the FP64 form.");
    ScatterClasses cls = build_classes(p, db, s);
    sass_plan_desc d{};
    d.scattering = p.scattering_type == "self" ? SASS_SCATTERING_SELF : SASS_SCATTERING_ALL;
    d.dsp_type = p.dsp_type == "square" ? SASS_DSP_SQUARE
                 : p.dsp_type == "plain" ? SASS_DSP_PLAIN
                                         : SASS_DSP_AUTOCORRELATE;
    d.dsp_method = p.dsp_method == "direct" ? SASS_METHOD_DIRECT : SASS_METHOD_FFTW;
    d.precision = (p.precision == "fp32" && !multipole) ? SASS_PRECISION_FP32 : SASS_PRECISION_FP64;
    d.na = na;
    d.nf = nf;
    d.nclass = cls.id.size();
    d.device = p.device;
    d.amplitude_budget_bytes = p.amplitude_budget;
    sass_plan* plan = nullptr;
    int rc = sass_plan_create(&d, &plan);
    if (rc != SASS_OK) {
        std::string m = plan ? sass_plan_error(plan) : "";
        sass_plan_destroy(plan);
        throw std::runtime_error(std::string("sass_plan_create: ") + sass_status_name(rc) + ": " + m);
    }
    struct Guard {
        sass_plan* p;
        ~Guard() { sass_plan_destroy(p); }
    } guard{plan};

    // sd:stage: frames read straight into page-locked memory, one copy to the device; with
    // alignments or motions the whole system goes up and the device applies them first
    double ts = now_s();
    {
        const bool prepass = !p.alignments.empty() || !p.motions.empty();
        const size_t nsys = s.atom_ids.size();
        const size_t bytes = nf * (prepass ? nsys : na) * 3 * sizeof(float);
        float* pinned = static_cast<float*>(sass_host_alloc(bytes));
        if (!pinned) throw std::runtime_error("sass_host_alloc: cannot allocate page-locked staging memory");
        struct Free {
            float* q;
            ~Free() { sass_host_free(q); }
        } release{pinned};
        if (p.stager_dump && p.stager_format != "dcd")
            throw std::runtime_error("Format for coordinate dumping not known: " + p.stager_format);
        if (!prepass) {
            s.stage_into(p.target, pinned);
            check(plan, sass_stage_frames(plan, pinned, 0), "sass_stage_frames");
            if (p.stager_dump) {
                info("Dumping coordinates to file: " + p.stager_filepath);
                write_dcd(p.stager_filepath, pinned, nf, na);
            }
        } else {
            s.stage_into("system", pinned);
            Prepass pp = build_prepass(p, db, s, pinned);
            std::vector<sass_prepass_step> steps(pp.steps.size());
            for (size_t i = 0; i < pp.steps.size(); ++i) {
                const PrepassStep& q = pp.steps[i];
                sass_prepass_step& e = steps[i];
                e = sass_prepass_step{};
                e.type = q.type;
                e.selection = q.selection.data();
                e.nselection = q.selection.size();
                e.reference_selection = q.reference_selection.data();
                e.nreference = q.reference_selection.size();
                e.reference = q.reference.empty() ? nullptr : q.reference.data();
                e.fit_target = q.fit_target.data();
                e.fit_source = q.fit_source.data();
                e.nfit = q.fit_target.size();
                e.translations = q.translations.empty() ? nullptr : q.translations.data();
                info("Staging pre-pass step: " + q.label);
            }
            const std::vector<size_t>& target = s.selection(p.target);
            std::vector<float> staged(p.stager_dump ? nf * na * 3 : 0);
            check(plan, sass_stage_frames_prepass(plan, pinned, nsys, pp.masses.data(), steps.data(), steps.size(),
                                                  target.data(), p.stager_dump ? staged.data() : nullptr),
                  "sass_stage_frames_prepass");
            if (p.stager_dump) {
                info("Dumping coordinates to file: " + p.stager_filepath);
                write_dcd(p.stager_filepath, staged.data(), nf, na);
            }
        }
    }
    check(plan, sass_set_atom_classes(plan, cls.atom_class.data(), 0), "sass_set_atom_classes");
    st.stage_s = now_s() - ts;
    info("Staged " + std::to_string(nf) + " frames x " + std::to_string(na) + " atoms (sd:stage " +
         std::to_string(st.stage_s) + " s)");

    std::vector<int32_t> moments;
    for (const auto& mm : p.moments) {
        moments.push_back((int32_t)mm.first);
        moments.push_back((int32_t)mm.second);
    }
    const double axis[3] = {p.axis[0], p.axis[1], p.axis[2]};

    // sd:compute in batches of whole q-vectors
    const size_t batch = p.batch_q ? p.batch_q : todo.size();
    double last_flush = now_s();
    for (size_t i0 = 0; i0 < todo.size(); i0 += batch) {
        const size_t i1 = std::min(todo.size(), i0 + batch), nq = i1 - i0;
        std::vector<size_t> offs(1, 0);
        std::vector<double> sv, cf, qv;
        for (size_t i = i0; i < i1; ++i) {
            if (multipole) {
                qv.insert(qv.end(), todo[i].begin(), todo[i].end());
                offs.push_back(offs.back() + p.moments.size());
            } else {
                std::vector<Vec3> sub = subvectors_for(p, todo[i]);
                for (const Vec3& v : sub) sv.insert(sv.end(), v.begin(), v.end());
                offs.push_back(offs.back() + sub.size());
            }
            std::vector<double> f = cls.factors(db, p.background_factor, len(todo[i]));
            cf.insert(cf.end(), f.begin(), f.end());
        }
        std::vector<double> fqt(nq * nf * 2), fq(nq * 2), fq2(nq * 2);
        double tc = now_s();
        if (multipole)
            check(plan,
                  sass_multipole_compute(plan, p.multipole_type == "sphere" ? SASS_MULTIPOLE_SPHERE : SASS_MULTIPOLE_CYLINDER,
                                         nq, qv.data(), cf.data(), p.moments.size(), moments.data(), axis, fqt.data(),
                                         fq.data(), fq2.data()),
                  "sass_multipole_compute");
        else
            check(plan, sass_compute(plan, nq, offs.data(), sv.data(), cf.data(), fqt.data(), fq.data(), fq2.data(), 0),
                  "sass_compute");
        st.compute_s += now_s() - tc;
        if (!multipole) {  // which phase kernel ran (sd:compute schedule)
            sass_schedule sch{};
            if (sass_plan_schedule(plan, &sch) == SASS_OK) {
                if (sch.rec_shells_per_lane > 0)
                    info("Phase sum: shell recurrence on " + std::to_string(sch.rec_shells) + " q-vectors (" +
                         std::to_string(sch.rec_shells_per_lane) + " shells per lane), direct kernel on " +
                         std::to_string(sch.direct_tiles) + " tiles");
                else
                    info("Phase sum: direct kernel, " + std::to_string(sch.direct_tiles) + " tiles of " +
                         std::to_string(sch.q_per_lane) + " q-vectors per lane");
            }
        }
        st.nsub += offs.back();
        st.terms += (double)offs.back() * (double)na * (double)nf;
        // rows in completion order (HDF5WriterClient::write, file_writer_service.cpp:504-531)
        for (size_t k = 0; k < nq; ++k) {
            out.qvectors.push_back(todo[i0 + k]);
            if (out.has_fqt) out.fqt.insert(out.fqt.end(), fqt.begin() + k * nf * 2, fqt.begin() + (k + 1) * nf * 2);
            if (out.has_fq0) out.fq0.insert(out.fq0.end(), fqt.begin() + k * nf * 2, fqt.begin() + k * nf * 2 + 2);
            if (out.has_fq) out.fq.insert(out.fq.end(), fq.begin() + 2 * k, fq.begin() + 2 * k + 2);
            if (out.has_fq2) out.fq2.insert(out.fq2.end(), fq2.begin() + 2 * k, fq2.begin() + 2 * k + 2);
        }
        st.nq_computed += nq;
        if (now_s() - last_flush > (double)p.serverflush_s && i1 < todo.size()) {
            double tw = now_s();
            write_signal_file(p.signal_filepath, out);
            st.write_s += now_s() - tw;
            last_flush = now_s();
        }
    }
    double tw = now_s();
    write_signal_file(p.signal_filepath, out);
    st.write_s += now_s() - tw;
    info("Computed " + std::to_string(st.nq_computed) + " q-vectors (" + std::to_string(st.nsub) +
         " sub-vectors, sd:compute " + std::to_string(st.compute_s) + " s, " +
         std::to_string(st.terms / std::max(st.compute_s, 1e-9)) + " terms/s); total " +
         std::to_string(now_s() - t0) + " s");
    return true;
}

}  // namespace sassgpu
