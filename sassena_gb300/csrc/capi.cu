// C ABI of the GB300 scattering path: plans (one scatter-device computation), batches
// (many systems in one graph-captured launch sequence), autotuning.
//
// A plan's sass_compute produces the rows the reference hands to HDF5WriterClient::write
// (src/services/file_writer_service.cpp:504-531): fqt [NF] complex, fq, fq2 per q.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sassena_gb300.h"
#include "engine.h"
#include "kernels.h"
#include "plan.h"

using namespace sassgpu;

namespace {

int ceil_log2(size_t n) {
    int lg = 0;
    while (((size_t)1 << lg) < n) ++lg;
    return lg;
}

int validate_desc(const sass_plan_desc& d, int& lg, std::string& msg) {
    if (d.scattering != SASS_SCATTERING_ALL && d.scattering != SASS_SCATTERING_SELF) return SASS_ERR_ARG;
    if (d.dsp_type < 0 || d.dsp_type > 2 || d.dsp_method < 0 || d.dsp_method > 1) return SASS_ERR_ARG;
    if (d.precision != SASS_PRECISION_FP64 && d.precision != SASS_PRECISION_FP32) return SASS_ERR_ARG;
    // NF < 1 is rejected as in file_writer_service.cpp:23-26
    if (d.na == 0 || d.nf == 0 || d.nclass == 0) return SASS_ERR_ARG;
    if (d.na > (size_t)1 << 30 || d.nf > (size_t)1 << 24) return SASS_ERR_ARG;
    lg = std::max(2, ceil_log2(2 * d.nf));
    // autocorrelation: shared-memory transforms up to 2^kMaxLg, the four-step transform
    // through HBM up to 2^kLongLgMax
    const int lg_limit = kLongLgMax;
    if (d.dsp_type == SASS_DSP_AUTOCORRELATE && lg > lg_limit) {
        char b[200];
        snprintf(b, sizeof(b), "autocorrelation supports NF <= %zu for this scattering type (padded FFT length <= %zu), got NF=%zu",
                 ((size_t)1 << lg_limit) / 2, (size_t)1 << lg_limit, d.nf);
        msg = b;
        return SASS_ERR_UNSUPPORTED;
    }
    if (d.scattering == SASS_SCATTERING_SELF && d.dsp_type == SASS_DSP_AUTOCORRELATE && lg <= kMaxLg &&
        fft_smem_bytes(d.precision, lg, (int)d.nf, true) > 227 * 1024) {
        msg = "incoherent FP64 autocorrelation with this NF exceeds shared memory";
        return SASS_ERR_UNSUPPORTED;
    }
    return SASS_OK;
}

EngineConfig engine_config(const sass_plan_desc& d) {
    EngineConfig c;
    c.scattering = d.scattering;
    c.dsp = d.dsp_type;
    c.method = d.dsp_method;
    c.precision = d.precision;
    c.device = d.device;
    return c;
}

// Process-wide autotuning cache: problem signature -> best configuration.
struct TuneChoice {
    PhaseShape shape{0, 0, 0};
    int split_atoms = 0, rec_k = 0;
};
std::mutex g_tune_lock;
std::map<std::string, TuneChoice> g_tune_cache;

// Product-set detection on host sub-vectors (copied from the device when needed).
int product_of(std::string& m, const double* qv, bool on_device, const std::vector<size_t>& offs,
               std::vector<double>& lam, int& base);

}  // namespace

struct sass_batch {
    sass_plan_desc d{};
    std::vector<SystemState*> systems;
    std::vector<size_t> nq, nv;
    std::vector<std::vector<size_t>> offs;
    DevBuf qv, cf, out;  // all systems' inputs / outputs, packed
    std::vector<size_t> qv_off, cf_off, fqt_off, fq_off, fq2_off;
    Engine eng;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool prepared = false;
    PhaseShape shape{0, 0, 0};
    int split_atoms = 0, rec_k = 0;
    std::vector<std::vector<double>> lam;  // product structure per system (empty: none)
    std::vector<int> lam_base;
    std::string msg;
    sass_timing timing{};
    cudaEvent_t ev[kEvents] = {};
    ~sass_batch() {
        for (SystemState* s : systems) delete s;
    }
};

namespace {

int set_msg(std::string& m, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    m = buf;
    return code;
}

int cuda_fail(std::string& m, cudaError_t e, const char* what) {
    int code = (e == cudaErrorMemoryAllocation) ? SASS_ERR_OOM : SASS_ERR_CUDA;
    cudaGetLastError();
    return set_msg(m, code, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(m, expr)                                           \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return cuda_fail(m, e_, #expr); \
    } while (0)

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();
        return 0.f;
    }
    return ms;
}

int read_err_word(std::string& m, unsigned* word, cudaStream_t st) {
    unsigned flag = 0;
    CK(m, cudaMemcpyAsync(&flag, word, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CK(m, cudaStreamSynchronize(st));
    if (flag == DEV_MBAR_TIMEOUT) return set_msg(m, SASS_ERR_TIMEOUT, "a device-side wait exceeded its iteration limit");
    if (flag != 0) return set_msg(m, SASS_ERR_CUDA, "device error flag %u", flag);
    return SASS_OK;
}

int init_stream(std::string& m, const sass_plan_desc& d, cudaStream_t& st, bool& own, cudaEvent_t* ev) {
    CK(m, cudaSetDevice(d.device));
    if (d.stream) {
        st = (cudaStream_t)d.stream;
    } else {
        CK(m, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        own = true;
    }
    for (int i = 0; i < kEvents; ++i) CK(m, cudaEventCreate(&ev[i]));
    return SASS_OK;
}

int init_system(std::string& m, SystemState& s, const sass_plan_desc& d, int lg, cudaStream_t st) {
    s.na = d.na;
    s.nf = d.nf;
    s.nclass = d.nclass;
    s.na_pad = ((d.na + kAtomGranule - 1) / kAtomGranule) * kAtomGranule;
    s.lg = lg;
    return build_system_tables(s, st, m);
}

int time_config(std::string& m, Engine& eng, const EngineConfig& c, const std::vector<WorkItem>& items,
                cudaStream_t st, cudaEvent_t* ev, int repeats, double& ms) {
    std::string err;
    ms = -1;
    if (eng.prepare(c, items, err) != SASS_OK) return SASS_OK;  // configuration not applicable
    if (eng.enqueue(st, err) != SASS_OK) return SASS_OK;         // warm-up
    CK(m, cudaEventRecord(ev[10], st));
    for (int r = 0; r < repeats; ++r)
        if (eng.enqueue(st, err) != SASS_OK) return set_msg(m, SASS_ERR_CUDA, "%s", err.c_str());
    CK(m, cudaEventRecord(ev[11], st));
    CK(m, cudaEventSynchronize(ev[11]));
    int rc = read_err_word(m, eng.err_word(), st);
    if (rc) return rc;
    ms = ev_ms(ev[10], ev[11]) / std::max(repeats, 1);
    return SASS_OK;
}

// Time the engine over candidate configurations and keep the best: first the shell
// recurrence width (FP32 product sets: off and every instantiated width, automatic tile),
// then the direct kernel's tile shapes x atom-split sizes with that width (only split
// sizes when the recurrence covers every shell).
int autotune_engine(std::string& m, Engine& eng, const EngineConfig& base, const std::vector<WorkItem>& items,
                    cudaStream_t st, cudaEvent_t* ev, int repeats, TuneChoice& best, double& best_ms) {
    best_ms = 1e300;
    bool any = false;
    auto consider = [&](const EngineConfig& c) -> int {
        double ms = 0;
        int rc = time_config(m, eng, c, items, st, ev, repeats, ms);
        if (rc) return rc;
        if (ms >= 0 && ms < best_ms) {
            best_ms = ms;
            // the shape the engine resolved (an automatic shape depends on the items, so a
            // choice made on a representative subset must name the shape it timed)
            best.shape = eng.stats().shape;
            best.split_atoms = c.split_atoms;
            best.rec_k = c.rec_k;
            any = true;
        }
        return SASS_OK;
    };
    // the recurrence widths are worth timing only where some shells form runs
    bool product = false;
    for (const WorkItem& it : items)
        product = product || (!it.lam.empty() && !arithmetic_runs(it.lam, 3).empty());
    int rec_k = -1;
    bool all_rec = false;
    if (base.precision == PREC_FP32 && product) {
        std::vector<int> ks = {-1};
        for (int k : rec_shell_counts()) ks.push_back(k);
        for (int k : ks) {
            EngineConfig c = base;
            c.rec_k = k;
            int rc = consider(c);
            if (rc) return rc;
        }
        rec_k = best.rec_k;
        if (rec_k > 0) {
            EngineConfig c = base;
            c.rec_k = rec_k;
            std::string err;
            if (eng.prepare(c, items, err) == SASS_OK) all_rec = eng.stats().phase_tiles == 0;
        }
    }
    std::vector<PhaseShape> shapes = all_rec ? std::vector<PhaseShape>{PhaseShape{0, 0, 0}} : phase_shapes(base.precision);
    for (const PhaseShape& sh : shapes)
        for (int sp : {0, 2048, 8192}) {
            EngineConfig c = base;
            c.shape = sh;
            c.split_atoms = sp;
            c.rec_k = rec_k;
            int rc = consider(c);
            if (rc) return rc;
        }
    if (!any) return set_msg(m, SASS_ERR_UNSUPPORTED, "no tile shape could be prepared");
    // leave the engine prepared with the choice, so that its schedule describes it
    EngineConfig c = base;
    c.shape = best.shape;
    c.split_atoms = best.split_atoms;
    c.rec_k = best.rec_k;
    std::string err;
    if (eng.prepare(c, items, err) != SASS_OK) return set_msg(m, SASS_ERR_CUDA, "%s", err.c_str());
    return SASS_OK;
}

int product_of(std::string& m, const double* qv, bool on_device, const std::vector<size_t>& offs,
               std::vector<double>& lam, int& base) {
    lam.clear();
    base = -1;
    const double* h = qv;
    std::vector<double> copy;
    if (on_device) {
        copy.resize(offs.back() * 3);
        CK(m, cudaMemcpy(copy.data(), qv, copy.size() * sizeof(double), cudaMemcpyDeviceToHost));
        h = copy.data();
    }
    detect_product(h, offs, lam, base);
    return SASS_OK;
}

void fill_schedule(const EngineStats& s, sass_schedule* out) {
    memset(out, 0, sizeof(*out));
    out->terms = s.terms;
    out->direct_tiles = s.phase_tiles;
    out->rec_tiles = s.rec_tiles;
    out->rec_shells = s.rec_shells;
    out->rec_shells_per_lane = s.rec_tiles ? s.rec_k : 0;
    out->q_per_lane = s.shape.q_per_lane;
    out->warps = s.shape.warps;
    out->atoms = s.shape.atoms;
    out->atom_splits = s.max_split;
    out->poly_pairs = s.phase_tiles ? s.shape.poly_pairs : 0;
}

std::string signature(const sass_plan_desc& d, const std::vector<WorkItem>& items) {
    std::string s = std::to_string(d.scattering) + "/" + std::to_string(d.dsp_type) + "/" + std::to_string(d.precision);
    for (const WorkItem& it : items) {
        s += "|" + std::to_string(it.sys->na) + "x" + std::to_string(it.sys->nf) + ":";
        for (size_t k = 0; k + 1 < it.offs.size(); ++k) s += std::to_string(it.offs[k + 1] - it.offs[k]) + ",";
    }
    return s;
}

}  // namespace

extern "C" {

const char* sass_version(void) { return "sassena_gb300 0.2 (sm_103a)"; }

const char* sass_status_name(int status) {
    switch (status) {
        case SASS_OK: return "SASS_OK";
        case SASS_ERR_ARG: return "SASS_ERR_ARG";
        case SASS_ERR_OOM: return "SASS_ERR_OOM";
        case SASS_ERR_UNSUPPORTED: return "SASS_ERR_UNSUPPORTED";
        case SASS_ERR_CUDA: return "SASS_ERR_CUDA";
        case SASS_ERR_TIMEOUT: return "SASS_ERR_TIMEOUT";
        case SASS_ERR_STATE: return "SASS_ERR_STATE";
        default: return "SASS_ERR_UNKNOWN";
    }
}

const char* sass_plan_error(const sass_plan* plan) { return plan ? plan->msg.c_str() : ""; }

int sass_plan_create(const sass_plan_desc* desc, sass_plan** out) {
    if (!out) return SASS_ERR_ARG;
    *out = nullptr;
    if (!desc) return SASS_ERR_ARG;
    std::string msg;
    int lg = 0;
    int rc = validate_desc(*desc, lg, msg);
    if (rc == SASS_ERR_ARG) return rc;
    sass_plan* p = new sass_plan();
    p->d = *desc;
    *out = p;
    if (rc) {
        p->msg = msg;
        return rc;
    }
    rc = init_stream(p->msg, p->d, p->st, p->own_stream, p->ev);
    if (rc) return rc;
    rc = init_system(p->msg, p->sys, p->d, lg, p->st);
    if (rc) return rc;
    p->msg.clear();
    return SASS_OK;
}

void sass_plan_destroy(sass_plan* p) {
    if (!p) return;
    cudaSetDevice(p->d.device);
    drop_prefetch(p->sys);
    if (p->side) cudaStreamDestroy(p->side);
    if (p->pf_done) cudaEventDestroy(p->pf_done);
    if (p->st) cudaStreamSynchronize(p->st);
    for (int i = 0; i < kEvents; ++i)
        if (p->ev[i]) cudaEventDestroy(p->ev[i]);
    p->eng.release();
    if (p->own_stream && p->st) cudaStreamDestroy(p->st);
    delete p;
}

int sass_stage_frames(sass_plan* p, const float* coords, int on_device) {
    if (!p) return SASS_ERR_ARG;
    CK(p->msg, cudaSetDevice(p->d.device));
    int rc = stage_system(p->sys, coords, on_device != 0, p->d.precision, p->st, p->msg);
    if (!rc) p->msg.clear();
    return rc;
}

int sass_prefetch_frames(sass_plan* p, const float* coords) {
    if (!p) return SASS_ERR_ARG;
    CK(p->msg, cudaSetDevice(p->d.device));
    if (!p->side) {
        CK(p->msg, cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
        CK(p->msg, cudaEventCreateWithFlags(&p->pf_done, cudaEventDisableTiming));
    }
    int rc = prefetch_system(p->sys, coords, p->msg);
    if (!rc) p->msg.clear();
    return rc;
}

int sass_set_atom_classes(sass_plan* p, const int32_t* atom_class, int on_device) {
    if (!p) return SASS_ERR_ARG;
    CK(p->msg, cudaSetDevice(p->d.device));
    int rc = set_system_classes(p->sys, atom_class, on_device != 0, p->st, p->msg);
    if (!rc) p->msg.clear();
    return rc;
}

int sass_set_phase_tile(sass_plan* p, int q_per_lane, int warps, int atoms, int atom_splits) {
    if (!p) return SASS_ERR_ARG;
    if (q_per_lane == 0) {
        p->shape = PhaseShape{0, 0, 0};
    } else {
        PhaseShape t{q_per_lane, warps, atoms};
        if (!phase_shape_supported(p->d.precision, t))
            return set_msg(p->msg, SASS_ERR_UNSUPPORTED, "phase tile Q=%d W=%d T=%d not instantiated", q_per_lane,
                           warps, atoms);
        p->shape = t;
    }
    // atom_splits > 0: that many slices of the atoms per tile row
    p->split_atoms = 0;
    if (atom_splits > 0) {
        int a = (int)((p->sys.na_pad + atom_splits - 1) / atom_splits);
        a = ((a + kAtomGranule - 1) / kAtomGranule) * kAtomGranule;
        p->split_atoms = std::max(a, kAtomGranule);
    }
    return SASS_OK;
}

int sass_frame_center(const sass_plan* p, double* c) {
    if (!p || !c) return SASS_ERR_ARG;
    memcpy(c, p->sys.center, sizeof(p->sys.center));
    return SASS_OK;
}

static bool rec_width_ok(int k) { return k == 0 || k == -1 || rec_shells_supported(k); }

int sass_set_phase_poly(sass_plan* p, int poly_pairs) {
    if (!p) return SASS_ERR_ARG;
    PhaseShape t = p->shape;
    t.poly_pairs = poly_pairs;
    if (poly_pairs != 0 && (t.q_per_lane == 0 || !phase_shape_supported(p->d.precision, t)))
        return set_msg(p->msg, SASS_ERR_UNSUPPORTED, "no instantiated tile shape Q=%d W=%d T=%d with %d polynomial pairs",
                       t.q_per_lane, t.warps, t.atoms, poly_pairs);
    p->shape.poly_pairs = poly_pairs;
    return SASS_OK;
}

int sass_set_shell_recurrence(sass_plan* p, int shells_per_lane) {
    if (!p) return SASS_ERR_ARG;
    if (!rec_width_ok(shells_per_lane))
        return set_msg(p->msg, SASS_ERR_UNSUPPORTED, "shell recurrence width %d not instantiated", shells_per_lane);
    p->rec_k = shells_per_lane;
    return SASS_OK;
}

int sass_plan_schedule(const sass_plan* p, sass_schedule* out) {
    if (!p || !out) return SASS_ERR_ARG;
    fill_schedule(p->eng.stats(), out);
    return SASS_OK;
}

static int check_ready(sass_plan* p) {
    if (!p->sys.staged) return set_msg(p->msg, SASS_ERR_STATE, "sass_stage_frames has not been called");
    if (!p->sys.classes_set) return set_msg(p->msg, SASS_ERR_STATE, "sass_set_atom_classes has not been called");
    return SASS_OK;
}

static int check_offsets(std::string& m, size_t nq, const size_t* offs) {
    if (!offs) return set_msg(m, SASS_ERR_ARG, "NULL argument");
    if (offs[0] != 0) return set_msg(m, SASS_ERR_ARG, "sub_offsets[0] must be 0");
    for (size_t i = 0; i < nq; ++i)
        if (offs[i + 1] <= offs[i]) return set_msg(m, SASS_ERR_ARG, "q-vector %zu has no sub-vectors", i);
    if (offs[nq] > (size_t)1 << 30) return set_msg(m, SASS_ERR_ARG, "too many sub-vectors");
    return SASS_OK;
}

// Inputs on the device for a plan call (copies host inputs into plan buffers).
static int plan_inputs(sass_plan* p, size_t nq, const size_t* offs, const double* subvectors,
                       const double* class_factors, int io_on_device, const double** d_qv, const double** d_cf) {
    const size_t nsub = offs[nq], nclass = p->d.nclass;
    *d_qv = subvectors;
    *d_cf = class_factors;
    if (!io_on_device) {
        CK(p->msg, p->qv.ensure(nsub * 3 * sizeof(double)));
        CK(p->msg, p->cf.ensure(nq * nclass * sizeof(double)));
        CK(p->msg, cudaMemcpyAsync(p->qv.p, subvectors, nsub * 3 * sizeof(double), cudaMemcpyHostToDevice, p->st));
        CK(p->msg, cudaMemcpyAsync(p->cf.p, class_factors, nq * nclass * sizeof(double), cudaMemcpyHostToDevice,
                                   p->st));
        *d_qv = p->qv.as<double>();
        *d_cf = p->cf.as<double>();
        p->timing.h2d_bytes = nsub * 3 * sizeof(double) + nq * nclass * sizeof(double);
    }
    return SASS_OK;
}

int sass_compute(sass_plan* p, size_t nq, const size_t* offs, const double* subvectors,
                 const double* class_factors, double* fqt, double* fq, double* fq2, int io_on_device) {
    if (!p) return SASS_ERR_ARG;
    int rc = check_ready(p);
    if (rc) return rc;
    if (nq == 0) return SASS_OK;
    if (!subvectors || !class_factors || !fqt || !fq || !fq2) return set_msg(p->msg, SASS_ERR_ARG, "NULL argument");
    rc = check_offsets(p->msg, nq, offs);
    if (rc) return rc;
    CK(p->msg, cudaSetDevice(p->d.device));
    memset(&p->timing, 0, sizeof(p->timing));
    CK(p->msg, cudaEventRecord(p->ev[4], p->st));
    const double* d_qv;
    const double* d_cf;
    rc = plan_inputs(p, nq, offs, subvectors, class_factors, io_on_device, &d_qv, &d_cf);
    if (rc) return rc;
    CK(p->msg, cudaEventRecord(p->ev[5], p->st));
    double2 *d_fqt = reinterpret_cast<double2*>(fqt), *d_fq = reinterpret_cast<double2*>(fq),
            *d_fq2 = reinterpret_cast<double2*>(fq2);
    const size_t nf = p->sys.nf, nclass = p->d.nclass;
    if (!io_on_device) {
        CK(p->msg, p->fqt.ensure(nq * nf * sizeof(double2)));
        CK(p->msg, p->fq.ensure(nq * sizeof(double2)));
        CK(p->msg, p->fq2.ensure(nq * sizeof(double2)));
        d_fqt = p->fqt.as<double2>();
        d_fq = p->fq.as<double2>();
        d_fq2 = p->fq2.as<double2>();
    }
    // batches of whole q-vectors bounded by the amplitude budget (coherent path)
    const size_t budget = p->d.amplitude_budget_bytes ? p->d.amplitude_budget_bytes : ((size_t)4 << 30);
    const size_t per_sub = nf * sizeof(double2);
    EngineConfig cfg = engine_config(p->d);
    cfg.shape = p->shape;
    cfg.split_atoms = p->split_atoms;
    cfg.rec_k = p->rec_k;
    const bool want_rec = p->d.precision == SASS_PRECISION_FP32 && p->d.scattering == SASS_SCATTERING_ALL &&
                          p->rec_k >= 0;
    size_t i = 0;
    while (i < nq) {
        size_t j = i + 1;
        if (p->d.scattering == SASS_SCATTERING_ALL) {
            while (j < nq && (offs[j + 1] - offs[i]) * per_sub <= budget) ++j;
        } else {
            j = nq;
        }
        std::vector<WorkItem> items(1);
        WorkItem& it = items[0];
        it.sys = &p->sys;
        for (size_t k = i; k <= j; ++k) it.offs.push_back(offs[k] - offs[i]);
        it.d_qv = d_qv + 3 * offs[i];
        if (want_rec) {
            rc = product_of(p->msg, io_on_device ? d_qv + 3 * offs[i] : subvectors + 3 * offs[i], io_on_device != 0,
                            it.offs, it.lam, it.lam_base);
            if (rc) return rc;
        }
        it.d_cf = d_cf + nclass * i;
        it.d_fqt = d_fqt + i * nf;
        it.d_fq = d_fq + i;
        it.d_fq2 = d_fq2 + i;
        rc = p->eng.prepare(cfg, items, p->msg);
        if (rc) return rc;
        rc = p->eng.enqueue(p->st, p->msg, p->ev);
        if (rc) return rc;
        // a requested frame prefetch goes to the copy engine now, behind this call's own
        // input copies, and overlaps the kernels just queued
        if (p->side) {
            rc = issue_prefetch(p->sys, p->side, p->pf_done, p->msg);
            if (rc) return rc;
        }
        // one host synchronisation: the error word's copy drains the stream, events included
        rc = read_err_word(p->msg, p->eng.err_word(), p->st);
        if (rc) return rc;
        p->timing.phase_ms += ev_ms(p->ev[0], p->ev[1]);
        p->timing.corr_ms += ev_ms(p->ev[1], p->ev[2]);
        p->timing.finalize_ms += ev_ms(p->ev[2], p->ev[3]);
        p->timing.kernel_launches += p->eng.stats().launches;
        p->timing.phase_launches += p->eng.stats().phase_launches;
        i = j;
    }
    CK(p->msg, cudaEventRecord(p->ev[6], p->st));
    if (!io_on_device) {
        CK(p->msg, cudaMemcpyAsync(fqt, d_fqt, nq * nf * sizeof(double2), cudaMemcpyDeviceToHost, p->st));
        CK(p->msg, cudaMemcpyAsync(fq, d_fq, nq * sizeof(double2), cudaMemcpyDeviceToHost, p->st));
        CK(p->msg, cudaMemcpyAsync(fq2, d_fq2, nq * sizeof(double2), cudaMemcpyDeviceToHost, p->st));
        p->timing.d2h_bytes = nq * (nf + 2) * sizeof(double2);
    }
    CK(p->msg, cudaEventRecord(p->ev[7], p->st));
    CK(p->msg, cudaEventSynchronize(p->ev[7]));
    p->timing.total_ms = ev_ms(p->ev[4], p->ev[7]);
    if (!io_on_device) {
        p->timing.h2d_ms = ev_ms(p->ev[4], p->ev[5]);
        p->timing.d2h_ms = ev_ms(p->ev[6], p->ev[7]);
    }
    p->msg.clear();
    return SASS_OK;
}

int sass_autotune(sass_plan* p, size_t nq, const size_t* offs, const double* subvectors,
                  const double* class_factors, int repeats, int* q_per_lane, int* warps, int* atoms,
                  int* split_atoms) {
    if (!p) return SASS_ERR_ARG;
    int rc = check_ready(p);
    if (rc) return rc;
    if (p->d.scattering != SASS_SCATTERING_ALL)
        return set_msg(p->msg, SASS_ERR_STATE, "autotuning applies to the coherent phase sum");
    if (nq == 0 || !subvectors || !class_factors) return set_msg(p->msg, SASS_ERR_ARG, "NULL argument");
    rc = check_offsets(p->msg, nq, offs);
    if (rc) return rc;
    CK(p->msg, cudaSetDevice(p->d.device));
    const double *d_qv, *d_cf;
    rc = plan_inputs(p, nq, offs, subvectors, class_factors, 0, &d_qv, &d_cf);
    if (rc) return rc;
    const size_t nf = p->sys.nf;
    CK(p->msg, p->fqt.ensure(nq * nf * sizeof(double2)));
    CK(p->msg, p->fq.ensure(nq * sizeof(double2)));
    CK(p->msg, p->fq2.ensure(nq * sizeof(double2)));
    std::vector<WorkItem> items(1);
    items[0].sys = &p->sys;
    items[0].offs.assign(offs, offs + nq + 1);
    items[0].d_qv = d_qv;
    items[0].d_cf = d_cf;
    items[0].d_fqt = p->fqt.as<double2>();
    items[0].d_fq = p->fq.as<double2>();
    items[0].d_fq2 = p->fq2.as<double2>();
    if (p->d.precision == SASS_PRECISION_FP32) {
        rc = product_of(p->msg, subvectors, false, items[0].offs, items[0].lam, items[0].lam_base);
        if (rc) return rc;
    }
    TuneChoice best;
    double ms = 0;
    std::string key = signature(p->d, items);
    key += items[0].lam.empty() ? "|general" : "|product";
    {
        std::lock_guard<std::mutex> g(g_tune_lock);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            best = it->second;
            ms = -1;
        }
    }
    if (ms == 0) {
        rc = autotune_engine(p->msg, p->eng, engine_config(p->d), items, p->st, p->ev, std::max(1, repeats), best, ms);
        if (rc) return rc;
        std::lock_guard<std::mutex> g(g_tune_lock);
        g_tune_cache[key] = best;
    }
    p->shape = best.shape;
    p->split_atoms = best.split_atoms;
    p->rec_k = best.rec_k;
    if (q_per_lane) *q_per_lane = best.shape.q_per_lane;
    if (warps) *warps = best.shape.warps;
    if (atoms) *atoms = best.shape.atoms;
    if (split_atoms) *split_atoms = best.split_atoms;
    p->msg.clear();
    return SASS_OK;
}

int sass_amplitudes(sass_plan* p, size_t nsub, const double* subvectors, const int32_t* sub_shell, size_t nshell,
                    const double* class_factors, double* out) {
    if (!p) return SASS_ERR_ARG;
    int rc = check_ready(p);
    if (rc) return rc;
    if (p->d.scattering != SASS_SCATTERING_ALL)
        return set_msg(p->msg, SASS_ERR_STATE, "amplitudes need a coherent (all) plan");
    if (nsub == 0) return SASS_OK;
    if (!subvectors || !sub_shell || !class_factors || !out || nshell == 0)
        return set_msg(p->msg, SASS_ERR_ARG, "NULL argument");
    for (size_t m = 0; m < nsub; ++m)
        if (sub_shell[m] < 0 || (size_t)sub_shell[m] >= nshell)
            return set_msg(p->msg, SASS_ERR_ARG, "sub_shell[%zu] out of range", m);
    CK(p->msg, cudaSetDevice(p->d.device));
    memset(&p->timing, 0, sizeof(p->timing));
    // runs of equal shell become the work item's "q-vectors", each with its factor row
    const size_t nclass = p->d.nclass, nf = p->sys.nf;
    std::vector<size_t> offs(1, 0);
    std::vector<double> cf;
    for (size_t m = 0; m < nsub;) {
        size_t e = m;
        while (e < nsub && sub_shell[e] == sub_shell[m]) ++e;
        offs.push_back(e);
        cf.insert(cf.end(), class_factors + nclass * sub_shell[m], class_factors + nclass * (sub_shell[m] + 1));
        m = e;
    }
    const size_t nrun = offs.size() - 1;
    const double *d_qv, *d_cf;
    rc = plan_inputs(p, nrun, offs.data(), subvectors, cf.data(), 0, &d_qv, &d_cf);
    if (rc) return rc;
    CK(p->msg, p->fqt.ensure(nrun * nf * sizeof(double2)));
    CK(p->msg, p->fq.ensure(nrun * sizeof(double2)));
    CK(p->msg, p->fq2.ensure(nrun * sizeof(double2)));
    std::vector<WorkItem> items(1);
    items[0].sys = &p->sys;
    items[0].offs = offs;
    items[0].d_qv = d_qv;
    items[0].d_cf = d_cf;
    items[0].d_fqt = p->fqt.as<double2>();
    items[0].d_fq = p->fq.as<double2>();
    items[0].d_fq2 = p->fq2.as<double2>();
    EngineConfig cfg = engine_config(p->d);
    cfg.dsp = SASS_DSP_PLAIN;  // the amplitudes are read before the store
    cfg.shape = p->shape;
    cfg.split_atoms = p->split_atoms;
    cfg.rec_k = -1;
    rc = p->eng.prepare(cfg, items, p->msg);
    if (rc) return rc;
    rc = p->eng.enqueue(p->st, p->msg, p->ev);
    if (rc) return rc;
    rc = read_err_word(p->msg, p->eng.err_word(), p->st);
    if (rc) return rc;
    p->timing.phase_ms = ev_ms(p->ev[0], p->ev[1]);
    p->timing.phase_launches = p->eng.stats().phase_launches;
    p->timing.kernel_launches = p->eng.stats().launches;
    const bool f32 = p->d.precision == SASS_PRECISION_FP32;
    const void* amp = p->eng.amplitudes(0);
    if (f32) {
        std::vector<float2> a32(nsub * nf);
        CK(p->msg, cudaMemcpy(a32.data(), amp, a32.size() * sizeof(float2), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < a32.size(); ++i) {
            out[2 * i] = a32[i].x;
            out[2 * i + 1] = a32[i].y;
        }
        // the FP32 form computes on centred coordinates: restore exp(i q.c) in FP64
        for (size_t v = 0; v < nsub; ++v) {
            const double* q = subvectors + 3 * v;
            double ph = q[0] * p->sys.center[0] + q[1] * p->sys.center[1] + q[2] * p->sys.center[2];
            double c = cos(ph), s = sin(ph);
            for (size_t f = 0; f < nf; ++f) {
                double* z = out + 2 * (v * nf + f);
                double re = z[0] * c - z[1] * s, im = z[0] * s + z[1] * c;
                z[0] = re;
                z[1] = im;
            }
        }
    } else {
        CK(p->msg, cudaMemcpy(out, amp, nsub * nf * sizeof(double2), cudaMemcpyDeviceToHost));
    }
    p->msg.clear();
    return SASS_OK;
}

int sass_last_timing(const sass_plan* p, sass_timing* out) {
    if (!p || !out) return SASS_ERR_ARG;
    *out = p->timing;
    return SASS_OK;
}

void* sass_host_alloc(size_t bytes) {
    void* ptr = nullptr;
    if (cudaHostAlloc(&ptr, bytes ? bytes : 16, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    return ptr;
}

void sass_host_free(void* ptr) {
    if (ptr) cudaFreeHost(ptr);
}

// ---------------------------------------------------------------------------------------------
// Batches: many systems in one graph-captured launch sequence.
// ---------------------------------------------------------------------------------------------
const char* sass_batch_error(const sass_batch* b) { return b ? b->msg.c_str() : ""; }

int sass_batch_create(const sass_plan_desc* desc, size_t nsystems, const sass_system* systems, sass_batch** out) {
    if (!out) return SASS_ERR_ARG;
    *out = nullptr;
    if (!desc || !systems || nsystems == 0) return SASS_ERR_ARG;
    sass_batch* b = new sass_batch();
    *out = b;
    b->d = *desc;
    int rc = init_stream(b->msg, b->d, b->st, b->own_stream, b->ev);
    if (rc) return rc;
    // sizes and validation
    size_t qv_n = 0, cf_n = 0, out_n = 0;
    for (size_t i = 0; i < nsystems; ++i) {
        const sass_system& s = systems[i];
        sass_plan_desc d = b->d;
        d.na = s.na;
        d.nf = s.nf;
        d.nclass = s.nclass;
        int lg = 0;
        std::string m;
        rc = validate_desc(d, lg, m);
        if (rc) return set_msg(b->msg, rc, "system %zu: %s", i, m.empty() ? "invalid sizes" : m.c_str());
        if (!s.coords || !s.atom_class || !s.sub_offsets || !s.subvectors || !s.class_factors || s.nq == 0)
            return set_msg(b->msg, SASS_ERR_ARG, "system %zu: NULL argument or no q-vectors", i);
        rc = check_offsets(b->msg, s.nq, s.sub_offsets);
        if (rc) return rc;
        b->offs.emplace_back(s.sub_offsets, s.sub_offsets + s.nq + 1);
        b->lam.emplace_back();
        b->lam_base.push_back(-1);
        if (b->d.precision == SASS_PRECISION_FP32 && b->d.scattering == SASS_SCATTERING_ALL)
            detect_product(s.subvectors, b->offs.back(), b->lam.back(), b->lam_base.back());
        b->nq.push_back(s.nq);
        b->nv.push_back(s.sub_offsets[s.nq]);
        b->qv_off.push_back(qv_n);
        b->cf_off.push_back(cf_n);
        qv_n += s.sub_offsets[s.nq] * 3;
        cf_n += s.nq * s.nclass;
        b->fqt_off.push_back(out_n);
        out_n += s.nq * s.nf * 2;
        b->fq_off.push_back(out_n);
        out_n += s.nq * 2;
        b->fq2_off.push_back(out_n);
        out_n += s.nq * 2;
        SystemState* st = new SystemState();
        b->systems.push_back(st);
        rc = init_system(b->msg, *st, d, lg, b->st);
        if (rc) return rc;
        rc = stage_system(*st, s.coords, false, b->d.precision, b->st, b->msg);
        if (rc) return rc;
        rc = set_system_classes(*st, s.atom_class, false, b->st, b->msg);
        if (rc) return rc;
    }
    CK(b->msg, b->qv.ensure(qv_n * sizeof(double)));
    CK(b->msg, b->cf.ensure(cf_n * sizeof(double)));
    CK(b->msg, b->out.ensure(out_n * sizeof(double)));
    for (size_t i = 0; i < nsystems; ++i) {
        const sass_system& s = systems[i];
        CK(b->msg, cudaMemcpy(b->qv.as<double>() + b->qv_off[i], s.subvectors, b->nv[i] * 3 * sizeof(double),
                              cudaMemcpyHostToDevice));
        CK(b->msg, cudaMemcpy(b->cf.as<double>() + b->cf_off[i], s.class_factors, s.nq * s.nclass * sizeof(double),
                              cudaMemcpyHostToDevice));
    }
    b->msg.clear();
    return SASS_OK;
}

static std::vector<WorkItem> batch_items(sass_batch* b) {
    std::vector<WorkItem> items(b->systems.size());
    for (size_t i = 0; i < items.size(); ++i) {
        WorkItem& it = items[i];
        it.sys = b->systems[i];
        it.offs = b->offs[i];
        it.d_qv = b->qv.as<double>() + b->qv_off[i];
        it.lam = b->lam[i];
        it.lam_base = b->lam_base[i];
        it.d_cf = b->cf.as<double>() + b->cf_off[i];
        it.d_fqt = reinterpret_cast<double2*>(b->out.as<double>() + b->fqt_off[i]);
        it.d_fq = reinterpret_cast<double2*>(b->out.as<double>() + b->fq_off[i]);
        it.d_fq2 = reinterpret_cast<double2*>(b->out.as<double>() + b->fq2_off[i]);
    }
    return items;
}

static void drop_graph(sass_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

int sass_batch_autotune(sass_batch* b, int repeats, int* q_per_lane, int* warps, int* atoms, int* split_atoms,
                        double* best_ms) {
    if (!b) return SASS_ERR_ARG;
    if (b->d.scattering != SASS_SCATTERING_ALL)
        return set_msg(b->msg, SASS_ERR_STATE, "autotuning applies to the coherent phase sum");
    CK(b->msg, cudaSetDevice(b->d.device));
    std::vector<WorkItem> items = batch_items(b);
    TuneChoice best;
    double ms = 0;
    int rc = autotune_engine(b->msg, b->eng, engine_config(b->d), items, b->st, b->ev, std::max(1, repeats), best, ms);
    if (rc) return rc;
    b->shape = best.shape;
    b->split_atoms = best.split_atoms;
    b->rec_k = best.rec_k;
    b->prepared = false;
    drop_graph(b);
    if (q_per_lane) *q_per_lane = best.shape.q_per_lane;
    if (warps) *warps = best.shape.warps;
    if (atoms) *atoms = best.shape.atoms;
    if (split_atoms) *split_atoms = best.split_atoms;
    if (best_ms) *best_ms = ms;
    b->msg.clear();
    return SASS_OK;
}

int sass_batch_set_tile(sass_batch* b, int q_per_lane, int warps, int atoms, int split_atoms) {
    if (!b) return SASS_ERR_ARG;
    PhaseShape t{q_per_lane, warps, atoms};
    if (q_per_lane != 0 && !phase_shape_supported(b->d.precision, t))
        return set_msg(b->msg, SASS_ERR_UNSUPPORTED, "phase tile Q=%d W=%d T=%d not instantiated", q_per_lane, warps,
                       atoms);
    if (split_atoms < 0 || split_atoms % kAtomGranule)
        return set_msg(b->msg, SASS_ERR_ARG, "split_atoms must be a non-negative multiple of %d", kAtomGranule);
    b->shape = q_per_lane ? t : PhaseShape{0, 0, 0};
    b->split_atoms = split_atoms;
    b->prepared = false;
    drop_graph(b);
    return SASS_OK;
}

int sass_batch_run(sass_batch* b) {
    if (!b) return SASS_ERR_ARG;
    CK(b->msg, cudaSetDevice(b->d.device));
    if (!b->prepared) {
        EngineConfig cfg = engine_config(b->d);
        cfg.shape = b->shape;
        cfg.split_atoms = b->split_atoms;
        cfg.rec_k = b->rec_k;
        std::vector<WorkItem> items = batch_items(b);
        int rc = b->eng.prepare(cfg, items, b->msg);
        if (rc) return rc;
        drop_graph(b);
        // capture the whole launch sequence once; replays need no host work
        CK(b->msg, cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        rc = b->eng.enqueue(b->st, b->msg, nullptr);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(b->st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return cuda_fail(b->msg, ce, "cudaStreamEndCapture");
        b->graph = g;
        CK(b->msg, cudaGraphInstantiate(&b->exec, b->graph, 0));
        b->prepared = true;
    }
    memset(&b->timing, 0, sizeof(b->timing));
    CK(b->msg, cudaEventRecord(b->ev[8], b->st));
    CK(b->msg, cudaGraphLaunch(b->exec, b->st));
    CK(b->msg, cudaEventRecord(b->ev[9], b->st));
    b->timing.kernel_launches = b->eng.stats().launches;
    b->timing.phase_launches = b->eng.stats().phase_launches;
    return SASS_OK;
}

int sass_batch_sync(sass_batch* b) {
    if (!b) return SASS_ERR_ARG;
    CK(b->msg, cudaEventSynchronize(b->ev[9]));
    b->timing.total_ms = ev_ms(b->ev[8], b->ev[9]);
    return read_err_word(b->msg, b->eng.err_word(), b->st);
}

int sass_batch_results(sass_batch* b, size_t system, double* fqt, double* fq, double* fq2) {
    if (!b || system >= b->systems.size()) return SASS_ERR_ARG;
    int rc = sass_batch_sync(b);
    if (rc) return rc;
    const double* o = b->out.as<double>();
    const size_t nq = b->nq[system], nf = b->systems[system]->nf;
    if (fqt) CK(b->msg, cudaMemcpy(fqt, o + b->fqt_off[system], nq * nf * 16, cudaMemcpyDeviceToHost));
    if (fq) CK(b->msg, cudaMemcpy(fq, o + b->fq_off[system], nq * 16, cudaMemcpyDeviceToHost));
    if (fq2) CK(b->msg, cudaMemcpy(fq2, o + b->fq2_off[system], nq * 16, cudaMemcpyDeviceToHost));
    return SASS_OK;
}

int sass_batch_timing(const sass_batch* b, sass_timing* out) {
    if (!b || !out) return SASS_ERR_ARG;
    *out = b->timing;
    return SASS_OK;
}

int sass_batch_info(const sass_batch* b, double* terms, uint64_t* phase_tiles, int* q_per_lane, int* warps,
                    int* atoms, int* split_atoms) {
    if (!b) return SASS_ERR_ARG;
    const EngineStats& s = b->eng.stats();
    if (terms) *terms = s.terms;
    if (phase_tiles) *phase_tiles = s.phase_tiles;
    if (q_per_lane) *q_per_lane = s.shape.q_per_lane;
    if (warps) *warps = s.shape.warps;
    if (atoms) *atoms = s.shape.atoms;
    if (split_atoms) *split_atoms = s.split_atoms;
    return SASS_OK;
}

int sass_batch_set_shell_recurrence(sass_batch* b, int shells_per_lane) {
    if (!b) return SASS_ERR_ARG;
    if (!rec_width_ok(shells_per_lane))
        return set_msg(b->msg, SASS_ERR_UNSUPPORTED, "shell recurrence width %d not instantiated", shells_per_lane);
    b->rec_k = shells_per_lane;
    b->prepared = false;
    drop_graph(b);
    return SASS_OK;
}

int sass_batch_set_phase_poly(sass_batch* b, int poly_pairs) {
    if (!b) return SASS_ERR_ARG;
    PhaseShape t = b->shape;
    t.poly_pairs = poly_pairs;
    if (poly_pairs != 0 && (t.q_per_lane == 0 || !phase_shape_supported(b->d.precision, t)))
        return set_msg(b->msg, SASS_ERR_UNSUPPORTED, "no instantiated tile shape Q=%d W=%d T=%d with %d polynomial pairs",
                       t.q_per_lane, t.warps, t.atoms, poly_pairs);
    b->shape.poly_pairs = poly_pairs;
    b->prepared = false;
    drop_graph(b);
    return SASS_OK;
}

int sass_batch_schedule(const sass_batch* b, sass_schedule* out) {
    if (!b || !out) return SASS_ERR_ARG;
    fill_schedule(b->eng.stats(), out);
    return SASS_OK;
}

void sass_batch_destroy(sass_batch* b) {
    if (!b) return;
    cudaSetDevice(b->d.device);
    if (b->st) cudaStreamSynchronize(b->st);
    drop_graph(b);
    b->eng.release();
    for (int i = 0; i < kEvents; ++i)
        if (b->ev[i]) cudaEventDestroy(b->ev[i]);
    if (b->own_stream && b->st) cudaStreamDestroy(b->st);
    delete b;
}

}  // extern "C"
