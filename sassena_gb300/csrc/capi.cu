// C ABI of the GB300 scattering path: plan object, staging, scheduling, launches.
//
// The plan owns every device buffer and the CUDA stream; sass_compute turns one
// batch of q-vectors into the rows the reference hands to HDF5WriterClient::write
// (src/services/file_writer_service.cpp:504-531): fqt [NF] complex, fq, fq2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sassena_gb300.h"
#include "kernels.h"

using namespace sassgpu;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
};

struct HostPinned {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaHostAlloc(&p, n ? n : 16, cudaHostAllocDefault);
        if (e == cudaSuccess) bytes = n ? n : 16;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
};

// Work schedule for one batch of shells (host copy + device copy).
struct Schedule {
    std::vector<VecGroup> groups;
    std::vector<SeriesChunk> chunks;
    std::vector<AtomChunk> achunks;
    std::vector<int> slot_begin;  // [nshell+1]
    std::vector<int> shell_v;     // [nshell+1]
    std::vector<double> inv_nm;   // [nshell]
    int nslots = 0;
};

constexpr int kEvents = 12;

}  // namespace

struct sass_plan {
    sass_plan_desc d{};
    int device = 0;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    size_t na = 0, nf = 0, na_pad = 0;
    int lg = 0;
    size_t L = 0;
    double center[3] = {0, 0, 0};
    bool staged = false, classes_set = false;
    DevBuf raw, xyz, cls, tw64, tw32, k64, k32, err;
    DevBuf qv, cf, bfac, sched, A, Apart, ppart, apart, a2part, fqt, fq, fq2;
    HostPinned hsched;
    std::string msg;
    sass_timing timing{};
    cudaEvent_t ev[kEvents] = {};
    PhaseTile tile{0, 0, 0};
    int nsplit_req = 0;
    // schedule cache key
    std::vector<size_t> last_offsets;
    PhaseTile last_tile{0, 0, 0};
    int last_nsplit = 0;
};

namespace {

int set_msg(sass_plan* p, int code, const char* fmt, ...) {
    if (p) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        p->msg = buf;
    }
    return code;
}

int cuda_fail(sass_plan* p, cudaError_t e, const char* what) {
    int code = (e == cudaErrorMemoryAllocation) ? SASS_ERR_OOM : SASS_ERR_CUDA;
    cudaGetLastError();  // clear sticky-free errors so the plan stays usable
    return set_msg(p, code, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(p, expr)                                           \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return cuda_fail(p, e_, #expr); \
    } while (0)

int ceil_log2(size_t n) {
    int lg = 0;
    while (((size_t)1 << lg) < n) ++lg;
    return lg;
}

unsigned bitrev(unsigned x, int lg) {
    unsigned r = 0;
    for (int i = 0; i < lg; ++i) {
        r = (r << 1) | (x & 1u);
        x >>= 1;
    }
    return r;
}

// tw[k] = exp(-2 pi i k / L), k < L/2; kbr[i] = K(bitrev(i)) with
// K(w) = sum_{tau<NF} exp(+2 pi i w tau / L) / (NF * L * (NF - tau)),
// so that mean_tau C(tau) = sum_w P(w) K(w) for C from an unnormalised inverse
// transform of the power spectrum P (smath.cpp:141-156 with the mean of
// all_vectors_scatter_device.cpp:232).
int build_tables(sass_plan* p) {
    const size_t L = p->L, nf = p->nf;
    const long double two_pi = 6.283185307179586476925286766559L;
    std::vector<long double> c(L), s(L);
    for (size_t k = 0; k < L; ++k) {
        long double a = two_pi * (long double)k / (long double)L;
        c[k] = cosl(a);
        s[k] = sinl(a);
    }
    std::vector<double2> tw64(L / 2);
    std::vector<float2> tw32(L / 2);
    for (size_t k = 0; k < L / 2; ++k) {
        tw64[k] = make_double2((double)c[k], (double)(-s[k]));
        tw32[k] = make_float2((float)c[k], (float)(-s[k]));
    }
    std::vector<double2> k64(L);
    std::vector<float2> k32(L);
    std::vector<long double> wt(nf);
    for (size_t t = 0; t < nf; ++t)
        wt[t] = 1.0L / ((long double)nf * (long double)L * (long double)(nf - t));
    for (size_t w = 0; w < L; ++w) {
        long double re = 0, im = 0;
        size_t idx = 0;  // (w * tau) mod L, advanced incrementally
        for (size_t t = 0; t < nf; ++t) {
            re += wt[t] * c[idx];
            im += wt[t] * s[idx];
            idx += w;
            if (idx >= L) idx %= L;
        }
        unsigned i = bitrev((unsigned)w, p->lg);
        k64[i] = make_double2((double)re, (double)im);
        k32[i] = make_float2((float)re, (float)im);
    }
    CK(p, p->tw64.ensure(tw64.size() * sizeof(double2)));
    CK(p, p->tw32.ensure(tw32.size() * sizeof(float2)));
    CK(p, p->k64.ensure(k64.size() * sizeof(double2)));
    CK(p, p->k32.ensure(k32.size() * sizeof(float2)));
    CK(p, cudaMemcpy(p->tw64.p, tw64.data(), tw64.size() * sizeof(double2), cudaMemcpyHostToDevice));
    CK(p, cudaMemcpy(p->tw32.p, tw32.data(), tw32.size() * sizeof(float2), cudaMemcpyHostToDevice));
    CK(p, cudaMemcpy(p->k64.p, k64.data(), k64.size() * sizeof(double2), cudaMemcpyHostToDevice));
    CK(p, cudaMemcpy(p->k32.p, k32.data(), k32.size() * sizeof(float2), cudaMemcpyHostToDevice));
    return SASS_OK;
}

int sm_count(int device) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0)
        n = 152;
    return n;
}

PhaseTile default_tile(const sass_plan* p, size_t nv_per_shell_min) {
    if (p->d.precision == SASS_PRECISION_FP64) return PhaseTile{nv_per_shell_min >= 64 ? 2 : 1, 4, 64};
    // 32*Q sub-vectors per CTA row: pick the largest Q that wastes little of a shell.
    int q = 1;
    for (int cand : {8, 4, 2}) {
        size_t per = 32 * (size_t)cand;
        size_t groups = (nv_per_shell_min + per - 1) / per;
        double waste = 1.0 - (double)nv_per_shell_min / (double)(groups * per);
        if (waste <= 0.15) {
            q = cand;
            break;
        }
    }
    return PhaseTile{q, 8, 128};
}

const void* tw_for(const sass_plan* p) {
    return p->d.precision == SASS_PRECISION_FP32 ? p->tw32.p : p->tw64.p;
}
const void* k_for(const sass_plan* p) {
    return p->d.precision == SASS_PRECISION_FP32 ? p->k32.p : p->k64.p;
}

size_t bsize(const sass_plan* p) { return p->d.precision == SASS_PRECISION_FP32 ? 4 : 8; }

void ev_record(sass_plan* p, int i) { cudaEventRecord(p->ev[i], p->st); }
float ev_ms(const sass_plan* p, int a, int b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p->ev[a], p->ev[b]) != cudaSuccess) return 0.f;
    return ms;
}

// Upload the schedule arrays of one batch into the plan's device schedule buffer.
struct SchedPtrs {
    VecGroup* groups;
    SeriesChunk* chunks;
    AtomChunk* achunks;
    int* slot_begin;
    int* shell_v;
    double* inv_nm;
};

template <class T>
size_t push_bytes(std::vector<unsigned char>& blob, const std::vector<T>& v) {
    size_t off = (blob.size() + 15) & ~(size_t)15;
    blob.resize(off + v.size() * sizeof(T));
    if (!v.empty()) memcpy(blob.data() + off, v.data(), v.size() * sizeof(T));
    return off;
}

int upload_schedule(sass_plan* p, const Schedule& s, SchedPtrs* out) {
    std::vector<unsigned char> blob;
    size_t og = push_bytes(blob, s.groups);
    size_t oc = push_bytes(blob, s.chunks);
    size_t oa = push_bytes(blob, s.achunks);
    size_t os = push_bytes(blob, s.slot_begin);
    size_t ov = push_bytes(blob, s.shell_v);
    size_t on = push_bytes(blob, s.inv_nm);
    CK(p, p->sched.ensure(blob.size()));
    CK(p, p->hsched.ensure(blob.size()));
    // the pinned staging buffer may still feed a previous async copy
    CK(p, cudaStreamSynchronize(p->st));
    memcpy(p->hsched.p, blob.data(), blob.size());
    CK(p, cudaMemcpyAsync(p->sched.p, p->hsched.p, blob.size(), cudaMemcpyHostToDevice, p->st));
    unsigned char* base = p->sched.as<unsigned char>();
    out->groups = reinterpret_cast<VecGroup*>(base + og);
    out->chunks = reinterpret_cast<SeriesChunk*>(base + oc);
    out->achunks = reinterpret_cast<AtomChunk*>(base + oa);
    out->slot_begin = reinterpret_cast<int*>(base + os);
    out->shell_v = reinterpret_cast<int*>(base + ov);
    out->inv_nm = reinterpret_cast<double*>(base + on);
    return SASS_OK;
}

// Split the series (coherent) or atoms (incoherent) of each shell into chunks so
// the correlation grid covers the GPU several times.
void plan_chunks(const sass_plan* p, size_t nshell, const size_t* offs, Schedule& s) {
    const int sms = sm_count(p->device);
    const size_t target = (size_t)sms * 4;
    s.slot_begin.assign(1, 0);
    s.chunks.clear();
    s.achunks.clear();
    int slot = 0;
    for (size_t i = 0; i < nshell; ++i) {
        size_t nm = offs[i + 1] - offs[i];
        size_t per_shell = std::max<size_t>(1, (target + nshell - 1) / nshell);
        if (p->d.scattering == SASS_SCATTERING_ALL) {
            size_t g = std::min(per_shell, nm);
            size_t len = (nm + g - 1) / g;
            for (size_t v = 0; v < nm; v += len) {
                SeriesChunk c;
                c.shell = (int)i;
                c.v_begin = (int)(offs[i] - offs[0] + v);
                c.v_end = (int)(offs[i] - offs[0] + std::min(nm, v + len));
                c.slot = slot++;
                s.chunks.push_back(c);
            }
        } else {
            size_t g = std::min(per_shell, p->na);
            size_t len = (p->na + g - 1) / g;
            for (size_t j = 0; j < p->na; j += len) {
                AtomChunk c;
                c.shell = (int)i;
                c.j_begin = (int)j;
                c.j_end = (int)std::min(p->na, j + len);
                c.slot = slot++;
                s.achunks.push_back(c);
            }
        }
        s.slot_begin.push_back(slot);
    }
    s.nslots = slot;
}

int run_batch(sass_plan* p, size_t nshell, const size_t* offs, const double* d_qv,
              const double* d_cf, double2* d_fqt, double2* d_fq, double2* d_fq2, bool& reuse) {
    const size_t nv = offs[nshell] - offs[0];
    const int dsp = p->d.dsp_type;
    // --- schedule -----------------------------------------------------------
    size_t min_nm = (size_t)-1;
    for (size_t i = 0; i < nshell; ++i) min_nm = std::min(min_nm, offs[i + 1] - offs[i]);
    PhaseTile tile = p->tile.q_per_lane ? p->tile : default_tile(p, min_nm);
    Schedule s;
    for (size_t i = 0; i < nshell; ++i) {
        s.shell_v.push_back((int)(offs[i] - offs[0]));
        s.inv_nm.push_back(1.0 / (double)(offs[i + 1] - offs[i]));
    }
    s.shell_v.push_back((int)nv);
    if (p->d.scattering == SASS_SCATTERING_ALL) {
        const int per = 32 * tile.q_per_lane;
        for (size_t i = 0; i < nshell; ++i)
            for (size_t v = offs[i]; v < offs[i + 1]; v += per) {
                VecGroup g;
                g.shell = (int)i;
                g.v0 = (int)(v - offs[0]);
                g.nv = (int)std::min<size_t>(per, offs[i + 1] - v);
                g.pad = 0;
                s.groups.push_back(g);
            }
    }
    plan_chunks(p, nshell, offs, s);
    // atom splits for the phase sum: enough CTAs to fill the GPU
    int nsplit = 1;
    if (p->d.scattering == SASS_SCATTERING_ALL) {
        const size_t ctas = ((p->nf + tile.warps - 1) / tile.warps) * s.groups.size();
        const size_t want = (size_t)sm_count(p->device) * 4;
        const int max_split = (int)(p->na_pad / tile.atoms);
        if (p->nsplit_req > 0) nsplit = std::min(p->nsplit_req, max_split);
        else if (ctas < want) nsplit = (int)std::min<size_t>(max_split, (want + ctas - 1) / ctas);
        nsplit = std::max(nsplit, 1);
    }
    SchedPtrs sp;
    int rc = upload_schedule(p, s, &sp);
    if (rc) return rc;
    (void)reuse;

    // --- scatter factors per shell ----------------------------------------------
    CK(p, p->bfac.ensure(nshell * p->na_pad * bsize(p)));
    CK(p, launch_expand_factors(d_cf, (int)p->d.nclass, (int)nshell, p->cls.as<int>(), (int)p->na_pad,
                                p->d.precision, p->bfac.p, p->st));
    p->timing.kernel_launches++;

    const bool autoc = dsp == SASS_DSP_AUTOCORRELATE;
    const size_t part_bytes = autoc ? (size_t)s.nslots * p->L * sizeof(double)
                                    : (size_t)s.nslots * p->nf * sizeof(double2);
    CK(p, p->ppart.ensure(part_bytes));
    CK(p, p->apart.ensure(s.nslots * sizeof(double2)));
    CK(p, p->a2part.ensure(s.nslots * sizeof(double)));

    CorrArgs ca{};
    ca.precision = p->d.precision;
    ca.nf = (int)p->nf;
    ca.lg = p->lg;
    ca.tw = tw_for(p);
    ca.kbr = k_for(p);
    ca.xyz = p->xyz.as<float4>();
    ca.na_pad = (int)p->na_pad;
    ca.qv = d_qv;
    ca.bfac = p->bfac.p;
    ca.shell_v = sp.shell_v;
    ca.cx = p->center[0];
    ca.cy = p->center[1];
    ca.cz = p->center[2];
    ca.restore_phase = p->d.precision == SASS_PRECISION_FP32;
    ca.ppart = p->ppart.as<double>();
    ca.apart = p->apart.as<double2>();
    ca.a2part = p->a2part.as<double>();
    ca.err = p->err.as<unsigned>();

    if (p->d.scattering == SASS_SCATTERING_ALL) {
        // --- phase sum ----------------------------------------------------------
        const bool f32 = p->d.precision == SASS_PRECISION_FP32;
        CK(p, p->A.ensure(nv * p->nf * (f32 ? sizeof(float2) : sizeof(double2))));
        double2* dst = f32 ? nullptr : p->A.as<double2>();
        if (nsplit > 1) {
            CK(p, p->Apart.ensure((size_t)nsplit * nv * p->nf * sizeof(double2)));
            dst = p->Apart.as<double2>();
        }
        PhaseSumArgs a{};
        a.precision = p->d.precision;
        a.xyz = p->xyz.as<float4>();
        a.na_pad = (int)p->na_pad;
        a.nf = (int)p->nf;
        a.bfac = p->bfac.p;
        a.qv = d_qv;
        a.groups = sp.groups;
        a.ngroups = (int)s.groups.size();
        a.nsplit = nsplit;
        size_t tiles = p->na_pad / tile.atoms;
        a.atoms_per_split = (int)(((tiles + nsplit - 1) / nsplit) * tile.atoms);
        a.out = dst;
        a.out_f32 = (f32 && nsplit == 1) ? p->A.as<float2>() : nullptr;
        a.split_stride = nv * p->nf;
        a.err = p->err.as<unsigned>();
        a.tile = tile;
        ev_record(p, 2);
        CK(p, launch_phase_sum(a, p->st));
        p->timing.kernel_launches++;
        p->timing.phase_launches++;
        if (nsplit > 1) {
            if (f32) CK(p, launch_split_reduce_f32(dst, nsplit, nv * p->nf, p->A.as<float2>(), p->st));
            else CK(p, launch_split_reduce(dst, nsplit, nv * p->nf, p->A.as<double2>(), p->st));
            p->timing.kernel_launches++;
        }
        ev_record(p, 3);
        // --- correlation / store -------------------------------------------------
        ca.A = p->A.p;
        ca.chunks = sp.chunks;
        ca.nchunks = (int)s.chunks.size();
        ev_record(p, 4);
        CK(p, launch_corr_accumulate(ca, dsp, p->st));
        p->timing.kernel_launches++;
    } else {
        ca.achunks = sp.achunks;
        ca.nchunks = (int)s.achunks.size();
        ev_record(p, 4);
        CK(p, launch_self_accumulate(ca, dsp, p->st));
        p->timing.kernel_launches++;
    }
    ev_record(p, 5);
    FinalizeArgs fa{};
    fa.nf = (int)p->nf;
    fa.lg = p->lg;
    fa.dsp = dsp;
    fa.conj_out = autoc && p->d.dsp_method == SASS_METHOD_DIRECT;
    fa.ppart = p->ppart.as<double>();
    fa.apart = p->apart.as<double2>();
    fa.a2part = p->a2part.as<double>();
    fa.slot_begin = sp.slot_begin;
    fa.inv_nm = sp.inv_nm;
    fa.tw = p->tw64.as<double2>();
    fa.fqt = d_fqt;
    fa.fq = d_fq;
    fa.fq2 = d_fq2;
    fa.nshell = (int)nshell;
    CK(p, launch_finalize(fa, p->st));
    p->timing.kernel_launches++;
    ev_record(p, 6);
    // event pairs are read after the caller synchronises; keep per-batch sums
    CK(p, cudaEventSynchronize(p->ev[6]));
    if (p->d.scattering == SASS_SCATTERING_ALL) p->timing.phase_ms += ev_ms(p, 2, 3);
    p->timing.corr_ms += ev_ms(p, 4, 5);
    p->timing.finalize_ms += ev_ms(p, 5, 6);
    return SASS_OK;
}

}  // namespace

extern "C" {

const char* sass_version(void) { return "sassena_gb300 0.1 (sm_103a)"; }

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
    const sass_plan_desc& d = *desc;
    if (d.scattering != SASS_SCATTERING_ALL && d.scattering != SASS_SCATTERING_SELF) return SASS_ERR_ARG;
    if (d.dsp_type < 0 || d.dsp_type > 2 || d.dsp_method < 0 || d.dsp_method > 1) return SASS_ERR_ARG;
    if (d.precision != SASS_PRECISION_FP64 && d.precision != SASS_PRECISION_FP32) return SASS_ERR_ARG;
    if (d.na == 0 || d.nf == 0 || d.nclass == 0) return SASS_ERR_ARG;  // NF<1 rejected as in
                                                                       // file_writer_service.cpp:23-26
    if (d.na > (size_t)1 << 30 || d.nf > (size_t)1 << 24) return SASS_ERR_ARG;
    sass_plan* p = new sass_plan();
    p->d = d;
    p->device = d.device;
    p->na = d.na;
    p->nf = d.nf;
    p->na_pad = ((d.na + kAtomGranule - 1) / kAtomGranule) * kAtomGranule;
    p->lg = std::max(2, ceil_log2(2 * d.nf));
    p->L = (size_t)1 << p->lg;
    *out = p;
    if (d.dsp_type == SASS_DSP_AUTOCORRELATE && p->lg > 13)
        return set_msg(p, SASS_ERR_UNSUPPORTED,
                       "autocorrelation supports NF <= 4096 (padded FFT length <= 8192), got NF=%zu",
                       d.nf);
    if (d.dsp_type != SASS_DSP_AUTOCORRELATE && d.nf > 4096)
        return set_msg(p, SASS_ERR_UNSUPPORTED, "dsp square/plain supports NF <= 4096, got NF=%zu",
                       d.nf);
    if (d.scattering == SASS_SCATTERING_SELF && d.dsp_type == SASS_DSP_AUTOCORRELATE &&
        fft_smem_bytes(d.precision, p->lg, (int)d.nf, true) > 227 * 1024)
        return set_msg(p, SASS_ERR_UNSUPPORTED,
                       "incoherent FP64 autocorrelation with NF=%zu exceeds shared memory", d.nf);
    CK(p, cudaSetDevice(d.device));
    if (d.stream) {
        p->st = (cudaStream_t)d.stream;
    } else {
        CK(p, cudaStreamCreateWithFlags(&p->st, cudaStreamNonBlocking));
        p->own_stream = true;
    }
    for (int i = 0; i < kEvents; ++i) CK(p, cudaEventCreate(&p->ev[i]));
    CK(p, p->err.ensure(sizeof(unsigned)));
    CK(p, p->xyz.ensure(p->nf * p->na_pad * sizeof(float4)));
    CK(p, p->cls.ensure(p->na_pad * sizeof(int)));
    int rc = build_tables(p);
    if (rc) return rc;
    p->msg.clear();
    return SASS_OK;
}

void sass_plan_destroy(sass_plan* p) {
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->st) cudaStreamSynchronize(p->st);
    DevBuf* bufs[] = {&p->raw, &p->xyz, &p->cls, &p->tw64, &p->tw32, &p->k64, &p->k32, &p->err,
                      &p->qv, &p->cf, &p->bfac, &p->sched, &p->A, &p->Apart, &p->ppart,
                      &p->apart, &p->a2part, &p->fqt, &p->fq, &p->fq2};
    for (DevBuf* b : bufs) b->release();
    p->hsched.release();
    for (int i = 0; i < kEvents; ++i)
        if (p->ev[i]) cudaEventDestroy(p->ev[i]);
    if (p->own_stream && p->st) cudaStreamDestroy(p->st);
    delete p;
}

int sass_stage_frames(sass_plan* p, const float* coords, int on_device) {
    if (!p) return SASS_ERR_ARG;
    if (!coords) return set_msg(p, SASS_ERR_ARG, "coords is NULL");
    CK(p, cudaSetDevice(p->device));
    const size_t n = p->nf * p->na * 3;
    const float* src = coords;
    std::vector<float> f0(p->na * 3);
    if (!on_device) {
        CK(p, p->raw.ensure(n * sizeof(float)));
        CK(p, cudaMemcpyAsync(p->raw.p, coords, n * sizeof(float), cudaMemcpyHostToDevice, p->st));
        src = p->raw.as<float>();
        memcpy(f0.data(), coords, f0.size() * sizeof(float));
    } else {
        CK(p, cudaMemcpyAsync(f0.data(), coords, f0.size() * sizeof(float), cudaMemcpyDeviceToHost,
                              p->st));
        CK(p, cudaStreamSynchronize(p->st));
    }
    // FP32 form: fixed centre = midpoint of frame 0's bounding box (FP64)
    double c[3] = {0, 0, 0};
    if (p->d.precision == SASS_PRECISION_FP32) {
        for (int k = 0; k < 3; ++k) {
            double lo = f0[k], hi = f0[k];
            for (size_t j = 1; j < p->na; ++j) {
                lo = std::min(lo, (double)f0[3 * j + k]);
                hi = std::max(hi, (double)f0[3 * j + k]);
            }
            c[k] = 0.5 * (lo + hi);
        }
        if (!std::isfinite(c[0]) || !std::isfinite(c[1]) || !std::isfinite(c[2]))
            return set_msg(p, SASS_ERR_ARG, "non-finite coordinates in frame 0");
    }
    memcpy(p->center, c, sizeof(c));
    CK(p, launch_stage(src, (int)p->nf, (int)p->na, (int)p->na_pad, c[0], c[1], c[2],
                       p->d.precision == SASS_PRECISION_FP32, p->xyz.as<float4>(), p->st));
    CK(p, cudaStreamSynchronize(p->st));
    p->staged = true;
    p->msg.clear();
    return SASS_OK;
}

int sass_set_atom_classes(sass_plan* p, const int32_t* atom_class, int on_device) {
    if (!p) return SASS_ERR_ARG;
    if (!atom_class) return set_msg(p, SASS_ERR_ARG, "atom_class is NULL");
    CK(p, cudaSetDevice(p->device));
    std::vector<int32_t> h(p->na_pad, -1);
    if (on_device) {
        CK(p, cudaMemcpy(h.data(), atom_class, p->na * sizeof(int32_t), cudaMemcpyDeviceToHost));
    } else {
        memcpy(h.data(), atom_class, p->na * sizeof(int32_t));
    }
    for (size_t j = 0; j < p->na; ++j)
        if (h[j] < 0 || (size_t)h[j] >= p->d.nclass)
            return set_msg(p, SASS_ERR_ARG, "atom %zu has class %d outside [0,%zu)", j, h[j],
                           p->d.nclass);
    CK(p, cudaMemcpyAsync(p->cls.p, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice, p->st));
    CK(p, cudaStreamSynchronize(p->st));
    p->classes_set = true;
    p->msg.clear();
    return SASS_OK;
}

int sass_set_phase_tile(sass_plan* p, int q_per_lane, int warps, int atoms, int atom_splits) {
    if (!p) return SASS_ERR_ARG;
    if (q_per_lane == 0) {
        p->tile = PhaseTile{0, 0, 0};
    } else {
        PhaseTile t{q_per_lane, warps, atoms};
        if (!phase_tile_supported(p->d.precision, t))
            return set_msg(p, SASS_ERR_UNSUPPORTED, "phase tile Q=%d W=%d T=%d not instantiated",
                           q_per_lane, warps, atoms);
        p->tile = t;
    }
    p->nsplit_req = atom_splits < 0 ? 0 : atom_splits;
    return SASS_OK;
}

int sass_frame_center(const sass_plan* p, double* c) {
    if (!p || !c) return SASS_ERR_ARG;
    memcpy(c, p->center, sizeof(p->center));
    return SASS_OK;
}

static int check_ready(sass_plan* p) {
    if (!p->staged) return set_msg(p, SASS_ERR_STATE, "sass_stage_frames has not been called");
    if (!p->classes_set) return set_msg(p, SASS_ERR_STATE, "sass_set_atom_classes has not been called");
    return SASS_OK;
}

static int read_device_error(sass_plan* p) {
    unsigned flag = 0;
    CK(p, cudaMemcpyAsync(&flag, p->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, p->st));
    CK(p, cudaStreamSynchronize(p->st));
    if (flag == DEV_MBAR_TIMEOUT)
        return set_msg(p, SASS_ERR_TIMEOUT, "a device-side wait exceeded its iteration limit");
    if (flag != 0) return set_msg(p, SASS_ERR_CUDA, "device error flag %u", flag);
    return SASS_OK;
}

int sass_compute(sass_plan* p, size_t nq, const size_t* offs, const double* subvectors,
                 const double* class_factors, double* fqt, double* fq, double* fq2,
                 int io_on_device) {
    if (!p) return SASS_ERR_ARG;
    int rc = check_ready(p);
    if (rc) return rc;
    if (nq == 0) return SASS_OK;
    if (!offs || !subvectors || !class_factors || !fqt || !fq || !fq2)
        return set_msg(p, SASS_ERR_ARG, "NULL argument");
    if (offs[0] != 0) return set_msg(p, SASS_ERR_ARG, "sub_offsets[0] must be 0");
    for (size_t i = 0; i < nq; ++i)
        if (offs[i + 1] <= offs[i])
            return set_msg(p, SASS_ERR_ARG, "q-vector %zu has no sub-vectors", i);
    const size_t nsub = offs[nq];
    if (nsub > (size_t)1 << 30) return set_msg(p, SASS_ERR_ARG, "too many sub-vectors");
    CK(p, cudaSetDevice(p->device));
    memset(&p->timing, 0, sizeof(p->timing));
    ev_record(p, 0);
    CK(p, cudaMemsetAsync(p->err.p, 0, sizeof(unsigned), p->st));
    const double* d_qv = subvectors;
    const double* d_cf = class_factors;
    double2 *d_fqt = reinterpret_cast<double2*>(fqt), *d_fq = reinterpret_cast<double2*>(fq),
            *d_fq2 = reinterpret_cast<double2*>(fq2);
    const size_t nclass = p->d.nclass;
    if (!io_on_device) {
        ev_record(p, 7);
        CK(p, p->qv.ensure(nsub * 3 * sizeof(double)));
        CK(p, p->cf.ensure(nq * nclass * sizeof(double)));
        CK(p, cudaMemcpyAsync(p->qv.p, subvectors, nsub * 3 * sizeof(double), cudaMemcpyHostToDevice, p->st));
        CK(p, cudaMemcpyAsync(p->cf.p, class_factors, nq * nclass * sizeof(double), cudaMemcpyHostToDevice,
                              p->st));
        ev_record(p, 8);
        p->timing.h2d_bytes = nsub * 3 * sizeof(double) + nq * nclass * sizeof(double);
        d_qv = p->qv.as<double>();
        d_cf = p->cf.as<double>();
        CK(p, p->fqt.ensure(nq * p->nf * sizeof(double2)));
        CK(p, p->fq.ensure(nq * sizeof(double2)));
        CK(p, p->fq2.ensure(nq * sizeof(double2)));
        d_fqt = p->fqt.as<double2>();
        d_fq = p->fq.as<double2>();
        d_fq2 = p->fq2.as<double2>();
    }
    // batches of whole shells bounded by the amplitude budget
    const size_t budget = p->d.amplitude_budget_bytes ? p->d.amplitude_budget_bytes : ((size_t)4 << 30);
    const size_t per_sub = p->nf * sizeof(double2);
    size_t i = 0;
    while (i < nq) {
        size_t j = i + 1;
        if (p->d.scattering == SASS_SCATTERING_ALL) {
            while (j < nq && (offs[j + 1] - offs[i]) * per_sub <= budget) ++j;
        } else {
            j = nq;  // the incoherent path keeps no amplitude buffer
        }
        bool reuse = false;
        rc = run_batch(p, j - i, offs + i, d_qv + 3 * offs[i], d_cf + nclass * i, d_fqt + i * p->nf,
                       d_fq + i, d_fq2 + i, reuse);
        if (rc) return rc;
        i = j;
    }
    if (!io_on_device) {
        ev_record(p, 9);
        CK(p, cudaMemcpyAsync(fqt, d_fqt, nq * p->nf * sizeof(double2), cudaMemcpyDeviceToHost, p->st));
        CK(p, cudaMemcpyAsync(fq, d_fq, nq * sizeof(double2), cudaMemcpyDeviceToHost, p->st));
        CK(p, cudaMemcpyAsync(fq2, d_fq2, nq * sizeof(double2), cudaMemcpyDeviceToHost, p->st));
        ev_record(p, 10);
        p->timing.d2h_bytes = nq * (p->nf + 2) * sizeof(double2);
    }
    ev_record(p, 1);
    rc = read_device_error(p);
    if (rc) return rc;
    p->timing.total_ms = ev_ms(p, 0, 1);
    if (!io_on_device) {
        p->timing.h2d_ms = ev_ms(p, 7, 8);
        p->timing.d2h_ms = ev_ms(p, 9, 10);
    }
    p->msg.clear();
    return SASS_OK;
}

int sass_amplitudes(sass_plan* p, size_t nsub, const double* subvectors, const int32_t* sub_shell,
                    size_t nshell, const double* class_factors, double* out) {
    if (!p) return SASS_ERR_ARG;
    int rc = check_ready(p);
    if (rc) return rc;
    if (p->d.scattering != SASS_SCATTERING_ALL)
        return set_msg(p, SASS_ERR_STATE, "amplitudes need a coherent (all) plan");
    if (nsub == 0) return SASS_OK;
    if (!subvectors || !sub_shell || !class_factors || !out || nshell == 0)
        return set_msg(p, SASS_ERR_ARG, "NULL argument");
    for (size_t m = 0; m < nsub; ++m)
        if (sub_shell[m] < 0 || (size_t)sub_shell[m] >= nshell)
            return set_msg(p, SASS_ERR_ARG, "sub_shell[%zu] out of range", m);
    CK(p, cudaSetDevice(p->device));
    memset(&p->timing, 0, sizeof(p->timing));
    CK(p, cudaMemsetAsync(p->err.p, 0, sizeof(unsigned), p->st));
    CK(p, p->qv.ensure(nsub * 3 * sizeof(double)));
    CK(p, p->cf.ensure(nshell * p->d.nclass * sizeof(double)));
    CK(p, cudaMemcpyAsync(p->qv.p, subvectors, nsub * 3 * sizeof(double), cudaMemcpyHostToDevice, p->st));
    CK(p, cudaMemcpyAsync(p->cf.p, class_factors, nshell * p->d.nclass * sizeof(double),
                          cudaMemcpyHostToDevice, p->st));
    CK(p, p->bfac.ensure(nshell * p->na_pad * bsize(p)));
    CK(p, launch_expand_factors(p->cf.as<double>(), (int)p->d.nclass, (int)nshell, p->cls.as<int>(),
                                (int)p->na_pad, p->d.precision, p->bfac.p, p->st));
    PhaseTile tile = p->tile.q_per_lane ? p->tile : default_tile(p, nsub);
    Schedule s;
    const int per = 32 * tile.q_per_lane;
    size_t m = 0;
    while (m < nsub) {
        size_t e = m;
        while (e < nsub && sub_shell[e] == sub_shell[m] && (int)(e - m) < per) ++e;
        VecGroup g;
        g.shell = sub_shell[m];
        g.v0 = (int)m;
        g.nv = (int)(e - m);
        g.pad = 0;
        s.groups.push_back(g);
        m = e;
    }
    SchedPtrs sp;
    rc = upload_schedule(p, s, &sp);
    if (rc) return rc;
    int nsplit = 1;
    const size_t ctas = ((p->nf + tile.warps - 1) / tile.warps) * s.groups.size();
    const int max_split = (int)(p->na_pad / tile.atoms);
    if (p->nsplit_req > 0) nsplit = std::min(p->nsplit_req, max_split);
    else if (ctas < (size_t)sm_count(p->device) * 4)
        nsplit = (int)std::min<size_t>(max_split, (sm_count(p->device) * 4 + ctas - 1) / ctas);
    nsplit = std::max(nsplit, 1);
    const bool f32 = p->d.precision == SASS_PRECISION_FP32;
    CK(p, p->A.ensure(nsub * p->nf * (f32 ? sizeof(float2) : sizeof(double2))));
    double2* dst = f32 ? nullptr : p->A.as<double2>();
    if (nsplit > 1) {
        CK(p, p->Apart.ensure((size_t)nsplit * nsub * p->nf * sizeof(double2)));
        dst = p->Apart.as<double2>();
    }
    PhaseSumArgs a{};
    a.precision = p->d.precision;
    a.xyz = p->xyz.as<float4>();
    a.na_pad = (int)p->na_pad;
    a.nf = (int)p->nf;
    a.bfac = p->bfac.p;
    a.qv = p->qv.as<double>();
    a.groups = sp.groups;
    a.ngroups = (int)s.groups.size();
    a.nsplit = nsplit;
    size_t tiles = p->na_pad / tile.atoms;
    a.atoms_per_split = (int)(((tiles + nsplit - 1) / nsplit) * tile.atoms);
    a.out = dst;
    a.out_f32 = (f32 && nsplit == 1) ? p->A.as<float2>() : nullptr;
    a.split_stride = nsub * p->nf;
    a.err = p->err.as<unsigned>();
    a.tile = tile;
    ev_record(p, 2);
    CK(p, launch_phase_sum(a, p->st));
    if (nsplit > 1) {
        if (f32) CK(p, launch_split_reduce_f32(dst, nsplit, nsub * p->nf, p->A.as<float2>(), p->st));
        else CK(p, launch_split_reduce(dst, nsplit, nsub * p->nf, p->A.as<double2>(), p->st));
    }
    ev_record(p, 3);
    std::vector<float2> a32;
    if (f32) {
        a32.resize(nsub * p->nf);
        CK(p, cudaMemcpyAsync(a32.data(), p->A.p, a32.size() * sizeof(float2), cudaMemcpyDeviceToHost, p->st));
    } else {
        CK(p, cudaMemcpyAsync(out, p->A.p, nsub * p->nf * sizeof(double2), cudaMemcpyDeviceToHost, p->st));
    }
    rc = read_device_error(p);
    if (rc) return rc;
    for (size_t i = 0; i < a32.size(); ++i) {
        out[2 * i] = a32[i].x;
        out[2 * i + 1] = a32[i].y;
    }
    p->timing.phase_ms = ev_ms(p, 2, 3);
    p->timing.phase_launches = 1;
    p->timing.kernel_launches = 2 + (nsplit > 1);
    // the FP32 form computes on centred coordinates: restore exp(i q.c) in FP64
    if (p->d.precision == SASS_PRECISION_FP32) {
        for (size_t v = 0; v < nsub; ++v) {
            const double* q = subvectors + 3 * v;
            double ph = q[0] * p->center[0] + q[1] * p->center[1] + q[2] * p->center[2];
            double c = cos(ph), s2 = sin(ph);
            for (size_t f = 0; f < p->nf; ++f) {
                double* z = out + 2 * (v * p->nf + f);
                double re = z[0] * c - z[1] * s2, im = z[0] * s2 + z[1] * c;
                z[0] = re;
                z[1] = im;
            }
        }
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

}  // extern "C"
