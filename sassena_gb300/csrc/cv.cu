// Learned control variate for the Monte Carlo orientational average (C ABI).
//
// The reference averages over NM random orientations with equal weights
// (all_vectors_scatter_device.cpp:355-360). Here a small network g(u, |q|) ~ |A(q u)|^2,
// trained on the GPU on exact intensities this library computes, is used as a control
// variate: with G = (1/4pi) integral g dOmega from dense quadrature,
//   S_cv(t) = (1/M) sum_i C_i(t) - beta(t) ((1/M) sum_i g(u_i) - G)
// is unbiased for any fixed beta. beta(t) = Cov(C(t), g)/Var(g) is estimated on one half
// of the directions and applied to the other half (cross-fitting), so the estimate stays
// unbiased. The needed sums (1/M) sum_i g_i C_i(t) come from one extra correlation pass
// over amplitudes scaled by sqrt(g_i) (the autocorrelation is quadratic in A).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sassena_gb300.h"
#include "engine.h"
#include "mlp.h"
#include "plan.h"

using namespace sassgpu;

struct sass_mlp {
    int device = 0;
    cudaStream_t st = nullptr;
    DevBuf master, w16, grad, m, v, loss, X, T, Y, qlen, gbar, wsqrt, outs;
    DevBuf scratch;  // per-CTA partial gradients and quadrature parts (fixed-order sums)
    double q_mid = 1.0, q_half = 1.0, y_mean = 0.0, y_std = 1.0;
    int step = 0;
    std::string msg;
};

namespace {

int fail(std::string& m, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    m = buf;
    return code;
}

int cfail(std::string& m, cudaError_t e, const char* what) {
    cudaGetLastError();
    return fail(m, e == cudaErrorMemoryAllocation ? SASS_ERR_OOM : SASS_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

#define CK(m, expr)                                         \
    do {                                                    \
        cudaError_t e_ = (expr);                            \
        if (e_ != cudaSuccess) return cfail(m, e_, #expr);  \
    } while (0)

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int upload_params(sass_mlp* n, const std::vector<float>& p) {
    std::vector<__nv_bfloat16> b(p.size());
    for (size_t i = 0; i < p.size(); ++i) b[i] = __float2bfloat16_rn(p[i]);
    CK(n->msg, cudaMemcpy(n->master.p, p.data(), p.size() * 4, cudaMemcpyHostToDevice));
    CK(n->msg, cudaMemcpy(n->w16.p, b.data(), b.size() * 2, cudaMemcpyHostToDevice));
    return SASS_OK;
}

int predict(sass_mlp* n, const float* x, size_t count, std::vector<float>& y) {
    CK(n->msg, n->X.ensure(count * 4 * sizeof(float)));
    CK(n->msg, n->Y.ensure(count * sizeof(float)));
    CK(n->msg, cudaMemcpy(n->X.p, x, count * 4 * sizeof(float), cudaMemcpyHostToDevice));
    CK(n->msg, launch_mlp_forward(n->w16.as<__nv_bfloat16>(), n->X.as<float>(), (int)count, n->Y.as<float>(),
                                  sm_count(n->device), n->st));
    y.resize(count);
    CK(n->msg, cudaMemcpyAsync(y.data(), n->Y.p, count * sizeof(float), cudaMemcpyDeviceToHost, n->st));
    CK(n->msg, cudaStreamSynchronize(n->st));
    return SASS_OK;
}

}  // namespace

extern "C" {

const char* sass_mlp_error(const sass_mlp* n) { return n ? n->msg.c_str() : ""; }

int sass_mlp_create(int device, uint64_t seed, sass_mlp** out) {
    if (!out) return SASS_ERR_ARG;
    sass_mlp* n = new sass_mlp();
    *out = n;
    n->device = device;
    CK(n->msg, cudaSetDevice(device));
    CK(n->msg, cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking));
    CK(n->msg, n->master.ensure(kMlpParams * 4));
    CK(n->msg, n->w16.ensure(kMlpParams * 2));
    CK(n->msg, n->grad.ensure(kMlpParams * 4));
    CK(n->msg, n->m.ensure(kMlpParams * 4));
    CK(n->msg, n->v.ensure(kMlpParams * 4));
    CK(n->msg, n->loss.ensure(8));
    CK(n->msg, cudaMemset(n->m.p, 0, kMlpParams * 4));
    CK(n->msg, cudaMemset(n->v.p, 0, kMlpParams * 4));
    // Glorot-uniform weights, zero biases (seeded)
    const int H = kMlpHidden;
    std::vector<float> p(kMlpParams, 0.f);
    uint64_t s = seed;
    auto uni = [&](double a) { return (float)(a * (2.0 * ((splitmix(s) >> 11) * (1.0 / 9007199254740992.0)) - 1.0)); };
    for (int i = 0; i < H * 4; ++i) p[i] = uni(std::sqrt(6.0 / (4 + H)));
    for (int i = 0; i < H * H; ++i) p[H * 4 + H + i] = uni(std::sqrt(6.0 / (2 * H)));
    for (int i = 0; i < H; ++i) p[H * 4 + H + H * H + H + i] = uni(std::sqrt(6.0 / (H + 1)));
    return upload_params(n, p);
}

void sass_mlp_destroy(sass_mlp* n) {
    if (!n) return;
    cudaSetDevice(n->device);
    if (n->st) {
        cudaStreamSynchronize(n->st);
        cudaStreamDestroy(n->st);
    }
    delete n;
}

int sass_mlp_set_scaling(sass_mlp* n, double q_mid, double q_half, double y_mean, double y_std) {
    if (!n || q_half <= 0 || y_std <= 0) return SASS_ERR_ARG;
    n->q_mid = q_mid;
    n->q_half = q_half;
    n->y_mean = y_mean;
    n->y_std = y_std;
    return SASS_OK;
}

int sass_mlp_param_count(void) { return kMlpParams; }

int sass_mlp_get_params(const sass_mlp* n, float* master, uint16_t* bf16) {
    if (!n) return SASS_ERR_ARG;
    if (master && cudaMemcpy(master, n->master.p, kMlpParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return SASS_ERR_CUDA;
    if (bf16 && cudaMemcpy(bf16, n->w16.p, kMlpParams * 2, cudaMemcpyDeviceToHost) != cudaSuccess) return SASS_ERR_CUDA;
    return SASS_OK;
}

int sass_mlp_set_params(sass_mlp* n, const float* master) {
    if (!n || !master) return SASS_ERR_ARG;
    CK(n->msg, cudaSetDevice(n->device));
    return upload_params(n, std::vector<float>(master, master + kMlpParams));
}

// Gradient of mean (y - t)^2 over all n samples at the current weights (no update).
int sass_mlp_gradient(sass_mlp* n, const float* x, const float* t, size_t count, float* grad, double* loss) {
    if (!n || !x || !t || !grad || count == 0) return SASS_ERR_ARG;
    CK(n->msg, cudaSetDevice(n->device));
    CK(n->msg, n->X.ensure(count * 16));
    CK(n->msg, n->T.ensure(count * 4));
    CK(n->msg, cudaMemcpy(n->X.p, x, count * 16, cudaMemcpyHostToDevice));
    CK(n->msg, cudaMemcpy(n->T.p, t, count * 4, cudaMemcpyHostToDevice));
    CK(n->msg, n->scratch.ensure(mlp_train_scratch_bytes(sm_count(n->device))));
    CK(n->msg, launch_mlp_train(n->w16.as<__nv_bfloat16>(), n->X.as<float>(), n->T.as<float>(), (int)count,
                                n->grad.as<float>(), n->loss.as<double>(), n->scratch.p, sm_count(n->device),
                                n->st));
    CK(n->msg, cudaMemcpyAsync(grad, n->grad.p, kMlpParams * 4, cudaMemcpyDeviceToHost, n->st));
    double l = 0;
    CK(n->msg, cudaMemcpyAsync(&l, n->loss.p, 8, cudaMemcpyDeviceToHost, n->st));
    CK(n->msg, cudaStreamSynchronize(n->st));
    if (loss) *loss = l;
    return SASS_OK;
}

// Adam on mini-batches (consecutive windows of the data, which the caller shuffles).
int sass_mlp_train(sass_mlp* n, const float* x, const float* t, size_t count, int steps, int batch, double lr,
                   double* last_loss) {
    if (!n || !x || !t || count == 0 || steps < 0 || batch <= 0) return SASS_ERR_ARG;
    CK(n->msg, cudaSetDevice(n->device));
    CK(n->msg, n->X.ensure(count * 16));
    CK(n->msg, n->T.ensure(count * 4));
    CK(n->msg, cudaMemcpy(n->X.p, x, count * 16, cudaMemcpyHostToDevice));
    CK(n->msg, cudaMemcpy(n->T.p, t, count * 4, cudaMemcpyHostToDevice));
    const size_t b = std::min<size_t>((size_t)batch, count);
    CK(n->msg, n->scratch.ensure(mlp_train_scratch_bytes(sm_count(n->device))));
    CK(n->msg, cudaMemsetAsync(n->loss.p, 0, 8, n->st));
    size_t off = 0;
    for (int k = 0; k < steps; ++k) {
        if (off + b > count) off = 0;
        CK(n->msg, launch_mlp_train(n->w16.as<__nv_bfloat16>(), n->X.as<float>() + off * 4, n->T.as<float>() + off,
                                    (int)b, n->grad.as<float>(), n->loss.as<double>(), n->scratch.p,
                                    sm_count(n->device), n->st));
        CK(n->msg, launch_mlp_adam(n->master.as<float>(), n->w16.as<__nv_bfloat16>(), n->grad.as<float>(),
                                   n->m.as<float>(), n->v.as<float>(), (float)lr, ++n->step, n->st));
        off += b;
    }
    double l = 0;
    CK(n->msg, cudaMemcpyAsync(&l, n->loss.p, 8, cudaMemcpyDeviceToHost, n->st));
    CK(n->msg, cudaStreamSynchronize(n->st));
    if (last_loss) *last_loss = l;
    return SASS_OK;
}

int sass_mlp_predict(sass_mlp* n, const float* x, size_t count, float* y) {
    if (!n || !x || !y) return SASS_ERR_ARG;
    if (count == 0) return SASS_OK;
    CK(n->msg, cudaSetDevice(n->device));
    std::vector<float> out;
    int rc = predict(n, x, count, out);
    if (rc) return rc;
    memcpy(y, out.data(), count * sizeof(float));
    return SASS_OK;
}

// G(|q|) = (1/4pi) integral g dOmega per shell on a spherical-Fibonacci set of npoints.
int sass_mlp_sphere_mean(sass_mlp* n, const double* qlen, size_t nshell, size_t npoints, double* gbar) {
    if (!n || !qlen || !gbar || nshell == 0 || npoints == 0) return SASS_ERR_ARG;
    CK(n->msg, cudaSetDevice(n->device));
    CK(n->msg, n->qlen.ensure(nshell * 8));
    CK(n->msg, n->gbar.ensure(nshell * 8));
    CK(n->msg, cudaMemcpy(n->qlen.p, qlen, nshell * 8, cudaMemcpyHostToDevice));
    CK(n->msg, n->scratch.ensure(std::max(mlp_sphere_scratch_bytes((int)nshell, (int)npoints, sm_count(n->device)),
                                          mlp_train_scratch_bytes(sm_count(n->device)))));
    CK(n->msg, launch_mlp_sphere(n->w16.as<__nv_bfloat16>(), n->qlen.as<double>(), (int)nshell, (int)npoints,
                                 (float)n->q_mid, (float)n->q_half, (float)n->y_mean, (float)n->y_std,
                                 n->gbar.as<double>(), n->scratch.as<double>(), sm_count(n->device), n->st));
    CK(n->msg, cudaMemcpyAsync(gbar, n->gbar.p, nshell * 8, cudaMemcpyDeviceToHost, n->st));
    CK(n->msg, cudaStreamSynchronize(n->st));
    return SASS_OK;
}

// Control-variate orientational average for a coherent plan (dsp autocorrelate or square).
//   qlen [nq], dirs [m][3] unit vectors (shared by all shells, as the reference's
//   orientation set is, abstract_vectors_scatter_device.cpp:123-129), class_factors
//   [nq][nclass]. Outputs [nq][nf][2] (fqt) and [nq][2] (fq): the control-variate
//   estimate and the plain Monte Carlo estimate on the same m directions. diag [nq][3]:
//   G (quadrature mean of g), mean g over the directions, Var g (optional).
int sass_compute_cv(sass_plan* p, sass_mlp* net, size_t nq, const double* qlen, size_t m, const double* dirs,
                    const double* class_factors, size_t nquad, double* fqt_cv, double* fqt_mc, double* fq_cv,
                    double* fq_mc, double* diag) {
    if (!p) return SASS_ERR_ARG;
    if (!net || !qlen || !dirs || !class_factors || !fqt_cv || !fqt_mc || !fq_cv || !fq_mc || nq == 0)
        return fail(p->msg, SASS_ERR_ARG, "NULL argument");
    if (!p->sys.staged || !p->sys.classes_set) return fail(p->msg, SASS_ERR_STATE, "plan not staged");
    if (p->d.scattering != SASS_SCATTERING_ALL || p->d.dsp_type == SASS_DSP_PLAIN)
        return fail(p->msg, SASS_ERR_UNSUPPORTED, "control variate needs coherent autocorrelate or square");
    if (m < 4) return fail(p->msg, SASS_ERR_ARG, "need at least 4 directions");
    CK(p->msg, cudaSetDevice(p->d.device));
    const size_t nf = p->sys.nf, nclass = p->d.nclass, h = m / 2, nsub = nq * m;
    // g at every (shell, direction)
    std::vector<float> x(nsub * 4);
    for (size_t s = 0; s < nq; ++s)
        for (size_t i = 0; i < m; ++i) {
            float* r = &x[(s * m + i) * 4];
            r[0] = (float)dirs[3 * i];
            r[1] = (float)dirs[3 * i + 1];
            r[2] = (float)dirs[3 * i + 2];
            r[3] = (float)((qlen[s] - net->q_mid) / net->q_half);
        }
    std::vector<float> y;
    int rc = predict(net, x.data(), nsub, y);
    if (rc) return fail(p->msg, rc, "%s", net->msg.c_str());
    std::vector<double> g(nsub), wsq(nsub);
    for (size_t k = 0; k < nsub; ++k) {
        g[k] = std::exp((double)y[k] * net->y_std + net->y_mean);
        wsq[k] = std::sqrt(g[k]);
    }
    std::vector<double> G(nq);
    rc = sass_mlp_sphere_mean(net, qlen, nq, nquad ? nquad : 32768, G.data());
    if (rc) return fail(p->msg, rc, "%s", net->msg.c_str());
    // Two work items over the same trajectory: every shell's directions [0, h) (half A)
    // and [h, m) (half B). Each half is a product set (|q_s| times one direction list), so
    // linear shell scans take the shell-recurrence kernel. Entries: half A rows [0, nq),
    // half B rows [nq, 2 nq); sub-vectors and sqrt(g) in the same half-major order.
    const size_t ne = 2 * nq;
    std::vector<double> sv(nsub * 3), wsq_h(nsub);
    std::vector<size_t> offs_half[2];
    {
        size_t k = 0;
        for (int half = 0; half < 2; ++half) {
            const size_t i0 = half ? h : 0, i1 = half ? m : h;
            offs_half[half].push_back(0);
            for (size_t s = 0; s < nq; ++s) {
                for (size_t i = i0; i < i1; ++i, ++k) {
                    for (int c = 0; c < 3; ++c) sv[3 * k + c] = qlen[s] * dirs[3 * i + c];
                    wsq_h[k] = wsq[s * m + i];
                }
                offs_half[half].push_back(offs_half[half].back() + (i1 - i0));
            }
        }
    }
    CK(p->msg, p->qv.ensure(sv.size() * 8));
    CK(p->msg, p->cf.ensure(nq * nclass * 8));
    CK(p->msg, net->wsqrt.ensure(nsub * 8));
    CK(p->msg, net->outs.ensure(2 * ne * (nf + 2) * 16));
    CK(p->msg, cudaMemcpy(p->qv.p, sv.data(), sv.size() * 8, cudaMemcpyHostToDevice));
    CK(p->msg, cudaMemcpy(p->cf.p, class_factors, nq * nclass * 8, cudaMemcpyHostToDevice));
    CK(p->msg, cudaMemcpy(net->wsqrt.p, wsq_h.data(), nsub * 8, cudaMemcpyHostToDevice));
    double2* o = net->outs.as<double2>();
    double2* ow = o + ne * (nf + 2);  // weighted block, same layout
    std::vector<WorkItem> items(2);
    for (int half = 0; half < 2; ++half) {
        WorkItem& it = items[half];
        const size_t first = half ? offs_half[0].back() : 0;  // sub-vector offset of the half
        const size_t row = half ? nq : 0;
        it.sys = &p->sys;
        it.offs = offs_half[half];
        it.d_qv = p->qv.as<double>() + 3 * first;
        if (p->d.precision == SASS_PRECISION_FP32 && p->rec_k >= 0)
            detect_product(sv.data() + 3 * first, it.offs, it.lam, it.lam_base);
        it.d_cf = p->cf.as<double>();
        it.d_fqt = o + row * nf;
        it.d_fq = o + ne * nf + row;
        it.d_fq2 = o + ne * nf + ne + row;
        it.d_wsqrt = net->wsqrt.as<double>() + first;
        it.d_fqt_w = ow + row * nf;
        it.d_fq_w = ow + ne * nf + row;
        it.d_fq2_w = ow + ne * nf + ne + row;
    }
    EngineConfig cfg;
    cfg.scattering = p->d.scattering;
    cfg.dsp = p->d.dsp_type;
    cfg.method = p->d.dsp_method;
    cfg.precision = p->d.precision;
    cfg.device = p->d.device;
    cfg.shape = p->shape;
    cfg.split_atoms = p->split_atoms;
    cfg.rec_k = p->rec_k;
    rc = p->eng.prepare(cfg, items, p->msg);
    if (rc) return rc;
    rc = p->eng.enqueue(p->st, p->msg, p->ev);
    if (rc) return rc;
    std::vector<double2> host(2 * ne * (nf + 2));
    CK(p->msg, cudaMemcpyAsync(host.data(), o, host.size() * 16, cudaMemcpyDeviceToHost, p->st));
    CK(p->msg, cudaStreamSynchronize(p->st));
    unsigned flag = 0;
    CK(p->msg, cudaMemcpy(&flag, p->eng.err_word(), 4, cudaMemcpyDeviceToHost));
    if (flag) return fail(p->msg, SASS_ERR_TIMEOUT, "device error flag %u", flag);
    const double2* S = host.data();
    const double2* Sq = S + ne * nf;
    const double2* W = S + ne * (nf + 2);
    const double2* Wq = W + ne * nf;
    for (size_t s = 0; s < nq; ++s) {
        double gb[2], var[2];
        for (int half = 0; half < 2; ++half) {
            const size_t i0 = s * m + (half ? h : 0), i1 = half ? (s + 1) * m : s * m + h;
            double a = 0, b = 0;
            for (size_t i = i0; i < i1; ++i) {
                a += g[i];
                b += g[i] * g[i];
            }
            gb[half] = a / (i1 - i0);
            var[half] = b / (i1 - i0) - gb[half] * gb[half];
        }
        // beta_X(t) from half X, applied to the other half (cross-fitting)
        auto combine = [&](const double2* sA, const double2* sB, const double2* wA, const double2* wB, double* cv,
                           double* mc) {
            double2 beta[2];
            const double2* sx[2] = {sA, sB};
            const double2* wx[2] = {wA, wB};
            for (int half = 0; half < 2; ++half) {
                const double v = var[half] > 1e-300 ? var[half] : 0.0;
                beta[half].x = v > 0 ? (wx[half]->x - gb[half] * sx[half]->x) / v : 0.0;
                beta[half].y = v > 0 ? (wx[half]->y - gb[half] * sx[half]->y) / v : 0.0;
            }
            const double dA = gb[0] - G[s], dB = gb[1] - G[s];
            cv[0] = 0.5 * ((sA->x - beta[1].x * dA) + (sB->x - beta[0].x * dB));
            cv[1] = 0.5 * ((sA->y - beta[1].y * dA) + (sB->y - beta[0].y * dB));
            mc[0] = 0.5 * (sA->x + sB->x);
            mc[1] = 0.5 * (sA->y + sB->y);
        };
        for (size_t t = 0; t < nf; ++t)
            combine(S + s * nf + t, S + (nq + s) * nf + t, W + s * nf + t, W + (nq + s) * nf + t,
                    fqt_cv + 2 * (s * nf + t), fqt_mc + 2 * (s * nf + t));
        combine(Sq + s, Sq + nq + s, Wq + s, Wq + nq + s, fq_cv + 2 * s, fq_mc + 2 * s);
        if (diag) {
            diag[3 * s] = G[s];
            diag[3 * s + 1] = 0.5 * (gb[0] + gb[1]);
            diag[3 * s + 2] = 0.5 * (var[0] + var[1]);
        }
    }
    p->msg.clear();
    return SASS_OK;
}

}  // extern "C"
