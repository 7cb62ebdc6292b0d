// Staging pre-pass on the device: the alignments and translation motions that the
// reference applies to every frame in CoordinateSets::load
// (src/sample/coordinate_sets.cpp:244-368), then the reduction to the stager target and
// the float32 staging (src/stager/data_stager.cpp:102-118).
//
// The reference works on each frame in FP64 (coor2_t, include/common.hpp:36-39) and stores
// float32 at the end. Here the whole trajectory is promoted once to an FP64 array
// W[nf][nsys][3] in HBM and every step runs over all frames at once:
//   * centres of mass: each frame's list is summed in list order with separately rounded
//     multiplies and adds (m += m_i; x += x_i * m_i), the reference's loop in
//     center_of_mass.cpp:160-264, so the centres are the reference's bit for bit (one lane
//     per frame over tiles of products staged in shared memory);
//   * translations and the fit's apply step: one thread per (frame, atom), again with
//     explicitly rounded operations in the reference's order;
//   * the fit's 3x3 correlation matrices (center_of_mass.cpp:79-98) are summed per frame on
//     the device; their SVDs (3x3, per frame) run on the host with a one-sided Jacobi
//     method, and the rotations go back to the device.
// Everything stays resident; the host sees nf x 9 doubles per fit step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sassena_gb300.h"
#include "engine.h"
#include "kernels.h"
#include "plan.h"

namespace sassgpu {
namespace {

constexpr int kPerFrameThreads = 32;  // one thread per frame (small per-frame kernels)

__global__ void pp_promote_kernel(const float* __restrict__ in, size_t n, double* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

// com[f] = sum_i m_i r_i / sum_i m_i over the list, r_i = base[f * stride + 3 idx[i]]
// (idx NULL: i), summed in list order without fused multiply-adds, as the reference's loop
// (center_of_mass.cpp:160-264). One CTA per 32 frames, one frame per lane: tiles of 32 list
// entries x 32 frames are loaded cooperatively (consecutive threads read consecutive atoms of a
// frame) and turned into the products m_i r_i in shared memory; then warp w runs accumulator w
// (m, x, y, z) with lane = frame through the tile in list order.
constexpr int kComFrames = 32, kComTile = 32, kComThreads = 128;

__global__ void __launch_bounds__(kComThreads) pp_com_kernel(const double* __restrict__ base, size_t stride,
                                                             const size_t* __restrict__ idx,
                                                             const double* __restrict__ mass, size_t n, int nf,
                                                             double* __restrict__ com) {
    __shared__ double S[4][kComTile][kComFrames + 1];
    const int f0 = blockIdx.x * kComFrames, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double acc = 0.0;
    for (size_t i0 = 0; i0 < n; i0 += kComTile) {
        for (int t = threadIdx.x; t < kComTile * kComFrames; t += kComThreads) {
            const int e = t % kComTile, fl = t / kComTile;
            const size_t i = i0 + e;
            double mi = 0.0, px = 0.0, py = 0.0, pz = 0.0;
            if (i < n && f0 + fl < nf) {
                const size_t j = idx ? idx[i] : i;
                const double* r = base + (size_t)(f0 + fl) * stride + 3 * j;
                mi = mass[i];
                px = __dmul_rn(r[0], mi);
                py = __dmul_rn(r[1], mi);
                pz = __dmul_rn(r[2], mi);
            }
            S[0][e][fl] = mi;
            S[1][e][fl] = px;
            S[2][e][fl] = py;
            S[3][e][fl] = pz;
        }
        __syncthreads();
        const int cnt = (int)min((size_t)kComTile, n - i0);
        for (int e = 0; e < cnt; ++e) acc = __dadd_rn(acc, S[warp][e][lane]);
        __syncthreads();
    }
    S[warp][0][lane] = acc;  // totals: m, x, y, z of frame f0 + lane
    __syncthreads();
    const int f = f0 + lane;
    if (warp == 0 && f < nf) {
        double* o = com + 3 * (size_t)f;
        const double m = S[0][0][lane];
        if (n == 0) {
            o[0] = o[1] = o[2] = 0.0;
        } else {
            o[0] = __ddiv_rn(S[1][0][lane], m);
            o[1] = __ddiv_rn(S[2][0][lane], m);
            o[2] = __ddiv_rn(S[3][0][lane], m);
        }
    }
}

// Per-frame translation vectors. a, b: [nf][3] or one row broadcast (a_one, b_one).
//   mode 0: t = -a;  mode 1: t = a - b;  mode 2: t = b
__global__ void pp_combine_kernel(const double* __restrict__ a, int a_one, const double* __restrict__ b, int b_one,
                                  int mode, int nf, double* __restrict__ t) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    for (int k = 0; k < 3; ++k) {
        const double av = a ? a[3 * (a_one ? 0 : f) + k] : 0.0;
        const double bv = b ? b[3 * (b_one ? 0 : f) + k] : 0.0;
        t[3 * f + k] = mode == 0 ? -av : mode == 1 ? __dsub_rn(av, bv) : bv;
    }
}

// W[f][sel[k]] += t[f] (CartesianCoordinateSet::translate, coordinate_set.cpp:107-143).
__global__ void pp_translate_kernel(double* __restrict__ W, size_t nsys, const size_t* __restrict__ sel, size_t nsel,
                                    int nf, const double* __restrict__ t) {
    const size_t n = (size_t)nf * nsel;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t f = i / nsel, k = i - f * nsel;
        double* r = W + (f * nsys + sel[k]) * 3;
        const double* tf = t + 3 * f;
        r[0] = __dadd_rn(r[0], tf[0]);
        r[1] = __dadd_rn(r[1], tf[1]);
        r[2] = __dadd_rn(r[2], tf[2]);
    }
}

// Translation motion: x -> ((x + (-c)) + t_f) + c, c = c[f] or c[0] (c_one)
// (coordinate_sets.cpp:296-315 with the walkers' 4x4 translation, motion_walker.cpp).
__global__ void pp_motion_kernel(double* __restrict__ W, size_t nsys, const size_t* __restrict__ sel, size_t nsel,
                                 int nf, const double* __restrict__ c, int c_one, const double* __restrict__ t) {
    const size_t n = (size_t)nf * nsel;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t f = i / nsel, k = i - f * nsel;
        double* r = W + (f * nsys + sel[k]) * 3;
        const double* cf = c + 3 * (c_one ? 0 : f);
        const double* tf = t + 3 * f;
        for (int d = 0; d < 3; ++d) r[d] = __dadd_rn(__dadd_rn(__dadd_rn(r[d], -cf[d]), tf[d]), cf[d]);
    }
}

// C[f][i] = W[f][idx[i]]: the fit's reduced copy (CoordinateSet(cs, system, ref), coordinate_set.cpp:32-67).
__global__ void pp_gather_kernel(const double* __restrict__ W, size_t nsys, const size_t* __restrict__ idx, size_t n,
                                 int nf, double* __restrict__ C) {
    const size_t tot = (size_t)nf * n * 3;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const size_t d = i % 3, e = i / 3, f = e / n, k = e - f * n;
        C[i] = W[(f * nsys + idx[k]) * 3 + d];
    }
}

// K[f] = sum_i m_i (u_i v_i^T), u_i = R_i - ref, v_i = C[f][i] - pos[f] (center_of_mass.cpp:79-98),
// R_i = reference[i] or (NULL) C[f][i]; each element m_i * (u_r * v_c), summed in order. Layout as
// pp_com_kernel: tiles of 16 entries x 32 frames of the nine products in shared memory, then warp w
// runs elements w, w + 4, w + 8 of K with lane = frame.
constexpr int kKmatTile = 16;

__global__ void __launch_bounds__(kComThreads) pp_kmat_kernel(const double* __restrict__ C, const double* __restrict__ ref_xyz,
                                                              const double* __restrict__ mass, size_t n, int nf,
                                                              const double* __restrict__ pos, const double* __restrict__ ref,
                                                              int ref_one, double* __restrict__ K) {
    __shared__ double S[9][kKmatTile][kComFrames + 1];
    const int f0 = blockIdx.x * kComFrames, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double acc[3] = {0.0, 0.0, 0.0};
    for (size_t i0 = 0; i0 < n; i0 += kKmatTile) {
        for (int t = threadIdx.x; t < kKmatTile * kComFrames; t += kComThreads) {
            const int e = t % kKmatTile, fl = t / kKmatTile;
            const size_t i = i0 + e;
            const int f = f0 + fl;
            double tv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (i < n && f < nf) {
                const double* cf = C + ((size_t)f * n + i) * 3;
                const double* rr = ref_xyz ? ref_xyz + 3 * i : cf;
                const double* pf = pos + 3 * (size_t)f;
                const double* qf = ref + 3 * (size_t)(ref_one ? 0 : f);
                const double mi = mass[i];
                double u[3], v[3];
                for (int d = 0; d < 3; ++d) {
                    v[d] = __dsub_rn(cf[d], pf[d]);
                    u[d] = __dsub_rn(rr[d], qf[d]);
                }
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) tv[3 * r + c] = __dmul_rn(mi, __dmul_rn(u[r], v[c]));
            }
#pragma unroll
            for (int q = 0; q < 9; ++q) S[q][e][fl] = tv[q];
        }
        __syncthreads();
        const int cnt = (int)min((size_t)kKmatTile, n - i0);
        for (int e = 0; e < cnt; ++e)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int q = warp + 4 * k;
                if (q < 9) acc[k] = __dadd_rn(acc[k], S[q][e][lane]);
            }
        __syncthreads();
    }
    const int f = f0 + lane;
    if (f < nf)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int q = warp + 4 * k;
            if (q < 9) K[9 * (size_t)f + q] = acc[k];
        }
}

// C[f][i] = R[f] (C[f][i] - pos[f]) + ref (center_of_mass.cpp:114-128; ublas prod order).
__global__ void pp_fit_apply_kernel(double* __restrict__ C, size_t n, int nf, const double* __restrict__ R,
                                    const double* __restrict__ pos, const double* __restrict__ ref, int ref_one) {
    const size_t tot = (size_t)nf * n;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const size_t f = i / n;
        double* c = C + 3 * i;
        const double* Rf = R + 9 * f;
        const double* pf = pos + 3 * f;
        const double* qf = ref + 3 * (ref_one ? 0 : f);
        const double b0 = __dsub_rn(c[0], pf[0]), b1 = __dsub_rn(c[1], pf[1]), b2 = __dsub_rn(c[2], pf[2]);
        for (int r = 0; r < 3; ++r) {
            const double a = __dadd_rn(__dadd_rn(__dmul_rn(Rf[3 * r], b0), __dmul_rn(Rf[3 * r + 1], b1)),
                                       __dmul_rn(Rf[3 * r + 2], b2));
            c[r] = __dadd_rn(a, qf[r]);
        }
    }
}

// W[f][sel[k]] = C[f][src[k]] (the write-back walk, center_of_mass.cpp:130-156).
__global__ void pp_scatter_kernel(double* __restrict__ W, size_t nsys, const size_t* __restrict__ sel,
                                  const size_t* __restrict__ src, size_t nsel, const double* __restrict__ C,
                                  size_t n, int nf) {
    const size_t tot = (size_t)nf * nsel;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const size_t f = i / nsel, k = i - f * nsel;
        const double* c = C + (f * n + src[k]) * 3;
        double* r = W + (f * nsys + sel[k]) * 3;
        r[0] = c[0];
        r[1] = c[1];
        r[2] = c[2];
    }
}

// out[f][t] = float(W[f][target[t]]) (the stager's float32 store).
__global__ void pp_target_kernel(const double* __restrict__ W, size_t nsys, const size_t* __restrict__ target,
                                 size_t na, int nf, float* __restrict__ out) {
    const size_t tot = (size_t)nf * na * 3;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const size_t d = i % 3, e = i / 3, f = e / na, t = e - f * na;
        out[i] = __double2float_rn(W[(f * nsys + target[t]) * 3 + d]);
    }
}

unsigned grid_for(size_t n, int threads) {
    return grid_blocks(n, threads, 32);
}

// ---------------------------------------------------------------------------------------
// 3x3 fit rotation (host)
// ---------------------------------------------------------------------------------------
double det3(const double* a) {
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) + a[2] * (a[3] * a[7] - a[4] * a[6]);
}

// K = U diag(S) V^T by one-sided Jacobi rotations of K's columns (Hestenes), singular
// values in descending order as LAPACK's gesvd returns them. Row-major 3x3.
void svd3(const double* K, double* U, double* S, double* V) {
    double A[9];
    memcpy(A, K, sizeof(A));
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 64; ++sweep) {
        bool rotated = false;
        for (const auto& pq : pairs) {
            const int p = pq[0], q = pq[1];
            double alpha = 0, beta = 0, gamma = 0;
            for (int r = 0; r < 3; ++r) {
                alpha += A[3 * r + p] * A[3 * r + p];
                beta += A[3 * r + q] * A[3 * r + q];
                gamma += A[3 * r + p] * A[3 * r + q];
            }
            if (gamma == 0.0 || std::fabs(gamma) <= 1e-17 * std::sqrt(alpha * beta)) continue;
            rotated = true;
            const double zeta = (beta - alpha) / (2.0 * gamma);
            const double t = std::copysign(1.0, zeta) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
            const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
            for (int r = 0; r < 3; ++r) {
                const double ap = A[3 * r + p], aq = A[3 * r + q];
                A[3 * r + p] = c * ap - s * aq;
                A[3 * r + q] = s * ap + c * aq;
                const double vp = V[3 * r + p], vq = V[3 * r + q];
                V[3 * r + p] = c * vp - s * vq;
                V[3 * r + q] = s * vp + c * vq;
            }
        }
        if (!rotated) break;
    }
    int order[3] = {0, 1, 2};
    double nrm[3];
    for (int j = 0; j < 3; ++j)
        nrm[j] = std::sqrt(A[j] * A[j] + A[3 + j] * A[3 + j] + A[6 + j] * A[6 + j]);
    std::sort(order, order + 3, [&](int a, int b) { return nrm[a] > nrm[b]; });
    double Vs[9];
    for (int j = 0; j < 3; ++j) {
        const int o = order[j];
        S[j] = nrm[o];
        for (int r = 0; r < 3; ++r) {
            U[3 * r + j] = nrm[o] > 0 ? A[3 * r + o] / nrm[o] : 0.0;
            Vs[3 * r + j] = V[3 * r + o];
        }
    }
    memcpy(V, Vs, sizeof(Vs));
    // complete U where singular values vanish: unit vectors orthogonal to the others
    const double tiny = 1e-300;
    if (S[0] <= tiny) {
        for (int i = 0; i < 9; ++i) U[i] = (i % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    if (S[1] <= tiny) {  // a unit vector orthogonal to u0
        const double u0[3] = {U[0], U[3], U[6]};
        const int m = std::fabs(u0[0]) <= std::fabs(u0[1]) && std::fabs(u0[0]) <= std::fabs(u0[2]) ? 0
                      : std::fabs(u0[1]) <= std::fabs(u0[2])                                      ? 1
                                                                                                  : 2;
        double e[3] = {0, 0, 0};
        e[m] = 1.0;
        double w[3] = {e[0] - u0[m] * u0[0], e[1] - u0[m] * u0[1], e[2] - u0[m] * u0[2]};
        const double n = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        for (int r = 0; r < 3; ++r) U[3 * r + 1] = w[r] / n;
    }
    if (S[2] <= tiny) {  // u2 = u0 x u1
        const double a[3] = {U[0], U[3], U[6]}, b[3] = {U[1], U[4], U[7]};
        U[2] = a[1] * b[2] - a[2] * b[1];
        U[5] = a[2] * b[0] - a[0] * b[2];
        U[8] = a[0] * b[1] - a[1] * b[0];
    }
}

// Rotation of Fit (center_of_mass.cpp:100-112): K = U S V^T, d = det(U V^T),
// R = U diag(1, 1, d) V^T.
void fit_rotation(const double* K, double* R) {
    double U[9], S[3], V[9];
    svd3(K, U, S, V);
    double UVt[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) UVt[3 * r + c] = U[3 * r] * V[3 * c] + U[3 * r + 1] * V[3 * c + 1] + U[3 * r + 2] * V[3 * c + 2];
    const double d = det3(UVt);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R[3 * r + c] = U[3 * r] * V[3 * c] + U[3 * r + 1] * V[3 * c + 1] + d * U[3 * r + 2] * V[3 * c + 2];
}

int fail(std::string& m, int code, const std::string& what) {
    m = what;
    return code;
}

}  // namespace
}  // namespace sassgpu

using namespace sassgpu;

extern "C" int sass_stage_frames_prepass(sass_plan* p, const float* frames, size_t nsys, const double* masses,
                                         const sass_prepass_step* steps, size_t nsteps, const size_t* target,
                                         float* staged) {
    if (!p) return SASS_ERR_ARG;
    SystemState& s = p->sys;
    const size_t nf = s.nf, na = s.na;
    if (!frames || !masses || !target || nsys == 0 || (nsteps && !steps))
        return fail(p->msg, SASS_ERR_ARG, "NULL argument or empty system");
    for (size_t t = 0; t < na; ++t)
        if (target[t] >= nsys) return fail(p->msg, SASS_ERR_ARG, "target atom outside the system");
    for (size_t i = 0; i < nsteps; ++i) {
        const sass_prepass_step& st = steps[i];
        if (st.type < SASS_STEP_CENTER || st.type > SASS_STEP_MOTION)
            return fail(p->msg, SASS_ERR_ARG, "prepass step " + std::to_string(i) + ": unknown type");
        if ((st.nselection && !st.selection) || (st.nreference && !st.reference_selection))
            return fail(p->msg, SASS_ERR_ARG, "prepass step " + std::to_string(i) + ": NULL list");
        for (size_t k = 0; k < st.nselection; ++k)
            if (st.selection[k] >= nsys) return fail(p->msg, SASS_ERR_ARG, "prepass step " + std::to_string(i) + ": atom outside the system");
        for (size_t k = 0; k < st.nreference; ++k)
            if (st.reference_selection[k] >= nsys)
                return fail(p->msg, SASS_ERR_ARG, "prepass step " + std::to_string(i) + ": reference atom outside the system");
        const bool fit = st.type == SASS_STEP_FITROTTRANS || st.type == SASS_STEP_FITROT;
        if (fit && st.nfit && (!st.fit_target || !st.fit_source))
            return fail(p->msg, SASS_ERR_ARG, "prepass step " + std::to_string(i) + ": fit without target/source lists");
        if (fit)
            for (size_t k = 0; k < st.nfit; ++k)
                if (st.fit_target[k] >= nsys || st.fit_source[k] >= st.nreference)
                    return fail(p->msg, SASS_ERR_ARG, "prepass step " + std::to_string(i) + ": fit pair outside the system or the fitted atoms");
        if (st.type == SASS_STEP_MOTION && !st.translations)
            return fail(p->msg, SASS_ERR_ARG, "prepass step " + std::to_string(i) + ": motion without translations");
    }

    std::string& m = p->msg;
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        cudaGetLastError();
        m = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? SASS_ERR_OOM : SASS_ERR_CUDA;
    };
#define PCK(expr)                                           \
    do {                                                    \
        cudaError_t e_ = (expr);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr); \
    } while (0)
    PCK(cudaSetDevice(p->d.device));
    cudaStream_t st = p->st;

    // every list of every step in one packed upload (16-byte aligned pieces)
    std::vector<unsigned char> blob;
    auto put = [&](const void* h, size_t bytes) {
        const size_t off = (blob.size() + 15) / 16 * 16;
        blob.resize(off + bytes);
        if (bytes) memcpy(blob.data() + off, h, bytes);
        return off;
    };
    struct Offs {
        size_t sel, ftg, fsrc, ref, rmass, smass, refxyz, trans;
    };
    std::vector<Offs> offs(nsteps);
    size_t max_ref = 0;
    for (size_t i = 0; i < nsteps; ++i) {
        const sass_prepass_step& q = steps[i];
        std::vector<double> rmass(q.nreference), smass(q.nselection);
        for (size_t k = 0; k < q.nreference; ++k) rmass[k] = masses[q.reference_selection[k]];
        for (size_t k = 0; k < q.nselection; ++k) smass[k] = masses[q.selection[k]];
        Offs& o = offs[i];
        o.sel = put(q.selection, q.nselection * sizeof(size_t));
        const bool fit = q.type == SASS_STEP_FITROTTRANS || q.type == SASS_STEP_FITROT;
        o.ftg = put(q.fit_target, fit ? q.nfit * sizeof(size_t) : 0);
        o.fsrc = put(q.fit_source, fit ? q.nfit * sizeof(size_t) : 0);
        o.ref = put(q.reference_selection, q.nreference * sizeof(size_t));
        o.rmass = put(rmass.data(), rmass.size() * sizeof(double));
        o.smass = put(smass.data(), smass.size() * sizeof(double));
        o.refxyz = put(q.reference, q.reference ? q.nreference * 3 * sizeof(double) : 0);
        o.trans = put(q.translations, q.type == SASS_STEP_MOTION ? nf * 3 * sizeof(double) : 0);
        if (q.type == SASS_STEP_FITROTTRANS || q.type == SASS_STEP_FITROT) max_ref = std::max(max_ref, q.nreference);
    }
    const size_t o_target = put(target, na * sizeof(size_t));
    PCK(p->pp_lists.ensure(blob.size()));
    PCK(p->pp_W.ensure(nf * nsys * 3 * sizeof(double)));
    PCK(p->pp_F.ensure(nf * nsys * 3 * sizeof(float)));
    PCK(p->pp_vec.ensure(nf * 3 * 4 * sizeof(double) + nf * 9 * 2 * sizeof(double)));
    if (max_ref) PCK(p->pp_C.ensure(nf * max_ref * 3 * sizeof(double)));
    PCK(s.raw.ensure(nf * na * 3 * sizeof(float)));
    unsigned char* dl = p->pp_lists.as<unsigned char>();
    PCK(cudaMemcpyAsync(dl, blob.data(), blob.size(), cudaMemcpyHostToDevice, st));
    PCK(cudaMemcpyAsync(p->pp_F.p, frames, nf * nsys * 3 * sizeof(float), cudaMemcpyHostToDevice, st));
    double* W = p->pp_W.as<double>();
    const size_t nW = nf * nsys * 3;
    pp_promote_kernel<<<grid_for(nW, 256), 256, 0, st>>>(p->pp_F.as<float>(), nW, W);
    PCK(cudaGetLastError());
    // per-frame vectors: a, b, t, c [nf][3] and K, R [nf][9]
    double* va = p->pp_vec.as<double>();
    double* vb = va + nf * 3;
    double* vt = vb + nf * 3;
    double* vc = vt + nf * 3;
    double* vK = vc + nf * 3;
    double* vR = vK + nf * 9;
    double* C = p->pp_C.as<double>();
    const int nfi = (int)nf;
    const unsigned gf = (unsigned)((nf + kPerFrameThreads - 1) / kPerFrameThreads);
    const unsigned gw = (unsigned)((nf + 31) / 32);  // the ordered sums: one CTA per 32 frames
    auto L = [&](size_t off) { return reinterpret_cast<const size_t*>(dl + off); };
    auto D = [&](size_t off) { return reinterpret_cast<const double*>(dl + off); };
    std::vector<double> hK(nf * 9), hR(nf * 9);

    for (size_t i = 0; i < nsteps; ++i) {
        const sass_prepass_step& q = steps[i];
        const Offs& o = offs[i];
        const size_t nsel = q.nselection, nref = q.nreference;
        // centre of mass of the reference structure -> va ([1][3] when it is constant)
        const bool ref_one = q.reference != nullptr;
        auto com_ref = [&](double* out) {
            if (ref_one)
                pp_com_kernel<<<1, kComThreads, 0, st>>>(D(o.refxyz), 0, nullptr, D(o.rmass), nref, 1, out);
            else
                pp_com_kernel<<<gw, kComThreads, 0, st>>>(W, nsys * 3, L(o.ref), D(o.rmass), nref, nfi, out);
        };
        switch (q.type) {
            case SASS_STEP_CENTER:
                com_ref(va);
                pp_combine_kernel<<<gf, kPerFrameThreads, 0, st>>>(va, ref_one, nullptr, 0, 0, nfi, vt);
                if (nsel) pp_translate_kernel<<<grid_for(nf * nsel, 256), 256, 0, st>>>(W, nsys, L(o.sel), nsel, nfi, vt);
                break;
            case SASS_STEP_FITTRANS:
                com_ref(va);
                pp_com_kernel<<<gw, kComThreads, 0, st>>>(W, nsys * 3, L(o.sel), D(o.smass), nsel, nfi, vb);
                pp_combine_kernel<<<gf, kPerFrameThreads, 0, st>>>(va, ref_one, vb, 0, 1, nfi, vt);
                if (nsel) pp_translate_kernel<<<grid_for(nf * nsel, 256), 256, 0, st>>>(W, nsys, L(o.sel), nsel, nfi, vt);
                break;
            case SASS_STEP_MOTION:
                com_ref(va);
                if (nsel)
                    pp_motion_kernel<<<grid_for(nf * nsel, 256), 256, 0, st>>>(W, nsys, L(o.sel), nsel, nfi, va, ref_one,
                                                                              D(o.trans));
                break;
            default: {  // FITROTTRANS, FITROT
                const bool rot_only = q.type == SASS_STEP_FITROT;
                if (rot_only)  // centre of mass of the moved atoms before the fit
                    pp_com_kernel<<<gw, kComThreads, 0, st>>>(W, nsys * 3, L(o.sel), D(o.smass), nsel, nfi, vc);
                if (nref) {
                    pp_gather_kernel<<<grid_for(nf * nref * 3, 256), 256, 0, st>>>(W, nsys, L(o.ref), nref, nfi, C);
                    // pos: the copy's centre; ref: the reference structure's (the copy itself when instant)
                    pp_com_kernel<<<gw, kComThreads, 0, st>>>(C, nref * 3, nullptr, D(o.rmass), nref, nfi, vb);
                    if (ref_one)
                        pp_com_kernel<<<1, kComThreads, 0, st>>>(D(o.refxyz), 0, nullptr, D(o.rmass), nref, 1, va);
                    else
                        pp_com_kernel<<<gw, kComThreads, 0, st>>>(C, nref * 3, nullptr, D(o.rmass), nref, nfi, va);
                    pp_kmat_kernel<<<gw, kComThreads, 0, st>>>(C, ref_one ? D(o.refxyz) : nullptr, D(o.rmass),
                                                                     nref, nfi, vb, va, ref_one, vK);
                    PCK(cudaGetLastError());
                    PCK(cudaMemcpyAsync(hK.data(), vK, nf * 9 * sizeof(double), cudaMemcpyDeviceToHost, st));
                    PCK(cudaStreamSynchronize(st));
                    for (size_t f = 0; f < nf; ++f) fit_rotation(&hK[9 * f], &hR[9 * f]);
                    PCK(cudaMemcpyAsync(vR, hR.data(), nf * 9 * sizeof(double), cudaMemcpyHostToDevice, st));
                    pp_fit_apply_kernel<<<grid_for(nf * nref, 256), 256, 0, st>>>(C, nref, nfi, vR, vb, va, ref_one);
                    if (q.nfit)
                        pp_scatter_kernel<<<grid_for(nf * q.nfit, 256), 256, 0, st>>>(W, nsys, L(o.ftg), L(o.fsrc), q.nfit,
                                                                                     C, nref, nfi);
                }
                if (rot_only && nsel) {
                    pp_combine_kernel<<<gf, kPerFrameThreads, 0, st>>>(nullptr, 0, vc, 0, 2, nfi, vt);
                    pp_translate_kernel<<<grid_for(nf * nsel, 256), 256, 0, st>>>(W, nsys, L(o.sel), nsel, nfi, vt);
                }
            }
        }
        PCK(cudaGetLastError());
    }
    pp_target_kernel<<<grid_for(nf * na * 3, 256), 256, 0, st>>>(W, nsys, L(o_target), na, nfi, s.raw.as<float>());
    PCK(cudaGetLastError());
    PCK(cudaStreamSynchronize(st));
    int rc = stage_system(s, s.raw.as<float>(), true, p->d.precision, st, p->msg);
    if (rc) return rc;
    if (staged) {
        PCK(cudaMemcpyAsync(staged, s.raw.p, nf * na * 3 * sizeof(float), cudaMemcpyDeviceToHost, st));
        PCK(cudaStreamSynchronize(st));
    }
    p->msg.clear();
    return SASS_OK;
#undef PCK
}
