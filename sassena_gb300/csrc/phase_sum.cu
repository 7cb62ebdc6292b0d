// Coherent phase sum A[v][f] = sum_j b_j(shell(v)) * exp(i q_v . r_j(f)).
//
// Replaces AllVectorsScatterDevice::scatter (src/scatter_devices/
// all_vectors_scatter_device.cpp:388-439): the reference runs one host thread per
// sub-vector and, for each frame, sums atoms sequentially in FP64 with libm cos/sin.
//
// GB300 layout. The work is a list of tiles; a tile is one group of 32*Q sub-vectors of
// one shell of one system (Q held in registers by every lane) x W consecutive frames
// (one warp per frame) x a range of atoms. The kernel is persistent: every CTA takes
// tiles from a global work counter (atomicAdd) until the list is exhausted, so one
// launch covers many systems of uneven size (the batched form) as well as a single
// system. Each warp streams its own frame's atoms through a private S-stage
// shared-memory ring filled by 1-D bulk copies (TMA engine, cp.async.bulk) of T float4
// coordinates plus T factors, completion tracked on mbarriers whose phases run on
// across tiles; every wait is bounded. All lanes of a warp read the same atom (shared-
// memory broadcast) and evaluate their Q sub-vectors. Results are transposed through
// shared memory so each sub-vector's frames are written as one contiguous row. Tiles
// never accumulate into each other (atom splits write separate FP64 partial slices), so
// results do not depend on which CTA processed which tile.
//
// Two arithmetic forms:
//   FP64 ("plain"): q.r and the atom sum in FP64 exactly as the reference writes
//     them (float coordinates promoted, products and sums rounded separately, no
//     FMA contraction, atoms in index order) with CUDA's double sincos.
//   FP32: coordinates centred on a fixed frame-0 centre (the constant phase
//     exp(i q.c) cancels in |A|^2 and in the autocorrelation and is restored in
//     FP64 for dsp=plain), q pre-scaled to revolutions (q/2pi), explicit range
//     reduction u - rint(u) (magic-number rounding, exact subtraction), SFU
//     sin/cos on the reduced angle, per-stage FP32 partial sums folded into a
//     Kahan-compensated FP32 accumulator; atom-split partials are FP64 and reduced
//     in FP64 (the cross-block reduction), single-split results are stored as FP32.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace sassgpu {

namespace {

template <int W, int T, int S, int BBYTES>
struct PipeLayout {
    static constexpr int kCoordBytes = W * S * T * 16;
    static constexpr int kFactorBytes = W * S * T * BBYTES;
    static constexpr int kBarOffset = kCoordBytes + kFactorBytes;
    static constexpr int kTileOffset = kBarOffset + W * S * 8;
    static constexpr int kBytes = kTileOffset + 16;
};

// Issue the bulk copies of one stage (T coordinates + T factors) into a ring slot.
template <int T, int BBYTES>
__device__ __forceinline__ void issue_stage(float4* sx, void* sb, uint64_t* bar, const float4* src_x,
                                            const unsigned char* src_b) {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, T * 16 + T * BBYTES);
    bulk_g2s(sx, src_x, T * 16, bar);
    bulk_g2s(sb, src_b, T * BBYTES, bar);
}

// FP32 form, Q = 1: one sub-vector per lane, scalar arithmetic.
template <int Q, int PP>
struct Fp32Acc {
    float qx[Q], qy[Q], qz[Q], sr[Q], si[Q], cr[Q], ci[Q];
    __device__ void load_q(const double* qv, int v0, int nv, int lane) {
        const double inv2pi = 0.15915494309189533577;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            int vl = lane + 32 * k;
            if (vl < nv) {
                const double* q = qv + 3 * (size_t)(v0 + vl);
                qx[k] = (float)(q[0] * inv2pi);
                qy[k] = (float)(q[1] * inv2pi);
                qz[k] = (float)(q[2] * inv2pi);
            } else {
                qx[k] = qy[k] = qz[k] = 0.f;
            }
            sr[k] = si[k] = cr[k] = ci[k] = 0.f;
        }
    }
    template <int T>
    __device__ __forceinline__ void stage(const float4* cx, const float* cb) {
        const float kMagic = 12582912.0f;  // 1.5 * 2^23: adds round to the nearest integer
        const float kTwoPi = 6.28318530717958647692f;
        float tr[Q], ti[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) tr[k] = ti[k] = 0.f;
#pragma unroll 2
        for (int jj = 0; jj < T; ++jj) {
            const float4 r = cx[jj];
            const float b = cb[jj];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                float u = fmaf(r.z, qz[k], fmaf(r.y, qy[k], r.x * qx[k]));
                float n = __fsub_rn(__fadd_rn(u, kMagic), kMagic);
                float fr = __fsub_rn(u, n);  // in [-1/2, 1/2], exact
                float s, c;
                __sincosf(fr * kTwoPi, &s, &c);
                tr[k] = fmaf(b, c, tr[k]);
                ti[k] = fmaf(b, s, ti[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) {  // Kahan: fold the stage sum into (s, c)
            float y = __fsub_rn(tr[k], cr[k]);
            float t = __fadd_rn(sr[k], y);
            cr[k] = __fsub_rn(__fsub_rn(t, sr[k]), y);
            sr[k] = t;
            y = __fsub_rn(ti[k], ci[k]);
            t = __fadd_rn(si[k], y);
            ci[k] = __fsub_rn(__fsub_rn(t, si[k]), y);
            si[k] = t;
        }
    }
    __device__ double2 result(int k) const {
        return make_double2((double)sr[k] - (double)cr[k], (double)si[k] - (double)ci[k]);
    }
    // the FP32 output: sum minus compensation rounded once, on the FP32 pipe
    __device__ float2 result_f32(int k) const { return make_float2(__fsub_rn(sr[k], cr[k]), __fsub_rn(si[k], ci[k])); }
};

// sin and cos of 2 pi f for a pair of reduced angles f in [-1/2, 1/2] revolutions on the
// FP32 pipe instead of the SFU: Taylor series of the half angle h = pi f in
// [-pi/2, pi/2] (sin through h^11, cos through h^12: truncation below 6e-8) and the
// double-angle formulas sin 2h = 2 sin h cos h, cos 2h = cos^2 h - sin^2 h (absolute error
// below 4.3e-7 over the range in float32, under the SFU approximation's 2^-21). Returns
// (cos 2h) and (sin h cos h) = (sin 2h) / 2.
__device__ __forceinline__ void sincos2_poly(float2 f, float2& c2h, float2& shch) {
    const float2 kPi = make_float2(3.14159265358979323846f, 3.14159265358979323846f);
    const float2 h = __fmul2_rn(f, kPi);
    const float2 h2 = __fmul2_rn(h, h);
    auto cst = [](float v) { return make_float2(v, v); };
    float2 ps = __ffma2_rn(cst(-1.f / 39916800.f), h2, cst(1.f / 362880.f));
    ps = __ffma2_rn(ps, h2, cst(-1.f / 5040.f));
    ps = __ffma2_rn(ps, h2, cst(1.f / 120.f));
    ps = __ffma2_rn(ps, h2, cst(-1.f / 6.f));
    ps = __ffma2_rn(ps, h2, cst(1.f));
    const float2 sh = __fmul2_rn(ps, h);
    float2 pc = __ffma2_rn(cst(1.f / 479001600.f), h2, cst(-1.f / 3628800.f));
    pc = __ffma2_rn(pc, h2, cst(1.f / 40320.f));
    pc = __ffma2_rn(pc, h2, cst(-1.f / 720.f));
    pc = __ffma2_rn(pc, h2, cst(1.f / 24.f));
    pc = __ffma2_rn(pc, h2, cst(-0.5f));
    const float2 ch = __ffma2_rn(pc, h2, cst(1.f));
    shch = __fmul2_rn(sh, ch);
    c2h = __ffma2_rn(ch, ch, __fmul2_rn(__fmul2_rn(sh, cst(-1.f)), sh));
}

// FP32 form, even Q: sub-vectors in pairs (lane + 32 (2j), lane + 32 (2j + 1)) evaluated
// with paired FP32 operations (FFMA2/FADD2/FMUL2). The last PP pairs take sin/cos from
// sincos2_poly on the FP32 pipe, the others from the SFU, so both units carry load.
template <int Q, int PP>
struct Fp32PairAcc {
    static constexpr int NP = Q / 2;
    static_assert(Q % 2 == 0 && PP <= NP, "pairs");
    float2 qx[NP], qy[NP], qz[NP], sr[NP], si[NP], cr[NP], ci[NP];
    __device__ void load_q(const double* qv, int v0, int nv, int lane) {
        const double inv2pi = 0.15915494309189533577;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
            float q[2][3];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int vl = lane + 32 * (2 * j + h);
                const double* p = qv + 3 * (size_t)(v0 + vl);
#pragma unroll
                for (int c = 0; c < 3; ++c) q[h][c] = vl < nv ? (float)(p[c] * inv2pi) : 0.f;
            }
            qx[j] = make_float2(q[0][0], q[1][0]);
            qy[j] = make_float2(q[0][1], q[1][1]);
            qz[j] = make_float2(q[0][2], q[1][2]);
            sr[j] = si[j] = cr[j] = ci[j] = make_float2(0.f, 0.f);
        }
    }
    template <int T>
    __device__ __forceinline__ void stage(const float4* cx, const float* cb) {
        const float2 kM = make_float2(12582912.0f, 12582912.0f), kNM = make_float2(-12582912.0f, -12582912.0f);
        const float2 kNeg = make_float2(-1.f, -1.f);
        const float2 kTwoPi = make_float2(6.28318530717958647692f, 6.28318530717958647692f);
        float2 tr[NP], ti[NP];
#pragma unroll
        for (int j = 0; j < NP; ++j) tr[j] = ti[j] = make_float2(0.f, 0.f);
#pragma unroll 2
        for (int jj = 0; jj < T; ++jj) {
            const float4 r = cx[jj];
            const float2 rx = make_float2(r.x, r.x), ry = make_float2(r.y, r.y), rz = make_float2(r.z, r.z);
            const float2 b = make_float2(cb[jj], cb[jj]);
            const float2 b2 = __fadd2_rn(b, b);
#pragma unroll
            for (int j = 0; j < NP; ++j) {
                const float2 u = __ffma2_rn(rz, qz[j], __ffma2_rn(ry, qy[j], __fmul2_rn(rx, qx[j])));
                const float2 n = __fadd2_rn(__fadd2_rn(u, kM), kNM);  // rint(u)
                const float2 fr = __ffma2_rn(n, kNeg, u);              // u - n in [-1/2, 1/2], exact
                if (j < NP - PP) {
                    const float2 x = __fmul2_rn(fr, kTwoPi);
                    float s0, c0, s1, c1;
                    __sincosf(x.x, &s0, &c0);
                    __sincosf(x.y, &s1, &c1);
                    tr[j] = __ffma2_rn(b, make_float2(c0, c1), tr[j]);
                    ti[j] = __ffma2_rn(b, make_float2(s0, s1), ti[j]);
                } else {
                    float2 c, sc;
                    sincos2_poly(fr, c, sc);
                    tr[j] = __ffma2_rn(b, c, tr[j]);
                    ti[j] = __ffma2_rn(b2, sc, ti[j]);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NP; ++j) {  // Kahan: fold the stage sums into (s, c)
            float2 y = __ffma2_rn(cr[j], kNeg, tr[j]);
            float2 t = __fadd2_rn(sr[j], y);
            cr[j] = __ffma2_rn(y, kNeg, __ffma2_rn(sr[j], kNeg, t));
            sr[j] = t;
            y = __ffma2_rn(ci[j], kNeg, ti[j]);
            t = __fadd2_rn(si[j], y);
            ci[j] = __ffma2_rn(y, kNeg, __ffma2_rn(si[j], kNeg, t));
            si[j] = t;
        }
    }
    __device__ double2 result(int k) const {
        const int j = k >> 1;
        const float s_r = (k & 1) ? sr[j].y : sr[j].x, c_r = (k & 1) ? cr[j].y : cr[j].x;
        const float s_i = (k & 1) ? si[j].y : si[j].x, c_i = (k & 1) ? ci[j].y : ci[j].x;
        return make_double2((double)s_r - (double)c_r, (double)s_i - (double)c_i);
    }
    __device__ float2 result_f32(int k) const {
        const int j = k >> 1;
        const float s_r = (k & 1) ? sr[j].y : sr[j].x, c_r = (k & 1) ? cr[j].y : cr[j].x;
        const float s_i = (k & 1) ? si[j].y : si[j].x, c_i = (k & 1) ? ci[j].y : ci[j].x;
        return make_float2(__fsub_rn(s_r, c_r), __fsub_rn(s_i, c_i));
    }
};

template <int Q>
struct Fp64Acc {
    double qx[Q], qy[Q], qz[Q], ar[Q], ai[Q];
    __device__ void load_q(const double* qv, int v0, int nv, int lane) {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            int vl = lane + 32 * k;
            if (vl < nv) {
                const double* q = qv + 3 * (size_t)(v0 + vl);
                qx[k] = q[0];
                qy[k] = q[1];
                qz[k] = q[2];
            } else {
                qx[k] = qy[k] = qz[k] = 0.0;
            }
            ar[k] = ai[k] = 0.0;
        }
    }
    template <int T>
    __device__ __forceinline__ void stage(const float4* cx, const double* cb) {
        for (int jj = 0; jj < T; ++jj) {
            const float4 r = cx[jj];
            const double b = cb[jj];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                // p = x*qx + y*qy + z*qz, rounded as the reference writes it
                double p = __dadd_rn(__dadd_rn(__dmul_rn((double)r.x, qx[k]), __dmul_rn((double)r.y, qy[k])),
                                     __dmul_rn((double)r.z, qz[k]));
                double s, c;
                sincos(p, &s, &c);
                ar[k] = __dadd_rn(ar[k], __dmul_rn(b, c));
                ai[k] = __dadd_rn(ai[k], __dmul_rn(b, s));
            }
        }
    }
    __device__ double2 result(int k) const { return make_double2(ar[k], ai[k]); }
};

template <bool F32, int Q, int PP, bool PAIRED = (Q % 2 == 0)>
struct AccSel;
template <int Q, int PP>
struct AccSel<true, Q, PP, false> {
    typedef Fp32Acc<Q, PP> type;
    typedef float B;
};
template <int Q, int PP>
struct AccSel<true, Q, PP, true> {
    typedef Fp32PairAcc<Q, PP> type;
    typedef float B;
};
template <int Q, int PP, bool PAIRED>
struct AccSel<false, Q, PP, PAIRED> {
    typedef Fp64Acc<Q> type;
    typedef double B;
};

template <bool F32, int Q, int W, int T, int S, int PP>
__global__ void __launch_bounds__(W * 32)
    phase_sum_kernel(const PhaseSystem* __restrict__ systems, const PhaseTileDesc* __restrict__ tiles,
                     int ntiles, unsigned int* __restrict__ counter, unsigned int* err) {
    typedef typename AccSel<F32, Q, PP>::type Acc;
    typedef typename AccSel<F32, Q, PP>::B B;
    constexpr int BB = sizeof(B);
    using L = PipeLayout<W, T, S, BB>;
    static_assert(S * T >= 32 * Q, "output staging must fit in the coordinate ring");
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* sx = reinterpret_cast<float4*>(smem) + warp * S * T;
    B* sb = reinterpret_cast<B*>(smem + L::kCoordBytes) + warp * S * T;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::kBarOffset) + warp * S;
    volatile int* s_tile = reinterpret_cast<volatile int*>(smem + L::kTileOffset);
    double2* so = reinterpret_cast<double2*>(smem);

    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncwarp();
    unsigned used = 0;    // stages this warp has consumed: ring slot and phase parity run on
    bool failed = false;  // a bounded wait gave up: this warp does no further work

    for (;;) {
        __syncthreads();  // the previous tile's output staging has been read by everyone
        if (threadIdx.x == 0) *s_tile = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int ti = *s_tile;
        if (ti >= ntiles) break;
        const PhaseTileDesc td = tiles[ti];
        const PhaseSystem sys = systems[td.system];
        const int f = td.f0 + warp;
        const int nst = (td.j_end - td.j_begin) / T;
        Acc acc;
        acc.load_q(sys.qv, td.v0, td.nv, lane);

        if (f < sys.nf && nst > 0 && !failed) {
            const float4* row = sys.xyz + (size_t)f * sys.na_pad + td.j_begin;
            const unsigned char* brow = reinterpret_cast<const unsigned char*>(sys.bfac) +
                                        ((size_t)td.shell * sys.na_pad + td.j_begin) * BB;
            if (lane == 0)
                for (int k = 0; k < S && k < nst; ++k) {
                    const unsigned slot = (used + k) % S;
                    issue_stage<T, BB>(sx + slot * T, sb + slot * T, &bars[slot], row + k * T,
                                       brow + (size_t)k * T * BB);
                }
            int t = 0;
            for (; t < nst; ++t) {
                const unsigned slot = (used + t) % S;
                const unsigned parity = ((used + t) / S) & 1u;
                bool ok = mbar_wait_parity(&bars[slot], parity);
                if (!__all_sync(0xffffffffu, ok)) break;
                acc.template stage<T>(sx + slot * T, sb + slot * T);
                __syncwarp();  // every lane is done with this slot: refill it with stage t+S
                if (lane == 0 && t + S < nst)
                    issue_stage<T, BB>(sx + slot * T, sb + slot * T, &bars[slot], row + (t + S) * T,
                                       brow + (size_t)(t + S) * T * BB);
            }
            if (t < nst) {  // timed out: record, let issued copies land (bounded), stop
                if (lane == 0) {
                    set_error(err, DEV_MBAR_TIMEOUT);
                    for (int k = t; k < nst && k < t + S; ++k)
                        mbar_wait_parity(&bars[(used + k) % S], ((used + k) / S) & 1u);
                }
                failed = true;
                __syncwarp();
            }
            used += nst;
        }

        __syncthreads();  // every pipeline of this tile is drained: the ring becomes staging
        if constexpr (F32) {
            // FP32 amplitudes or FP32 split partials (the FP32 form always writes FP32):
            // results formed and staged in FP32
            float2* so32 = reinterpret_cast<float2*>(smem);
#pragma unroll
            for (int k = 0; k < Q; ++k) so32[(lane + 32 * k) * W + warp] = acc.result_f32(k);
            __syncthreads();
            float2* dst = sys.out_f32 + (size_t)td.split * sys.split_stride;
            for (int idx = threadIdx.x; idx < td.nv * W; idx += W * 32) {
                int vl = idx / W, w = idx - vl * W, ff = td.f0 + w;
                if (ff < sys.nf) dst[(size_t)(td.v0 + vl) * sys.nf + ff] = so32[vl * W + w];
            }
        } else {
#pragma unroll
            for (int k = 0; k < Q; ++k) so[(lane + 32 * k) * W + warp] = acc.result(k);
            __syncthreads();
            double2* dst = sys.out + (size_t)td.split * sys.split_stride;
            for (int idx = threadIdx.x; idx < td.nv * W; idx += W * 32) {
                int vl = idx / W, w = idx - vl * W, ff = td.f0 + w;
                if (ff < sys.nf) dst[(size_t)(td.v0 + vl) * sys.nf + ff] = so[vl * W + w];
            }
        }
    }
}

template <class OUT>
__device__ __forceinline__ OUT store_as(double2 v);
template <>
__device__ __forceinline__ double2 store_as<double2>(double2 v) {
    return v;
}
template <>
__device__ __forceinline__ float2 store_as<float2>(double2 v) {
    return make_float2((float)v.x, (float)v.y);
}

template <class OUT>
__global__ void split_reduce_kernel(const double2* __restrict__ part, int nsplit, size_t n,
                                    OUT* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        double2 a = part[i];
        for (int s = 1; s < nsplit; ++s) {
            double2 b = part[(size_t)s * n + i];
            a.x += b.x;
            a.y += b.y;
        }
        out[i] = store_as<OUT>(a);
    }
}

// s + e = a + b exactly (Knuth's TwoSum), in FP32
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// FP32 form: the partials are FP32 pairs, summed in split order in float-float arithmetic
// (TwoSum, the rounding errors gathered in a low word) and rounded once to FP32: the sum
// of two partials is the correctly rounded FP32 sum. On GB300 the FP64 adds and
// conversions this took before bounded the kernel on the narrow FP64 pipe (0.15 ms for the
// coherent workload's 2 x 82 MB of partials, a quarter of HBM bandwidth).
__global__ void split_reduce32_kernel(const float2* __restrict__ part, int nsplit, size_t n,
                                     float2* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float2 p0 = part[i];
        float hx = p0.x, hy = p0.y, lx = 0.f, ly = 0.f;
        for (int s = 1; s < nsplit; ++s) {
            const float2 b = part[(size_t)s * n + i];
            float ex, ey;
            two_sum(hx, b.x, hx, ex);
            two_sum(hy, b.y, hy, ey);
            lx = __fadd_rn(lx, ex);
            ly = __fadd_rn(ly, ey);
        }
        out[i] = make_float2(__fadd_rn(hx, lx), __fadd_rn(hy, ly));
    }
}

template <bool F32, int Q, int W, int T, int S, int PP>
cudaError_t launch_tiles(const PhaseLaunch& a, cudaStream_t st) {
    auto k = phase_sum_kernel<F32, Q, W, T, S, PP>;
    const int smem = PipeLayout<W, T, S, F32 ? 4 : 8>::kBytes;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, W * 32, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (long long)std::max(per_sm, 1) * std::max(sms, 1);
    if (a.max_ctas > 0 && grid > a.max_ctas) grid = a.max_ctas;
    if (grid > a.ntiles) grid = a.ntiles;
    if (grid < 1) return cudaSuccess;
    k<<<(unsigned)grid, W * 32, smem, st>>>(a.systems, a.tiles, a.ntiles, a.counter, a.err);
    return cudaGetLastError();
}

}  // namespace

// Instantiated tile shapes (q per lane, warps = frames per CTA, atoms per stage, pairs of
// q-vectors whose sin/cos come from the FP32 pipe instead of the SFU).
#define SASS_FP32_SHAPES(X)                                                                  \
    X(1, 8, 128, 0) X(2, 8, 128, 0) X(4, 8, 128, 0) X(8, 8, 128, 0) X(8, 8, 128, 1) X(4, 4, 128, 0) \
        X(8, 4, 128, 0) X(8, 4, 128, 1) X(2, 8, 64, 0) X(4, 8, 64, 0)
#define SASS_FP64_SHAPES(X) X(1, 4, 64, 0) X(2, 4, 64, 0) X(2, 8, 64, 0)

bool phase_shape_supported(int precision, PhaseShape t) {
#define CHECK(Q, W, T, PP) \
    if (t.q_per_lane == Q && t.warps == W && t.atoms == T && t.poly_pairs == PP) return true;
    if (precision == PREC_FP32) {
        SASS_FP32_SHAPES(CHECK)
    } else {
        SASS_FP64_SHAPES(CHECK)
    }
#undef CHECK
    return false;
}

std::vector<PhaseShape> phase_shapes(int precision) {
    std::vector<PhaseShape> v;
#define ADD(Q, W, T, PP) v.push_back(PhaseShape{Q, W, T, PP});
    if (precision == PREC_FP32) {
        SASS_FP32_SHAPES(ADD)
    } else {
        SASS_FP64_SHAPES(ADD)
    }
#undef ADD
    return v;
}

cudaError_t launch_phase_sum(const PhaseLaunch& a, cudaStream_t st) {
    if (a.ntiles <= 0) return cudaSuccess;
    const PhaseShape& t = a.shape;
#define L32(Q, W, T, PP)                                                                       \
    if (t.q_per_lane == Q && t.warps == W && t.atoms == T && t.poly_pairs == PP)               \
        return launch_tiles<true, Q, W, T, 2, PP>(a, st);
#define L64(Q, W, T, PP)                                                                       \
    if (t.q_per_lane == Q && t.warps == W && t.atoms == T && t.poly_pairs == PP)               \
        return launch_tiles<false, Q, W, T, 2, PP>(a, st);
    if (a.precision == PREC_FP32) {
        SASS_FP32_SHAPES(L32)
    } else {
        SASS_FP64_SHAPES(L64)
    }
#undef L32
#undef L64
    return cudaErrorInvalidValue;
}

cudaError_t launch_split_reduce(const double2* part, int nsplit, size_t n, double2* out,
                                cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    int blocks = (int)grid_blocks(n, 256, 16);
    split_reduce_kernel<double2><<<blocks, 256, 0, st>>>(part, nsplit, n, out);
    return cudaGetLastError();
}

cudaError_t launch_split_reduce_f32(const float2* part, int nsplit, size_t n, float2* out,
                                    cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    int blocks = (int)grid_blocks(n, 256, 16);
    split_reduce32_kernel<<<blocks, 256, 0, st>>>(part, nsplit, n, out);
    return cudaGetLastError();
}

}  // namespace sassgpu
