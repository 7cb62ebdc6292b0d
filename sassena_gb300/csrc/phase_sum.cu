// Coherent phase sum A[v][f] = sum_j b_j(shell(v)) * exp(i q_v . r_j(f)).
//
// Replaces AllVectorsScatterDevice::scatter (src/scatter_devices/
// all_vectors_scatter_device.cpp:388-439): the reference runs one host thread per
// sub-vector and, for each frame, sums atoms sequentially in FP64 with libm cos/sin.
//
// GB300 layout: one CTA = one group of sub-vectors of a single shell (32*Q of
// them, Q held in registers by every lane) x W consecutive frames (one warp per
// frame). Each warp streams its own frame's atoms through a private S-stage
// shared-memory ring filled by 1-D bulk copies (TMA engine, cp.async.bulk) of
// T float4 coordinates plus T factors, completion tracked on mbarriers with
// bounded waits. Every lane of a warp reads the same atom (shared-memory
// broadcast) and evaluates its Q sub-vectors. Results are transposed through
// shared memory so that each sub-vector's frames are written as one contiguous
// row.
//
// Two arithmetic forms:
//   FP64 ("plain"): q.r and the atom sum in FP64 exactly as the reference writes
//     them (float coordinates promoted, products and sums rounded separately, no
//     FMA contraction, atoms in index order) with CUDA's double sincos.
//   FP32: coordinates centred on a fixed frame-0 centre (the constant phase
//     exp(i q.c) cancels in |A|^2 and in the autocorrelation and is restored in
//     FP64 for dsp=plain), q pre-scaled to revolutions (q/2pi), explicit range
//     reduction u - rint(u) (magic-number rounding, exact subtraction), SFU
//     sin/cos on the reduced angle, per-tile FP32 partial sums folded into a
//     Kahan-compensated FP32 accumulator; the per-thread result is converted to
//     FP64 for the cross-block (atom-split) reduction.
#include "common.cuh"
#include "kernels.h"

namespace sassgpu {

namespace {

template <int W, int T, int S, int BBYTES>
struct PipeLayout {
    static constexpr int kCoordBytes = W * S * T * 16;
    static constexpr int kFactorBytes = W * S * T * BBYTES;
    static constexpr int kBarOffset = kCoordBytes + kFactorBytes;
    static constexpr int kBytes = kBarOffset + W * S * 8;
};

// Issue the bulk copies of tile `t` of this warp's frame into ring stage `st`.
template <int T, int BBYTES>
__device__ __forceinline__ void issue_tile(float4* sx, void* sb, uint64_t* bar, const float4* src_x,
                                           const unsigned char* src_b) {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, T * 16 + T * BBYTES);
    bulk_g2s(sx, src_x, T * 16, bar);
    bulk_g2s(sb, src_b, T * BBYTES, bar);
}

// Drain: after a timeout, wait (bounded) for any copy still in flight so that no
// asynchronous write lands in shared memory after the CTA has moved on.
template <int S>
__device__ void drain(uint64_t* bars, int first_pending, int issued) {
    for (int t = first_pending; t < issued; ++t) mbar_wait_parity(&bars[t % S], (t / S) & 1);
}

template <int Q, int W, int T, int S>
__global__ void __launch_bounds__(W * 32)
    phase_sum_fp32_kernel(const float4* __restrict__ xyz, int na_pad, int nf,
                          const float* __restrict__ bfac, const double* __restrict__ qv,
                          const VecGroup* __restrict__ groups, int atoms_per_split,
                          double2* __restrict__ out, float2* __restrict__ out_f32,
                          size_t split_stride, unsigned int* err) {
    using L = PipeLayout<W, T, S, 4>;
    static_assert(S * T >= 32 * Q, "output staging must fit in the coordinate ring");
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int f = blockIdx.x * W + warp;
    const VecGroup g = groups[blockIdx.y];
    const int j_begin = blockIdx.z * atoms_per_split;
    const int j_end = min(j_begin + atoms_per_split, na_pad);
    const int ntiles = j_end > j_begin ? (j_end - j_begin) / T : 0;

    float4* sx = reinterpret_cast<float4*>(smem) + warp * S * T;
    float* sb = reinterpret_cast<float*>(smem + L::kCoordBytes) + warp * S * T;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::kBarOffset) + warp * S;

    // q in revolutions per Angstrom, rounded once from FP64.
    const double inv2pi = 0.15915494309189533577;
    float qx[Q], qy[Q], qz[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        int vl = lane + 32 * k;
        if (vl < g.nv) {
            const double* q = qv + 3 * (size_t)(g.v0 + vl);
            qx[k] = (float)(q[0] * inv2pi);
            qy[k] = (float)(q[1] * inv2pi);
            qz[k] = (float)(q[2] * inv2pi);
        } else {
            qx[k] = qy[k] = qz[k] = 0.f;
        }
    }

    float sr[Q], si[Q], cr[Q], ci[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) sr[k] = si[k] = cr[k] = ci[k] = 0.f;

    if (f < nf && ntiles > 0) {
        const float4* row = xyz + (size_t)f * na_pad;
        const unsigned char* brow =
            reinterpret_cast<const unsigned char*>(bfac + (size_t)g.shell * na_pad);
        if (lane == 0) {
#pragma unroll
            for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
            fence_mbar_init();
        }
        __syncwarp();
        int issued = 0;
        if (lane == 0)
            for (; issued < S && issued < ntiles; ++issued)
                issue_tile<T, 4>(sx + issued * T, sb + issued * T, &bars[issued],
                                 row + j_begin + issued * T,
                                 brow + (size_t)(j_begin + issued * T) * 4);
        issued = __shfl_sync(0xffffffffu, issued, 0);

        const float kMagic = 12582912.0f;  // 1.5 * 2^23: adds round to nearest integer
        const float kTwoPi = 6.28318530717958647692f;
        int t = 0;
        for (; t < ntiles; ++t) {
            const int st = t % S;
            bool ok = mbar_wait_parity(&bars[st], (t / S) & 1);
            if (!__all_sync(0xffffffffu, ok)) break;
            const float4* cx = sx + st * T;
            const float* cb = sb + st * T;
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
            for (int k = 0; k < Q; ++k) {  // Kahan: fold the tile sum into (s, c)
                float y = __fsub_rn(tr[k], cr[k]);
                float tt = __fadd_rn(sr[k], y);
                cr[k] = __fsub_rn(__fsub_rn(tt, sr[k]), y);
                sr[k] = tt;
                y = __fsub_rn(ti[k], ci[k]);
                tt = __fadd_rn(si[k], y);
                ci[k] = __fsub_rn(__fsub_rn(tt, si[k]), y);
                si[k] = tt;
            }
            __syncwarp();  // every lane is done with stage st: refill it with tile t+S
            if (t + S < ntiles) {
                if (lane == 0)
                    issue_tile<T, 4>(sx + st * T, sb + st * T, &bars[st],
                                     row + j_begin + (t + S) * T,
                                     brow + (size_t)(j_begin + (t + S) * T) * 4);
                ++issued;
            }
        }
        if (t < ntiles) {  // timed out: record, let in-flight copies land, stop
            if (lane == 0) {
                set_error(err, DEV_MBAR_TIMEOUT);
                drain<S>(bars, t, issued);
            }
            __syncwarp();
        }
    }

    // Transpose through shared memory: so[vl][w], then rows of W frames per v.
    __syncthreads();
    double2* so = reinterpret_cast<double2*>(smem);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        int vl = lane + 32 * k;
        so[vl * W + warp] =
            make_double2((double)sr[k] - (double)cr[k], (double)si[k] - (double)ci[k]);
    }
    __syncthreads();
    if (out_f32) {  // single atom split: the result goes straight to FP32 amplitudes
        for (int idx = threadIdx.x; idx < g.nv * W; idx += W * 32) {
            int vl = idx / W, w = idx - vl * W;
            int ff = blockIdx.x * W + w;
            if (ff < nf) {
                double2 v = so[vl * W + w];
                out_f32[(size_t)(g.v0 + vl) * nf + ff] = make_float2((float)v.x, (float)v.y);
            }
        }
        return;
    }
    double2* dst = out + (size_t)blockIdx.z * split_stride;  // FP64 partial of this atom split
    for (int idx = threadIdx.x; idx < g.nv * W; idx += W * 32) {
        int vl = idx / W, w = idx - vl * W;
        int ff = blockIdx.x * W + w;
        if (ff < nf) dst[(size_t)(g.v0 + vl) * nf + ff] = so[vl * W + w];
    }
}

template <int Q, int W, int T, int S>
__global__ void __launch_bounds__(W * 32)
    phase_sum_fp64_kernel(const float4* __restrict__ xyz, int na_pad, int nf,
                          const double* __restrict__ bfac, const double* __restrict__ qv,
                          const VecGroup* __restrict__ groups, int atoms_per_split,
                          double2* __restrict__ out, float2* __restrict__ out_f32,
                          size_t split_stride, unsigned int* err) {
    using L = PipeLayout<W, T, S, 8>;
    (void)out_f32;
    static_assert(S * T >= 32 * Q, "output staging must fit in the coordinate ring");
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int f = blockIdx.x * W + warp;
    const VecGroup g = groups[blockIdx.y];
    const int j_begin = blockIdx.z * atoms_per_split;
    const int j_end = min(j_begin + atoms_per_split, na_pad);
    const int ntiles = j_end > j_begin ? (j_end - j_begin) / T : 0;

    float4* sx = reinterpret_cast<float4*>(smem) + warp * S * T;
    double* sb = reinterpret_cast<double*>(smem + L::kCoordBytes) + warp * S * T;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::kBarOffset) + warp * S;

    double qx[Q], qy[Q], qz[Q], ar[Q], ai[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        int vl = lane + 32 * k;
        if (vl < g.nv) {
            const double* q = qv + 3 * (size_t)(g.v0 + vl);
            qx[k] = q[0];
            qy[k] = q[1];
            qz[k] = q[2];
        } else {
            qx[k] = qy[k] = qz[k] = 0.0;
        }
        ar[k] = ai[k] = 0.0;
    }

    if (f < nf && ntiles > 0) {
        const float4* row = xyz + (size_t)f * na_pad;
        const unsigned char* brow =
            reinterpret_cast<const unsigned char*>(bfac + (size_t)g.shell * na_pad);
        if (lane == 0) {
#pragma unroll
            for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
            fence_mbar_init();
        }
        __syncwarp();
        int issued = 0;
        if (lane == 0)
            for (; issued < S && issued < ntiles; ++issued)
                issue_tile<T, 8>(sx + issued * T, sb + issued * T, &bars[issued],
                                 row + j_begin + issued * T,
                                 brow + (size_t)(j_begin + issued * T) * 8);
        issued = __shfl_sync(0xffffffffu, issued, 0);

        int t = 0;
        for (; t < ntiles; ++t) {
            const int st = t % S;
            bool ok = mbar_wait_parity(&bars[st], (t / S) & 1);
            if (!__all_sync(0xffffffffu, ok)) break;
            const float4* cx = sx + st * T;
            const double* cb = sb + st * T;
            for (int jj = 0; jj < T; ++jj) {
                const float4 r = cx[jj];
                const double b = cb[jj];
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    // p = x*qx + y*qy + z*qz, rounded as the reference writes it
                    double p = __dadd_rn(__dadd_rn(__dmul_rn((double)r.x, qx[k]),
                                                   __dmul_rn((double)r.y, qy[k])),
                                         __dmul_rn((double)r.z, qz[k]));
                    double s, c;
                    sincos(p, &s, &c);
                    ar[k] = __dadd_rn(ar[k], __dmul_rn(b, c));
                    ai[k] = __dadd_rn(ai[k], __dmul_rn(b, s));
                }
            }
            __syncwarp();  // every lane is done with stage st: refill it with tile t+S
            if (t + S < ntiles) {
                if (lane == 0)
                    issue_tile<T, 8>(sx + st * T, sb + st * T, &bars[st],
                                     row + j_begin + (t + S) * T,
                                     brow + (size_t)(j_begin + (t + S) * T) * 8);
                ++issued;
            }
        }
        if (t < ntiles) {
            if (lane == 0) {
                set_error(err, DEV_MBAR_TIMEOUT);
                drain<S>(bars, t, issued);
            }
            __syncwarp();
        }
    }

    __syncthreads();
    double2* so = reinterpret_cast<double2*>(smem);
#pragma unroll
    for (int k = 0; k < Q; ++k) so[(lane + 32 * k) * W + warp] = make_double2(ar[k], ai[k]);
    __syncthreads();
    double2* dst = out + (size_t)blockIdx.z * split_stride;
    for (int idx = threadIdx.x; idx < g.nv * W; idx += W * 32) {
        int vl = idx / W, w = idx - vl * W;
        int ff = blockIdx.x * W + w;
        if (ff < nf) dst[(size_t)(g.v0 + vl) * nf + ff] = so[vl * W + w];
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

}  // namespace

#define SASS_FP32_TILES(X) X(1, 8, 128, 2) X(2, 8, 128, 2) X(4, 8, 128, 2) X(8, 8, 128, 2)
#define SASS_FP64_TILES(X) X(1, 4, 64, 2) X(2, 4, 64, 2)

bool phase_tile_supported(int precision, PhaseTile t) {
#define CHECK(Q, W, T, S) \
    if (t.q_per_lane == Q && t.warps == W && t.atoms == T) return true;
    if (precision == PREC_FP32) {
        SASS_FP32_TILES(CHECK)
    } else {
        SASS_FP64_TILES(CHECK)
    }
#undef CHECK
    return false;
}

cudaError_t launch_phase_sum(const PhaseSumArgs& a, cudaStream_t st) {
    if (a.ngroups == 0 || a.nf == 0) return cudaSuccess;
#define LAUNCH32(Q, W, T, S)                                                                    \
    if (a.tile.q_per_lane == Q && a.tile.warps == W && a.tile.atoms == T) {                     \
        constexpr int smem = PipeLayout<W, T, S, 4>::kBytes;                                    \
        auto k = phase_sum_fp32_kernel<Q, W, T, S>;                                             \
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem); \
        if (e != cudaSuccess) return e;                                                         \
        for (int g0 = 0; g0 < a.ngroups; g0 += 65535) {                                         \
        dim3 grid((a.nf + W - 1) / W, min(65535, a.ngroups - g0), a.nsplit);                    \
        k<<<grid, W * 32, smem, st>>>(a.xyz, a.na_pad, a.nf, (const float*)a.bfac, a.qv,        \
                                      a.groups + g0, a.atoms_per_split, a.out, a.out_f32,       \
                                      a.split_stride,                                           \
                                      a.err);                                                   \
        }                                                                                       \
        return cudaGetLastError();                                                              \
    }
#define LAUNCH64(Q, W, T, S)                                                                    \
    if (a.tile.q_per_lane == Q && a.tile.warps == W && a.tile.atoms == T) {                     \
        constexpr int smem = PipeLayout<W, T, S, 8>::kBytes;                                    \
        auto k = phase_sum_fp64_kernel<Q, W, T, S>;                                             \
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem); \
        if (e != cudaSuccess) return e;                                                         \
        for (int g0 = 0; g0 < a.ngroups; g0 += 65535) {                                         \
        dim3 grid((a.nf + W - 1) / W, min(65535, a.ngroups - g0), a.nsplit);                    \
        k<<<grid, W * 32, smem, st>>>(a.xyz, a.na_pad, a.nf, (const double*)a.bfac, a.qv,       \
                                      a.groups + g0, a.atoms_per_split, a.out, a.out_f32,       \
                                      a.split_stride,                                           \
                                      a.err);                                                   \
        }                                                                                       \
        return cudaGetLastError();                                                              \
    }
    if (a.precision == PREC_FP32) {
        SASS_FP32_TILES(LAUNCH32)
    } else {
        SASS_FP64_TILES(LAUNCH64)
    }
#undef LAUNCH32
#undef LAUNCH64
    return cudaErrorInvalidValue;
}

cudaError_t launch_split_reduce(const double2* part, int nsplit, size_t n, double2* out,
                                cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    split_reduce_kernel<double2><<<blocks, 256, 0, st>>>(part, nsplit, n, out);
    return cudaGetLastError();
}

cudaError_t launch_split_reduce_f32(const double2* part, int nsplit, size_t n, float2* out,
                                    cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    split_reduce_kernel<float2><<<blocks, 256, 0, st>>>(part, nsplit, n, out);
    return cudaGetLastError();
}

}  // namespace sassgpu
