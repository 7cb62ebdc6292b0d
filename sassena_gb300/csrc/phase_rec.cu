// Shell-recurrence phase sum (FP32 form) for shells that share one direction set.
//
// The reference builds the sub-vectors of every |q| from the same orientation set
// (init_subvectors, src/scatter_devices/abstract_vectors_scatter_device.cpp:112-130:
// ql * vectors[i] for the "file" and "sphere" types), and its q-vector scans are linear
// in the usual case (Params::create_from_scans, src/control/parameters.cpp). For a run of
// shells lam_k = lam_0 + k dlam along the base vectors u_d, the phase of shell k is
// phi_0 + k theta with phi_0 = lam_0 u.r and theta = dlam u.r, so
//     z_k = exp(i (phi_0 + k theta)),  z_{k+1} = 2 cos(theta) z_k - z_{k-1},
// a three-term (Chebyshev) recurrence with one FMA per component. One lane evaluates K
// shells of one direction with two SFU sin/cos pairs per atom instead of K; the
// recurrence restarts for every group of at most K shells, which bounds its rounding
// growth (O(K^2) ulp for theta near 0 or pi).
//
// Layout: atoms are sorted by scattering class into segments padded to 32 atoms, so every
// 32-atom block has one class; padding atoms sit at the origin, where every shell's term
// is exactly 1, and are subtracted by count. The lane keeps plain FP32 block sums per
// shell in registers and, where the class changes or every few pipeline stages, folds them
// times the class factor into Kahan-compensated FP32 running sums held in shared memory
// (so registers grow by 2 per shell, allowing groups of up to 32 shells). Lanes run over
// (group, direction) pairs of a system, so ragged direction counts leave no idle lanes
// except in the last tile. Staging, the per-warp bulk-copy ring, bounded mbarrier waits
// and the persistent work queue follow the direct kernel.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace sassgpu {

namespace {

constexpr int kRecWarps = 8, kRecAtoms = 128, kRecStages = 2, kRecBlock = 32;
// Block sums are folded into the Kahan state where the class changes and at least every
// kRecFoldStages stages (512 atoms of plain FP32 sums: relative rounding about 1e-5).
constexpr int kRecFoldStages = 4;

// Shared memory: per warp a ring of coordinate stages, the stage barriers, the tile
// slot and the Kahan state (sum re, sum im, compensation re, compensation im) of every
// (shell, lane) as float4 [warp][k][lane].
template <int K>
struct RecLayout {
    static constexpr int kCoordBytes = kRecWarps * kRecStages * kRecAtoms * 16;
    static constexpr int kBarOffset = kCoordBytes;
    static constexpr int kTileOffset = kBarOffset + kRecWarps * kRecStages * 8;
    static constexpr int kKahanOffset = (kTileOffset + 16 + 127) / 128 * 128;
    static constexpr int kBytes = kKahanOffset + kRecWarps * K * 32 * 16;
};

__device__ __forceinline__ void issue_coords(float4* sx, uint64_t* bar, const float4* src) {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, kRecAtoms * 16);
    bulk_g2s(sx, src, kRecAtoms * 16, bar);
}

// Per-block sums are kept on the sign-patterned sequence w_k = s_k z_k with
// s = (+1, +1, -1, -1, +1, +1, ...): then w_{k+1} = r_k 2cos(theta) w_k + w_{k-1} with
// r_k = -1 for odd k and +1 for even k, so every step is one paired FMA whose addend
// needs no negation, and the sign s_k is applied once when the block sums are folded.
__host__ __device__ constexpr float rec_sign(int k) { return ((k >> 1) & 1) ? -1.f : 1.f; }

// Fold the block sums (minus the padding atoms' exact contribution: z_k = 1 each) times
// the class factors into the Kahan state (sum re, sum im, compensation re, im) and clear.
template <int K>
__device__ __forceinline__ void kahan_fold(float4* __restrict__ ks, float2 (&acc)[K], float npad,
                                           const float* __restrict__ bf) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const float b = __ldg(bf + k);
        const float sg = rec_sign(k);
        float4 a = ks[k * 32];
        float y = fmaf(b, __fsub_rn(sg * acc[k].x, npad), -a.z);
        float t = __fadd_rn(a.x, y);
        a.z = __fsub_rn(__fsub_rn(t, a.x), y);
        a.x = t;
        y = fmaf(b, sg * acc[k].y, -a.w);
        t = __fadd_rn(a.y, y);
        a.w = __fsub_rn(__fsub_rn(t, a.y), y);
        a.y = t;
        ks[k * 32] = a;
        acc[k] = make_float2(0.f, 0.f);
    }
}

template <int K>
__global__ void __launch_bounds__(kRecWarps * 32, K <= 20 ? 2 : 1) phase_rec_kernel(const RecLaunch a) {
    using L = RecLayout<K>;
    constexpr int T = kRecAtoms, S = kRecStages, NB = kRecAtoms / kRecBlock;
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* sx = reinterpret_cast<float4*>(smem) + warp * S * T;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::kBarOffset) + warp * S;
    volatile int* s_tile = reinterpret_cast<volatile int*>(smem + L::kTileOffset);
    float4* ks = reinterpret_cast<float4*>(smem + L::kKahanOffset) + warp * K * 32 + lane;

    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncwarp();
    unsigned used = 0;
    bool failed = false;
    const double inv2pi = 0.15915494309189533577;
    // Thread 0 takes the next tile from the queue when the current one starts and publishes
    // it at the next loop head, so the atomic's round trip overlaps the tile's work.
    int next_tile = 0;
    if (threadIdx.x == 0) next_tile = (int)atomicAdd(a.counter, 1u);

    for (;;) {
        if (threadIdx.x == 0) *s_tile = next_tile;
        __syncthreads();  // also: the previous tile's results are read out of the Kahan state
        const int ti_ = *s_tile;
        if (ti_ >= a.ntiles) break;
        if (threadIdx.x == 0) next_tile = (int)atomicAdd(a.counter, 1u);
        const RecTileDesc td = a.tiles[ti_];
        const RecSystem& sys = a.systems[td.system];
        const int nf = sys.nf;
        // this lane's (group, direction) pair
        const bool act = lane < td.np;
        const int p = td.p0 + (act ? lane : 0);
        const int gl = p / sys.nd, d = p - gl * sys.nd;
        const RecGroup g = a.groups[sys.g_begin + gl];
        const float* bf = a.bfac + (size_t)(sys.g_begin + gl) * kRecMaxClass * K;
        const double* u = sys.dirs + 3 * (size_t)d;
        const float ux = (float)(u[0] * inv2pi), uy = (float)(u[1] * inv2pi), uz = (float)(u[2] * inv2pi);
        const float q0 = (float)g.lam0, dq = (float)g.dlam;

#pragma unroll
        for (int k = 0; k < K; ++k) ks[k * 32] = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 acc[K];
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = make_float2(0.f, 0.f);
        const float2 qd = make_float2(q0, dq);
        const float2 k2pi = make_float2(6.28318530717958647692f, 6.28318530717958647692f);
        const float2 kTwo = make_float2(2.f, -2.f);
        const int f = td.f0 + warp;
        const int nst = (td.j_end - td.j_begin) / T;

        if (f < nf && nst > 0 && !failed) {
            const float4* row = sys.xyzw + (size_t)f * sys.na_rec + td.j_begin;
            const int* binfo = sys.block_class + td.j_begin / kRecBlock;
            if (lane == 0)
                for (int k = 0; k < S && k < nst; ++k) {
                    const unsigned slot = (used + k) % S;
                    issue_coords(sx + slot * T, &bars[slot], row + k * T);
                }
            int t = 0;
            int info = __ldg(binfo);
            float npad = 0.f;
            for (; t < nst; ++t) {
                const unsigned slot = (used + t) % S;
                const bool ok = mbar_wait_parity(&bars[slot], ((used + t) / S) & 1u);
                if (!__all_sync(0xffffffffu, ok)) break;
                const float4* cx = sx + slot * T;
#pragma unroll 1
                for (int b = 0; b < NB; ++b) {
#pragma unroll 4
                    for (int jj = 0; jj < kRecBlock; ++jj) {
                        const float4 r = cx[b * kRecBlock + jj];
                        const float du = fmaf(r.z, uz, fmaf(r.y, uy, __fmul_rn(r.x, ux)));
                        const float2 dd = make_float2(du, du);
                        // (lam0, dlam) x u.r in revolutions, reduced to [-1/2, 1/2]: n is the
                        // nearest integer of the rounded product, then f = lam u.r - n by FMA
                        // (magic-number rounding took two more operations per pair on the FMA
                        // pipe, which bounds this kernel: 1.7 % slower on the GB300)
                        const float2 pr = __fmul2_rn(qd, dd);
                        const float2 nn = make_float2(-rintf(pr.x), -rintf(pr.y));
                        const float2 x = __fmul2_rn(__ffma2_rn(qd, dd, nn), k2pi);
                        float s0, c0, s1, c1;
                        __sincosf(x.x, &s0, &c0);
                        __sincosf(x.y, &s1, &c1);
                        const float2 w0 = make_float2(c0, s0);
                        // w1 = z1 = z0 exp(i theta) by a complex product on the FMA pipe: a third
                        // SFU pair for z1 instead (one more SFU result per atom) made the kernel
                        // 5.5 % slower on the GB300, whose SFU pipe then limits
                        const float2 w1 = __ffma2_rn(make_float2(-s0, c0), make_float2(s1, s1),
                                                     __fmul2_rn(w0, make_float2(c1, c1)));
                        const float2 c2 = __fmul2_rn(make_float2(c1, c1), kTwo);  // (2c, -2c)
                        const float2 cp = make_float2(c2.x, c2.x), cn = make_float2(c2.y, c2.y);
                        acc[0] = __fadd2_rn(acc[0], w0);
                        if (K > 1) {
                            acc[1] = __fadd2_rn(acc[1], w1);
                            float2 wa = w0, wb = w1;
#pragma unroll
                            for (int k = 2; k < K; ++k) {
                                const float2 wc = __ffma2_rn((k & 1) ? cp : cn, wb, wa);
                                acc[k] = __fadd2_rn(acc[k], wc);
                                wa = wb;
                                wb = wc;
                            }
                        }
                    }
                    npad += (float)(info >> 16);
                    const int nb = t * NB + b + 1;  // the tile's next 32-atom block
                    const int next = nb < nst * NB ? __ldg(binfo + nb) : -1;
                    const bool fold_stage = b + 1 == NB && (t + 1) % kRecFoldStages == 0;
                    // warp-uniform: every lane reads the same block information; the
                    // tile's last block always folds (next = -1 is no class)
                    if (fold_stage || (next & 0xffff) != (info & 0xffff)) {
                        kahan_fold<K>(ks, acc, npad, bf + (info & 0xffff) * K);
                        npad = 0.f;
                    }
                    info = next;
                }
                __syncwarp();
                if (lane == 0 && t + S < nst) issue_coords(sx + slot * T, &bars[slot], row + (t + S) * T);
            }
            if (t < nst) {
                if (lane == 0) {
                    set_error(a.err, DEV_MBAR_TIMEOUT);
                    for (int k = t; k < nst && k < t + S; ++k)
                        mbar_wait_parity(&bars[(used + k) % S], ((used + k) / S) & 1u);
                }
                failed = true;
                __syncwarp();
            }
            used += nst;
        }
        // Results from the Kahan state of all warps: thread (l, w) = (tid / 8, tid % 8) writes
        // frame f0 + w of lane l's (group, direction) pair for every shell of the group, so 8
        // consecutive threads write one (shell, direction) row's frames [f0, f0 + 8) as one
        // contiguous segment. Every (split, shell, direction, frame) slot is written, also for
        // empty atom ranges.
        __syncthreads();
        {
            static_assert(kRecWarps == 8, "8 frames per tile: one per warp, 8 threads per output row");
            const int w = threadIdx.x % kRecWarps, l = threadIdx.x / kRecWarps;
            if (td.f0 + w < nf && l < td.np) {
                const int pl = td.p0 + l;
                const int gw = pl / sys.nd, dw = pl - gw * sys.nd;
                const RecGroup gr = a.groups[sys.g_begin + gw];
                const size_t row_stride = (size_t)sys.nd * nf;
                float2* dst = sys.out_f32 + (size_t)td.split * sys.split_stride +
                              ((size_t)gr.s0 * sys.nd + dw) * nf + td.f0 + w;
                const float4* ks_all = reinterpret_cast<const float4*>(smem + L::kKahanOffset) + w * K * 32 + l;
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    if (k >= gr.ks) break;
                    const float4 st = ks_all[k * 32];
                    // sum minus compensation, rounded once in FP32 (through FP64 these two
                    // subtractions and six conversions per value made every tile's epilogue
                    // wait about 9 us on GB300's narrow FP64 pipe)
                    dst[k * row_stride] = make_float2(__fsub_rn(st.x, st.z), __fsub_rn(st.y, st.w));
                }
            }
        }
    }
}

template <int K>
cudaError_t launch_rec(const RecLaunch& a, cudaStream_t st) {
    auto k = phase_rec_kernel<K>;
    const int smem = RecLayout<K>::kBytes;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kRecWarps * 32, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    long long grid = (long long)std::max(per_sm, 1) * std::max(sms, 1);
    if (a.max_ctas > 0) grid = std::min<long long>(grid, a.max_ctas);
    if (grid > a.ntiles) grid = a.ntiles;
    if (grid < 1) return cudaSuccess;
    k<<<(unsigned)grid, kRecWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

// bfac[g][c][k] = class_factors[s0 + k][c] (float) for k < ks, else 0
__global__ void rec_factors_kernel(const RecSystem* __restrict__ systems, const RecGroup* __restrict__ groups,
                                   int ngroups, int K, float* __restrict__ bfac) {
    const size_t n = (size_t)ngroups * kRecMaxClass * K;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int g = (int)(i / ((size_t)kRecMaxClass * K));
        const int r = (int)(i - (size_t)g * kRecMaxClass * K);
        const int c = r / K, k = r - c * K;
        const RecGroup gr = groups[g];
        const RecSystem& s = systems[gr.system];
        float v = 0.f;
        if (k < gr.ks && c < s.nclass) v = (float)s.cf[(size_t)(gr.s0 + k) * s.nclass + c];
        bfac[i] = v;
    }
}

}  // namespace

std::vector<int> rec_shell_counts() { return {4, 8, 12, 16, 20, 24, 32}; }

bool rec_shells_supported(int K) {
    for (int k : rec_shell_counts())
        if (k == K) return true;
    return false;
}

cudaError_t launch_rec_factors(const RecLaunch& a, int ngroups, cudaStream_t st) {
    if (ngroups <= 0) return cudaSuccess;
    const size_t n = (size_t)ngroups * kRecMaxClass * a.K;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 1024);
    rec_factors_kernel<<<blocks, 256, 0, st>>>(a.systems, a.groups, ngroups, a.K, a.bfac);
    return cudaGetLastError();
}

cudaError_t launch_phase_rec(const RecLaunch& a, cudaStream_t st) {
    if (a.ntiles <= 0) return cudaSuccess;
    switch (a.K) {
        case 4: return launch_rec<4>(a, st);
        case 8: return launch_rec<8>(a, st);
        case 12: return launch_rec<12>(a, st);
        case 16: return launch_rec<16>(a, st);
        case 20: return launch_rec<20>(a, st);
        case 24: return launch_rec<24>(a, st);
        case 32: return launch_rec<32>(a, st);
    }
    return cudaErrorInvalidValue;
}

// Class-sorted copy of the staged coordinates: dst[f][j] = src[f][map[j]] (w = 1), or
// the origin (w = 0) where map[j] < 0; a padding atom at the origin contributes exactly
// 1 to the real part of every shell, which the kernel subtracts by count.
__global__ void permute_stage_kernel(const float4* __restrict__ src, int na_pad_src, const int* __restrict__ map,
                                     int na_dst, int nf, float4* __restrict__ dst) {
    const size_t n = (size_t)nf * na_dst;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t f = i / na_dst;
        const int j = (int)(i - f * na_dst);
        const int s = map[j];
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (s >= 0) {
            r = src[f * na_pad_src + s];
            r.w = 1.f;
        }
        dst[i] = r;
    }
}

cudaError_t launch_permute_stage(const float4* src, int na_pad_src, const int* map, int na_dst, int nf, float4* dst,
                                 cudaStream_t st) {
    const size_t n = (size_t)nf * na_dst;
    const int blocks = (int)grid_blocks(n, 256, 32);
    permute_stage_kernel<<<std::max(blocks, 1), 256, 0, st>>>(src, na_pad_src, map, na_dst, nf, dst);
    return cudaGetLastError();
}

}  // namespace sassgpu
