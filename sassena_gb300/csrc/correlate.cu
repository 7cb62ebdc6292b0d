// Correlation, store and orientational-average kernels.
//
// Replaces, per sub-vector, alignpad + dsp + store of the reference
// (src/scatter_devices/all_vectors_scatter_device.cpp:186-236, smath.cpp:141-247)
// and the 1/NM normalisation (:355-360), and the whole incoherent series loop of
// SelfVectorsScatterDevice (self_vectors_scatter_device.cpp:145-239, 288-322).
//
// The reference computes, per sub-vector v, C_v = IFFT(|FFT(pad(A_v))|^2)/(2NF(NF-tau)),
// then accumulates atfinal += C_v, afinal += mean(C_v), a2final += |mean(C_v)|^2.
// Both sums over v are linear in the power spectrum P_v = |X_v|^2, so here:
//   * one forward FFT per series (cuFFT-free radix-2 DIF in shared memory, input
//     natural order, output bit-reversed; the zero upper half of the padded series
//     folds the first stage into the load),
//   * P_v is accumulated per shell (Kahan FP32 or FP64 per CTA, FP64 across CTAs),
//   * mean_tau C_v = sum_w P_v(w) K(w) with a precomputed kernel K (so no per-series
//     inverse transform is needed for afinal/a2final),
//   * ONE inverse FFT per shell (FP64 radix-2 DIT taking the bit-reversed spectrum,
//     output natural order) gives sum_v C_v, normalised in FP64.
// The padded length L is the next power of two >= 2NF; the linear correlation for
// tau < NF is the same for any L >= 2NF-1, and the normalisation uses L. Work items
// carry their system, so one launch serves systems of different NF (twiddles come from
// one table at the largest length of the launch, indexed with a per-system stride).
#include <algorithm>

#include "common.cuh"
#include "fft_util.cuh"
#include "kernels.h"

namespace sassgpu {

namespace {

// Shared memory of the FFT accumulate kernels:
//   buf [L] T2 | tw [L/2] T2 (FP32 only; FP64 twiddles are read through L1) |
//   red [NT/32] double2 | rj [nf] float4 (incoherent only)
template <class T>
size_t fft_smem(int lg, int nt, int nf, bool self) {
    size_t L = (size_t)1 << lg;
    size_t b = L * sizeof(typename cplx<T>::type);
    if (sizeof(T) == 4) b += (L / 2) * sizeof(typename cplx<T>::type);
    b += (nt / 32) * sizeof(double2);
    if (self) b += (size_t)nf * sizeof(float4);
    return b;
}

// ---------------------------------------------------------------------------------------
// Coherent autocorrelation: one CTA per chunk of series of one shell.
// ---------------------------------------------------------------------------------------
template <class T, int NT, int MAXR>
__global__ void __launch_bounds__(NT) corr_fft_kernel(CorrLaunch a) {
    typedef typename cplx<T>::type T2;
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int lg = sys.lg, L = 1 << lg, half = L >> 1, tws = a.lg_max - lg;
    T2* buf = reinterpret_cast<T2*>(smem);
    T2* twsm = buf + (1 << a.lg_max);
    const T2* tw = stage_twiddles<T, NT>(twsm, a.tw, a.lg_max);
    double2* red = reinterpret_cast<double2*>(sizeof(T) == 4 ? twsm + (1 << (a.lg_max - 1)) : twsm);
    const T2* kbr = reinterpret_cast<const T2*>(sys.kbr);
    PowerAcc<T, MAXR> acc;
    acc.clear();
    SeriesAcc<T> sacc;
    __syncthreads();
    for (int v = c.v_begin; v < c.v_end; ++v) {
        const T2* src = reinterpret_cast<const T2*>(sys.A) + (size_t)v * sys.nf;
        for (int p = threadIdx.x; p < half; p += NT) {
            T2 x = zero2<T2>();
            if (p < sys.nf) x = src[p];
            buf[p] = x;
            buf[p + half] = cmul(x, tw[p << tws]);
        }
        __syncthreads();
        dif_tail<T2, NT>(buf, tw, lg, tws);
        const T2 pv = absorb_power_t<T, NT, MAXR>(buf, L, kbr, acc);
        const T2 av = block_sum_t<T, NT>(pv.x, pv.y, reinterpret_cast<T2*>(red));
        if (threadIdx.x == 0) sacc.add(av.x, av.y);
    }
    if constexpr (sizeof(T) == 4) write_power_pair<NT, MAXR>(acc, L, a.ppart + c.part_off);
    else write_power<T, NT, MAXR>(acc, L, a.ppart + c.part_off);
    if (threadIdx.x == 0) {
        a.apart[c.slot] = sacc.mean_sum();
        a.a2part[c.slot] = sacc.sq_sum();
    }
}

// ---------------------------------------------------------------------------------------
// Incoherent autocorrelation: one CTA per chunk of atoms of one shell; each atom's
// trajectory is staged once and reused for every direction of the shell.
// ---------------------------------------------------------------------------------------
template <class T, int NT, int MAXR>
__global__ void __launch_bounds__(NT) self_fft_kernel(CorrLaunch a) {
    typedef typename cplx<T>::type T2;
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int lg = sys.lg, L = 1 << lg, half = L >> 1, tws = a.lg_max - lg, nf = sys.nf;
    T2* buf = reinterpret_cast<T2*>(smem);
    T2* twsm = buf + (1 << a.lg_max);
    const T2* tw = stage_twiddles<T, NT>(twsm, a.tw, a.lg_max);
    double2* red = reinterpret_cast<double2*>(sizeof(T) == 4 ? twsm + (1 << (a.lg_max - 1)) : twsm);
    float4* rj = reinterpret_cast<float4*>(red + NT / 32);
    const T2* kbr = reinterpret_cast<const T2*>(sys.kbr);
    const T* bfac = reinterpret_cast<const T*>(sys.bfac);
    const int v0 = sys.shell_v[c.shell], v1 = sys.shell_v[c.shell + 1];
    PowerAcc<T, MAXR> acc;
    acc.clear();
    SeriesAcc<T> sacc;
    for (int j = c.v_begin; j < c.v_end; ++j) {
        __syncthreads();  // previous atom's series fully consumed
        for (int t = threadIdx.x; t < nf; t += NT) rj[t] = sys.xyz[(size_t)t * sys.na_pad + j];
        const T b = bfac[(size_t)c.shell * sys.na_pad + j];
        __syncthreads();
        for (int v = v0; v < v1; ++v) {
            T qx, qy, qz;
            load_qv(sys.qv, sys.qrev, (size_t)v, qx, qy, qz);
            for (int p = threadIdx.x; p < half; p += NT) {
                T2 x = zero2<T2>();
                if (p < nf) x = self_term(b, rj[p], qx, qy, qz);
                buf[p] = x;
                buf[p + half] = cmul(x, tw[p << tws]);
            }
            __syncthreads();
            dif_tail<T2, NT>(buf, tw, lg, tws);
            const T2 pv = absorb_power_t<T, NT, MAXR>(buf, L, kbr, acc);
            const T2 av = block_sum_t<T, NT>(pv.x, pv.y, reinterpret_cast<T2*>(red));
            if (threadIdx.x == 0) sacc.add(av.x, av.y);
        }
    }
    if constexpr (sizeof(T) == 4) write_power_pair<NT, MAXR>(acc, L, a.ppart + c.part_off);
    else write_power<T, NT, MAXR>(acc, L, a.ppart + c.part_off);
    if (threadIdx.x == 0) {
        a.apart[c.slot] = sacc.mean_sum();
        a.a2part[c.slot] = sacc.sq_sum();
    }
}

// ---------------------------------------------------------------------------------------
// Warp-per-series form for padded lengths L <= 512: every warp transforms its own series
// in a private shared-memory buffer with warp-level barriers only, keeps its share of the
// power spectrum (bins lane + 32 r) in registers and its series sums in lane 0. The
// warps' partials are added in warp order at the end of the chunk. Same outputs as the
// CTA-per-series kernels above (used for longer series).
// ---------------------------------------------------------------------------------------
constexpr int kWarpFftMaxLg = 9, kWarpFftWarps = 8;

template <class T>
size_t warp_fft_smem(int lg_max, int nf, bool self) {
    typedef typename cplx<T>::type T2;
    const size_t Lm = (size_t)1 << lg_max;
    size_t b = (sizeof(T) == 4 ? Lm / 2 : 0) * sizeof(T2);           // twiddles (FP32)
    b += std::max(kWarpFftWarps * Lm * sizeof(T2), kWarpFftWarps * Lm * sizeof(double));  // buffers / reduce
    b += kWarpFftWarps * sizeof(double2) + kWarpFftWarps * sizeof(double);
    if (self) b += (size_t)nf * sizeof(float4);
    return b;
}

template <class T, bool SELF>
__global__ void __launch_bounds__(kWarpFftWarps * 32) warp_fft_kernel(CorrLaunch a) {
    typedef typename cplx<T>::type T2;
    constexpr int NW = kWarpFftWarps, NT = NW * 32, MAXR = (1 << kWarpFftMaxLg) / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int lg = sys.lg, L = 1 << lg, half = L >> 1, tws = a.lg_max - lg, nf = sys.nf;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int Lm = 1 << a.lg_max;
    T2* twsm = reinterpret_cast<T2*>(smem);
    unsigned char* region = smem + (sizeof(T) == 4 ? (size_t)(Lm / 2) * sizeof(T2) : 0);
    T2* buf = reinterpret_cast<T2*>(region) + (size_t)warp * Lm;
    const size_t region_bytes = NW * (size_t)Lm * (sizeof(T2) > sizeof(double) ? sizeof(T2) : sizeof(double));
    double2* red = reinterpret_cast<double2*>(region + region_bytes);
    double* red2 = reinterpret_cast<double*>(red + NW);
    float4* rj = reinterpret_cast<float4*>(red2 + NW);
    const T2* tw = stage_twiddles<T, NT>(twsm, a.tw, a.lg_max);
    const T2* kbr = reinterpret_cast<const T2*>(sys.kbr);
    PowerAcc<T, MAXR> acc;
    acc.clear();
    SeriesAcc<T> sacc;
    __syncthreads();

    // one series: folded first DIF stage on load, the other stages, power + K-weighted sum
    auto transform = [&](auto gen) {
        for (int p = lane; p < half; p += 32) {
            T2 x = zero2<T2>();
            if (p < nf) x = gen(p);
            buf[p] = x;
            buf[p + half] = cmul(x, tw[p << tws]);
        }
        __syncwarp();
        for (int lh = lg - 2; lh >= 0; --lh) {
            const int h = 1 << lh, sh = lg - 1 - lh + tws;
            for (int b = lane; b < half; b += 32) {
                const int q = b & (h - 1);
                const int i0 = ((b >> lh) << (lh + 1)) + q;
                const T2 u = buf[i0], w = buf[i0 + h];
                buf[i0] = cadd(u, w);
                buf[i0 + h] = cmul(csub(u, w), tw[q << sh]);
            }
            __syncwarp();
        }
        T ax = 0, ay = 0;
#pragma unroll
        for (int r = 0; r < MAXR; ++r) {
            const int i = lane + 32 * r;
            if (i < L) {
                const T2 X = buf[i];
                const T P = X.x * X.x + X.y * X.y;
                acc.add(r, P);
                const T2 k = kbr[i];
                ax += P * k.x;
                ay += P * k.y;
            }
        }
        const T2 av = warp_sum_t<T>(ax, ay);
        if (lane == 0) sacc.add(av.x, av.y);
        __syncwarp();  // the buffer is free for the next series
    };

    if (SELF) {
        const T* bfac = reinterpret_cast<const T*>(sys.bfac);
        const int v0 = sys.shell_v[c.shell], v1 = sys.shell_v[c.shell + 1];
        for (int j = c.v_begin; j < c.v_end; ++j) {
            __syncthreads();  // every warp is done with the previous atom's trajectory
            for (int t = threadIdx.x; t < nf; t += NT) rj[t] = sys.xyz[(size_t)t * sys.na_pad + j];
            const T b = bfac[(size_t)c.shell * sys.na_pad + j];
            __syncthreads();
            for (int v = v0 + warp; v < v1; v += NW) {
                T qx, qy, qz;
                load_qv(sys.qv, sys.qrev, (size_t)v, qx, qy, qz);
                transform([&](int p) { return self_term(b, rj[p], qx, qy, qz); });
            }
        }
    } else {
        for (int v = c.v_begin + warp; v < c.v_end; v += NW) {
            const T2* src = reinterpret_cast<const T2*>(sys.A) + (size_t)v * sys.nf;
            transform([&](int p) { return src[p]; });
        }
    }

    // partials of the warps, added in warp order
    __syncthreads();
    double* pw = reinterpret_cast<double*>(region);  // [NW][L]
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
        const int i = lane + 32 * r;
        if (i < L) pw[(size_t)warp * L + i] = acc.get(r);
    }
    if (lane == 0) {
        red[warp] = sacc.mean_sum();
        red2[warp] = sacc.sq_sum();
    }
    __syncthreads();
    double* dst = a.ppart + c.part_off;
    for (int i = threadIdx.x; i < L; i += NT) {
        double s = 0.0;
        for (int w = 0; w < NW; ++w) s += pw[(size_t)w * L + i];
        dst[i] = s;
    }
    if (threadIdx.x == 0) {
        double2 as = make_double2(0.0, 0.0);
        double a2 = 0.0;
        for (int w = 0; w < NW; ++w) {
            as.x += red[w].x;
            as.y += red[w].y;
            a2 += red2[w];
        }
        a.apart[c.slot] = as;
        a.a2part[c.slot] = a2;
    }
}

// ---------------------------------------------------------------------------------------
// dsp = square | plain (no transform): C_v(t) = |A_v(t)|^2 or A_v(t) * exp(i q_v.c).
// Partials are complex per frame (double2 [nf] at part_off).
// ---------------------------------------------------------------------------------------
template <class AT, int NT, int MAXT>
__global__ void __launch_bounds__(NT) corr_direct_kernel(CorrLaunch a) {
    __shared__ double2 red[NT / 32];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int nf = sys.nf;
    const bool square = a.dsp == DSP_SQUARE;
    const AT* A = reinterpret_cast<const AT*>(sys.A);
    if (nf > NT * MAXT) {
        // long series: the chunk's per-frame sums live in its slot; each thread owns the
        // frames t = threadIdx.x + k NT, summed over series in order as below
        double2* dst = reinterpret_cast<double2*>(a.ppart + c.part_off);
        double2 asum = make_double2(0.0, 0.0);
        double a2sum = 0.0;
        for (int v = c.v_begin; v < c.v_end; ++v) {
            double2 ph = make_double2(1.0, 0.0);
            if (!square && a.restore_phase) {
                const double* q = sys.qv + 3 * (size_t)v;
                sincos(q[0] * sys.cx + q[1] * sys.cy + q[2] * sys.cz, &ph.y, &ph.x);
            }
            double2 part = make_double2(0.0, 0.0);
            for (int t = threadIdx.x; t < nf; t += NT) {
                double2 x = to_d2(A[(size_t)v * nf + t]);
                double2 cv = square ? make_double2(x.x * x.x + x.y * x.y, 0.0) : cmul(x, ph);
                const double2 o = v == c.v_begin ? make_double2(0.0, 0.0) : dst[t];
                dst[t] = make_double2(o.x + cv.x, o.y + cv.y);
                part.x += cv.x;
                part.y += cv.y;
            }
            double2 s = block_sum<NT>(part, red);
            if (threadIdx.x == 0) {
                double2 av = make_double2(s.x * (1.0 / nf), s.y * (1.0 / nf));
                asum.x += av.x;
                asum.y += av.y;
                a2sum += av.x * av.x + av.y * av.y;
            }
        }
        if (c.v_begin == c.v_end)  // no series in the chunk: an all-zero slot
            for (int t = threadIdx.x; t < nf; t += NT) dst[t] = make_double2(0.0, 0.0);
        if (threadIdx.x == 0) {
            a.apart[c.slot] = asum;
            a.a2part[c.slot] = a2sum;
        }
        return;
    }
    double2 acc[MAXT];
#pragma unroll
    for (int r = 0; r < MAXT; ++r) acc[r] = make_double2(0.0, 0.0);
    double2 asum = make_double2(0.0, 0.0);
    double a2sum = 0.0;
    for (int v = c.v_begin; v < c.v_end; ++v) {
        double2 ph = make_double2(1.0, 0.0);
        if (!square && a.restore_phase) {
            const double* q = sys.qv + 3 * (size_t)v;
            sincos(q[0] * sys.cx + q[1] * sys.cy + q[2] * sys.cz, &ph.y, &ph.x);
        }
        double2 part = make_double2(0.0, 0.0);
#pragma unroll
        for (int r = 0; r < MAXT; ++r) {
            const int t = threadIdx.x + r * NT;
            if (t < nf) {
                double2 x = to_d2(A[(size_t)v * nf + t]);
                double2 cv = square ? make_double2(x.x * x.x + x.y * x.y, 0.0) : cmul(x, ph);
                acc[r].x += cv.x;
                acc[r].y += cv.y;
                part.x += cv.x;
                part.y += cv.y;
            }
        }
        double2 s = block_sum<NT>(part, red);
        if (threadIdx.x == 0) {
            double2 av = make_double2(s.x * (1.0 / nf), s.y * (1.0 / nf));
            asum.x += av.x;
            asum.y += av.y;
            a2sum += av.x * av.x + av.y * av.y;
        }
    }
    double2* dst = reinterpret_cast<double2*>(a.ppart + c.part_off);
#pragma unroll
    for (int r = 0; r < MAXT; ++r) {
        const int t = threadIdx.x + r * NT;
        if (t < nf) dst[t] = acc[r];
    }
    if (threadIdx.x == 0) {
        a.apart[c.slot] = asum;
        a.a2part[c.slot] = a2sum;
    }
}

template <class T, int NT, int MAXT>
__global__ void __launch_bounds__(NT) self_direct_kernel(CorrLaunch a) {
    typedef typename cplx<T>::type T2;
    __shared__ double2 red[NT / 32];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int nf = sys.nf;
    const bool square = a.dsp == DSP_SQUARE;
    const T* bfac = reinterpret_cast<const T*>(sys.bfac);
    const int v0 = sys.shell_v[c.shell], v1 = sys.shell_v[c.shell + 1];
    if (nf > NT * MAXT) {  // long series: per-frame sums in the chunk's slot (see corr_direct_kernel)
        double2* dst = reinterpret_cast<double2*>(a.ppart + c.part_off);
        double2 asum = make_double2(0.0, 0.0);
        double a2sum = 0.0;
        bool first = true;
        for (int j = c.v_begin; j < c.v_end; ++j) {
            const T b = bfac[(size_t)c.shell * sys.na_pad + j];
            for (int v = v0; v < v1; ++v) {
                const double* q = sys.qv + 3 * (size_t)v;
                double2 ph = make_double2(1.0, 0.0);
                if (!square && a.restore_phase) sincos(q[0] * sys.cx + q[1] * sys.cy + q[2] * sys.cz, &ph.y, &ph.x);
                T qx, qy, qz;
                load_qv(sys.qv, sys.qrev, (size_t)v, qx, qy, qz);
                double2 part = make_double2(0.0, 0.0);
                for (int t = threadIdx.x; t < nf; t += NT) {
                    T2 x = self_term(b, sys.xyz[(size_t)t * sys.na_pad + j], qx, qy, qz);
                    double2 xd = to_d2(x);
                    double2 cv = square ? make_double2(xd.x * xd.x + xd.y * xd.y, 0.0) : cmul(xd, ph);
                    const double2 o = first ? make_double2(0.0, 0.0) : dst[t];
                    dst[t] = make_double2(o.x + cv.x, o.y + cv.y);
                    part.x += cv.x;
                    part.y += cv.y;
                }
                first = false;
                double2 s = block_sum<NT>(part, red);
                if (threadIdx.x == 0) {
                    double2 av = make_double2(s.x * (1.0 / nf), s.y * (1.0 / nf));
                    asum.x += av.x;
                    asum.y += av.y;
                    a2sum += av.x * av.x + av.y * av.y;
                }
            }
        }
        if (first)  // no series in the chunk: an all-zero slot
            for (int t = threadIdx.x; t < nf; t += NT) dst[t] = make_double2(0.0, 0.0);
        if (threadIdx.x == 0) {
            a.apart[c.slot] = asum;
            a.a2part[c.slot] = a2sum;
        }
        return;
    }
    double2 acc[MAXT];
#pragma unroll
    for (int r = 0; r < MAXT; ++r) acc[r] = make_double2(0.0, 0.0);
    double2 asum = make_double2(0.0, 0.0);
    double a2sum = 0.0;
    for (int j = c.v_begin; j < c.v_end; ++j) {
        const T b = bfac[(size_t)c.shell * sys.na_pad + j];
        for (int v = v0; v < v1; ++v) {
            const double* q = sys.qv + 3 * (size_t)v;
            double2 ph = make_double2(1.0, 0.0);
            if (!square && a.restore_phase) sincos(q[0] * sys.cx + q[1] * sys.cy + q[2] * sys.cz, &ph.y, &ph.x);
            T qx, qy, qz;
            load_qv(sys.qv, sys.qrev, (size_t)v, qx, qy, qz);
            double2 part = make_double2(0.0, 0.0);
#pragma unroll
            for (int r = 0; r < MAXT; ++r) {
                const int t = threadIdx.x + r * NT;
                if (t < nf) {
                    T2 x = self_term(b, sys.xyz[(size_t)t * sys.na_pad + j], qx, qy, qz);
                    double2 xd = to_d2(x);
                    double2 cv = square ? make_double2(xd.x * xd.x + xd.y * xd.y, 0.0) : cmul(xd, ph);
                    acc[r].x += cv.x;
                    acc[r].y += cv.y;
                    part.x += cv.x;
                    part.y += cv.y;
                }
            }
            double2 s = block_sum<NT>(part, red);
            if (threadIdx.x == 0) {
                double2 av = make_double2(s.x * (1.0 / nf), s.y * (1.0 / nf));
                asum.x += av.x;
                asum.y += av.y;
                a2sum += av.x * av.x + av.y * av.y;
            }
        }
    }
    double2* dst = reinterpret_cast<double2*>(a.ppart + c.part_off);
#pragma unroll
    for (int r = 0; r < MAXT; ++r) {
        const int t = threadIdx.x + r * NT;
        if (t < nf) dst[t] = acc[r];
    }
    if (threadIdx.x == 0) {
        a.apart[c.slot] = asum;
        a.a2part[c.slot] = a2sum;
    }
}

// ---------------------------------------------------------------------------------------
// Per-shell finalisation in FP64: sum partial slots, inverse FFT (autocorrelate),
// normalise by 1/(L (NF - tau)) and 1/NM, conjugate for dsp.method = direct.
// ---------------------------------------------------------------------------------------
// Sums over a shell's partial slots, in slot order. The slots' loads are issued eight at a
// time ahead of their additions, so a thread waits on memory once per eight slots instead
// of once per slot (the finalisation runs one CTA per shell, too few to hide latency with
// warps). FP64 slots are added in FP64 in the order of a plain loop.
constexpr int kSlotBatch = 8;

__device__ __forceinline__ double slot_sum(const double* __restrict__ src, size_t stride, int n, int f32pair) {
    if (f32pair) {
        // FP32 Kahan pairs (sum s_k, compensation c_k) with value s_k - c_k, added in
        // float-float arithmetic on the FP32 pipe (Knuth's TwoSum for the sums, the
        // compensations and rounding errors in the low word), converted to FP64 once:
        // on GB300 an FP64 conversion and two FP64 adds per slot made this loop the
        // bound of the finalisation. Relative rounding ~n * 2^-48, far below the FP32
        // form's partials' own.
        float hi = 0.f, lo = 0.f;
        for (int k0 = 0; k0 < n; k0 += kSlotBatch) {
            float2 v[kSlotBatch];
#pragma unroll
            for (int u = 0; u < kSlotBatch; ++u)
                v[u] = k0 + u < n ? __ldg(reinterpret_cast<const float2*>(src + (size_t)(k0 + u) * stride))
                                  : make_float2(0.f, 0.f);
#pragma unroll
            for (int u = 0; u < kSlotBatch; ++u) {
                const float s = __fadd_rn(hi, v[u].x), bb = __fsub_rn(s, hi);
                const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v[u].x, bb));
                hi = s;
                lo = __fadd_rn(lo, __fsub_rn(e, v[u].y));
            }
        }
        return (double)hi + (double)lo;
    }
    double p = 0.0;
    for (int k0 = 0; k0 < n; k0 += kSlotBatch) {
        double v[kSlotBatch];
#pragma unroll
        for (int u = 0; u < kSlotBatch; ++u) v[u] = k0 + u < n ? __ldg(src + (size_t)(k0 + u) * stride) : 0.0;
#pragma unroll
        for (int u = 0; u < kSlotBatch; ++u)
            if (k0 + u < n) p += v[u];
    }
    return p;
}

template <int NT>
__global__ void __launch_bounds__(NT) finalize_kernel(FinalLaunch a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const FinalEntry e = a.entries[blockIdx.x];
    const int nf = e.nf, ns = e.slot_end - e.slot_begin;
    const double sgn = a.conj_out ? -1.0 : 1.0;
    const double* part = a.ppart + e.part_off;
    if (a.dsp == DSP_AUTOCORRELATE) {
        const int L = 1 << e.lg;
        double2* buf = reinterpret_cast<double2*>(smem);
        if (L < NT) {
            // fewer bins than threads: G = NT / L threads per bin, each summing a contiguous
            // range of the slots; the G partial sums are then added in range order (a short
            // series' shell otherwise left most threads idle while a quarter of them walked
            // every slot: 112 chunk slots of the 256-point incoherent spectra)
            double* gp = reinterpret_cast<double*>(smem + ((size_t)1 << a.lg_max) * sizeof(double2));
            const int G = NT / L, i = threadIdx.x % L, g = threadIdx.x / L;
            const int s0 = (int)((long long)ns * g / G), s1 = (int)((long long)ns * (g + 1) / G);
            gp[threadIdx.x] = slot_sum(part + (size_t)s0 * e.part_len + i, e.part_len, s1 - s0, e.f32pair);
            __syncthreads();
            if (threadIdx.x < L) {
                double v = 0.0;
                for (int k = 0; k < G; ++k) v += gp[k * L + threadIdx.x];
                buf[threadIdx.x] = make_double2(v, 0.0);
            }
        } else {
            for (int i = threadIdx.x; i < L; i += NT)
                buf[i] = make_double2(slot_sum(part + i, e.part_len, ns, e.f32pair), 0.0);
        }
        __syncthreads();
        dit_inverse<NT>(buf, a.tw, e.lg, a.lg_max - e.lg);
        for (int t = threadIdx.x; t < nf; t += NT) {
            double f = (1.0 / ((double)L * (double)(nf - t))) * e.inv_nm;
            e.fqt[t] = make_double2(buf[t].x * f, sgn * buf[t].y * f);
        }
    } else {
        for (int t = threadIdx.x; t < nf; t += NT) {
            const double vx = slot_sum(part + 2 * t, e.part_len, ns, 0);
            const double vy = slot_sum(part + 2 * t + 1, e.part_len, ns, 0);
            e.fqt[t] = make_double2(vx * e.inv_nm, sgn * vy * e.inv_nm);
        }
    }
    if (threadIdx.x == 0) {
        double2 as = make_double2(0.0, 0.0);
        double a2 = 0.0;
        for (int k0 = e.slot_begin; k0 < e.slot_end; k0 += kSlotBatch) {
            double2 va[kSlotBatch];
            double v2[kSlotBatch];
#pragma unroll
            for (int u = 0; u < kSlotBatch; ++u) {
                const bool in = k0 + u < e.slot_end;
                va[u] = in ? a.apart[k0 + u] : make_double2(0.0, 0.0);
                v2[u] = in ? a.a2part[k0 + u] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kSlotBatch; ++u)
                if (k0 + u < e.slot_end) {
                    as.x += va[u].x;
                    as.y += va[u].y;
                    a2 += v2[u];
                }
        }
        *e.fq = make_double2(as.x * e.inv_nm, sgn * as.y * e.inv_nm);
        *e.fq2 = make_double2(a2 * e.inv_nm, 0.0);
    }
}

__global__ void twiddle_kernel(double2* tw64, float2* tw32, int L) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L / 2; k += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(-2.0 * (double)k / (double)L, &s, &c);
        tw64[k] = make_double2(c, s);
        tw32[k] = make_float2((float)c, (float)s);
    }
}

// K(w) = sum_{tau<NF} exp(+2 pi i w tau / L) / (NF L (NF - tau)) at bit-reversed position
// of w; exp(+2 pi i m / L) = conj(tw[m]) for m < L/2 and -conj(tw[m - L/2]) otherwise,
// with tw the table of length 2^lg_tw >= L read at stride 2^(lg_tw - lg).
__global__ void store_kernel_kernel(const double2* __restrict__ tw, int lg_tw, double2* k64,
                                    float2* k32, int nf, int lg) {
    const int L = 1 << lg, sh = lg_tw - lg;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < L; w += gridDim.x * blockDim.x) {
        double re = 0.0, im = 0.0;
        long long m = 0;
        for (int t = 0; t < nf; ++t) {
            const double wt = 1.0 / ((double)nf * (double)L * (double)(nf - t));
            const bool lo = m < L / 2;
            double2 z = tw[(lo ? m : m - L / 2) << sh];
            const double sg = lo ? 1.0 : -1.0;
            re += wt * sg * z.x;
            im -= wt * sg * z.y;
            m += w;
            if (m >= L) m -= L;
        }
        const int i = (int)(__brev((unsigned)w) >> (32 - lg));
        k64[i] = make_double2(re, im);
        k32[i] = make_float2((float)re, (float)im);
    }
}

// x - (h + l) rounded to FP32: s + e = x - h exactly (TwoSum), then s + (e - l)
__device__ __forceinline__ float centred(float x, float h, float l) {
    const float s = __fsub_rn(x, h), bb = __fsub_rn(s, x);
    const float e = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(-h, bb));
    return __fadd_rn(s, __fsub_rn(e, l));
}

__global__ void stage_kernel(const float* __restrict__ raw, int nf, int na, int na_pad, double cx,
                             double cy, double cz, int center, float4* __restrict__ xyz,
                             const int* __restrict__ rec_inv, int na_rec, float4* __restrict__ xyz_rec) {
    const size_t n = (size_t)nf * na_pad;
    // the centre as float pairs hi + lo: x - c is formed by TwoSum in FP32 and rounded once
    // (per coordinate an FP64 subtraction and two conversions made this kernel bound by
    // GB300's narrow FP64 pipe once its input came from device memory)
    const float hx = (float)cx, hy = (float)cy, hz = (float)cz;
    const float lx = (float)(cx - (double)hx), ly = (float)(cy - (double)hy), lz = (float)(cz - (double)hz);
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const size_t f = idx / na_pad;
        const int j = (int)(idx - f * na_pad);
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j < na) {
            const float* p = raw + (f * na + j) * 3;
            if (center) {
                r.x = centred(p[0], hx, lx);
                r.y = centred(p[1], hy, ly);
                r.z = centred(p[2], hz, lz);
            } else {
                r.x = p[0];
                r.y = p[1];
                r.z = p[2];
            }
            if (xyz_rec) xyz_rec[f * na_rec + rec_inv[j]] = make_float4(r.x, r.y, r.z, 1.f);
        }
        xyz[idx] = r;
    }
}

template <class T>
__global__ void expand_factors_kernel(const double* __restrict__ cf, int nclass, int nshell,
                                      const int* __restrict__ cls, int na_pad, T* __restrict__ b) {
    const size_t n = (size_t)nshell * na_pad;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const size_t s = idx / na_pad;
        const int j = (int)(idx - s * na_pad);
        const int c = cls[j];
        b[idx] = (c >= 0 && c < nclass) ? (T)cf[s * nclass + c] : (T)0;
    }
}

// ---------------------------------------------------------------------------------------
// dsp = square / plain, coherent, series of at most 32 K frames: warp per series. Lane l holds
// frames l + 32 k (k < K) of the chunk's per-frame sums in registers (Kahan FP32 in the FP32
// form, FP64 in the FP64 form); each series' mean is one warp reduction; the warps' frame
// sums and series sums are combined in warp order at the end of the chunk. Replaces a CTA per
// series with two CTA-wide FP64 reductions each (short series left most of its threads idle).
// ---------------------------------------------------------------------------------------
constexpr int kSqWarps = 8;

template <class T>
struct FrameAcc;  // per-frame complex sums of one lane

template <>
struct FrameAcc<float> {
    float sx, sy, cx, cy;
    __device__ void clear() { sx = sy = cx = cy = 0.f; }
    __device__ __forceinline__ void add(float x, float y) {
        SeriesAcc<float>::kahan(sx, cx, x);
        SeriesAcc<float>::kahan(sy, cy, y);
    }
    __device__ double2 get() const { return make_double2((double)sx - (double)cx, (double)sy - (double)cy); }
};

template <>
struct FrameAcc<double> {
    double sx, sy;
    __device__ void clear() { sx = sy = 0.0; }
    __device__ __forceinline__ void add(double x, double y) {
        sx += x;
        sy += y;
    }
    __device__ double2 get() const { return make_double2(sx, sy); }
};

// exp(i q_v . c), the centring phase restored for dsp = plain in the FP32 form: in
// revolutions with the nearest integer removed, then the SFU (phase error about 1e-5 rad
// for |q . c| up to 25 revolutions, far inside the FP32 form's 1e-3). FP64 form: FP64.
__device__ __forceinline__ float2 restore_phase(const CorrSystem& sys, size_t v, float) {
    const float4 q = sys.qrev[v];
    const float u = fmaf(q.z, (float)sys.cz, fmaf(q.y, (float)sys.cy, q.x * (float)sys.cx));
    float s, c;
    __sincosf(__fsub_rn(u, rintf(u)) * 6.28318530717958647692f, &s, &c);
    return make_float2(c, s);
}
__device__ __forceinline__ double2 restore_phase(const CorrSystem& sys, size_t v, double) {
    const double* q = sys.qv + 3 * v;
    double s, c;
    sincos(q[0] * sys.cx + q[1] * sys.cy + q[2] * sys.cz, &s, &c);
    return make_double2(c, s);
}

template <class T, int K>
__global__ void __launch_bounds__(kSqWarps * 32) corr_sq_warp_kernel(CorrLaunch a) {
    typedef typename cplx<T>::type T2;
    constexpr int NW = kSqWarps, NT = NW * 32;
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int nf = sys.nf, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool square = a.dsp == DSP_SQUARE;
    const T2* A = reinterpret_cast<const T2*>(sys.A);
    double2* pw = reinterpret_cast<double2*>(smem);  // [NW][nf] frame sums, then [NW] series sums
    FrameAcc<T> acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k].clear();
    SeriesAcc<T> sacc;
    const T inv_nf = T(1) / T(nf);
    for (int v = c.v_begin + warp; v < c.v_end; v += NW) {
        T2 ph;
        ph.x = T(1);
        ph.y = T(0);
        if (!square && a.restore_phase) ph = restore_phase(sys, (size_t)v, T());
        T px = 0, py = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int t = lane + 32 * k;
            if (t < nf) {
                const T2 x = A[(size_t)v * nf + t];
                T2 cv;
                if (square) {
                    cv.x = x.x * x.x + x.y * x.y;
                    cv.y = T(0);
                } else {
                    cv = cmul(x, ph);
                }
                acc[k].add(cv.x, cv.y);
                px += cv.x;
                py += cv.y;
            }
        }
        const T2 sv = warp_sum_t<T>(px, py);
        if (lane == 0) sacc.add(sv.x * inv_nf, sv.y * inv_nf);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int t = lane + 32 * k;
        if (t < nf) pw[(size_t)warp * nf + t] = acc[k].get();
    }
    double2* red = pw + (size_t)NW * nf;
    double* red2 = reinterpret_cast<double*>(red + NW);
    if (lane == 0) {
        red[warp] = sacc.mean_sum();
        red2[warp] = sacc.sq_sum();
    }
    __syncthreads();
    double* dst = a.ppart + c.part_off;
    for (int t = threadIdx.x; t < nf; t += NT) {
        double2 s = make_double2(0.0, 0.0);
        for (int w = 0; w < NW; ++w) {
            s.x += pw[(size_t)w * nf + t].x;
            s.y += pw[(size_t)w * nf + t].y;
        }
        dst[2 * t] = s.x;
        dst[2 * t + 1] = s.y;
    }
    if (threadIdx.x == 0) {
        double2 as = make_double2(0.0, 0.0);
        double a2 = 0.0;
        for (int w = 0; w < NW; ++w) {
            as.x += red[w].x;
            as.y += red[w].y;
            a2 += red2[w];
        }
        a.apart[c.slot] = as;
        a.a2part[c.slot] = a2;
    }
}

template <class T, int K>
cudaError_t launch_sq_warp_k(const CorrLaunch& a, cudaStream_t st) {
    const size_t sm = (size_t)kSqWarps * a.nf_max * sizeof(double2) + kSqWarps * (sizeof(double2) + sizeof(double));
    auto k = corr_sq_warp_kernel<T, K>;
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<a.nchunks, kSqWarps * 32, sm, st>>>(a);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_sq_warp(const CorrLaunch& a, cudaStream_t st) {
    const int k = (a.nf_max + 31) / 32;
    if (k <= 2) return launch_sq_warp_k<T, 2>(a, st);
    if (k <= 4) return launch_sq_warp_k<T, 4>(a, st);
    if (k <= 8) return launch_sq_warp_k<T, 8>(a, st);
    return launch_sq_warp_k<T, 16>(a, st);
}

constexpr int kSqWarpMaxNf = 512;

// The same for the incoherent device: trajectories of kSqAtoms atoms of the chunk are staged
// per barrier (coalesced over atoms), and the warps share out their (atom, direction) series,
// generated in registers.
constexpr int kSqAtoms = 4;

template <class T, int K>
__global__ void __launch_bounds__(kSqWarps * 32) self_sq_warp_kernel(CorrLaunch a) {
    typedef typename cplx<T>::type T2;
    constexpr int NW = kSqWarps, NT = NW * 32, NAS = kSqAtoms;
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int nf = sys.nf, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool square = a.dsp == DSP_SQUARE;
    const T* bfac = reinterpret_cast<const T*>(sys.bfac);
    const int v0 = sys.shell_v[c.shell], nd = sys.shell_v[c.shell + 1] - v0;
    float4* rj = reinterpret_cast<float4*>(smem);                          // [NAS][nf]
    double2* pw = reinterpret_cast<double2*>(rj + (size_t)NAS * a.nf_max);  // [NW][nf], then series sums
    T* bsm = reinterpret_cast<T*>(pw + (size_t)NW * a.nf_max + 2 * NW);     // [NAS]
    FrameAcc<T> acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k].clear();
    SeriesAcc<T> sacc;
    const T inv_nf = T(1) / T(nf);
    for (int j0 = c.v_begin; j0 < c.v_end; j0 += NAS) {
        const int na = min(NAS, c.v_end - j0);
        __syncthreads();  // every warp is done with the previous atoms' trajectories
        for (int i = threadIdx.x; i < na * nf; i += NT) {
            const int t = i / na, at = i - t * na;
            rj[at * nf + t] = sys.xyz[(size_t)t * sys.na_pad + j0 + at];
        }
        if (threadIdx.x < na) bsm[threadIdx.x] = bfac[(size_t)c.shell * sys.na_pad + j0 + threadIdx.x];
        __syncthreads();
        for (int pr = warp; pr < na * nd; pr += NW) {
            const int at = pr / nd, v = v0 + (pr - at * nd);
            T qx, qy, qz;
            load_qv(sys.qv, sys.qrev, (size_t)v, qx, qy, qz);
            const T b = bsm[at];
            const float4* ra = rj + (size_t)at * nf;
            T2 ph;
            ph.x = T(1);
            ph.y = T(0);
            if (!square && a.restore_phase) ph = restore_phase(sys, (size_t)v, T());
            T px = 0, py = 0;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int t = lane + 32 * k;
                if (t < nf) {
                    const T2 x = self_term(b, ra[t], qx, qy, qz);
                    T2 cv;
                    if (square) {
                        cv.x = x.x * x.x + x.y * x.y;
                        cv.y = T(0);
                    } else {
                        cv = cmul(x, ph);
                    }
                    acc[k].add(cv.x, cv.y);
                    px += cv.x;
                    py += cv.y;
                }
            }
            const T2 sv = warp_sum_t<T>(px, py);
            if (lane == 0) sacc.add(sv.x * inv_nf, sv.y * inv_nf);
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int t = lane + 32 * k;
        if (t < nf) pw[(size_t)warp * nf + t] = acc[k].get();
    }
    double2* red = pw + (size_t)NW * nf;
    double* red2 = reinterpret_cast<double*>(red + NW);
    if (lane == 0) {
        red[warp] = sacc.mean_sum();
        red2[warp] = sacc.sq_sum();
    }
    __syncthreads();
    double* dst = a.ppart + c.part_off;
    for (int t = threadIdx.x; t < nf; t += NT) {
        double2 s = make_double2(0.0, 0.0);
        for (int w = 0; w < NW; ++w) {
            s.x += pw[(size_t)w * nf + t].x;
            s.y += pw[(size_t)w * nf + t].y;
        }
        dst[2 * t] = s.x;
        dst[2 * t + 1] = s.y;
    }
    if (threadIdx.x == 0) {
        double2 as = make_double2(0.0, 0.0);
        double a2 = 0.0;
        for (int w = 0; w < NW; ++w) {
            as.x += red[w].x;
            as.y += red[w].y;
            a2 += red2[w];
        }
        a.apart[c.slot] = as;
        a.a2part[c.slot] = a2;
    }
}

template <class T, int K>
cudaError_t launch_self_sq_warp_k(const CorrLaunch& a, cudaStream_t st) {
    const size_t sm = (size_t)kSqAtoms * a.nf_max * sizeof(float4) + (size_t)kSqWarps * a.nf_max * sizeof(double2) +
                      2 * kSqWarps * sizeof(double2) + kSqAtoms * sizeof(double);
    auto k = self_sq_warp_kernel<T, K>;
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<a.nchunks, kSqWarps * 32, sm, st>>>(a);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_self_sq_warp(const CorrLaunch& a, cudaStream_t st) {
    const int k = (a.nf_max + 31) / 32;
    if (k <= 2) return launch_self_sq_warp_k<T, 2>(a, st);
    if (k <= 4) return launch_self_sq_warp_k<T, 4>(a, st);
    if (k <= 8) return launch_self_sq_warp_k<T, 8>(a, st);
    return launch_self_sq_warp_k<T, 16>(a, st);
}

template <class T, int NT, int MAXR>
cudaError_t launch_fft(const CorrLaunch& a, bool self, cudaStream_t st) {
    const size_t sm = fft_smem<T>(a.lg_max, NT, a.nf_max, self);
    auto k = self ? self_fft_kernel<T, NT, MAXR> : corr_fft_kernel<T, NT, MAXR>;
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<a.nchunks, NT, sm, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Register-resident warp FFT for one padded length L = 32 E (64 <= L <= 512) shared by
// every system of the launch. Lane l holds elements l + 32 m (m < E), generated or loaded
// in place: the folded first DIF stage and the stages of span >= 32 pair elements inside
// a lane; the five stages of span 16 .. 1 pair lanes l and l ^ h through shuffles. The
// output is in bit-reversed order at the same positions l + 32 m, which are exactly the
// power-spectrum bins this lane accumulates, so no shared memory holds series data.
// ---------------------------------------------------------------------------------------
__host__ __device__ constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v >> 1); }

template <class T2>
__device__ __forceinline__ T2 shfl_xor2(T2 v, int m) {
    v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
    v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
    return v;
}

constexpr int kRegFftAtoms = 8;  // incoherent: atoms whose trajectories are staged together

template <class T>
size_t reg_fft_smem(int lg, int nf, bool self) {
    typedef typename cplx<T>::type T2;
    size_t b = (sizeof(T) == 4 ? ((size_t)1 << lg) / 2 : 0) * sizeof(T2);
    b += (size_t)kWarpFftWarps * ((size_t)1 << lg) * sizeof(double);  // warp partials
    b += kWarpFftWarps * sizeof(double2) + kWarpFftWarps * sizeof(double);
    if (self) b += (size_t)kRegFftAtoms * nf * sizeof(float4) + kRegFftAtoms * sizeof(double);
    return b;
}

template <class T, int LG, bool SELF>
__global__ void __launch_bounds__(kWarpFftWarps * 32, (LG <= 8 && sizeof(T) == 4) ? 3 : 2) reg_fft_kernel(CorrLaunch a) {
    typedef typename cplx<T>::type T2;
    constexpr int NW = kWarpFftWarps, NT = NW * 32, L = 1 << LG, E = L / 32, EH = E / 2;
    static_assert(E >= 2 && E <= 16, "register FFT lengths 64 .. 512");
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int nf = sys.nf, tws = a.lg_max - LG;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T2* twsm = reinterpret_cast<T2*>(smem);
    unsigned char* region = smem + (sizeof(T) == 4 ? (size_t)(L / 2) * sizeof(T2) : 0);
    double* pw = reinterpret_cast<double*>(region);  // [NW][L] warp partials at the end
    double2* red = reinterpret_cast<double2*>(pw + (size_t)NW * L);
    double* red2 = reinterpret_cast<double*>(red + NW);
    float4* rj = reinterpret_cast<float4*>(red2 + NW);
    const T2* tw = stage_twiddles<T, NT>(twsm, a.tw, a.lg_max);
    const T2* kbr = reinterpret_cast<const T2*>(sys.kbr);
    PowerAcc<T, E> acc;
    acc.clear();
    SeriesAcc<T> sacc;
    __syncthreads();

    auto transform = [&](auto gen) {
        T2 x[E];
#pragma unroll
        for (int m = 0; m < EH; ++m) {  // load with the folded first stage (upper half zero)
            const int p = lane + 32 * m;
            const T2 v = p < nf ? gen(p) : zero2<T2>();
            x[m] = v;
            x[m + EH] = cmul(v, tw[p << tws]);
        }
#pragma unroll
        for (int hm = E / 4; hm >= 1; hm >>= 1) {  // spans 32 hm inside the lane
            const int sh = LG - 1 - (5 + ilog2c(hm)) + tws;
#pragma unroll
            for (int m = 0; m < E; ++m) {
                if ((m & hm) == 0) {
                    const T2 u = x[m], w = x[m + hm];
                    x[m] = cadd(u, w);
                    x[m + hm] = cmul(csub(u, w), tw[(lane + 32 * (m & (hm - 1))) << sh]);
                }
            }
        }
#pragma unroll
        for (int lh = 4; lh >= 0; --lh) {  // spans 16 .. 1 across lanes
            const int h = 1 << lh, sh = LG - 1 - lh + tws;
            const bool upper = (lane & h) != 0;
            const T sg = upper ? T(-1) : T(1);
            T2 tv = tw[(lane & (h - 1)) << sh];
            if (!upper) {
                tv.x = T(1);
                tv.y = T(0);
            }
#pragma unroll
            for (int m = 0; m < E; ++m) {
                const T2 o = shfl_xor2(x[m], h);
                T2 d;  // lower lane: x + o; upper lane: o - x (then times the twiddle)
                d.x = fma(sg, x[m].x, o.x);
                d.y = fma(sg, x[m].y, o.y);
                x[m] = cmul(d, tv);
            }
        }
        T ax = 0, ay = 0;
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const T P = x[m].x * x[m].x + x[m].y * x[m].y;
            acc.add(m, P);
            const T2 kv = __ldg(kbr + lane + 32 * m);  // this lane's bins of the store kernel (L1)
            ax += P * kv.x;
            ay += P * kv.y;
        }
        const T2 av = warp_sum_t<T>(ax, ay);
        if (lane == 0) sacc.add(av.x, av.y);
    };

    if (SELF) {
        // trajectories of up to kRegFftAtoms atoms staged at once (coalesced over atoms);
        // the warps share out their (atom, direction) pairs evenly
        constexpr int NAS = kRegFftAtoms;
        T* bsm = reinterpret_cast<T*>(rj + (size_t)NAS * nf);
        const T* bfac = reinterpret_cast<const T*>(sys.bfac);
        const int v0 = sys.shell_v[c.shell], nd = sys.shell_v[c.shell + 1] - v0;
        for (int j0 = c.v_begin; j0 < c.v_end; j0 += NAS) {
            const int na = min(NAS, c.v_end - j0);
            __syncthreads();  // every warp is done with the previous atoms' trajectories
            for (int i = threadIdx.x; i < na * nf; i += NT) {
                const int t = i / na, at = i - t * na;
                rj[at * nf + t] = sys.xyz[(size_t)t * sys.na_pad + j0 + at];
            }
            if (threadIdx.x < na) bsm[threadIdx.x] = bfac[(size_t)c.shell * sys.na_pad + j0 + threadIdx.x];
            __syncthreads();
            for (int pr = warp; pr < na * nd; pr += NW) {
                const int at = pr / nd, v = v0 + (pr - at * nd);
                T qx, qy, qz;
                load_qv(sys.qv, sys.qrev, (size_t)v, qx, qy, qz);
                const T b = bsm[at];
                const float4* ra = rj + (size_t)at * nf;
                transform([&](int p) { return self_term(b, ra[p], qx, qy, qz); });
            }
        }
    } else {
        for (int v = c.v_begin + warp; v < c.v_end; v += NW) {
            const T2* src = reinterpret_cast<const T2*>(sys.A) + (size_t)v * sys.nf;
            transform([&](int p) { return src[p]; });
        }
    }

    __syncthreads();
#pragma unroll
    for (int m = 0; m < E; ++m) pw[(size_t)warp * L + lane + 32 * m] = acc.get(m);
    if (lane == 0) {
        red[warp] = sacc.mean_sum();
        red2[warp] = sacc.sq_sum();
    }
    __syncthreads();
    double* dst = a.ppart + c.part_off;
    for (int i = threadIdx.x; i < L; i += NT) {
        double s = 0.0;
        for (int w = 0; w < NW; ++w) s += pw[(size_t)w * L + i];
        dst[i] = s;
    }
    if (threadIdx.x == 0) {
        double2 as = make_double2(0.0, 0.0);
        double a2 = 0.0;
        for (int w = 0; w < NW; ++w) {
            as.x += red[w].x;
            as.y += red[w].y;
            a2 += red2[w];
        }
        a.apart[c.slot] = as;
        a.a2part[c.slot] = a2;
    }
}

// ---------------------------------------------------------------------------------------
// Transposed register FFT (FP32) for one padded length L = 16 C, C = 4, 8, 16 (64 .. 256
// points), G = 32 / C series per warp. With n = a + C b (a < C, b < 16) and k = k_b + 16 k_a,
//     X[k] = sum_a W_C^{a k_a} [ W_L^{a k_b} sum_b x[a + C b] W_16^{b k_b} ],
// so lane (g, a) of pass 1 generates or loads its column b = 0 .. 7 of series g (the upper
// half is the zero padding), runs the 16-point DFT over b in registers (the first stage
// folded, constant twiddles), multiplies by W_L^{a k_b} and writes the 16 values into the
// warp's shared-memory tile; after one __syncwarp, lane l of pass 2 reads the rows
// (g = l / 16 + 2 j, k_b = l % 16), j < G / 2, and runs the C-point DFTs over a in
// registers. One transpose through shared memory replaces the five shuffle stages of the
// lane-strided form. Lane l then owns the bins k_b = l % 16 + 16 k_a of its series: their
// power is summed in plain FP32 for a few rounds and folded into Kahan-compensated FP32
// state in shared memory, and each series' sum_k P K (its mean over lags) is reduced over
// the half warp. Tile rows are padded and the per-lane twiddle and store-kernel tables are
// laid out lane-contiguous, so shared-memory accesses are free of bank conflicts. All
// twiddle choices are resolved at compile time.
// ---------------------------------------------------------------------------------------
constexpr int kReg2Warps = 8, kReg2MinLg = 6, kReg2MaxLg = 8;

// W_L^m for 0 <= m < L from the half table of the launch's largest length (W^m = -W^{m-L/2}).
template <class T2>
__device__ __forceinline__ T2 tw_full(const T2* tw, int m, int lg, int tws) {
    const int h = 1 << (lg - 1);
    if (m < h) return tw[m << tws];
    T2 v = tw[(m - h) << tws];
    v.x = -v.x;
    v.y = -v.y;
    return v;
}

template <int LG>
struct Reg2Shape {
    static constexpr int L = 1 << LG, C = L / 16, G = 32 / C, RPL = G / 2;
    static constexpr int S = 2 * C + 4;          // words per tile row (C complex + 2 padding)
    static constexpr int GS = 16 * S + 2 * C;    // words per series
    static constexpr int WW = G * GS;            // words per warp
    static constexpr int FOLD = 8;               // rounds of plain FP32 power sums between Kahan folds
    static constexpr int NAS = LG >= 8 ? 4 : 8;  // atoms staged per barrier (shared memory of three CTAs per SM)
};

__host__ __device__ constexpr int brev_bits(int v, int bits) {
    return bits == 0 ? 0 : (((v & 1) << (bits - 1)) | brev_bits(v >> 1, bits - 1));
}

// cos / sin of -2 pi j / 16 (the forward transform's W_16^j)
__host__ __device__ constexpr float w16_re(int j) {
    return j == 0 ? 1.f : j == 1 ? 0.923879532511286756f : j == 2 ? 0.707106781186547524f
         : j == 3 ? 0.382683432365089772f : j == 4 ? 0.f : j == 5 ? -0.382683432365089772f
         : j == 6 ? -0.707106781186547524f : j == 7 ? -0.923879532511286756f : j == 8 ? -1.f
         : j == 9 ? -0.923879532511286756f : j == 10 ? -0.707106781186547524f : j == 11 ? -0.382683432365089772f
         : j == 12 ? 0.f : j == 13 ? 0.382683432365089772f : j == 14 ? 0.707106781186547524f
         : 0.923879532511286756f;
}
__host__ __device__ constexpr float w16_im(int j) { return -w16_re((j + 12) & 15); }

__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// v * W_16^J: products in scalar FP32, so no register pairs need rebuilding; the factors
// 1, -i, -1, +i cost no multiplications.
template <int J>
__device__ __forceinline__ float2 mul_w16c(float2 v) {
    constexpr int j = J & 15;
    if constexpr (j == 0) return v;
    else if constexpr (j == 4) return make_float2(v.y, -v.x);
    else if constexpr (j == 8) return make_float2(-v.x, -v.y);
    else if constexpr (j == 12) return make_float2(-v.y, v.x);
    else {
        constexpr float c = w16_re(j), s = w16_im(j);
        return make_float2(fmaf(v.x, c, -v.y * s), fmaf(v.x, s, v.y * c));
    }
}

// DIF butterfly: a' = a + b (paired), b' = (a - b) W_16^J
template <int J>
__device__ __forceinline__ void bfly16c(float2& a, float2& b) {
    constexpr int j = J & 15;
    const float2 u = a, w = b;
    a = __fadd2_rn(u, w);
    if constexpr (j == 0) b = sub2(u, w);
    else if constexpr (j == 4) b = make_float2(u.y - w.y, w.x - u.x);
    else if constexpr (j == 8) b = sub2(w, u);
    else if constexpr (j == 12) b = make_float2(w.y - u.y, u.x - w.x);
    else b = mul_w16c<j>(sub2(u, w));
}

// Radix-2 DIF stages of span H .. 1 over x[OFF .. OFF + N) (N <= 16, natural order in,
// bit-reversed order out), unrolled by template recursion.
template <int N, int OFF, int H, int M, int TOT>
__device__ __forceinline__ void dif_stage(float2 (&x)[TOT]) {
    if constexpr (M < N) {
        if constexpr ((M & H) == 0) bfly16c<(M & (H - 1)) * (8 / H)>(x[OFF + M], x[OFF + M + H]);
        dif_stage<N, OFF, H, M + 1, TOT>(x);
    }
}
template <int N, int OFF, int H, int TOT>
__device__ __forceinline__ void dif_lane(float2 (&x)[TOT]) {
    if constexpr (H >= 1) {
        dif_stage<N, OFF, H, 0, TOT>(x);
        dif_lane<N, OFF, H / 2, TOT>(x);
    }
}

// the folded first stage of pass 1 (upper half zero): x[b + 8] = x[b] W_16^b
template <int B = 0>
__device__ __forceinline__ void fold_first(float2 (&x)[16]) {
    if constexpr (B < 8) {
        x[B + 8] = mul_w16c<B>(x[B]);
        fold_first<B + 1>(x);
    }
}

// pass-1 results into the tile: register p holds k_b = br16(p)
template <int S, int P = 0>
__device__ __forceinline__ void store_tile(float* base, const float2 (&x)[16]) {
    if constexpr (P < 16) {
        *reinterpret_cast<float2*>(base + brev_bits(P, 4) * S) = x[P];
        store_tile<S, P + 1>(base, x);
    }
}

// the RPL row transforms of pass 2: x[J C .. J C + C) for J < RPL
template <int C, int RPL, int J = 0>
__device__ __forceinline__ void dif_rows(float2 (&x)[16]) {
    if constexpr (J < RPL) {
        dif_lane<C, J * C, C / 2, 16>(x);
        dif_rows<C, RPL, J + 1>(x);
    }
}

// Shared memory of reg2_fft_kernel, in bytes from the start.
template <int LG>
struct Reg2Layout {
    typedef Reg2Shape<LG> Sh;
    static constexpr size_t kTiles = (size_t)kReg2Warps * Sh::WW * 4, kBins = (size_t)kReg2Warps * Sh::L * 8;
    static constexpr size_t kTw = 0;                          // float4 [8][C]: W_L^{a br16(p)}, p = 2 pp, 2 pp + 1
    static constexpr size_t kK = kTw + (size_t)Sh::L * 8;     // float4 [C / 2][16]: K of bins k_b + 16 br_C(q), q = 2 qq, 2 qq + 1
    static constexpr size_t kKahan = kK + (size_t)Sh::L * 8;  // float2 [NW][C][16]: power (sum, compensation)
    static constexpr size_t kTile = kKahan + (size_t)kReg2Warps * Sh::C * 16 * 8;
    static constexpr size_t kRed = kTile + (kTiles > kBins ? kTiles : kBins);  // tiles, then partial bins
    static constexpr size_t kTraj = kRed + kReg2Warps * (16 + 8);  // float4 [NAS][nf], then float [NAS]
};

template <int LG>
size_t reg2_fft_smem(int nf, bool self) {
    size_t b = Reg2Layout<LG>::kTraj;
    if (self) b += (size_t)Reg2Shape<LG>::NAS * nf * sizeof(float4) + Reg2Shape<LG>::NAS * sizeof(float);
    return b;
}

template <int LG, bool SELF>
__global__ void __launch_bounds__(kReg2Warps * 32, SELF ? 2 : 3) reg2_fft_kernel(CorrLaunch a) {
    typedef Reg2Shape<LG> Sh;
    typedef Reg2Layout<LG> Ly;
    constexpr int NW = kReg2Warps, NT = NW * 32, L = Sh::L, C = Sh::C, G = Sh::G, RPL = Sh::RPL;
    constexpr int BC = ilog2c(C);
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int nf = sys.nf, tws = a.lg_max - LG;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* ttab = reinterpret_cast<float4*>(smem + Ly::kTw);
    float4* ktab = reinterpret_cast<float4*>(smem + Ly::kK);
    float2* kst = reinterpret_cast<float2*>(smem + Ly::kKahan) + (size_t)warp * C * 16;
    float* tile = reinterpret_cast<float*>(smem + Ly::kTile) + (size_t)warp * Sh::WW;
    double* pw = reinterpret_cast<double*>(smem + Ly::kTile);  // [NW][L] after the loop
    double2* red = reinterpret_cast<double2*>(smem + Ly::kRed);
    double* red2 = reinterpret_cast<double*>(red + NW);
    float4* rj = reinterpret_cast<float4*>(smem + Ly::kTraj);
    {
        // lane-contiguous tables: entry (pp, col) and (qq, kb) are read by consecutive lanes
        const float2* twg = reinterpret_cast<const float2*>(a.tw);
        const float2* kbr = reinterpret_cast<const float2*>(sys.kbr);
        for (int i = threadIdx.x; i < L / 2; i += NT) {
            const int pp = i / C, col = i - pp * C;
            const float2 t0 = tw_full(twg, col * brev_bits(2 * pp, 4), LG, tws);
            const float2 t1 = tw_full(twg, col * brev_bits(2 * pp + 1, 4), LG, tws);
            ttab[i] = make_float4(t0.x, t0.y, t1.x, t1.y);
            const int qq = i >> 4, kb = i & 15;
            const int k0 = kb + 16 * brev_bits(2 * qq, BC), k1 = kb + 16 * brev_bits(2 * qq + 1, BC);
            const float2 a0 = kbr[__brev((unsigned)k0) >> (32 - LG)], a1 = kbr[__brev((unsigned)k1) >> (32 - LG)];
            ktab[i] = make_float4(a0.x, a0.y, a1.x, a1.y);
        }
        for (int i = threadIdx.x; i < NW * C * 16; i += NT)
            reinterpret_cast<float2*>(smem + Ly::kKahan)[i] = make_float2(0.f, 0.f);
    }
    // pass-1 role: series g1, column col; pass-2 role: row k_b of series half + 2 j
    const int g1 = lane / C, col = lane - g1 * C, kb = lane & 15, half = lane >> 4;
    float pacc[C];
#pragma unroll
    for (int q = 0; q < C; ++q) pacc[q] = 0.f;
    SeriesAcc<float> sacc;
    int rounds = 0;
    __syncthreads();

    // Kahan fold of the plain sums; lanes l and l + 16 hold the same bins
    auto fold = [&]() {
#pragma unroll
        for (int q = 0; q < C; ++q) {
            const float v = pacc[q] + __shfl_xor_sync(0xffffffffu, pacc[q], 16);
            pacc[q] = 0.f;
            if (half == 0) {
                float2 st = kst[q * 16 + kb];
                const float y = __fsub_rn(v, st.y), t = __fadd_rn(st.x, y);
                st.y = __fsub_rn(__fsub_rn(t, st.x), y);
                st.x = t;
                kst[q * 16 + kb] = st;
            }
        }
    };

    // the warp's G series: get(b, n, m) is point n = col + C b (< NF) of this lane's pass-1
    // series times m (0 for the zero padding), valid(g) whether series g exists this round, w2 this
    // lane's pass-1 series' power weight (the incoherent series are generated with unit
    // length and weighted by b^2 in the power sums: |b X|^2 = b^2 |X|^2)
    auto transform = [&](auto get, auto valid, float w2) {
        float2 x[16];
#pragma unroll
        for (int b = 0; b < 8; ++b) {  // points beyond NF read the last point, scaled by 0
            const int n = col + C * b;
            x[b] = get(b, min(n, nf - 1), n < nf ? 1.f : 0.f);
        }
        fold_first(x);  // first stage, upper half zero
        dif_lane<16, 0, 4, 16>(x);
#pragma unroll
        for (int p = 0; p < 16; p += 2) {  // times W_L^{col k1}, k1 = br16(p) (p = 0: k1 = 0)
            const float4 w = ttab[(p / 2) * C + col];
            if (p > 0) x[p] = make_float2(fmaf(x[p].x, w.x, -x[p].y * w.y), fmaf(x[p].x, w.y, x[p].y * w.x));
            x[p + 1] = make_float2(fmaf(x[p + 1].x, w.z, -x[p + 1].y * w.w), fmaf(x[p + 1].x, w.w, x[p + 1].y * w.z));
        }
        __syncwarp();  // the previous round's pass 2 has read the tile
        store_tile<Sh::S>(tile + g1 * Sh::GS + 2 * col, x);
        __syncwarp();
#pragma unroll
        for (int j = 0; j < RPL; ++j) {
            const float* row = tile + (half + 2 * j) * Sh::GS + kb * Sh::S;
#pragma unroll
            for (int q = 0; q < C; q += 2) {
                const float4 v = *reinterpret_cast<const float4*>(row + 2 * q);
                x[j * C + q] = make_float2(v.x, v.y);
                x[j * C + q + 1] = make_float2(v.z, v.w);
            }
        }
        dif_rows<C, RPL>(x);
        // power weights of the pass-2 series half + 2 j, from a pass-1 lane of each
        float wj[RPL];
#pragma unroll
        for (int j = 0; j < RPL; ++j) wj[j] = __shfl_sync(0xffffffffu, w2, (half + 2 * j) * C);
        // power of the lane's bins k = k_b + 16 br_C(q) and each series' sum_k P K
        float sx[RPL], sy[RPL];
#pragma unroll
        for (int j = 0; j < RPL; ++j) sx[j] = sy[j] = 0.f;
#pragma unroll
        for (int q = 0; q < C; q += 2) {
            const float4 kv = ktab[(q / 2) * 16 + kb];
#pragma unroll
            for (int j = 0; j < RPL; ++j) {
                const float2 v0 = x[j * C + q], v1 = x[j * C + q + 1];
                const float P0 = fmaf(v0.x, v0.x, v0.y * v0.y), P1 = fmaf(v1.x, v1.x, v1.y * v1.y);
                pacc[q] = fmaf(P0, wj[j], pacc[q]);
                pacc[q + 1] = fmaf(P1, wj[j], pacc[q + 1]);
                sx[j] = fmaf(P1, kv.z, fmaf(P0, kv.x, sx[j]));
                sy[j] = fmaf(P1, kv.w, fmaf(P0, kv.y, sy[j]));
            }
        }
#pragma unroll
        for (int j = 0; j < RPL; ++j) {
            float tx = sx[j] * wj[j], ty = sy[j] * wj[j];
#pragma unroll
            for (int o = 8; o >= 1; o >>= 1) {  // within the half warp: the series' total
                tx += __shfl_xor_sync(0xffffffffu, tx, o);
                ty += __shfl_xor_sync(0xffffffffu, ty, o);
            }
            if (kb == 0 && valid(half + 2 * j)) sacc.add(tx, ty);
        }
        if (++rounds == Sh::FOLD) {
            fold();
            rounds = 0;
        }
    };

    if (SELF) {
        constexpr int NAS = Sh::NAS;
        float* bsm = reinterpret_cast<float*>(rj + (size_t)NAS * nf);
        const float* bfac = reinterpret_cast<const float*>(sys.bfac);
        const int v0 = sys.shell_v[c.shell], nd = sys.shell_v[c.shell + 1] - v0;
        for (int j0 = c.v_begin; nd > 0 && j0 < c.v_end; j0 += NAS) {  // (no directions: no series)
            const int na = min(NAS, c.v_end - j0), npair = na * nd;
            __syncthreads();  // every warp is done with the previous atoms' trajectories
            for (int i = threadIdx.x; i < na * nf; i += NT) {
                const int t = i / na, at = i - t * na;
                rj[at * nf + t] = sys.xyz[(size_t)t * sys.na_pad + j0 + at];
            }
            if (threadIdx.x < na) bsm[threadIdx.x] = bfac[(size_t)c.shell * sys.na_pad + j0 + threadIdx.x];
            __syncthreads();
            // pair pr = atom * nd + direction (nd >= 1), walked without divisions
            int at0 = 0, d0 = warp * G;
            while (d0 >= nd) {
                d0 -= nd;
                ++at0;
            }
            // the lane's 8 points of its atom's trajectory, kept in registers while the lane's
            // pairs stay on that atom (consecutive rounds take the next directions)
            float cx[8], cy[8], cz[8];
            int cached = -1;
            for (int pr0 = warp * G; pr0 < npair; pr0 += NW * G) {
                int at = at0, d = d0 + g1;
                while (d >= nd) {
                    d -= nd;
                    ++at;
                }
                const bool ok = at < na;
                if (!ok) {
                    at = na - 1;
                    d = 0;
                }
                float qx, qy, qz;
                load_qv(sys.qv, sys.qrev, (size_t)(v0 + d), qx, qy, qz);
                const float b = ok ? bsm[at] : 0.f;
                if (at != cached) {
                    const float4* ra = rj + (size_t)at * nf;
#pragma unroll
                    for (int p = 0; p < 8; ++p) {
                        const float4 r = ra[min(col + C * p, nf - 1)];
                        cx[p] = r.x;
                        cy[p] = r.y;
                        cz[p] = r.z;
                    }
                    cached = at;
                }
                transform(
                    [&](int p, int, float m) {  // unit length; the zero padding selected, not multiplied
                        const float2 v = self_term(1.f, make_float4(cx[p], cy[p], cz[p], 0.f), qx, qy, qz);
                        return m != 0.f ? v : make_float2(0.f, 0.f);
                    },
                    [&](int g) { return pr0 + g < npair; }, b * b);
                d0 += NW * G;
                while (d0 >= nd) {
                    d0 -= nd;
                    ++at0;
                }
            }
        }
    } else {
        const int nser = c.v_end - c.v_begin;
        for (int s0 = warp * G; s0 < nser; s0 += NW * G) {
            const bool mine = s0 + g1 < nser;
            const float mm = mine ? 1.f : 0.f;
            const float2* src = reinterpret_cast<const float2*>(sys.A) + (size_t)(c.v_begin + (mine ? s0 + g1 : 0)) * nf;
            transform([&](int, int n, float m) {
                const float2 v = src[n];
                return make_float2(v.x * (m * mm), v.y * (m * mm));
            },
                      [&](int g) { return s0 + g < nser; }, 1.f);
        }
    }
    fold();

    // the warp's bins and series sums (lanes 0 and 16), then the chunk's partial slot in
    // bit-reversed order
    __syncthreads();  // every warp is done with its tile: the region now holds partial bins
    if (half == 0) {
#pragma unroll
        for (int q = 0; q < C; ++q) {
            const float2 st = kst[q * 16 + kb];
            const int k = kb + 16 * brev_bits(q, BC);
            pw[(size_t)warp * L + (__brev((unsigned)k) >> (32 - LG))] = (double)st.x - (double)st.y;
        }
    }
    double2 ms = sacc.mean_sum();
    double s2 = sacc.sq_sum();
    ms.x += __shfl_xor_sync(0xffffffffu, ms.x, 16);
    ms.y += __shfl_xor_sync(0xffffffffu, ms.y, 16);
    s2 += __shfl_xor_sync(0xffffffffu, s2, 16);
    if (lane == 0) {
        red[warp] = ms;
        red2[warp] = s2;
    }
    __syncthreads();
    double* dst = a.ppart + c.part_off;
    for (int i = threadIdx.x; i < L; i += NT) {
        double sum = 0.0;
        for (int w = 0; w < NW; ++w) sum += pw[(size_t)w * L + i];
        dst[i] = sum;
    }
    if (threadIdx.x == 0) {
        double2 as = make_double2(0.0, 0.0);
        double a2 = 0.0;
        for (int w = 0; w < NW; ++w) {
            as.x += red[w].x;
            as.y += red[w].y;
            a2 += red2[w];
        }
        a.apart[c.slot] = as;
        a.a2part[c.slot] = a2;
    }
}

// ---------------------------------------------------------------------------------------
// Block-register FFT for series of one padded length L = 512 B (B = 2, 4, 8: 1,024 .. 4,096
// points). The first log2 B DIF stages are folded into the load: after them, position
// 512 b + j of the DIF array holds
//     v_b[j] = W_L^{j br(b)} sum_{u < B/2} x[j + 512 u] W_B^{u br(b)}
// (br: reversal of the log2 B bits of b; the upper half of x is the zero padding), and the
// remaining stages are the 512-point DIF of each block on its own. So a warp transforms one
// block of one series with no exchange between warps: lane l holds positions 512 b + l + 32 m
// (m < 16), runs the in-lane stages of span 256 .. 32 and the shuffle stages of span 16 .. 1
// of the register warp FFT, and accumulates the power of exactly those (bit-reversed) bins.
// Warps b, b + B, ... take block b of G = 8 / B series per round; each round's series sums
// add their blocks' partial means in block order. Coherent series load straight from the
// amplitudes in global memory; incoherent series are generated once per round into shared
// memory from the atom's staged trajectory. Replaces 11 barrier-separated radix-2 stages in
// shared memory per series.
// ---------------------------------------------------------------------------------------
constexpr int kBlkFftWarps = 8, kBlkFftMinLg = 10, kBlkFftMaxLg = 12;

template <class T, int LG>
struct BlkFft {
    typedef typename cplx<T>::type T2;
    static constexpr int NW = kBlkFftWarps, NT = NW * 32, L = 1 << LG, B = L / 512, E = 16, G = NW / B;
    static_assert(B >= 2 && B <= NW && NW % B == 0, "block FFT lengths 1,024 .. 4,096");
    const T2* tw;
    int tws, lane, b, br;
    T2 cu[B / 2];  // W_B^{u br(b)} of the folded stages

    __device__ void init(const T2* tw_, int tws_) {
        tw = tw_;
        tws = tws_;
        lane = threadIdx.x & 31;
        b = (threadIdx.x >> 5) % B;
        br = (int)(__brev((unsigned)b) >> (32 - ilog2c(B)));
#pragma unroll
        for (int u = 0; u < B / 2; ++u) cu[u] = tw_full(tw, (512 * u * br) & (L - 1), LG, tws);
    }

    // x[m] = v_b[lane + 32 m] from get(n), the series' first L / 2 points (0 beyond NF)
    template <class Get>
    __device__ __forceinline__ void load(T2 (&x)[E], Get get) const {
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const int j = lane + 32 * m;
            T2 sv = get(j);
#pragma unroll
            for (int u = 1; u < B / 2; ++u) sv = cadd(sv, cmul(get(j + 512 * u), cu[u]));
            x[m] = br == 0 ? sv : cmul(sv, tw_full(tw, j * br, LG, tws));
        }
    }

    // the 512-point DIF of the block: bit-reversed order at the same positions
    __device__ __forceinline__ void stages(T2 (&x)[E]) const {
#pragma unroll
        for (int hm = E / 2; hm >= 1; hm >>= 1) {  // spans 32 hm inside the lane
            const int sh = LG - 6 - ilog2c(hm) + tws;
#pragma unroll
            for (int m = 0; m < E; ++m) {
                if ((m & hm) == 0) {
                    const T2 u = x[m], w = x[m + hm];
                    x[m] = cadd(u, w);
                    x[m + hm] = cmul(csub(u, w), tw[(lane + 32 * (m & (hm - 1))) << sh]);
                }
            }
        }
#pragma unroll
        for (int lh = 4; lh >= 0; --lh) {  // spans 16 .. 1 across lanes
            const int h = 1 << lh, sh = LG - 1 - lh + tws;
            const bool upper = (lane & h) != 0;
            const T sg = upper ? T(-1) : T(1);
            T2 tv = tw[(lane & (h - 1)) << sh];
            if (!upper) {
                tv.x = T(1);
                tv.y = T(0);
            }
#pragma unroll
            for (int m = 0; m < E; ++m) {
                const T2 o = shfl_xor2(x[m], h);
                T2 d;
                d.x = fma(sg, x[m].x, o.x);
                d.y = fma(sg, x[m].y, o.y);
                x[m] = cmul(d, tv);
            }
        }
    }

    // accumulate |X|^2 of the lane's bins; the warp's part of sum_w P(w) K(w)
    __device__ __forceinline__ T2 power(const T2 (&x)[E], const T2* __restrict__ kbr, PowerAcc<T, E>& acc) const {
        T ax = 0, ay = 0;
#pragma unroll
        for (int m = 0; m < E; ++m) {
            const T P = x[m].x * x[m].x + x[m].y * x[m].y;
            acc.add(m, P);
            const T2 kv = __ldg(kbr + 512 * b + lane + 32 * m);
            ax += P * kv.x;
            ay += P * kv.y;
        }
        return warp_sum_t<T>(ax, ay);
    }

    // end of a chunk: the bins of warps b, b + B, ... combined in warp order into the
    // chunk's partial slot (FP32: float-float sum of (sum - compensation), stored as a
    // (sum, compensation) pair; FP64: plain sums), and the series sums. `pwb`: NW x 512 bins.
    __device__ void finish(const PowerAcc<T, E>& acc, const SeriesAcc<T>& sacc, unsigned char* pwb,
                           const CorrLaunch& a, const CorrChunk& c) const {
        const int warp = threadIdx.x >> 5;
        if constexpr (sizeof(T) == 4) {
            float2* pw = reinterpret_cast<float2*>(pwb);
#pragma unroll
            for (int m = 0; m < E; ++m) pw[warp * 512 + lane + 32 * m] = make_float2(acc.s[m], acc.c[m]);
            __syncthreads();
            float2* dst = reinterpret_cast<float2*>(a.ppart + c.part_off);
            for (int i = threadIdx.x; i < L; i += NT) {
                const int bb = i >> 9, loc = i & 511;
                float hi = 0.f, lo = 0.f;
                for (int w = bb; w < NW; w += B) {
                    const float2 p = pw[w * 512 + loc];
                    const float s = __fadd_rn(hi, p.x), bv = __fsub_rn(s, hi);
                    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(p.x, bv));
                    hi = s;
                    lo = __fadd_rn(lo, __fsub_rn(e, p.y));
                }
                dst[i] = make_float2(hi, -lo);  // read back as (sum, compensation): hi + lo
            }
        } else {
            double* pw = reinterpret_cast<double*>(pwb);
#pragma unroll
            for (int m = 0; m < E; ++m) pw[warp * 512 + lane + 32 * m] = acc.get(m);
            __syncthreads();
            double* dst = a.ppart + c.part_off;
            for (int i = threadIdx.x; i < L; i += NT) {
                const int bb = i >> 9, loc = i & 511;
                double s = 0.0;
                for (int w = bb; w < NW; w += B) s += pw[w * 512 + loc];
                dst[i] = s;
            }
        }
        if (threadIdx.x == 0) {
            a.apart[c.slot] = sacc.mean_sum();
            a.a2part[c.slot] = sacc.sq_sum();
        }
    }

    // after a round's barrier: thread 0 adds the round's series (block partials in block order)
    __device__ __forceinline__ static void add_round(const T2* pmr, int nser_round, SeriesAcc<T>& sacc) {
        for (int gg = 0; gg < nser_round; ++gg) {
            T2 tot = pmr[gg * B];
#pragma unroll
            for (int bb = 1; bb < B; ++bb) tot = cadd(tot, pmr[gg * B + bb]);
            sacc.add(tot.x, tot.y);
        }
    }
};

template <class T>
size_t blk_fft_smem(int lg_max, int nf, bool self) {
    typedef typename cplx<T>::type T2;
    const size_t H = ((size_t)1 << lg_max) / 2;
    size_t b = (sizeof(T) == 4 ? H : 0) * sizeof(T2);  // FP32 twiddles
    if (self) b += (size_t)kBlkFftWarps * 256 * sizeof(T2) + (size_t)nf * sizeof(float4);  // G series, trajectory
    b += 2 * kBlkFftWarps * sizeof(T2);                                                     // partial means
    b += (size_t)kBlkFftWarps * 512 * (sizeof(T) == 4 ? sizeof(float2) : sizeof(double));  // bins
    return b;
}

template <class T, int LG>
__global__ void __launch_bounds__(kBlkFftWarps * 32, sizeof(T) == 4 ? 2 : 1) blk_fft_kernel(CorrLaunch a) {
    typedef BlkFft<T, LG> F;
    typedef typename F::T2 T2;
    constexpr int NW = F::NW, NT = F::NT, L = F::L, E = F::E, G = F::G;
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int nf = sys.nf, warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = warp / F::B;
    T2* twsm = reinterpret_cast<T2*>(smem);
    unsigned char* region = smem + (sizeof(T) == 4 ? (size_t)(L / 2) * sizeof(T2) : 0);
    T2* pm = reinterpret_cast<T2*>(region);  // [2][NW]: round parity x warp
    unsigned char* pwb = region + 2 * NW * sizeof(T2);
    const T2* tw = stage_twiddles<T, NT>(twsm, a.tw, a.lg_max);
    const T2* kbr = reinterpret_cast<const T2*>(sys.kbr);
    __syncthreads();
    F f;
    f.init(tw, a.lg_max - LG);
    PowerAcc<T, E> acc;
    acc.clear();
    SeriesAcc<T> sacc;
    const int nser = c.v_end - c.v_begin, rounds = (nser + G - 1) / G;
    for (int r = 0; r < rounds; ++r) {
        const int sl = r * G + g;  // warp-uniform
        T2 pv = zero2<T2>();
        if (sl < nser) {
            const T2* src = reinterpret_cast<const T2*>(sys.A) + (size_t)(c.v_begin + sl) * nf;
            T2 x[E];
            f.load(x, [&](int n) { return n < nf ? src[n] : zero2<T2>(); });
            f.stages(x);
            pv = f.power(x, kbr, acc);
        }
        if (lane == 0) pm[(r & 1) * NW + warp] = pv;
        __syncthreads();
        if (threadIdx.x == 0) F::add_round(pm + (r & 1) * NW, min(G, nser - r * G), sacc);
    }
    f.finish(acc, sacc, pwb, a, c);
}

// Incoherent series of one padded length L (1,024 .. 4,096): CTA per chunk of atoms of one
// shell. Per atom its trajectory is staged; per round the G series (atom, direction d0 .. d0
// + G - 1) are generated into shared memory, then transformed block-wise as above.
template <class T, int LG>
__global__ void __launch_bounds__(kBlkFftWarps * 32, sizeof(T) == 4 ? 2 : 1) self_blk_fft_kernel(CorrLaunch a) {
    typedef BlkFft<T, LG> F;
    typedef typename F::T2 T2;
    constexpr int NW = F::NW, NT = F::NT, L = F::L, E = F::E, G = F::G, H = L / 2;
    extern __shared__ __align__(16) unsigned char smem[];
    const CorrChunk c = a.chunks[blockIdx.x];
    const CorrSystem sys = a.systems[c.system];
    const int nf = sys.nf, warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = warp / F::B;
    T2* twsm = reinterpret_cast<T2*>(smem);
    unsigned char* region = smem + (sizeof(T) == 4 ? (size_t)H * sizeof(T2) : 0);
    T2* xs = reinterpret_cast<T2*>(region);  // [G][H] the round's series
    T2* pm = xs + G * H;                     // [2][NW]
    float4* rj = reinterpret_cast<float4*>(pm + 2 * NW);  // [nf] the atom's trajectory
    unsigned char* pwb = reinterpret_cast<unsigned char*>(rj + nf);
    const T2* tw = stage_twiddles<T, NT>(twsm, a.tw, a.lg_max);
    const T2* kbr = reinterpret_cast<const T2*>(sys.kbr);
    const T* bfac = reinterpret_cast<const T*>(sys.bfac);
    const int v0 = sys.shell_v[c.shell], nd = sys.shell_v[c.shell + 1] - v0;
    __syncthreads();
    F f;
    f.init(tw, a.lg_max - LG);
    PowerAcc<T, E> acc;
    acc.clear();
    SeriesAcc<T> sacc;
    int r = 0;
    for (int j = c.v_begin; j < c.v_end; ++j) {
        __syncthreads();  // the previous atom's series are consumed
        for (int t = threadIdx.x; t < nf; t += NT) rj[t] = sys.xyz[(size_t)t * sys.na_pad + j];
        const T bj = bfac[(size_t)c.shell * sys.na_pad + j];
        __syncthreads();
        for (int d0 = 0; d0 < nd; d0 += G, ++r) {
            for (int i = threadIdx.x; i < G * H; i += NT) {
                const int gg = i / H, n = i - gg * H, d = d0 + gg;
                T2 v = zero2<T2>();
                if (d < nd && n < nf) {
                    T qx, qy, qz;
                    load_qv(sys.qv, sys.qrev, (size_t)(v0 + d), qx, qy, qz);
                    v = self_term(bj, rj[n], qx, qy, qz);
                }
                xs[i] = v;
            }
            __syncthreads();
            T2 pv = zero2<T2>();
            if (d0 + g < nd) {  // warp-uniform
                const T2* xg = xs + g * H;
                T2 x[E];
                f.load(x, [&](int n) { return xg[n]; });
                f.stages(x);
                pv = f.power(x, kbr, acc);
            }
            if (lane == 0) pm[(r & 1) * NW + warp] = pv;
            __syncthreads();
            if (threadIdx.x == 0) F::add_round(pm + (r & 1) * NW, min(G, nd - d0), sacc);
        }
    }
    __syncthreads();
    f.finish(acc, sacc, pwb, a, c);
}

template <class T, int LG>
cudaError_t launch_blk_fft_lg(const CorrLaunch& a, bool self, cudaStream_t st) {
    const size_t sm = blk_fft_smem<T>(a.lg_max, a.nf_max, self);
    auto k = self ? self_blk_fft_kernel<T, LG> : blk_fft_kernel<T, LG>;
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<a.nchunks, kBlkFftWarps * 32, sm, st>>>(a);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_blk_fft(const CorrLaunch& a, bool self, cudaStream_t st) {
    switch (a.lg_max) {
        case 10: return launch_blk_fft_lg<T, 10>(a, self, st);
        case 11: return launch_blk_fft_lg<T, 11>(a, self, st);
        case 12: return launch_blk_fft_lg<T, 12>(a, self, st);
    }
    return cudaErrorInvalidValue;
}

template <int LG>
cudaError_t launch_reg2_fft_lg(const CorrLaunch& a, bool self, cudaStream_t st) {
    const size_t sm = reg2_fft_smem<LG>(a.nf_max, self);
    auto k = self ? reg2_fft_kernel<LG, true> : reg2_fft_kernel<LG, false>;
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<a.nchunks, kReg2Warps * 32, sm, st>>>(a);
    return cudaGetLastError();
}

template <class T, int LG>
cudaError_t launch_reg_fft_lg(const CorrLaunch& a, bool self, cudaStream_t st) {
    if constexpr (sizeof(T) == 4 && LG >= kReg2MinLg && LG <= kReg2MaxLg) return launch_reg2_fft_lg<LG>(a, self, st);
    const size_t sm = reg_fft_smem<T>(LG, a.nf_max, self);
    auto k = self ? reg_fft_kernel<T, LG, true> : reg_fft_kernel<T, LG, false>;
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<a.nchunks, kWarpFftWarps * 32, sm, st>>>(a);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_reg_fft(const CorrLaunch& a, bool self, cudaStream_t st) {
    switch (a.lg_max) {
        case 6: return launch_reg_fft_lg<T, 6>(a, self, st);
        case 7: return launch_reg_fft_lg<T, 7>(a, self, st);
        case 8: return launch_reg_fft_lg<T, 8>(a, self, st);
        case 9: return launch_reg_fft_lg<T, 9>(a, self, st);
    }
    return cudaErrorInvalidValue;
}

template <class T>
cudaError_t launch_warp_fft(const CorrLaunch& a, bool self, cudaStream_t st) {
    const size_t sm = warp_fft_smem<T>(a.lg_max, a.nf_max, self);
    auto k = self ? warp_fft_kernel<T, true> : warp_fft_kernel<T, false>;
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<a.nchunks, kWarpFftWarps * 32, sm, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_accumulate(const CorrLaunch& a, bool self, cudaStream_t st) {
    if (a.nchunks == 0) return cudaSuccess;
    if (a.dsp == DSP_AUTOCORRELATE) {
        if (a.lg_max < 2 || a.lg_max > kMaxLg) return cudaErrorInvalidValue;
        if (a.lg_min == a.lg_max && a.lg_max >= 6 && a.lg_max <= kWarpFftMaxLg)
            return a.precision == PREC_FP32 ? launch_reg_fft<float>(a, self, st) : launch_reg_fft<double>(a, self, st);
        if (a.lg_max <= kWarpFftMaxLg)
            return a.precision == PREC_FP32 ? launch_warp_fft<float>(a, self, st) : launch_warp_fft<double>(a, self, st);
        if (a.lg_min == a.lg_max && a.lg_max >= kBlkFftMinLg && a.lg_max <= kBlkFftMaxLg)
            return a.precision == PREC_FP32 ? launch_blk_fft<float>(a, self, st) : launch_blk_fft<double>(a, self, st);
        // per-thread spectrum bins sized to the longest series of the launch (registers)
        switch (a.lg_max) {
            case 10: return a.precision == PREC_FP32 ? launch_fft<float, 256, 4>(a, self, st) : launch_fft<double, 256, 4>(a, self, st);
            case 11: return a.precision == PREC_FP32 ? launch_fft<float, 256, 8>(a, self, st) : launch_fft<double, 256, 8>(a, self, st);
            case 12: return a.precision == PREC_FP32 ? launch_fft<float, 256, 16>(a, self, st) : launch_fft<double, 256, 16>(a, self, st);
            default: return a.precision == PREC_FP32 ? launch_fft<float, 256, 32>(a, self, st) : launch_fft<double, 256, 32>(a, self, st);
        }
    }
    if (self && a.dsp != DSP_AUTOCORRELATE && a.nf_max <= kSqWarpMaxNf) {
        return a.precision == PREC_FP32 ? launch_self_sq_warp<float>(a, st) : launch_self_sq_warp<double>(a, st);
    } else if (self) {
        if (a.precision == PREC_FP32) self_direct_kernel<float, 256, 16><<<a.nchunks, 256, 0, st>>>(a);
        else self_direct_kernel<double, 256, 16><<<a.nchunks, 256, 0, st>>>(a);
    } else if (a.dsp != DSP_AUTOCORRELATE && a.nf_max <= kSqWarpMaxNf) {
        return a.precision == PREC_FP32 ? launch_sq_warp<float>(a, st) : launch_sq_warp<double>(a, st);
    } else {
        if (a.precision == PREC_FP32) corr_direct_kernel<float2, 256, 16><<<a.nchunks, 256, 0, st>>>(a);
        else corr_direct_kernel<double2, 256, 16><<<a.nchunks, 256, 0, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace

bool corr_writes_f32_pairs(int precision, int dsp, int lg_max) {
    // the CTA-per-series kernels (padded length above the warp forms') in the FP32 form
    return precision == PREC_FP32 && dsp == DSP_AUTOCORRELATE && lg_max > kWarpFftMaxLg;
}

__global__ void q_revolutions_kernel(const double* __restrict__ qv, size_t nv, float4* __restrict__ out) {
    const double inv2pi = 0.15915494309189533577;
    for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x)
        out[v] = make_float4((float)(qv[3 * v] * inv2pi), (float)(qv[3 * v + 1] * inv2pi), (float)(qv[3 * v + 2] * inv2pi),
                             0.f);
}

cudaError_t launch_q_revolutions(const double* qv, size_t nv, float4* out, cudaStream_t st) {
    if (nv == 0) return cudaSuccess;
    q_revolutions_kernel<<<grid_for(nv, 256), 256, 0, st>>>(qv, nv, out);
    return cudaGetLastError();
}

size_t fft_smem_bytes(int precision, int lg, int nf, bool self) {
    if (lg <= kWarpFftMaxLg)
        return precision == PREC_FP32 ? warp_fft_smem<float>(lg, nf, self) : warp_fft_smem<double>(lg, nf, self);
    return precision == PREC_FP32 ? fft_smem<float>(lg, 256, nf, self) : fft_smem<double>(lg, 256, nf, self);
}

cudaError_t launch_corr_accumulate(const CorrLaunch& a, cudaStream_t st) { return launch_accumulate(a, false, st); }

cudaError_t launch_self_accumulate(const CorrLaunch& a, cudaStream_t st) { return launch_accumulate(a, true, st); }

cudaError_t launch_finalize(const FinalLaunch& a, cudaStream_t st) {
    if (a.nentries == 0) return cudaSuccess;
    constexpr int NT = 1024;  // one CTA per shell: as many threads as a CTA takes
    // the spectrum, then one FP64 partial sum per thread (short series)
    const size_t sm = a.dsp == DSP_AUTOCORRELATE ? ((size_t)1 << a.lg_max) * sizeof(double2) + NT * sizeof(double) : 0;
    auto k = finalize_kernel<NT>;
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<a.nentries, NT, sm, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_twiddles(double2* tw64, float2* tw32, int lg, cudaStream_t st) {
    const int L = 1 << lg;
    twiddle_kernel<<<grid_for(L / 2, 256), 256, 0, st>>>(tw64, tw32, L);
    return cudaGetLastError();
}

cudaError_t launch_store_kernel(const double2* tw64, int lg_tw, double2* k64, float2* k32, int nf,
                                int lg, cudaStream_t st) {
    const int L = 1 << lg;
    store_kernel_kernel<<<grid_for(L, 128), 128, 0, st>>>(tw64, lg_tw, k64, k32, nf, lg);
    return cudaGetLastError();
}

cudaError_t launch_stage(const float* raw, int nf, int na, int na_pad, double cx, double cy,
                         double cz, int center, float4* xyz, const int* rec_inv, int na_rec,
                         float4* xyz_rec, cudaStream_t st) {
    size_t n = (size_t)nf * na_pad;
    stage_kernel<<<grid_for(n, 256), 256, 0, st>>>(raw, nf, na, na_pad, cx, cy, cz, center, xyz, rec_inv,
                                                   na_rec, xyz_rec);
    return cudaGetLastError();
}

cudaError_t launch_expand_factors(const double* class_factors, int nclass, int nshell,
                                  const int* cls, int na_pad, int precision, void* b,
                                  cudaStream_t st) {
    size_t n = (size_t)nshell * na_pad;
    if (n == 0) return cudaSuccess;
    if (precision == PREC_FP32)
        expand_factors_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(class_factors, nclass, nshell, cls,
                                                                       na_pad, (float*)b);
    else
        expand_factors_kernel<double><<<grid_for(n, 256), 256, 0, st>>>(class_factors, nclass, nshell, cls,
                                                                        na_pad, (double*)b);
    return cudaGetLastError();
}


}  // namespace sassgpu
