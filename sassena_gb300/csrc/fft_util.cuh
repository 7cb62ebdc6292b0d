// Device helpers shared by the correlation kernels (correlate.cu) and the long-series
// transforms (corr_long.cu): radix-2 stages on shared-memory buffers, CTA sums, the
// power-spectrum accumulator, the incoherent series term, and launch helpers.
#pragma once

#include "common.cuh"
#include "kernels.h"

namespace sassgpu {
namespace {

template <class T2>
__device__ __forceinline__ T2 zero2();
template <>
__device__ __forceinline__ float2 zero2<float2>() {
    return make_float2(0.f, 0.f);
}
template <>
__device__ __forceinline__ double2 zero2<double2>() {
    return make_double2(0.0, 0.0);
}

__device__ __forceinline__ double2 to_d2(float2 a) { return make_double2(a.x, a.y); }
__device__ __forceinline__ double2 to_d2(double2 a) { return a; }

// Remaining DIF stages (half-size L/4 .. 1) after the folded first stage; twiddles
// of length L are tw[k << tws] of the table for the launch's largest length.
template <class T2, int NT>
__device__ void dif_tail(T2* buf, const T2* tw, int lg, int tws) {
    const int half = 1 << (lg - 1);
    for (int lh = lg - 2; lh >= 0; --lh) {
        const int h = 1 << lh;
        const int sh = lg - 1 - lh + tws;
        for (int b = threadIdx.x; b < half; b += NT) {
            const int p = b & (h - 1);
            const int i0 = ((b >> lh) << (lh + 1)) + p;
            T2 u = buf[i0], w = buf[i0 + h];
            buf[i0] = cadd(u, w);
            buf[i0 + h] = cmul(csub(u, w), tw[p << sh]);
        }
        __syncthreads();
    }
}

// Unnormalised inverse DIT FFT: bit-reversed input, natural output, twiddles conj(tw).
template <int NT>
__device__ void dit_inverse(double2* buf, const double2* __restrict__ tw, int lg, int tws) {
    const int half = 1 << (lg - 1);
    for (int lh = 0; lh < lg; ++lh) {
        const int h = 1 << lh;
        const int sh = lg - 1 - lh + tws;
        for (int b = threadIdx.x; b < half; b += NT) {
            const int p = b & (h - 1);
            const int i0 = ((b >> lh) << (lh + 1)) + p;
            double2 u = buf[i0];
            double2 w = cmulc(buf[i0 + h], __ldg(tw + (p << sh)));
            buf[i0] = cadd(u, w);
            buf[i0 + h] = csub(u, w);
        }
        __syncthreads();
    }
}

// Sum of a double2 over the CTA; valid in thread 0. Ends with a barrier so the
// caller may reuse shared memory afterwards.
template <int NT>
__device__ double2 block_sum(double2 v, double2* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double2 s = make_double2(0.0, 0.0);
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; ++w) {
            s.x += red[w].x;
            s.y += red[w].y;
        }
    __syncthreads();
    return s;
}

// Per-thread power-spectrum accumulator: Kahan FP32 (FP32 form) or plain FP64.
template <class T, int MAXR>
struct PowerAcc;

template <int MAXR>
struct PowerAcc<float, MAXR> {
    float s[MAXR], c[MAXR];
    __device__ void clear() {
#pragma unroll
        for (int r = 0; r < MAXR; ++r) s[r] = c[r] = 0.f;
    }
    __device__ __forceinline__ void add(int r, float p) {
        float y = __fsub_rn(p, c[r]);
        float t = __fadd_rn(s[r], y);
        c[r] = __fsub_rn(__fsub_rn(t, s[r]), y);
        s[r] = t;
    }
    __device__ double get(int r) const { return (double)s[r] - (double)c[r]; }
};

template <int MAXR>
struct PowerAcc<double, MAXR> {
    double s[MAXR];
    __device__ void clear() {
#pragma unroll
        for (int r = 0; r < MAXR; ++r) s[r] = 0.0;
    }
    __device__ __forceinline__ void add(int r, double p) { s[r] += p; }
    __device__ double get(int r) const { return s[r]; }
};

// Series generation for the incoherent path: b * exp(i q . r(t)).
__device__ __forceinline__ double2 self_term(double b, float4 r, double qx, double qy, double qz) {
    // p1 = x1*qx+y1*qy+z1*qz, rounded as self_vectors_scatter_device.cpp:312 writes it
    double p = __dadd_rn(__dadd_rn(__dmul_rn((double)r.x, qx), __dmul_rn((double)r.y, qy)),
                         __dmul_rn((double)r.z, qz));
    double s, c;
    sincos(p, &s, &c);
    return make_double2(__dmul_rn(b, c), __dmul_rn(b, s));
}
__device__ __forceinline__ float2 self_term(float b, float4 r, float qx, float qy, float qz) {
    float u = fmaf(r.z, qz, fmaf(r.y, qy, r.x * qx));  // revolutions, centred coordinates
    float n = __fsub_rn(__fadd_rn(u, 12582912.0f), 12582912.0f);
    float s, c;
    __sincosf(__fsub_rn(u, n) * 6.28318530717958647692f, &s, &c);
    return make_float2(b * c, b * s);
}

// The sub-vector v of a system in the form's units: FP32 from the per-call table in
// revolutions, FP64 as given.
__device__ __forceinline__ void load_qv(const double* qv, const float4* qrev, size_t v, float& qx, float& qy,
                                        float& qz) {
    const float4 r = qrev[v];
    qx = r.x;
    qy = r.y;
    qz = r.z;
}
__device__ __forceinline__ void load_qv(const double* qv, const float4* qrev, size_t v, double& qx, double& qy,
                                        double& qz) {
    const double* q = qv + 3 * v;
    qx = q[0];
    qy = q[1];
    qz = q[2];
}

template <class T>
__device__ __forceinline__ void load_q(const double* q, T& qx, T& qy, T& qz) {
    if (sizeof(T) == 4) {  // FP32 form: revolutions per Angstrom
        const double inv2pi = 0.15915494309189533577;
        qx = (T)(q[0] * inv2pi);
        qy = (T)(q[1] * inv2pi);
        qz = (T)(q[2] * inv2pi);
    } else {
        qx = (T)q[0];
        qy = (T)q[1];
        qz = (T)q[2];
    }
}

// Sum of (x, y) over the CTA in T, valid in thread 0 (FP32 in the FP32 form: GB300's FP64 pipe
// is a narrow fraction of its FP32 pipe, and a warp instruction occupies it whole even with one
// active lane). `red` holds NT / 32 pairs of T. Ends with a barrier so the caller may reuse
// shared memory afterwards.
template <class T, int NT>
__device__ typename cplx<T>::type block_sum_t(T x, T y, typename cplx<T>::type* red) {
    typedef typename cplx<T>::type T2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        T2 v;
        v.x = x;
        v.y = y;
        red[warp] = v;
    }
    __syncthreads();
    T2 s;
    s.x = 0;
    s.y = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; ++w) {
            s.x += red[w].x;
            s.y += red[w].y;
        }
    __syncthreads();
    return s;
}

// Sum of (x, y) over the warp in T, valid in every lane.
template <class T>
__device__ __forceinline__ typename cplx<T>::type warp_sum_t(T x, T y) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_xor_sync(0xffffffffu, x, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    typename cplx<T>::type v;
    v.x = x;
    v.y = y;
    return v;
}

// Per-series bookkeeping of the afinal / a2final partials: the sum of the series means and of
// their squared moduli. FP32 form: Kahan-compensated FP32, converted once at the end; FP64
// form: plain FP64.
template <class T>
struct SeriesAcc;

template <>
struct SeriesAcc<float> {
    float sx = 0.f, sy = 0.f, s2 = 0.f, cx = 0.f, cy = 0.f, c2 = 0.f;
    __device__ static void kahan(float& s, float& c, float v) {
        const float y = __fsub_rn(v, c), t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ void add(float x, float y) {
        kahan(sx, cx, x);
        kahan(sy, cy, y);
        kahan(s2, c2, fmaf(x, x, y * y));
    }
    __device__ double2 mean_sum() const { return make_double2((double)sx - (double)cx, (double)sy - (double)cy); }
    __device__ double sq_sum() const { return (double)s2 - (double)c2; }
};

template <>
struct SeriesAcc<double> {
    double sx = 0.0, sy = 0.0, s2 = 0.0;
    __device__ void add(double x, double y) {
        sx += x;
        sy += y;
        s2 += x * x + y * y;
    }
    __device__ double2 mean_sum() const { return make_double2(sx, sy); }
    __device__ double sq_sum() const { return s2; }
};

// Power spectrum of the series in buf (bit-reversed order): accumulate P and return this
// thread's part of sum_w P(w) K(w) in T (reduce it with block_sum_t).
template <class T, int NT, int MAXR>
__device__ __forceinline__ typename cplx<T>::type absorb_power_t(const typename cplx<T>::type* buf, int L,
                                                                  const typename cplx<T>::type* __restrict__ kbr,
                                                                  PowerAcc<T, MAXR>& acc) {
    typedef typename cplx<T>::type T2;
    T ax = 0, ay = 0;
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
        const int i = threadIdx.x + r * NT;
        if (i < L) {
            T2 X = buf[i];
            T P = X.x * X.x + X.y * X.y;
            acc.add(r, P);
            T2 k = kbr[i];
            ax += P * k.x;
            ay += P * k.y;
        }
    }
    T2 v;
    v.x = ax;
    v.y = ay;
    return v;
}

// Power spectrum of the series in buf (bit-reversed order): accumulate P and return
// this thread's part of sum_w P(w) K(w).
template <class T, int NT, int MAXR>
__device__ __forceinline__ double2 absorb_power(const typename cplx<T>::type* buf, int L,
                                                const typename cplx<T>::type* __restrict__ kbr,
                                                PowerAcc<T, MAXR>& acc) {
    typedef typename cplx<T>::type T2;
    T ax = 0, ay = 0;
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
        const int i = threadIdx.x + r * NT;
        if (i < L) {
            T2 X = buf[i];
            T P = X.x * X.x + X.y * X.y;
            acc.add(r, P);
            T2 k = kbr[i];
            ax += P * k.x;
            ay += P * k.y;
        }
    }
    return make_double2((double)ax, (double)ay);
}

template <class T, int NT, int MAXR>
__device__ __forceinline__ void write_power(const PowerAcc<T, MAXR>& acc, int L, double* dst) {
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
        const int i = threadIdx.x + r * NT;
        if (i < L) dst[i] = acc.get(r);
    }
}

// FP32 Kahan partials stored as (sum, compensation) float pairs in the double slot: the FP64
// finalisation combines them, so the kernels spend no FP64 conversions at the end.
template <int NT, int MAXR>
__device__ __forceinline__ void write_power_pair(const PowerAcc<float, MAXR>& acc, int L, double* dst) {
    float2* d2 = reinterpret_cast<float2*>(dst);
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
        const int i = threadIdx.x + r * NT;
        if (i < L) d2[i] = make_float2(acc.s[r], acc.c[r]);
    }
}

// Shared twiddle table of the launch: FP32 copies into shared memory, FP64 reads L1.
template <class T, int NT>
__device__ __forceinline__ const typename cplx<T>::type* stage_twiddles(
    typename cplx<T>::type* tws, const void* tw_, int lg_max) {
    typedef typename cplx<T>::type T2;
    const T2* twg = reinterpret_cast<const T2*>(tw_);
    if (sizeof(T) != 4) return twg;
    for (int i = threadIdx.x; i < (1 << (lg_max - 1)); i += NT) tws[i] = twg[i];
    return tws;
}

inline int grid_for(size_t n, int threads) {
    size_t b = (n + threads - 1) / threads;
    const size_t cap = (size_t)current_sms() * 32;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

template <class K>
cudaError_t set_smem(K k, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace
}  // namespace sassgpu
