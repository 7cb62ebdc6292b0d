// Long-series correlation (padded FFT length 2^14 .. 2^20, NF up to 524,288 frames).
//
// The shared-memory kernels of correlate.cu hold one padded series per CTA (L <= 8192);
// longer series go through HBM in four steps (see the section comment below). Same outputs
// as the short path: per-shell power spectra in partial slots, series means for afinal and
// a2final, and an FP64 finalisation per shell.
#include <algorithm>

#include "common.cuh"
#include "fft_util.cuh"
#include "kernels.h"

namespace sassgpu {
// ---------------------------------------------------------------------------------------
// Long series: padded length L = 2^14 .. 2^20 (NF up to 524,288 frames), four-step FFT
// through HBM with L = R x C, C = 4096:
//   X[k1 + R k2] = sum_n2 W_C^{n2 k2} W_L^{n2 k1} [sum_n1 x[C n1 + n2] W_R^{n1 k1}]
//   column pass: per series, length-R transforms over n1 for 16 columns n2 at a time in
//                shared memory, times W_L^{n2 k1}, stored as rows Y[k1][n2];
//   row pass:    per (row k1, chunk of series), the length-C transform of each row in shared
//                memory; |X|^2 accumulates in the chunk's slot and sum P K gives the row's part
//                of the series mean;
//   finalisation: slots summed per shell, then the inverse in the opposite order (rows with
//                conj twiddles, W_L^{-n2 k1}, columns), FP64, normalised as the short path.
// Spectra stay in (k1, bit-reversed k2) order; K is built in that order by the same passes.
// ---------------------------------------------------------------------------------------

// ---------------------------------------------------------------------------------------
// Float-float arithmetic for the FP32 form's long transforms. A value is h + l with
// |l| <= ulp(h) / 2; additions use Knuth's TwoSum, products the FMA-exact product (Dekker's
// method with the FMA instruction), each renormalised once ("sloppy" addition: absolute
// error about 2^-44 (|a| + |b|), the bound FFT butterflies need). These run on the FP32
// pipe: GB300's FP64 pipe made the FP64 transforms of this path its bound.
// ---------------------------------------------------------------------------------------
struct ffs {
    float h, l;
    ffs() = default;
    __device__ __forceinline__ ffs(float v) : h(v), l(0.f) {}
    __device__ __forceinline__ ffs(float hi, float lo) : h(hi), l(lo) {}
    __device__ __forceinline__ explicit operator double() const { return (double)h + (double)l; }
};
struct __align__(16) ff2 {
    ffs x, y;
};

__device__ __forceinline__ ffs ff_renorm(float s, float e) {
    const float h = __fadd_rn(s, e);
    return ffs(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ ffs operator+(ffs a, ffs b) {
    const float s = __fadd_rn(a.h, b.h), bb = __fsub_rn(s, a.h);
    float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    return ff_renorm(s, e);
}
__device__ __forceinline__ ffs operator-(ffs a) { return ffs(-a.h, -a.l); }
__device__ __forceinline__ ffs operator-(ffs a, ffs b) { return a + (-b); }
__device__ __forceinline__ ffs operator*(ffs a, ffs b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return ff_renorm(p, e);
}
__device__ __forceinline__ ffs& operator+=(ffs& a, ffs b) { return a = a + b; }
__device__ __forceinline__ ffs ff_from(double v) {
    const float h = (float)v;
    return ffs(h, (float)(v - (double)h));
}

template <>
struct cplx<ffs> {
    typedef ff2 type;
};
__device__ __forceinline__ ff2 make_ff2(ffs x, ffs y) {
    ff2 r;
    r.x = x;
    r.y = y;
    return r;
}
__device__ __forceinline__ ff2 cadd(ff2 a, ff2 b) { return make_ff2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ ff2 csub(ff2 a, ff2 b) { return make_ff2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ ff2 cmul(ff2 a, ff2 b) {
    return make_ff2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
namespace {

template <>
__device__ __forceinline__ ff2 zero2<ff2>() {
    return make_ff2(ffs(0.f), ffs(0.f));
}

// power spectrum accumulator of the float-float transforms (float-float sums)
template <int MAXR>
struct PowerAcc<ffs, MAXR> {
    ffs s[MAXR];
    __device__ void clear() {
#pragma unroll
        for (int r = 0; r < MAXR; ++r) s[r] = ffs(0.f);
    }
    __device__ __forceinline__ void add(int r, ffs p) { s[r] += p; }
    __device__ double get(int r) const { return (double)s[r]; }
};

// float-float tables from the FP64 ones
__global__ void to_ff2_kernel(const double2* __restrict__ src, size_t n, ff2* __restrict__ dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = make_ff2(ff_from(src[i].x), ff_from(src[i].y));
}

constexpr int kLongC = 1 << kLongRowLg;
constexpr int kLongTile = 16;  // columns per CTA in the column passes
constexpr int kLongNT = 256;

__device__ __forceinline__ float2 cneg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ ff2 cneg(ff2 a) { return make_ff2(-a.x, -a.y); }
__device__ __forceinline__ ff2 cconj(ff2 a) { return make_ff2(a.x, -a.y); }
__device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// W_L^m for 0 <= m < L from the half table tw[j] = W_L^j (j < L/2).
template <class T2>
__device__ __forceinline__ T2 tw_full(const T2* tw, int m, int L) {
    return m < (L >> 1) ? tw[m] : cneg(tw[m - (L >> 1)]);
}

__device__ __forceinline__ int brev_bits(int x, int bits) {
    return bits ? (int)(__brev((unsigned)x) >> (32 - bits)) : 0;
}

__device__ __forceinline__ float2 as_t2(float2 x, float2) { return x; }
__device__ __forceinline__ double2 as_t2(float2 x, double2) { return make_double2(x.x, x.y); }
__device__ __forceinline__ double2 as_t2(double2 x, double2) { return x; }
__device__ __forceinline__ float2 as_t2(double2 x, float2) { return make_float2((float)x.x, (float)x.y); }
__device__ __forceinline__ ff2 as_t2(float2 x, ff2) { return make_ff2(ffs(x.x), ffs(x.y)); }
__device__ __forceinline__ ff2 as_t2(double2 x, ff2) { return make_ff2(ff_from(x.x), ff_from(x.y)); }

template <class T, class AT2>
__global__ void __launch_bounds__(kLongNT) long_col_kernel(LongArgs a) {
    typedef typename cplx<T>::type T2;
    extern __shared__ __align__(16) unsigned char smem[];
    T2* buf = reinterpret_cast<T2*>(smem);  // [kLongTile][R]
    const int r = a.lg - kLongRowLg, R = 1 << r, half = R >> 1, L = 1 << a.lg;
    const int n2base = blockIdx.x * kLongTile;
    const AT2* A = reinterpret_cast<const AT2*>(a.A) + (size_t)blockIdx.y * a.nf;
    const T2* tw = reinterpret_cast<const T2*>(a.tw);
    // first stage folded into the load: x[C n1 + n2] = 0 for n1 >= R/2 (C R / 2 = L / 2 >= nf)
    for (int idx = threadIdx.x; idx < kLongTile * half; idx += kLongNT) {
        const int c = idx % kLongTile, n1 = idx / kLongTile;
        const int t = kLongC * n1 + n2base + c;
        const T2 x = t < a.nf ? as_t2(A[t], T2()) : zero2<T2>();
        buf[c * R + n1] = x;
        buf[c * R + n1 + half] = cmul(x, tw[n1 << kLongRowLg]);  // W_R^n1 = W_L^{n1 C}
    }
    __syncthreads();
    for (int lh = r - 2; lh >= 0; --lh) {
        const int h = 1 << lh, sh = kLongRowLg + (r - 1 - lh);
        for (int b = threadIdx.x; b < kLongTile * half; b += kLongNT) {
            const int c = b / half, bb = b - c * half;
            const int p = bb & (h - 1), i0 = ((bb >> lh) << (lh + 1)) + p;
            T2* col = buf + c * R;
            const T2 u = col[i0], w = col[i0 + h];
            col[i0] = cadd(u, w);
            col[i0 + h] = cmul(csub(u, w), tw[p << sh]);
        }
        __syncthreads();
    }
    T2* Y = reinterpret_cast<T2*>(a.Y) + (size_t)blockIdx.y * L;
    for (int idx = threadIdx.x; idx < kLongTile * R; idx += kLongNT) {
        const int c = idx % kLongTile, k1 = idx / kLongTile, n2 = n2base + c;
        Y[(size_t)k1 * kLongC + n2] = cmul(buf[c * R + brev_bits(k1, r)], tw_full(tw, n2 * k1, L));
    }
}

// MODE 0: power and mean parts of every series of the CTA's chunk, for row k1 = blockIdx.x.
// MODE 1: the transform of series 0 written conjugated to xout.
template <class T, int MODE>
__global__ void __launch_bounds__(kLongNT) long_row_kernel(LongArgs a) {
    typedef typename cplx<T>::type T2;
    constexpr int MAXR = kLongC / kLongNT;
    extern __shared__ __align__(16) unsigned char smem[];
    T2* buf = reinterpret_cast<T2*>(smem);            // [C]
    T2* twc = buf + kLongC;                            // [C/2] W_C^p
    double2* red = reinterpret_cast<double2*>(twc + kLongC / 2);
    const int r = a.lg - kLongRowLg, R = 1 << r, L = 1 << a.lg;
    const int k1 = blockIdx.x;
    const T2* tw = reinterpret_cast<const T2*>(a.tw);
    for (int p = threadIdx.x; p < kLongC / 2; p += kLongNT) twc[p] = tw[p << r];  // W_C^p = W_L^{p R}
    int v_begin = 0, v_end = 1;
    size_t part_off = 0;
    if (MODE == 0) {
        const CorrChunk c = a.chunks[blockIdx.y];
        v_begin = c.v_begin;
        v_end = c.v_end;
        part_off = c.part_off;
    }
    PowerAcc<T, MAXR> acc;
    acc.clear();
    const T2* kbr = MODE == 0 ? reinterpret_cast<const T2*>(a.kbr) + (size_t)k1 * kLongC : nullptr;
    __syncthreads();
    for (int v = v_begin; v < v_end; ++v) {
        const T2* row = reinterpret_cast<const T2*>(a.Y) + (size_t)(v - a.v0) * L + (size_t)k1 * kLongC;
        for (int i = threadIdx.x; i < kLongC / 2; i += kLongNT) {
            const T2 u = row[i], w = row[i + kLongC / 2];
            buf[i] = cadd(u, w);
            buf[i + kLongC / 2] = cmul(csub(u, w), twc[i]);
        }
        __syncthreads();
        dif_tail<T2, kLongNT>(buf, twc, kLongRowLg, 0);
        if (MODE == 1) {
            T2* out = reinterpret_cast<T2*>(a.xout) + (size_t)k1 * kLongC;
            for (int i = threadIdx.x; i < kLongC; i += kLongNT) out[i] = cconj(buf[i]);
            __syncthreads();
        } else {
            const double2 m = block_sum<kLongNT>(absorb_power<T, kLongNT, MAXR>(buf, kLongC, kbr, acc), red);
            if (threadIdx.x == 0) a.mpart[(size_t)v * R + k1] = m;
        }
    }
    if (MODE == 0) write_power<T, kLongNT, MAXR>(acc, kLongC, a.ppart + part_off + (size_t)k1 * kLongC);
}

__global__ void long_mean_kernel(const CorrChunk* __restrict__ chunks, int nchunks, const double2* __restrict__ mpart,
                                 int R, double2* apart, double* a2part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nchunks) return;
    const CorrChunk c = chunks[i];
    double2 as = make_double2(0.0, 0.0);
    double a2 = 0.0;
    for (int v = c.v_begin; v < c.v_end; ++v) {
        double2 m = make_double2(0.0, 0.0);
        for (int k = 0; k < R; ++k) {
            const double2 x = mpart[(size_t)v * R + k];
            m.x += x.x;
            m.y += x.y;
        }
        as.x += m.x;
        as.y += m.y;
        a2 += m.x * m.x + m.y * m.y;
    }
    apart[c.slot] = as;
    a2part[c.slot] = a2;
}

// Finalisation, rows: sum the shell's slots for row k1, inverse length-C transform
// (bit-reversed k2 in, natural n2 out), times W_L^{-n2 k1}.
__global__ void __launch_bounds__(kLongNT) long_final_rows_kernel(LongFinal a) {
    extern __shared__ __align__(16) unsigned char smem[];
    double2* buf = reinterpret_cast<double2*>(smem);
    const FinalEntry e = a.entries[blockIdx.y];
    const int k1 = blockIdx.x, r = a.lg - kLongRowLg, L = 1 << a.lg;
    for (int i = threadIdx.x; i < kLongC; i += kLongNT) {
        double p = 0.0;
        for (int k = e.slot_begin; k < e.slot_end; ++k)
            p += a.ppart[e.part_off + (size_t)(k - e.slot_begin) * e.part_len + (size_t)k1 * kLongC + i];
        buf[i] = make_double2(p, 0.0);
    }
    __syncthreads();
    dit_inverse<kLongNT>(buf, a.tw, kLongRowLg, r);  // W_C^p = tw[p << r]
    double2* Z = a.Z + (size_t)blockIdx.y * L + (size_t)k1 * kLongC;
    for (int n2 = threadIdx.x; n2 < kLongC; n2 += kLongNT) Z[n2] = cmulc(buf[n2], tw_full(a.tw, n2 * k1, L));
}

// Finalisation, columns: inverse length-R transforms over k1 for 16 columns n2, then
// tau = C n1 + n2 < NF normalised by 1/(L (NF - tau)) and 1/NM; fq, fq2 from the slots.
__global__ void __launch_bounds__(kLongNT) long_final_cols_kernel(LongFinal a) {
    extern __shared__ __align__(16) unsigned char smem[];
    double2* buf = reinterpret_cast<double2*>(smem);  // [kLongTile][R]
    const FinalEntry e = a.entries[blockIdx.y];
    const int r = a.lg - kLongRowLg, R = 1 << r, half = R >> 1, L = 1 << a.lg;
    const int n2base = blockIdx.x * kLongTile;
    const double2* Z = a.Z + (size_t)blockIdx.y * L;
    for (int idx = threadIdx.x; idx < kLongTile * R; idx += kLongNT) {
        const int c = idx % kLongTile, k1 = idx / kLongTile;
        buf[c * R + brev_bits(k1, r)] = Z[(size_t)k1 * kLongC + n2base + c];
    }
    __syncthreads();
    for (int lh = 0; lh < r; ++lh) {
        const int h = 1 << lh, sh = kLongRowLg + (r - 1 - lh);
        for (int b = threadIdx.x; b < kLongTile * half; b += kLongNT) {
            const int c = b / half, bb = b - c * half;
            const int p = bb & (h - 1), i0 = ((bb >> lh) << (lh + 1)) + p;
            double2* col = buf + c * R;
            const double2 u = col[i0];
            const double2 w = cmulc(col[i0 + h], __ldg(a.tw + (p << sh)));
            col[i0] = cadd(u, w);
            col[i0 + h] = csub(u, w);
        }
        __syncthreads();
    }
    const int nf = e.nf;
    const double sgn = a.conj_out ? -1.0 : 1.0;
    for (int idx = threadIdx.x; idx < kLongTile * R; idx += kLongNT) {
        const int c = idx % kLongTile, n1 = idx / kLongTile;
        const int tau = kLongC * n1 + n2base + c;
        if (tau < nf) {
            const double2 x = buf[c * R + n1];
            const double f = (1.0 / ((double)L * (double)(nf - tau))) * e.inv_nm;
            e.fqt[tau] = make_double2(x.x * f, sgn * x.y * f);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double2 as = make_double2(0.0, 0.0);
        double a2 = 0.0;
        for (int k = e.slot_begin; k < e.slot_end; ++k) {
            as.x += a.apart[k].x;
            as.y += a.apart[k].y;
            a2 += a.a2part[k];
        }
        *e.fq = make_double2(as.x * e.inv_nm, sgn * as.y * e.inv_nm);
        *e.fq2 = make_double2(a2 * e.inv_nm, 0.0);
    }
}

template <class T>
__global__ void long_self_series_kernel(LongSelfArgs a) {
    typedef typename cplx<T>::type T2;
    const T* b = reinterpret_cast<const T*>(a.bfac);
    T2* G = reinterpret_cast<T2*>(a.G);
    const size_t n = (size_t)a.nseries * a.nf;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int s = (int)(idx / a.nf), t = (int)(idx - (size_t)s * a.nf);
        const int p = a.p0 + s, j = p / a.nm, m = p - j * a.nm;
        T qx, qy, qz;
        load_qv(a.qv, a.qrev, (size_t)m, qx, qy, qz);
        G[idx] = self_term(b[j], a.xyz[(size_t)t * a.na_pad + j], qx, qy, qz);
    }
}

__global__ void long_window_kernel(int nf, int L, double2* w) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += gridDim.x * blockDim.x)
        w[t] = make_double2(1.0 / ((double)nf * (double)L * (double)(nf - t)), 0.0);
}

__global__ void long_k32_kernel(const double2* k64, int L, float2* k32) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x)
        k32[i] = make_float2((float)k64[i].x, (float)k64[i].y);
}

size_t long_elem(int precision) { return precision == PREC_FP32 ? sizeof(float2) : precision == PREC_FF ? sizeof(ff2) : sizeof(double2); }

size_t long_col_smem(int precision, int lg) {
    return (size_t)kLongTile * ((size_t)1 << (lg - kLongRowLg)) * long_elem(precision);
}

size_t long_row_smem(int precision) {
    const size_t e = long_elem(precision);
    return (size_t)kLongC * e + (size_t)(kLongC / 2) * e + (kLongNT / 32) * sizeof(double2);
}

bool long_ok(int lg) { return lg > kLongRowLg + 1 && lg <= kLongLgMax; }

}  // namespace

cudaError_t launch_long_columns(const LongArgs& a, cudaStream_t st) {
    if (!long_ok(a.lg)) return cudaErrorInvalidValue;
    if (a.nseries == 0) return cudaSuccess;
    const size_t sm = long_col_smem(a.precision, a.lg);
    dim3 grid(kLongC / kLongTile, (unsigned)a.nseries);
    auto k = a.precision == PREC_FP32 ? (a.amp_f32 ? long_col_kernel<float, float2> : long_col_kernel<float, double2>)
             : a.precision == PREC_FF ? (a.amp_f32 ? long_col_kernel<ffs, float2> : long_col_kernel<ffs, double2>)
                                      : (a.amp_f32 ? long_col_kernel<double, float2> : long_col_kernel<double, double2>);
    cudaError_t e = set_smem(k, sm);
    if (e != cudaSuccess) return e;
    k<<<grid, kLongNT, sm, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_long_rows(const LongArgs& a, cudaStream_t st) {
    if (!long_ok(a.lg)) return cudaErrorInvalidValue;
    if (a.nchunks == 0) return cudaSuccess;
    if (a.nchunks > 65535) return cudaErrorInvalidValue;  // grid y: the engine's batches hold fewer
    const size_t sm = long_row_smem(a.precision);
    dim3 grid((unsigned)(1 << (a.lg - kLongRowLg)), (unsigned)a.nchunks);
    if (a.precision == PREC_FP32) {
        cudaError_t e = set_smem(long_row_kernel<float, 0>, sm);
        if (e != cudaSuccess) return e;
        long_row_kernel<float, 0><<<grid, kLongNT, sm, st>>>(a);
    } else if (a.precision == PREC_FF) {
        cudaError_t e = set_smem(long_row_kernel<ffs, 0>, sm);
        if (e != cudaSuccess) return e;
        long_row_kernel<ffs, 0><<<grid, kLongNT, sm, st>>>(a);
    } else {
        cudaError_t e = set_smem(long_row_kernel<double, 0>, sm);
        if (e != cudaSuccess) return e;
        long_row_kernel<double, 0><<<grid, kLongNT, sm, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_long_transform(const LongArgs& a, cudaStream_t st) {
    if (!long_ok(a.lg) || a.precision != PREC_FP64) return cudaErrorInvalidValue;
    LongArgs b = a;
    b.nseries = 1;
    cudaError_t e = launch_long_columns(b, st);
    if (e != cudaSuccess) return e;
    const size_t sm = long_row_smem(PREC_FP64);
    e = set_smem(long_row_kernel<double, 1>, sm);
    if (e != cudaSuccess) return e;
    long_row_kernel<double, 1><<<dim3((unsigned)(1 << (a.lg - kLongRowLg)), 1), kLongNT, sm, st>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_long_self_series(const LongSelfArgs& a, cudaStream_t st) {
    const size_t n = (size_t)a.nseries * a.nf;
    if (n == 0) return cudaSuccess;
    if (a.precision == PREC_FP32) long_self_series_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(a);
    else long_self_series_kernel<double><<<grid_for(n, 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_long_means(const CorrChunk* chunks, int nchunks, const double2* mpart, int R, double2* apart,
                              double* a2part, cudaStream_t st) {
    if (nchunks == 0) return cudaSuccess;
    long_mean_kernel<<<(nchunks + 127) / 128, 128, 0, st>>>(chunks, nchunks, mpart, R, apart, a2part);
    return cudaGetLastError();
}

cudaError_t launch_long_finalize(const LongFinal& a, cudaStream_t st) {
    if (a.nentries == 0) return cudaSuccess;
    if (!long_ok(a.lg)) return cudaErrorInvalidValue;
    const int R = 1 << (a.lg - kLongRowLg);
    const size_t sm_rows = (size_t)kLongC * sizeof(double2);
    const size_t sm_cols = long_col_smem(PREC_FP64, a.lg);
    cudaError_t e = set_smem(long_final_rows_kernel, sm_rows);
    if (e != cudaSuccess) return e;
    if ((e = set_smem(long_final_cols_kernel, sm_cols)) != cudaSuccess) return e;
    for (int e0 = 0; e0 < a.nentries; e0 += 65535) {  // entries in grid y, at most 65,535 per launch
        LongFinal b = a;
        b.entries = a.entries + e0;
        b.nentries = std::min(65535, a.nentries - e0);
        b.Z = a.Z + (size_t)e0 * ((size_t)1 << a.lg);
        long_final_rows_kernel<<<dim3((unsigned)R, (unsigned)b.nentries), kLongNT, sm_rows, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        long_final_cols_kernel<<<dim3(kLongC / kLongTile, (unsigned)b.nentries), kLongNT, sm_cols, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_to_ff2(const double2* src, size_t n, void* dst, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    to_ff2_kernel<<<grid_for(n, 256), 256, 0, st>>>(src, n, static_cast<ff2*>(dst));
    return cudaGetLastError();
}

cudaError_t launch_long_store_kernel(const double2* tw64, int lg, int nf, double2* scratch, double2* k64,
                                     float2* k32, cudaStream_t st) {
    if (!long_ok(lg)) return cudaErrorInvalidValue;
    const int L = 1 << lg;
    long_window_kernel<<<grid_for(nf, 256), 256, 0, st>>>(nf, L, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    LongArgs a{};
    a.precision = PREC_FP64;
    a.lg = lg;
    a.nf = nf;
    a.A = scratch;
    a.Y = scratch + nf;
    a.nseries = 1;
    a.tw = tw64;
    a.xout = k64;
    e = launch_long_transform(a, st);
    if (e != cudaSuccess) return e;
    long_k32_kernel<<<grid_for(L, 256), 256, 0, st>>>(k64, L, k32);
    return cudaGetLastError();
}

}  // namespace sassgpu
