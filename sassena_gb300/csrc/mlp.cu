// Learned control variate: a small MLP g(u, |q|) ~ |A(q u)|^2 used to reduce the variance
// of the Monte Carlo orientational average.
//
// Network: x = (ux, uy, uz, s) with s = (|q| - q_mid)/q_half -> tanh(W1 x + b1) [128]
// -> tanh(W2 h1 + b2) [128] -> y = W3 h2 + b3, the prediction of the normalised log
// intensity. Weights are held in BF16 for the forward and backward passes (FP32 master
// copy for the optimiser); every product is accumulated in FP32. g = exp(y*y_std + y_mean).
//
// Kernels (all hand-written, no library calls):
//   mlp_train_kernel   fused forward + loss + backward over tiles of 32 samples; weight
//                      gradients accumulate in shared memory per CTA (persistent loop) and
//                      are added to the global FP32 gradient once per CTA
//   mlp_adam_kernel    Adam on the FP32 master weights, refreshes the BF16 copy
//   mlp_forward_kernel inference y for arbitrary inputs
//   mlp_sphere_kernel  dense spherical-Fibonacci quadrature of g on each shell (FP64 sums)
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "mlp.h"

namespace sassgpu {

namespace {

constexpr int H = kMlpHidden;  // 128
constexpr int TB = 32;         // samples per tile
constexpr int NT = 128;        // threads per CTA (one per hidden unit)

// Parameter offsets in the packed vector.
constexpr int OW1 = 0, OB1 = OW1 + H * 4, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + H;
static_assert(OB3 + 1 == kMlpParams, "parameter layout");

struct Smem {
    float w1[H * 4], b1[H], w2[H * (H + 1)], b2[H], w3[H], b3;
    float x[TB * 4], t[TB];
    float h1[TB * H], z2n[TB * H];  // h1 = tanh(z1); then dz2 for the backward
    float y[TB], dy[TB];
};

__device__ __forceinline__ float bf(const __nv_bfloat16* p, int i) { return __bfloat162float(p[i]); }

__device__ void load_weights(Smem& s, const __nv_bfloat16* __restrict__ w) {
    for (int i = threadIdx.x; i < H * 4; i += NT) s.w1[i] = bf(w, OW1 + i);
    for (int i = threadIdx.x; i < H * H; i += NT) s.w2[(i / H) * (H + 1) + (i % H)] = bf(w, OW2 + i);
    for (int i = threadIdx.x; i < H; i += NT) {
        s.b1[i] = bf(w, OB1 + i);
        s.b2[i] = bf(w, OB2 + i);
        s.w3[i] = bf(w, OW3 + i);
    }
    if (threadIdx.x == 0) s.b3 = bf(w, OB3);
}

// Forward of one tile: thread j owns hidden unit j. Leaves h1 in s.h1, h2 in regs h2[],
// y in s.y. n = valid samples of the tile.
__device__ void forward_tile(Smem& s, float* h2, int n) {
    const int j = threadIdx.x;
    for (int b = 0; b < TB; ++b) {
        float z = s.b1[j];
#pragma unroll
        for (int k = 0; k < 4; ++k) z = fmaf(s.w1[j * 4 + k], s.x[b * 4 + k], z);
        s.h1[b * H + j] = b < n ? tanhf(z) : 0.f;
    }
    __syncthreads();
    float acc[TB];
#pragma unroll
    for (int b = 0; b < TB; ++b) acc[b] = s.b2[j];
    const float* wr = s.w2 + j * (H + 1);
    for (int k = 0; k < H; ++k) {
        const float w = wr[k];
#pragma unroll
        for (int b = 0; b < TB; ++b) acc[b] = fmaf(w, s.h1[b * H + k], acc[b]);
    }
#pragma unroll
    for (int b = 0; b < TB; ++b) {
        h2[b] = tanhf(acc[b]);
        s.z2n[b * H + j] = s.w3[j] * h2[b];
    }
    __syncthreads();
    if (j < TB) {  // y_b = sum_j w3_j h2_bj + b3
        float y = s.b3;
        for (int k = 0; k < H; ++k) y += s.z2n[j * H + k];
        s.y[j] = y;
    }
    __syncthreads();
}

}  // namespace

__global__ void __launch_bounds__(NT) mlp_train_kernel(const __nv_bfloat16* __restrict__ w,
                                                       const float* __restrict__ X, const float* __restrict__ T,
                                                       int n, float inv_n, float* __restrict__ grad,
                                                       double* __restrict__ loss) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    float* gw2 = reinterpret_cast<float*>(smem_raw + sizeof(Smem));  // [H][H+1] gradient of W2
    load_weights(s, w);
    const int j = threadIdx.x;
    for (int k = 0; k < H; ++k) gw2[j * (H + 1) + k] = 0.f;
    float gw1[4] = {0, 0, 0, 0}, gb1 = 0, gb2 = 0, gw3 = 0, gb3 = 0;
    double l = 0.0;
    __syncthreads();
    const int ntiles = (n + TB - 1) / TB;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int b0 = tile * TB, nb = min(TB, n - b0);
        for (int i = threadIdx.x; i < TB * 4; i += NT) s.x[i] = (i / 4) < nb ? X[(size_t)b0 * 4 + i] : 0.f;
        if (j < TB) s.t[j] = j < nb ? T[b0 + j] : 0.f;
        __syncthreads();
        float h2[TB];
        forward_tile(s, h2, nb);
        if (j < TB) {  // d loss / d y for loss = mean (y - t)^2
            float d = j < nb ? s.y[j] - s.t[j] : 0.f;
            s.dy[j] = 2.f * d * inv_n;
            l += (double)d * d;
        }
        __syncthreads();
        // layer 3 and dz2 = dy * w3 * (1 - h2^2)
#pragma unroll
        for (int b = 0; b < TB; ++b) {
            const float dy = s.dy[b];
            gw3 = fmaf(dy, h2[b], gw3);
            s.z2n[b * H + j] = dy * s.w3[j] * (1.f - h2[b] * h2[b]);
        }
        if (j == 0)
            for (int b = 0; b < TB; ++b) gb3 += s.dy[b];
        __syncthreads();
        // dW2[j][k] += sum_b dz2[b][j] h1[b][k]; db2
        for (int b = 0; b < TB; ++b) gb2 += s.z2n[b * H + j];
        for (int k = 0; k < H; ++k) {
            float g = 0.f;
#pragma unroll 8
            for (int b = 0; b < TB; ++b) g = fmaf(s.z2n[b * H + j], s.h1[b * H + k], g);
            gw2[j * (H + 1) + k] += g;
        }
        // dh1[b][k=j] = sum_i W2[i][j] dz2[b][i]; dz1 = dh1 (1 - h1^2)
        float dz1[TB];
#pragma unroll
        for (int b = 0; b < TB; ++b) dz1[b] = 0.f;
        for (int i = 0; i < H; ++i) {
            const float wij = s.w2[i * (H + 1) + j];
#pragma unroll
            for (int b = 0; b < TB; ++b) dz1[b] = fmaf(wij, s.z2n[b * H + i], dz1[b]);
        }
#pragma unroll
        for (int b = 0; b < TB; ++b) {
            const float h = s.h1[b * H + j];
            const float d = dz1[b] * (1.f - h * h);
            gb1 += d;
#pragma unroll
            for (int k = 0; k < 4; ++k) gw1[k] = fmaf(d, s.x[b * 4 + k], gw1[k]);
        }
        __syncthreads();
    }
    for (int k = 0; k < 4; ++k) atomicAdd(&grad[OW1 + j * 4 + k], gw1[k]);
    atomicAdd(&grad[OB1 + j], gb1);
    for (int k = 0; k < H; ++k) atomicAdd(&grad[OW2 + j * H + k], gw2[j * (H + 1) + k]);
    atomicAdd(&grad[OB2 + j], gb2);
    atomicAdd(&grad[OW3 + j], gw3);
    if (j == 0) atomicAdd(&grad[OB3], gb3);
    if (j < TB) atomicAdd(loss, l * inv_n);
}

__global__ void mlp_adam_kernel(float* __restrict__ master, __nv_bfloat16* __restrict__ w,
                                const float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v,
                                float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpParams; i += gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * g;
        const float vi = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        const float p = master[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        master[i] = p;
        w[i] = __float2bfloat16_rn(p);
    }
}

__global__ void __launch_bounds__(NT) mlp_forward_kernel(const __nv_bfloat16* __restrict__ w,
                                                         const float* __restrict__ X, int n, float* __restrict__ Y) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    load_weights(s, w);
    __syncthreads();
    const int ntiles = (n + TB - 1) / TB;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int b0 = tile * TB, nb = min(TB, n - b0);
        for (int i = threadIdx.x; i < TB * 4; i += NT) s.x[i] = (i / 4) < nb ? X[(size_t)b0 * 4 + i] : 0.f;
        __syncthreads();
        float h2[TB];
        forward_tile(s, h2, nb);
        if (threadIdx.x < nb) Y[b0 + threadIdx.x] = s.y[threadIdx.x];
        __syncthreads();
    }
}

// Mean of g = exp(y * y_std + y_mean) over a spherical-Fibonacci set of P points on
// each shell: gbar[s] (FP64). One CTA per (shell, chunk of points); per-CTA FP64
// partials are added with atomics (fixed count per shell, order-independent to ~1e-16).
__global__ void __launch_bounds__(NT) mlp_sphere_kernel(const __nv_bfloat16* __restrict__ w,
                                                        const double* __restrict__ qlen, int nshell, int P,
                                                        int chunks, float q_mid, float q_half, float y_mean,
                                                        float y_std, double* __restrict__ gbar) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    __shared__ double red[NT / 32];
    load_weights(s, w);
    __syncthreads();
    const int sh = blockIdx.x / chunks, c = blockIdx.x % chunks;
    const int per = (P + chunks - 1) / chunks, p0 = c * per, p1 = min(P, p0 + per);
    const float sq = (float)((qlen[sh] - q_mid) / q_half);
    const double golden = 3.14159265358979323846 * (3.0 - 2.23606797749978969641);
    double acc = 0.0;
    for (int b0 = p0; b0 < p1; b0 += TB) {
        const int nb = min(TB, p1 - b0);
        if (threadIdx.x < TB) {
            const int i = b0 + threadIdx.x;
            const double z = 1.0 - 2.0 * (i + 0.5) / P;
            const double r = sqrt(fmax(0.0, 1.0 - z * z));
            double sn, cs;
            sincos(golden * (i + 0.5), &sn, &cs);
            s.x[threadIdx.x * 4 + 0] = (float)(r * cs);
            s.x[threadIdx.x * 4 + 1] = (float)(r * sn);
            s.x[threadIdx.x * 4 + 2] = (float)z;
            s.x[threadIdx.x * 4 + 3] = sq;
        }
        __syncthreads();
        float h2[TB];
        forward_tile(s, h2, nb);
        if (threadIdx.x < nb) acc += exp((double)s.y[threadIdx.x] * y_std + y_mean);
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < NT / 32; ++k) t += red[k];
        atomicAdd(&gbar[sh], t / P);
    }
}

// A_v(t) *= sqrt(g_v): the autocorrelation of the scaled series is g_v C_v(t).
template <class T2>
__global__ void scale_series_kernel(T2* __restrict__ A, const double* __restrict__ wsqrt, size_t nv, int nf) {
    const size_t n = nv * (size_t)nf;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double f = wsqrt[i / nf];
        T2 a = A[i];
        a.x = (decltype(a.x))(a.x * f);
        a.y = (decltype(a.y))(a.y * f);
        A[i] = a;
    }
}

size_t mlp_smem_bytes(bool train) {
    return sizeof(Smem) + (train ? (size_t)H * (H + 1) * sizeof(float) : 0);
}

cudaError_t launch_mlp_train(const __nv_bfloat16* w, const float* X, const float* T, int n, float* grad,
                             double* loss, int sms, cudaStream_t st) {
    const size_t sm = mlp_smem_bytes(true);
    cudaError_t e = cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const int tiles = (n + TB - 1) / TB;
    const int grid = max(1, min(tiles, sms));
    mlp_train_kernel<<<grid, NT, sm, st>>>(w, X, T, n, 1.f / n, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* master, __nv_bfloat16* w, const float* grad, float* m, float* v, float lr,
                            int step, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
    mlp_adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(master, w, grad, m, v, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_mlp_forward(const __nv_bfloat16* w, const float* X, int n, float* Y, int sms, cudaStream_t st) {
    const size_t sm = mlp_smem_bytes(false);
    cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const int tiles = (n + TB - 1) / TB;
    mlp_forward_kernel<<<max(1, min(tiles, sms * 4)), NT, sm, st>>>(w, X, n, Y);
    return cudaGetLastError();
}

cudaError_t launch_mlp_sphere(const __nv_bfloat16* w, const double* qlen, int nshell, int P, float q_mid,
                              float q_half, float y_mean, float y_std, double* gbar, int sms, cudaStream_t st) {
    const size_t sm = mlp_smem_bytes(false);
    cudaError_t e = cudaFuncSetAttribute(mlp_sphere_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(gbar, 0, nshell * sizeof(double), st);
    if (e != cudaSuccess) return e;
    const int chunks = max(1, min((P + 1023) / 1024, (sms * 4 + nshell - 1) / nshell));
    mlp_sphere_kernel<<<nshell * chunks, NT, sm, st>>>(w, qlen, nshell, P, chunks, q_mid, q_half, y_mean, y_std,
                                                       gbar);
    return cudaGetLastError();
}

cudaError_t launch_scale_series(void* A, bool f32, const double* wsqrt, size_t nv, int nf, cudaStream_t st) {
    const size_t n = nv * (size_t)nf;
    int blocks = n ? (int)grid_blocks(n, 256, 16) : 0;
    if (blocks < 1) return cudaSuccess;
    if (f32) scale_series_kernel<float2><<<blocks, 256, 0, st>>>((float2*)A, wsqrt, nv, nf);
    else scale_series_kernel<double2><<<blocks, 256, 0, st>>>((double2*)A, wsqrt, nv, nf);
    return cudaGetLastError();
}

}  // namespace sassgpu
