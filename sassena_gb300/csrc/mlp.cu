// Learned control variate: a small MLP g(u, |q|) ~ |A(q u)|^2 used to reduce the variance
// of the Monte Carlo orientational average.
//
// Network: x = (ux, uy, uz, s) with s = (|q| - q_mid)/q_half -> tanh(W1 x + b1) [128]
// -> tanh(W2 h1 + b2) [128] -> y = W3 h2 + b3, the prediction of the normalised log
// intensity. Weights are held in BF16 for the forward and backward passes (FP32 master
// copy for the optimiser); every product is accumulated in FP32. g = exp(y*y_std + y_mean).
//
// The 128 x 128 layer is the one dense contraction. Its three products per tile of 32
// samples run on the tensor cores as BF16 mma.sync (m16n8k16) with FP32 accumulation:
//   forward        z2 = h1 W2^T            (32 x 128, K = 128)
//   weight grad    dW2 += dz2^T h1         (128 x 128, K = 32), held in registers
//   input grad     dh1 = dz2 W2            (32 x 128, K = 128)
// so their operands h1 and dz2 are rounded to BF16 (the weights already are); tanh, the
// derivatives, the biases and the two small layers stay in FP32.
//
// Kernels (all hand-written, no library calls):
//   mlp_train_kernel   fused forward + loss + backward over tiles of 32 samples; each CTA
//                      (persistent loop) writes its partial gradient to its own slot
//   mlp_reduce_kernel  sums the CTAs' slots in CTA order: the gradient and the loss are the
//                      same bits from run to run (no floating-point atomics)
//   mlp_adam_kernel    Adam on the FP32 master weights, refreshes the BF16 copy
//   mlp_forward_kernel inference y for arbitrary inputs
//   mlp_sphere_kernel  dense spherical-Fibonacci quadrature of g on each shell (FP64 sums,
//                      parts combined in a fixed order by mlp_sphere_reduce_kernel)
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "mlp.h"

namespace sassgpu {

namespace {

constexpr int H = kMlpHidden;  // 128
constexpr int TB = 32;         // samples per tile
constexpr int NT = 128;        // threads per CTA: thread j owns hidden unit j; warp w owns units 32w ..
constexpr int HP = H + 8;      // padded BF16 row of 128 (272 bytes): conflict-free fragment loads
constexpr int TBP = TB + 8;    // padded BF16 row of 32 (80 bytes)

// Parameter offsets in the packed vector.
constexpr int OW1 = 0, OB1 = OW1 + H * 4, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + H;
static_assert(OB3 + 1 == kMlpParams, "parameter layout");

struct Smem {
    float w1[H * 4], b1[H], b2[H], w3[H], b3, pad0[3];
    float x[TB * 4], t[TB], y[TB], dy[TB], ypart[NT / 32][TB];
    float h1f[TB * H];  // h1 in FP32 [b][j] (its derivative)
    float h2[TB * H];   // h2 in FP32 [b][j]
    float dz1[TB * H];  // dz1 in FP32 [b][j]
    __nv_bfloat16 w2[H * HP];     // W2 [j][k]
    __nv_bfloat16 w2t[H * HP];    // W2 transposed [k][j] (the input gradient's operand)
    __nv_bfloat16 h1[TB * HP];    // h1 [b][k]
    __nv_bfloat16 h1t[H * TBP];   // h1 transposed [k][b]
    __nv_bfloat16 dz2[TB * HP];   // dz2 [b][j]
    __nv_bfloat16 dz2t[H * TBP];  // dz2 transposed [j][b]
};

__device__ __forceinline__ float bf(const __nv_bfloat16* p, int i) { return __bfloat162float(p[i]); }

// two consecutive BF16 as one 32-bit fragment register
__device__ __forceinline__ uint32_t ld2(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// D = A B + D, A 16 x 16 (row), B 16 x 8 (column), BF16 in, FP32 accumulate
__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// One 16 x 8 output block over K = 16 KS: A rows [ar, ar + 16) of a row-major [*][lda] array,
// B columns [bn, bn + 8) of an array stored as [n][ldb] (k contiguous), from k = k0.
// Fragment layout of m16n8k16 (g = lane / 4, t = lane % 4): A rows g, g + 8, columns 2t,
// 2t + 1 and 2t + 8, 2t + 9; B column g, rows 2t, 2t + 1 and 2t + 8, 2t + 9; D rows g, g + 8,
// columns 2t, 2t + 1.
template <int KS>
__device__ __forceinline__ void mma_block(float (&d)[4], const __nv_bfloat16* A, int lda, int ar,
                                          const __nv_bfloat16* B, int ldb, int bn, int k0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
        const int k = k0 + 16 * ks + 2 * t;
        const __nv_bfloat16* a = A + (size_t)(ar + g) * lda + k;
        const __nv_bfloat16* b = B + (size_t)(bn + g) * ldb + k;
        mma_bf16(d, ld2(a), ld2(a + 8 * lda), ld2(a + 8), ld2(a + 8 * lda + 8), ld2(b), ld2(b + 8));
    }
}

__device__ void load_weights(Smem& s, const __nv_bfloat16* __restrict__ w, bool transposed) {
    for (int i = threadIdx.x; i < H * 4; i += NT) s.w1[i] = bf(w, OW1 + i);
    for (int i = threadIdx.x; i < H * H; i += NT) {
        const int r = i / H, c = i % H;
        s.w2[r * HP + c] = w[OW2 + i];
        if (transposed) s.w2t[c * HP + r] = w[OW2 + i];
    }
    for (int i = threadIdx.x; i < H; i += NT) {
        s.b1[i] = bf(w, OB1 + i);
        s.b2[i] = bf(w, OB2 + i);
        s.w3[i] = bf(w, OW3 + i);
    }
    if (threadIdx.x == 0) s.b3 = bf(w, OB3);
}

// Forward of one tile. Layer 1: thread j computes unit j for the 32 samples (h1 in FP32 and
// as BF16 [b][k] and [k][b]). Layer 2 on the tensor cores: warp w computes units 32w .. 32w
// + 31 for all samples, h2 = tanh(z2 + b2) into s.h2. Layer 3: each warp's part of
// sum_j w3_j h2_bj, added in warp order into s.y. n = valid samples of the tile.
__device__ void forward_tile(Smem& s, int n) {
    const int j = threadIdx.x, warp = j >> 5, lane = j & 31, g = lane >> 2, t = lane & 3;
    for (int b = 0; b < TB; ++b) {
        float z = s.b1[j];
#pragma unroll
        for (int k = 0; k < 4; ++k) z = fmaf(s.w1[j * 4 + k], s.x[b * 4 + k], z);
        const float h = b < n ? tanhf(z) : 0.f;
        const __nv_bfloat16 hb = __float2bfloat16_rn(h);
        s.h1f[b * H + j] = h;
        s.h1[b * HP + j] = hb;
        s.h1t[j * TBP + b] = hb;
    }
    __syncthreads();
    float yp[2][2] = {{0.f, 0.f}, {0.f, 0.f}};  // [m-tile][row g, g + 8]
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const int j0 = 32 * warp + 8 * nt;
            float d[4] = {0.f, 0.f, 0.f, 0.f};
            mma_block<8>(d, s.h1, HP, 16 * mt, s.w2, HP, j0, 0);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int b = 16 * mt + g + (e >> 1) * 8, jj = j0 + 2 * t + (e & 1);
                const float h2 = tanhf(d[e] + s.b2[jj]);
                s.h2[b * H + jj] = h2;
                yp[mt][e >> 1] = fmaf(s.w3[jj], h2, yp[mt][e >> 1]);
            }
        }
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            float v = yp[mt][r];
            v += __shfl_xor_sync(0xffffffffu, v, 1);
            v += __shfl_xor_sync(0xffffffffu, v, 2);
            if (t == 0) s.ypart[warp][16 * mt + g + 8 * r] = v;
        }
    __syncthreads();
    if (j < TB) {
        float y = s.b3;
        for (int w = 0; w < NT / 32; ++w) y += s.ypart[w][j];
        s.y[j] = y;
    }
    __syncthreads();
}

}  // namespace

__global__ void __launch_bounds__(NT) mlp_train_kernel(const __nv_bfloat16* __restrict__ w,
                                                       const float* __restrict__ X, const float* __restrict__ T,
                                                       int n, float inv_n, float* __restrict__ gpart,
                                                       double* __restrict__ lpart) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    load_weights(s, w, true);
    const int j = threadIdx.x, warp = j >> 5, lane = j & 31, g = lane >> 2, t = lane & 3;
    float gw1[4] = {0, 0, 0, 0}, gb1 = 0, gb2 = 0, gw3 = 0, gb3 = 0;
    float gw2[2][16][4];  // dW2 rows 32 warp + 16 mt + (g, g + 8), columns 8 nt + 2t (+1)
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 16; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) gw2[mt][nt][e] = 0.f;
    double l = 0.0;
    __syncthreads();
    const int ntiles = (n + TB - 1) / TB;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int b0 = tile * TB, nb = min(TB, n - b0);
        for (int i = threadIdx.x; i < TB * 4; i += NT) s.x[i] = (i / 4) < nb ? X[(size_t)b0 * 4 + i] : 0.f;
        if (j < TB) s.t[j] = j < nb ? T[b0 + j] : 0.f;
        __syncthreads();
        forward_tile(s, nb);
        if (j < TB) {  // d loss / d y for loss = mean (y - t)^2
            float d = j < nb ? s.y[j] - s.t[j] : 0.f;
            s.dy[j] = 2.f * d * inv_n;
            l += (double)d * d;
        }
        __syncthreads();
        // layer 3 and dz2 = dy * w3 * (1 - h2^2) (FP32 for b2, BF16 for the products)
        for (int b = 0; b < TB; ++b) {
            const float dy = s.dy[b], h2 = s.h2[b * H + j];
            gw3 = fmaf(dy, h2, gw3);
            const float dz = dy * s.w3[j] * (1.f - h2 * h2);
            gb2 += dz;
            const __nv_bfloat16 db = __float2bfloat16_rn(dz);
            s.dz2[b * HP + j] = db;
            s.dz2t[j * TBP + b] = db;
        }
        if (j == 0)
            for (int b = 0; b < TB; ++b) gb3 += s.dy[b];
        __syncthreads();
        // dW2[j][k] += sum_b dz2[b][j] h1[b][k]: warp w, rows j in [32 w, 32 w + 32)
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 16; ++nt) mma_block<2>(gw2[mt][nt], s.dz2t, TBP, 32 * warp + 16 * mt, s.h1t, TBP, 8 * nt, 0);
        // dh1[b][j] = sum_i dz2[b][i] W2[i][j]; dz1 = dh1 (1 - h1^2): warp w, columns j in [32 w, 32 w + 32)
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int j0 = 32 * warp + 8 * nt;
                float d[4] = {0.f, 0.f, 0.f, 0.f};
                mma_block<8>(d, s.dz2, HP, 16 * mt, s.w2t, HP, j0, 0);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int b = 16 * mt + g + (e >> 1) * 8, jj = j0 + 2 * t + (e & 1);
                    const float h = s.h1f[b * H + jj];
                    s.dz1[b * H + jj] = d[e] * (1.f - h * h);
                }
            }
        __syncthreads();
        for (int b = 0; b < TB; ++b) {
            const float d = s.dz1[b * H + j];
            gb1 += d;
#pragma unroll
            for (int k = 0; k < 4; ++k) gw1[k] = fmaf(d, s.x[b * 4 + k], gw1[k]);
        }
        __syncthreads();
    }
    // this CTA's partial gradient and loss into its own slot
    float* gp = gpart + (size_t)blockIdx.x * kMlpParams;
    for (int k = 0; k < 4; ++k) gp[OW1 + j * 4 + k] = gw1[k];
    gp[OB1 + j] = gb1;
    gp[OB2 + j] = gb2;
    gp[OW3 + j] = gw3;
    if (j == 0) gp[OB3] = gb3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 16; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int r = 32 * warp + 16 * mt + g + (e >> 1) * 8, c = 8 * nt + 2 * t + (e & 1);
                gp[OW2 + r * H + c] = gw2[mt][nt][e];
            }
    if (j < TB) {  // warp 0: the tile losses of threads 0 .. 31, summed in lane order
        double lt = l * inv_n;
        for (int o = 1; o < 32; o <<= 1) lt += __shfl_xor_sync(0xffffffffu, lt, o);
        if (j == 0) lpart[blockIdx.x] = lt;
    }
}

// grad[i] = sum over CTAs c (in order) of gpart[c][i]; *loss = sum of lpart in order.
__global__ void mlp_reduce_kernel(const float* __restrict__ gpart, const double* __restrict__ lpart, int nparts,
                                  float* __restrict__ grad, double* __restrict__ loss) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpParams; i += gridDim.x * blockDim.x) {
        float sum = 0.f;
        for (int c = 0; c < nparts; ++c) sum += gpart[(size_t)c * kMlpParams + i];
        grad[i] = sum;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double sum = 0.0;
        for (int c = 0; c < nparts; ++c) sum += lpart[c];
        *loss = sum;
    }
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
    load_weights(s, w, false);
    __syncthreads();
    const int ntiles = (n + TB - 1) / TB;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int b0 = tile * TB, nb = min(TB, n - b0);
        for (int i = threadIdx.x; i < TB * 4; i += NT) s.x[i] = (i / 4) < nb ? X[(size_t)b0 * 4 + i] : 0.f;
        __syncthreads();
        forward_tile(s, nb);
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
                                                        float y_std, double* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    __shared__ double red[NT / 32];
    load_weights(s, w, false);
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
        forward_tile(s, nb);
        if (threadIdx.x < nb) acc += exp((double)s.y[threadIdx.x] * y_std + y_mean);
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < NT / 32; ++k) t += red[k];
        part[blockIdx.x] = t;  // this (shell, chunk) part of the sum
    }
}

// gbar[s] = (sum of shell s's chunk parts, in chunk order) / P
__global__ void mlp_sphere_reduce_kernel(const double* __restrict__ part, int nshell, int chunks, int P,
                                         double* __restrict__ gbar) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nshell; s += gridDim.x * blockDim.x) {
        double t = 0.0;
        for (int c = 0; c < chunks; ++c) t += part[(size_t)s * chunks + c];
        gbar[s] = t / P;
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

size_t mlp_smem_bytes(bool) { return sizeof(Smem); }

size_t mlp_train_scratch_bytes(int sms) {
    return (size_t)std::max(sms, 1) * ((size_t)kMlpParams * sizeof(float) + sizeof(double));
}

cudaError_t launch_mlp_train(const __nv_bfloat16* w, const float* X, const float* T, int n, float* grad,
                             double* loss, void* scratch, int sms, cudaStream_t st) {
    const size_t sm = mlp_smem_bytes(true);
    cudaError_t e = cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const int tiles = (n + TB - 1) / TB;
    const int grid = max(1, min(tiles, max(sms, 1)));
    float* gpart = reinterpret_cast<float*>(scratch);
    double* lpart = reinterpret_cast<double*>(gpart + (size_t)max(sms, 1) * kMlpParams);
    mlp_train_kernel<<<grid, NT, sm, st>>>(w, X, T, n, 1.f / n, gpart, lpart);
    mlp_reduce_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(gpart, lpart, grid, grad, loss);
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

static int sphere_chunks(int nshell, int P, int sms) {
    return max(1, min((P + 1023) / 1024, (max(sms, 1) * 4 + nshell - 1) / nshell));
}

size_t mlp_sphere_scratch_bytes(int nshell, int P, int sms) {
    return (size_t)nshell * sphere_chunks(nshell, P, sms) * sizeof(double);
}

cudaError_t launch_mlp_sphere(const __nv_bfloat16* w, const double* qlen, int nshell, int P, float q_mid,
                              float q_half, float y_mean, float y_std, double* gbar, double* scratch, int sms,
                              cudaStream_t st) {
    const size_t sm = mlp_smem_bytes(false);
    cudaError_t e = cudaFuncSetAttribute(mlp_sphere_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const int chunks = sphere_chunks(nshell, P, sms);
    mlp_sphere_kernel<<<nshell * chunks, NT, sm, st>>>(w, qlen, nshell, P, chunks, q_mid, q_half, y_mean, y_std,
                                                       scratch);
    mlp_sphere_reduce_kernel<<<(nshell + 127) / 128, 128, 0, st>>>(scratch, nshell, chunks, P, gbar);
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
