// Pipe-throughput microbenchmarks for the roofline of the phase sum.
//
// The FP32 phase sum is bounded by the special-function unit (one sin and one cos
// per atom.q.frame term) or, if the SFU is not the limit, by FP32 issue. Neither
// rate is in the measured peaks (those cover HBM copy and bf16 GEMM), so the
// library measures them on the device it runs on:
//   * SFU: independent chains of __sinf/__cosf (sin.approx / cos.approx);
//   * FP32: independent chains of fmaf;
//   * FP64: independent chains of fma (the FP64 forms and the multipole devices).
// Each kernel runs a fixed number of dependent iterations on 8 independent chains per
// thread over a grid that fills every SM; rates are results / elapsed device time.
#include <cuda_runtime.h>

#include "../../include/sassena_gb300.h"

namespace {

__global__ void __launch_bounds__(256) sfu_chains(float* out, int iters, float seed) {
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = seed + 0.001f * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float s, c;
            __sincosf(x[k], &s, &c);
            x[k] = s + c;  // stays in [-sqrt2, sqrt2]
        }
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) acc += x[k];
    if (acc == 12345.678f) out[blockIdx.x] = acc;  // keep the work observable
}

__global__ void __launch_bounds__(256) fma_chains(float* out, int iters, float seed) {
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = seed + 0.001f * (threadIdx.x + k);
    const float a = 0.999999f, b = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) acc += x[k];
    if (acc == 12345.678f) out[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(256) dfma_chains(float* out, int iters, float seed) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = seed + 0.001 * (threadIdx.x + k);
    const double a = 0.9999999999, b = 1e-12;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) acc += x[k];
    if (acc == 12345.678) out[blockIdx.x] = (float)acc;
}

template <class K>
double time_kernel(K k, int blocks, int iters, float* out, cudaStream_t st) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k<<<blocks, 256, 0, st>>>(out, iters / 8, 0.5f);  // warm-up
    cudaEventRecord(a, st);
    k<<<blocks, 256, 0, st>>>(out, iters, 0.5f);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms * 1e-3;
}

}  // namespace

extern "C" int sass_probe_pipes(int device, double* sfu_ops_per_s, double* fp32_fma_per_s) {
    if (!sfu_ops_per_s || !fp32_fma_per_s) return SASS_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SASS_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8;
    float* out = nullptr;
    if (cudaMalloc(&out, blocks * sizeof(float)) != cudaSuccess) return SASS_ERR_OOM;
    cudaStream_t st;
    cudaStreamCreate(&st);
    const int iters = 4096;
    double t_sfu = time_kernel(sfu_chains, blocks, iters, out, st);
    double t_fma = time_kernel(fma_chains, blocks, iters * 4, out, st);
    const double threads = (double)blocks * 256;
    *sfu_ops_per_s = threads * 8.0 * iters * 2.0 / t_sfu;       // sin + cos per chain step
    *fp32_fma_per_s = threads * 8.0 * (iters * 4.0) / t_fma;    // one FMA per chain step
    cudaStreamDestroy(st);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? SASS_OK : SASS_ERR_CUDA;
}

extern "C" int sass_probe_fp64(int device, double* fp64_fma_per_s) {
    if (!fp64_fma_per_s) return SASS_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SASS_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8;
    float* out = nullptr;
    if (cudaMalloc(&out, blocks * sizeof(float)) != cudaSuccess) return SASS_ERR_OOM;
    cudaStream_t st;
    cudaStreamCreate(&st);
    const int iters = 1024;
    double t = time_kernel(dfma_chains, blocks, iters, out, st);
    *fp64_fma_per_s = (double)blocks * 256 * 8.0 * iters / t;  // one FMA per chain step
    cudaStreamDestroy(st);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? SASS_OK : SASS_ERR_CUDA;
}
