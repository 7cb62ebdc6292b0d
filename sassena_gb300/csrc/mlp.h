// Launch interface of the control-variate MLP kernels (internal).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>

namespace sassgpu {

constexpr int kMlpHidden = 128;
// W1 [128][4], b1 [128], W2 [128][128], b2 [128], W3 [128], b3
constexpr int kMlpParams = 128 * 4 + 128 + 128 * 128 + 128 + 128 + 1;

size_t mlp_smem_bytes(bool train);
// Writes d(mean (y - t)^2)/d params to grad and the loss to *loss, summed over the CTAs in
// a fixed order (the same bits on every run). scratch: mlp_train_scratch_bytes(sms) bytes.
size_t mlp_train_scratch_bytes(int sms);
cudaError_t launch_mlp_train(const __nv_bfloat16* w, const float* X, const float* T, int n, float* grad,
                             double* loss, void* scratch, int sms, cudaStream_t st);
cudaError_t launch_mlp_adam(float* master, __nv_bfloat16* w, const float* grad, float* m, float* v, float lr,
                            int step, cudaStream_t st);
cudaError_t launch_mlp_forward(const __nv_bfloat16* w, const float* X, int n, float* Y, int sms, cudaStream_t st);
// gbar[s]: mean of g over P spherical-Fibonacci points of shell s, parts summed in a fixed
// order. scratch: mlp_sphere_scratch_bytes(nshell, P, sms) bytes.
size_t mlp_sphere_scratch_bytes(int nshell, int P, int sms);
cudaError_t launch_mlp_sphere(const __nv_bfloat16* w, const double* qlen, int nshell, int P, float q_mid,
                              float q_half, float y_mean, float y_std, double* gbar, double* scratch, int sms,
                              cudaStream_t st);
// A_v(t) *= wsqrt[v] for float2 (f32) or double2 amplitudes [nv][nf].
cudaError_t launch_scale_series(void* A, bool f32, const double* wsqrt, size_t nv, int nf, cudaStream_t st);

}  // namespace sassgpu
