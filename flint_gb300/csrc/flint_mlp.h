// flint_mlp.h -- the BF16 tensor-core GEMM and elementwise kernels of the
// surrogate MLP (flint_mlp.cu), shared with the surrogate driver.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

namespace flint {

enum { EPI_STORE = 0, EPI_BIAS = 1, EPI_BIAS_GELU = 2, EPI_GELU_BWD = 3 };

struct GemmArgs {
  int M, N, K;
  const void* A; int a_bf16; int64_t sa_m, sa_k;
  const void* B; int b_bf16; int64_t sb_k, sb_n;
  const float* bias;                 // [N]
  float* C; int64_t ldc;             // FP32 output (pre-activation or result)
  __nv_bfloat16* Cb; int64_t ldcb;   // optional BF16 activation output
  float* Cf; int64_t ldcf;           // optional FP32 activation output (GELU applied for EPI_BIAS_GELU)
  const float* Zprev; int64_t ldz;   // GELU_BWD: pre-activation of the previous layer
  int epi;
  int accumulate;                    // C += result
  int split;                         // operands as BF16 hi + lo pairs, three MMAs per fragment
};

cudaError_t launch_gemm(const GemmArgs& g, cudaStream_t st);
cudaError_t launch_colsum(const float* dZ, int M, int N, int64_t ld, float* db, int acc, cudaStream_t st);
cudaError_t launch_mse(const float* yhat, const float* y, int64_t total, float scale, float* grad, double* loss,
                       cudaStream_t st);
cudaError_t launch_adam(float* w, const float* gw, float* m1, float* m2, __nv_bfloat16* wb, int64_t n, float lr,
                        float b1, float b2, float eps, float bc1, float bc2, float wd, cudaStream_t st);
cudaError_t launch_to_bf16(const float* x, __nv_bfloat16* y, int64_t n, cudaStream_t st);

}  // namespace flint
