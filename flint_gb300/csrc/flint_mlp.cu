// flint_mlp.cu -- BF16 tensor-core MLP kernels of the learned reactor surrogate.
//
// The surrogate is a multilayer perceptron (33 -> 256 -> 256 -> 256 -> 256 -> 32,
// GELU) with BF16 weights and activations as MMA operands and FP32
// accumulation.  One generic tiled GEMM serves the forward layers and both
// backward products:
//
//   C[m][n] = sum_k A(m,k) * B(k,n)      A, B read through strides (FP32 or BF16),
//                                        staged as BF16 tiles in shared memory,
//                                        multiplied by mma.sync.m16n8k16 (BF16 in,
//                                        FP32 accumulate),
//   epilogues: +bias and GELU (writes FP32 pre-activation and BF16 activation),
//              +bias, plain FP32, or (for back-propagation) C * GELU'(Z).
//
// Elementwise kernels: MSE loss and its gradient, bias gradients (column sums),
// Adam on FP32 master weights with BF16 shadow copies.
//
// Tiles: 64 x 64 per block, 4 warps of 32 x 32, K staged 32 at a time with rows
// padded to 40 BF16 (80 bytes) so the fragment loads are bank-conflict free.
//
// Split mode (the forward pass): every operand x is staged as the BF16 pair
// hi = bf16(x), lo = bf16(x - hi), and each fragment product is accumulated as
// lo*hi + hi*lo + hi*hi in FP32.  A single BF16 operand carries 8 significant
// bits; the pair carries about 16, which moves the network's rounding floor
// from ~1e-3 to ~1e-5 of its output scale at three times the MMA work (the
// lo*lo term is below the FP32 accumulation error and is skipped).
#include <cstdint>
#include <algorithm>
#include <cuda_bf16.h>
#include "flint_host.h"
#include "flint_mlp.h"

namespace flint {

constexpr int GBM = 64, GBN = 64, GBK = 32, GKP = 40, GTHREADS = 128;

__device__ __forceinline__ float gelu_f(float x) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  return 0.5f * x * (1.0f + tanhf(k0 * (x + k1 * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float u = k0 * (x + k1 * x * x * x);
  const float t = tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * k0 * (1.0f + 3.0f * k1 * x * x);
}

__device__ __forceinline__ float ld_any(const void* p, int bf16, int64_t idx) {
  return bf16 ? __bfloat162float(static_cast<const __nv_bfloat16*>(p)[idx]) : static_cast<const float*>(p)[idx];
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool SPLIT>
__global__ void __launch_bounds__(GTHREADS) k_gemm_bf16(GemmArgs g) {
  constexpr int NP = SPLIT ? 2 : 1;   // hi (and lo) planes
  __shared__ __align__(16) __nv_bfloat16 sA[NP][GBM][GKP];
  __shared__ __align__(16) __nv_bfloat16 sB[NP][GBN][GKP];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const int grp = lane >> 2, tig = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[i][j][c] = 0.f;

  for (int k0 = 0; k0 < g.K; k0 += GBK) {
    // stage A tile (GBM x GBK) and B tile (GBN x GBK, n-major) as BF16
    for (int e = tid; e < GBM * GBK; e += GTHREADS) {
      const int r = e / GBK, c = e % GBK;
      const int m = m0 + r, k = k0 + c;
      float v = 0.f;
      if (m < g.M && k < g.K) v = ld_any(g.A, g.a_bf16, (int64_t)m * g.sa_m + (int64_t)k * g.sa_k);
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      sA[0][r][c] = hi;
      if (SPLIT) sA[NP - 1][r][c] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
    for (int e = tid; e < GBN * GBK; e += GTHREADS) {
      const int r = e / GBK, c = e % GBK;
      const int n = n0 + r, k = k0 + c;
      float v = 0.f;
      if (n < g.N && k < g.K) v = ld_any(g.B, g.b_bf16, (int64_t)k * g.sb_k + (int64_t)n * g.sb_n);
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      sB[0][r][c] = hi;
      if (SPLIT) sB[NP - 1][r][c] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; kk += 16) {
      uint32_t af[NP][2][4], bfr[NP][4][2];
#pragma unroll
      for (int pl = 0; pl < NP; ++pl) {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const int r = wm + i * 16 + grp;
          af[pl][i][0] = *reinterpret_cast<const uint32_t*>(&sA[pl][r][kk + tig * 2]);
          af[pl][i][1] = *reinterpret_cast<const uint32_t*>(&sA[pl][r + 8][kk + tig * 2]);
          af[pl][i][2] = *reinterpret_cast<const uint32_t*>(&sA[pl][r][kk + tig * 2 + 8]);
          af[pl][i][3] = *reinterpret_cast<const uint32_t*>(&sA[pl][r + 8][kk + tig * 2 + 8]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int n = wn + j * 8 + grp;
          bfr[pl][j][0] = *reinterpret_cast<const uint32_t*>(&sB[pl][n][kk + tig * 2]);
          bfr[pl][j][1] = *reinterpret_cast<const uint32_t*>(&sB[pl][n][kk + tig * 2 + 8]);
        }
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (SPLIT) {
            mma_bf16(acc[i][j], af[NP - 1][i], bfr[0][j]);
            mma_bf16(acc[i][j], af[0][i], bfr[NP - 1][j]);
          }
          mma_bf16(acc[i][j], af[0][i], bfr[0][j]);
        }
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int m = m0 + wm + i * 16 + grp + (c >= 2 ? 8 : 0);
        const int n = n0 + wn + j * 8 + tig * 2 + (c & 1);
        if (m >= g.M || n >= g.N) continue;
        float v = acc[i][j][c];
        if (g.epi == EPI_BIAS || g.epi == EPI_BIAS_GELU) v += g.bias[n];
        if (g.epi == EPI_GELU_BWD) v *= gelu_grad(g.Zprev[(int64_t)m * g.ldz + n]);
        if (g.C) {
          float* cp = g.C + (int64_t)m * g.ldc + n;
          *cp = g.accumulate ? *cp + v : v;
        }
        if (g.Cb || g.Cf) {
          const float a = g.epi == EPI_BIAS_GELU ? gelu_f(v) : v;
          if (g.Cb) g.Cb[(int64_t)m * g.ldcb + n] = __float2bfloat16_rn(a);
          if (g.Cf) g.Cf[(int64_t)m * g.ldcf + n] = a;
        }
      }
}

// Column sums: db[n] (+)= sum_m dZ[m][n].
__global__ void k_colsum(const float* __restrict__ dZ, int M, int N, int64_t ld, float* __restrict__ db, int accumulate) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += dZ[(int64_t)m * ld + n];
  db[n] = accumulate ? db[n] + s : s;
}

// MSE over an (M x N) output: grad = 2 (yhat - y) / (M N); loss partial sums per block.
__global__ void k_mse(const float* __restrict__ yhat, const float* __restrict__ y, int64_t total, float scale,
                      float* __restrict__ grad, double* __restrict__ loss_acc) {
  double part = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = yhat[i] - y[i];
    grad[i] = 2.f * d * scale;
    part += (double)d * d;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss_acc, part * scale);
}

// Adam on FP32 master weights; writes the BF16 shadow used as MMA operand.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ gw, float* __restrict__ m1,
                       float* __restrict__ m2, __nv_bfloat16* __restrict__ wb, int64_t n, float lr, float b1, float b2,
                       float eps, float bc1, float bc2, float wd) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float g = gw[i] + wd * w[i];
    const float a = b1 * m1[i] + (1.f - b1) * g;
    const float b = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = a;
    m2[i] = b;
    const float upd = lr * (a / bc1) / (sqrtf(b / bc2) + eps);
    const float nw = w[i] - upd;
    w[i] = nw;
    if (wb) wb[i] = __float2bfloat16_rn(nw);
  }
}

__global__ void k_f32_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

cudaError_t launch_gemm(const GemmArgs& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return cudaSuccess;
  dim3 grid((g.N + GBN - 1) / GBN, (g.M + GBM - 1) / GBM);
  if (g.split) k_gemm_bf16<true><<<grid, GTHREADS, 0, st>>>(g);
  else k_gemm_bf16<false><<<grid, GTHREADS, 0, st>>>(g);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_colsum(const float* dZ, int M, int N, int64_t ld, float* db, int acc, cudaStream_t st) {
  k_colsum<<<(N + 127) / 128, 128, 0, st>>>(dZ, M, N, ld, db, acc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_mse(const float* yhat, const float* y, int64_t total, float scale, float* grad, double* loss,
                       cudaStream_t st) {
  int blocks = (int)std::min<int64_t>((total + 255) / 256, 4 * device_sms());
  k_mse<<<blocks, 256, 0, st>>>(yhat, y, total, scale, grad, loss);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_adam(float* w, const float* gw, float* m1, float* m2, __nv_bfloat16* wb, int64_t n, float lr,
                        float b1, float b2, float eps, float bc1, float bc2, float wd, cudaStream_t st) {
  int blocks = (int)std::min<int64_t>((n + 255) / 256, 4 * device_sms());
  k_adam<<<blocks, 256, 0, st>>>(w, gw, m1, m2, wb, n, lr, b1, b2, eps, bc1, bc2, wd);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float* x, __nv_bfloat16* y, int64_t n, cudaStream_t st) {
  int blocks = (int)std::min<int64_t>((n + 255) / 256, 4 * device_sms());
  k_f32_to_bf16<<<blocks, 256, 0, st>>>(x, y, n);
  count_launch();
  return cudaGetLastError();
}

}  // namespace flint
