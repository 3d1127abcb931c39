// flint_umma.h -- the fused tcgen05 inference forward of the surrogate MLP
// (flint_umma.cu), used by the surrogate driver.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace flint {

constexpr int UMMA_MAXL = 8;

// One network as the fused kernel sees it: per layer the true (K, N), the
// padded (Kp, Np) of the packed weights and the byte offset of the layer's
// chunks in the packed buffer.
struct UmmaNet {
  int nl, N_in, N_out;
  int K[UMMA_MAXL], N[UMMA_MAXL], Kp[UMMA_MAXL], Np[UMMA_MAXL];
  int64_t off[UMMA_MAXL];
};

// dims[0..nl]: input, hidden (all 256), output widths; the fused kernel takes
// inputs and outputs of up to 64 and hidden layers of exactly 256.
bool umma_fits(int nl, const int* dims);
// fills *u, returns the bytes of the packed weights
int64_t umma_describe(int nl, const int* dims, UmmaNet* u);
size_t umma_smem_bytes();
// FP32 weights (the network's storage; off_w/off_b device arrays of per-layer
// offsets) -> packed BF16 hi/lo chunks and zero-padded biases [nl][256]
cudaError_t umma_pack(const UmmaNet& u, const float* w, const int64_t* off_w_dev, const int64_t* off_b_dev,
                      uint8_t* packed, float* bias, cudaStream_t st);
// out[n][N_out] = network(X[n][N_in]); err: device word set non-zero if a wait timed out
cudaError_t launch_mlp_umma(const UmmaNet& u, const uint8_t* packed, const float* bias, int64_t n, const float* X,
                            float* out, int* err, cudaStream_t st);

}  // namespace flint
