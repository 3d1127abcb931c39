// flint_umma.cu -- the surrogate MLP's inference forward as one fused
// Blackwell kernel: tcgen05 MMAs with the accumulator in tensor memory (TMEM).
//
// One CTA (8 warps) per SM walks tiles of 128 cells.  Per tile the five layers
// run back to back without leaving the SM: the layer input A (128 x K, BF16
// hi and lo planes, 128 KB) stays in shared memory, the weights stream from
// the L2-resident packed copy (BF16 hi and lo, 1.7 MB for two networks) in
// K-chunks of 32 through a two-stage shared-memory ring filled by
// cp.async.bulk, and one thread issues tcgen05.mma (M = 128, N = 256 or the
// padded output width, K = 16) into a 128 x 256 FP32 accumulator in TMEM.
// Each product is split as in the mma.sync path: a = a_hi + a_lo, w = w_hi +
// w_lo (BF16 each) and a*w ~ a_hi*w_hi + a_hi*w_lo + a_lo*w_hi, three MMAs
// accumulating in FP32 (about 16 significant bits per operand instead of 8).
// After a layer's MMAs complete (tcgen05.commit -> mbarrier), the 8 warps
// read the accumulator (tcgen05.ld, warp w: TMEM lanes 32 (w % 4) .. + 31,
// half w / 4 of the columns), add the bias, apply GELU, split into BF16 and
// overwrite A for the next layer; the last layer adds the bias and writes
// FP32 rows to global memory.
//
// Operand layout in shared memory (no swizzle, K-major): 8 x 8 BF16 "core
// matrices" of 128 contiguous bytes (row r at 16 r); core matrix (row group g,
// K group j) of A at (g * 32 + j) * 128 (K = 256 columns), of a weight chunk at
// (g * 4 + j) * 128 (K = 32).  The matrix descriptors give the K-direction
// core stride (leading byte offset, 128) and the row-group stride (stride byte
// offset: 4096 for A, 512 for a chunk).
//
// Every wait on an mbarrier is bounded: on a timeout the CTA records an error
// word, stops issuing work, waits (bounded) for what it has in flight, frees
// its TMEM and returns; flint_surrogate_check reports the word.
#include <cstdint>
#include <cuda_bf16.h>

#include "flint_host.h"
#include "flint_umma.h"

namespace flint {

constexpr int UM = 128;                 // cells per tile (MMA M, TMEM lanes)
constexpr int UH = 256;                 // hidden width (TMEM columns)
constexpr int UKC = 32;                 // K per weight chunk
constexpr int UTHREADS = 256;
constexpr int A_PLANE = UM * UH * 2;    // bytes per BF16 plane of A
constexpr int B_STAGE = 2 * UH * UKC * 2;   // bytes per stage (hi + lo planes, N <= 256)
constexpr int UMMA_SMEM = 2 * A_PLANE + 2 * B_STAGE + 128;
constexpr long long WAIT_LIMIT = 1ll << 26;   // polls of an mbarrier before giving up (~seconds)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// blocked K-major offset of element (row, k) in a plane whose rows hold kw
// K-elements (kw a multiple of 8)
__host__ __device__ __forceinline__ uint32_t core_off(int row, int k, int kw) {
  return (uint32_t)((((row >> 3) * (kw >> 3) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

// shared-memory matrix descriptor: start address, leading (K-direction) and
// stride (row-group) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both
// K-major, N and M as given
__host__ __device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// true when the phase with this parity completed; false after WAIT_LIMIT polls
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu_u(float x) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  return 0.5f * x * (1.0f + tanhf(k0 * (x + k1 * x * x * x)));
}

// 8 consecutive values -> one 16-byte store of BF16 hi and one of BF16 lo
__device__ __forceinline__ void store_split8(uint8_t* hi, uint8_t* lo, const float* v) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __nv_bfloat16 a = __float2bfloat16_rn(v[2 * i]), b = __float2bfloat16_rn(v[2 * i + 1]);
    const __nv_bfloat16 c = __float2bfloat16_rn(v[2 * i] - __bfloat162float(a));
    const __nv_bfloat16 d = __float2bfloat16_rn(v[2 * i + 1] - __bfloat162float(b));
    h[i] = (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
    l[i] = (uint32_t)__bfloat16_as_ushort(c) | ((uint32_t)__bfloat16_as_ushort(d) << 16);
  }
  *reinterpret_cast<uint4*>(hi) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4*>(lo) = make_uint4(l[0], l[1], l[2], l[3]);
}

// ---------------------------------------------------------------- weights
// FP32 W[l][n][k] (row-major, the network's own storage) -> per layer and
// K-chunk the blocked hi plane then the lo plane, zero-padded to (N', K');
// biases zero-padded to 256 per layer.
__global__ void k_umma_pack(UmmaNet u, const float* __restrict__ w, const int64_t* __restrict__ off_w,
                            const int64_t* __restrict__ off_b, uint8_t* __restrict__ packed,
                            float* __restrict__ bias) {
  for (int l = 0; l < u.nl; ++l) {
    const int N = u.N[l], K = u.K[l], Np = u.Np[l], Kp = u.Kp[l];
    const int64_t total = (int64_t)Np * Kp;
    const int64_t chunk = 2ll * Np * UKC * 2;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
      const int n = (int)(e / Kp), k = (int)(e % Kp);
      const float v = (n < N && k < K) ? w[off_w[l] + (int64_t)n * K + k] : 0.f;
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(h));
      uint8_t* base = packed + u.off[l] + (int64_t)(k / UKC) * chunk;
      const uint32_t o = core_off(n, k % UKC, UKC);
      *reinterpret_cast<__nv_bfloat16*>(base + o) = h;
      *reinterpret_cast<__nv_bfloat16*>(base + (int64_t)Np * UKC * 2 + o) = lo;
    }
    for (int n = (int)(blockIdx.x * blockDim.x + threadIdx.x); n < UH; n += gridDim.x * blockDim.x)
      bias[l * UH + n] = n < N ? w[off_b[l] + n] : 0.f;
  }
}

// ---------------------------------------------------------------- forward
__global__ void __launch_bounds__(UTHREADS, 1)
k_mlp_umma(UmmaNet u, const uint8_t* __restrict__ packed, const float* __restrict__ bias, int64_t n,
           const float* __restrict__ X, float* __restrict__ out, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t* A_hi = sm;
  uint8_t* A_lo = sm + A_PLANE;
  uint8_t* Bst = sm + 2 * A_PLANE;                                  // 2 stages
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 2 * A_PLANE + 2 * B_STAGE);   // full[2], empty[2], done
  volatile uint32_t* tslot = reinterpret_cast<volatile uint32_t*>(bars + 5);
  volatile int* abort_f = reinterpret_cast<volatile int*>(bars + 6);
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[2]), done = smem_u32(&bars[4]);

  if (tid == 0) {
    mbar_init(full0, 1); mbar_init(full0 + 8, 1);
    mbar_init(empty0, 1); mbar_init(empty0 + 8, 1);
    mbar_init(done, 1);
    *abort_f = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32((const void*)tslot)),
                 "r"(UH));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  // barrier phases (every commit / expect_tx is matched by one wait)
  uint32_t ph_full[2] = {0, 0}, ph_empty[2] = {0, 0}, ph_done = 0;
  int pend_full[2] = {0, 0};   // a copy into the stage was issued and not yet waited for
  const int q = warp & 3, half = warp >> 2;
  const int row = q * 32 + (tid & 31);   // the TMEM lane / tile row this thread reads

  const int64_t ntiles = (n + UM - 1) / UM;
  for (int64_t tile = blockIdx.x; tile < ntiles && !*abort_f; tile += gridDim.x) {
    // ---- layer 0 input: the features of 128 cells, split into hi / lo
    {
      const int r = tid & (UM - 1), h2 = tid >> 7;
      const int64_t cell = tile * UM + r;
      const int kw = u.Kp[0] / 2;
      for (int k0 = h2 * kw; k0 < (h2 + 1) * kw; k0 += 8) {
        float v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int k = k0 + i;
          v[i] = (cell < n && k < u.N_in) ? X[cell * u.N_in + k] : 0.f;
        }
        store_split8(A_hi + core_off(r, k0, UH), A_lo + core_off(r, k0, UH), v);
      }
      proxy_fence();
    }
    __syncthreads();
    for (int l = 0; l < u.nl && !*abort_f; ++l) {
      const int Np = u.Np[l], nch = u.Kp[l] / UKC;
      const uint32_t cbytes = (uint32_t)(2 * Np * UKC * 2);
      const uint8_t* wl = packed + u.off[l];
      const uint32_t idesc = idesc_bf16(UM, Np);
      // ---- one thread: stream the weight chunks and issue the MMAs
      if (tid == 0) {
        tc_fence_after();
        bool ok = true;
        for (int c = 0; c < 2 && c < nch; ++c) {
          mbar_expect_tx(full0 + 8 * c, cbytes);
          bulk_g2s(smem_u32(Bst + c * B_STAGE), wl + (int64_t)c * cbytes, cbytes, full0 + 8 * c);
          pend_full[c] = 1;
        }
        for (int c = 0; c < nch && ok; ++c) {
          const int s = c & 1;
          ok = mbar_wait(full0 + 8 * s, ph_full[s]);
          ph_full[s] ^= 1;
          if (!ok) break;
          pend_full[s] = 0;
          const uint32_t bh = smem_u32(Bst + s * B_STAGE), bl = bh + (uint32_t)(Np * UKC * 2);
#pragma unroll
          for (int j = 0; j < UKC / 16; ++j) {
            const int kg = c * (UKC / 8) + 2 * j;   // K core-matrix index of this K = 16 step in A
            const uint64_t ah = smem_desc(smem_u32(A_hi) + kg * 128, 128, 4096);
            const uint64_t al = smem_desc(smem_u32(A_lo) + kg * 128, 128, 4096);
            const uint64_t wh = smem_desc(bh + 2 * j * 128, 128, 512);
            const uint64_t wlo = smem_desc(bl + 2 * j * 128, 128, 512);
            umma_f16(tmem, ah, wh, idesc, (c | j) ? 1u : 0u);
            umma_f16(tmem, ah, wlo, idesc, 1u);
            umma_f16(tmem, al, wh, idesc, 1u);
          }
          umma_commit(empty0 + 8 * s);
          if (c >= 1 && c + 1 < nch) {   // refill the stage chunk c - 1 used with chunk c + 1
            const int s2 = (c + 1) & 1;
            ok = mbar_wait(empty0 + 8 * s2, ph_empty[s2]);
            ph_empty[s2] ^= 1;
            if (!ok) break;
            mbar_expect_tx(full0 + 8 * s2, cbytes);
            bulk_g2s(smem_u32(Bst + s2 * B_STAGE), wl + (int64_t)(c + 1) * cbytes, cbytes, full0 + 8 * s2);
            pend_full[s2] = 1;
          }
        }
        if (ok) umma_commit(done);
        // the stages of the last two chunks: their MMAs end with the layer
        for (int c = (nch >= 2 ? nch - 2 : 0); c < nch && ok; ++c) {
          const int s = c & 1;
          ok = mbar_wait(empty0 + 8 * s, ph_empty[s]);
          ph_empty[s] ^= 1;
        }
        if (!ok) {
          // stop: wait (bounded) for the copies still in flight and for every
          // MMA issued so far, so nothing writes this CTA's memory after it ends
          for (int s = 0; s < 2; ++s)
            if (pend_full[s]) (void)mbar_wait(full0 + 8 * s, ph_full[s]);
          umma_commit(done);
          (void)mbar_wait(done, ph_done);
          *abort_f = 1;
          atomicExch(err, 1);
        }
      }
      __syncthreads();
      if (*abort_f) break;
      // ---- all threads: wait for the accumulator (lane 0 of each warp polls,
      // so the warp stays converged for tcgen05.ld), then the epilogue
      int okd = 1;
      if ((tid & 31) == 0) okd = mbar_wait(done, ph_done) ? 1 : 0;
      okd = __shfl_sync(0xffffffffu, okd, 0);
      ph_done ^= 1;
      if (!okd) { *abort_f = 1; atomicExch(err, 2); }
      tc_fence_after();
      const int cols = Np / 2, c0 = half * cols;
      const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16);
      const int64_t cell = tile * UM + row;
      if (okd) {
        for (int cc = 0; cc < cols; cc += 16) {
          float v[16];
          tmem_ld16(tl + (uint32_t)(c0 + cc), v);
#pragma unroll
          for (int i = 0; i < 16; ++i) v[i] += bias[l * UH + c0 + cc + i];
          if (l < u.nl - 1) {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = gelu_u(v[i]);
            store_split8(A_hi + core_off(row, c0 + cc, UH), A_lo + core_off(row, c0 + cc, UH), v);
            store_split8(A_hi + core_off(row, c0 + cc + 8, UH), A_lo + core_off(row, c0 + cc + 8, UH), v + 8);
          } else if (cell < n) {
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (c0 + cc + i < u.N_out) out[cell * u.N_out + c0 + cc + i] = v[i];
          }
        }
      }
      proxy_fence();
      tc_fence_before();
      __syncthreads();
    }
  }
  // leave: nothing of this CTA in flight (every commit was waited), free TMEM
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UH));
}

// ---------------------------------------------------------------- host
bool umma_fits(int nl, const int* dims) {
  if (nl < 2 || nl > UMMA_MAXL) return false;
  if (dims[0] < 1 || dims[0] > 64 || dims[nl] < 1 || dims[nl] > 64) return false;
  for (int l = 1; l < nl; ++l)
    if (dims[l] != UH) return false;
  return true;
}

size_t umma_smem_bytes() { return UMMA_SMEM; }

static int rup(int x, int m) { return (x + m - 1) / m * m; }

int64_t umma_describe(int nl, const int* dims, UmmaNet* u) {
  u->nl = nl;
  u->N_in = dims[0];
  u->N_out = dims[nl];
  int64_t off = 0;
  for (int l = 0; l < nl; ++l) {
    u->K[l] = dims[l];
    u->N[l] = dims[l + 1];
    u->Kp[l] = l == 0 ? rup(dims[0], 2 * UKC) : rup(dims[l], UKC);   // layer 0: two halves of whole chunks
    u->Np[l] = dims[l + 1] <= 32 ? 32 : (dims[l + 1] <= 64 ? 64 : UH);
    u->off[l] = off;
    off += (int64_t)(u->Kp[l] / UKC) * 2 * u->Np[l] * UKC * 2;
  }
  return off;
}

cudaError_t umma_pack(const UmmaNet& u, const float* w, const int64_t* off_w_dev, const int64_t* off_b_dev,
                      uint8_t* packed, float* bias, cudaStream_t st) {
  k_umma_pack<<<device_sms() * 4, 256, 0, st>>>(u, w, off_w_dev, off_b_dev, packed, bias);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_mlp_umma(const UmmaNet& u, const uint8_t* packed, const float* bias, int64_t n, const float* X,
                            float* out, int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = set_smem((const void*)k_mlp_umma, UMMA_SMEM);
  if (e != cudaSuccess) return e;
  const int64_t tiles = (n + UM - 1) / UM;
  const int64_t grid = tiles < device_sms() ? tiles : device_sms();
  k_mlp_umma<<<(unsigned)grid, UTHREADS, UMMA_SMEM, st>>>(u, packed, bias, n, X, out, err);
  count_launch();
  return cudaGetLastError();
}

}  // namespace flint
