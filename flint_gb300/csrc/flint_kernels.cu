// flint_kernels.cu -- batched source-term, Jacobian and thermo kernels.
//
//  k_wdot_small   one thread per cell, for small mechanisms (ns <= 16): the
//                 2-step CH4/air case.  Mechanism staged in shared memory;
//                 every thread reads the same reaction word at the same time
//                 (broadcast), per-thread species arrays live in shared memory
//                 as [species][thread] (conflict-free).
//  k_wdot_warp    one warp per cell (ns <= 63, species k on lane k % 32): reaction-parallel rates of
//                 progress, species-parallel sums; optional analytic Jacobian
//                 written coalesced (lane = row, one column per store).
//  k_rhs_warp     constant-pressure reactor right-hand side.
//
// All kernels are grid-stride loops over cells sized to whole waves of the 152
// SMs, so any N (including 0 and ragged tails) is handled without a tail kernel.
#include <algorithm>
#include <atomic>
#include "flint_dev.cuh"
#include "flint_host.h"

namespace flint {

constexpr int SMALL_NSMAX = 16;
constexpr int SMALL_THREADS = 128;
constexpr int WARP_THREADS = 256;

// ---------------------------------------------------------------- small
__global__ void __launch_bounds__(SMALL_THREADS)
k_wdot_small(const uint8_t* __restrict__ img, ImageLayout L, int64_t n, int layout,
             const double* __restrict__ Tg, const double* __restrict__ pg,
             const double* __restrict__ Yg, double* __restrict__ wdot,
             double* __restrict__ cpo, double* __restrict__ ho, int roi_mode, double* roi_io) {
  extern __shared__ __align__(16) uint8_t smem[];
  stage_image(smem, img, L.bytes);
  MechView m;
  m.bind(L, smem);
  const int ns = m.ns, P = m.nrpad;
  double* cs = reinterpret_cast<double*>(smem + L.bytes);      // [NSMAX][threads]
  double* gs = cs + SMALL_NSMAX * SMALL_THREADS;
  double* ws = gs + SMALL_NSMAX * SMALL_THREADS;
  const int t = threadIdx.x;
#define CS(k) cs[(k) * SMALL_THREADS + t]
#define GS(k) gs[(k) * SMALL_THREADS + t]
#define WS(k) ws[(k) * SMALL_THREADS + t]
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + t; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double T = Tg[i];
    const double lnT = flog(T, m.logtab), invT = 1.0 / T;
    double rho;
    double cpm = 0.0, hm = 0.0, ctot = 0.0;
    if (roi_mode) {
      // chemistry_source(roi, T, omegadot): c = max(roi,0)/W (WD.f90:18-21)
      rho = 0.0;
      for (int k = 0; k < ns; ++k) {
        double r = roi_io[i * ns + k];
        r = r > 0.0 ? r : 0.0;
        roi_io[i * ns + k] = r;
        CS(k) = r * m.invmw[k];
        ctot += CS(k);
      }
    } else {
      double sumYW = 0.0;
      for (int k = 0; k < ns; ++k) {
        double y = (layout == 1) ? Yg[(int64_t)k * n + i] : Yg[i * ns + k];
        CS(k) = y;
        sumYW += y * m.invmw[k];
      }
      rho = pg[i] / (m.r_eos * T * sumYW);
      for (int k = 0; k < ns; ++k) {
        double y = CS(k);
        SpThermo th = nasa7(m, k, T, lnT, invT);
        cpm += y * th.cpR * m.invmw[k];
        hm += y * th.hRT * m.invmw[k];
        CS(k) = rho * y * m.invmw[k];
        ctot += CS(k);
        GS(k) = th.hRT - th.sR;
      }
    }
    if (roi_mode) {
      for (int k = 0; k < ns; ++k) {
        SpThermo th = nasa7(m, k, T, lnT, invT);
        GS(k) = th.hRT - th.sR;
      }
    }
    for (int k = 0; k < ns; ++k) WS(k) = 0.0;
    const double lnC0 = m.lnpref_rth - lnT;
    for (int r = 0; r < m.nr; ++r) {
      const uint32_t w = m.code[r];
      const int type = rx_type(w);
      double kf = m.A[r] * fexp(m.b[r] * lnT - m.E[r] * invT, m.exptab);
      double Pf = 1.0, d;
#pragma unroll
      for (int sl = 0; sl < MAXSIDE; ++sl) {
        int sp = m.rsp[sl * P + r];
        if (sp >= 0) Pf *= powc(CS(sp), rx_ordcode(w, sl), m.rord[sl * P + r], &d, m.exptab, m.logtab);
      }
      double rvsf = 0.0;
      if (rx_rev(w)) {
        double dG = 0.0, Pr = 1.0;
#pragma unroll
        for (int sl = 0; sl < MAXSIDE; ++sl) {
          int sp = m.psp[sl * P + r];
          if (sp >= 0) {
            double nu = m.pnu[sl * P + r];
            dG += nu * GS(sp);
            Pr *= powc(CS(sp), (m.pcode[r] >> (4 * sl)) & 0xf, nu, &d, m.exptab, m.logtab);
          }
          int sq = m.rsp[sl * P + r];
          if (sq >= 0) dG -= m.rnu[sl * P + r] * GS(sq);
        }
        rvsf = fexp(dG - m.dnu[r] * lnC0, m.exptab) * Pr;
      }
      double keff = kf, Mfac = 1.0;
      if (type != 0) {
        const int row = rx_tbrow(w);
        double M = m.tbd[row] * ctot;
        for (int e = m.tbp[row]; e < m.tbp[row + 1]; ++e) M = fma(m.tbv[e], CS(m.tbs[e]), M);
        if (type == 1) Mfac = M;
        else keff = falloff_eval(m, r, type, kf, 0.0, M, T, lnT, invT).keff;
      }
      const double q = Mfac * keff * (Pf - rvsf);
#pragma unroll
      for (int sl = 0; sl < MAXSIDE; ++sl) {
        int sp = m.rsp[sl * P + r];
        if (sp >= 0) WS(sp) -= m.rnu[sl * P + r] * q;
        int sq = m.psp[sl * P + r];
        if (sq >= 0) WS(sq) += m.pnu[sl * P + r] * q;
      }
    }
    if (wdot) {
      for (int k = 0; k < ns; ++k) {
        double v = m.mw[k] * WS(k);
        if (roi_mode || layout == 0) wdot[i * ns + k] = v;
        else wdot[(int64_t)k * n + i] = v;
      }
    }
    (void)rho;
    if (cpo) cpo[i] = cpm * m.r_thermo;
    if (ho) ho[i] = hm * m.r_thermo * T;
  }
#undef CS
#undef GS
#undef WS
}

// ---------------------------------------------------------------- warp
// SPL species per lane; GJ: the Jacobian work area is a per-warp slot of
// global memory (mechanisms of 33-63 species, and smaller ones whose shared
// memory layout would not fit a block).
template <bool JAC, int SPL, bool GJ>
__global__ void __launch_bounds__(WARP_THREADS)
k_wdot_warp(const uint8_t* __restrict__ img, ImageLayout L, int64_t n, int layout,
            const double* __restrict__ Tg, const double* __restrict__ pg,
            const double* __restrict__ Yg, double* __restrict__ wdot, double* __restrict__ cpo,
            double* __restrict__ ho, double* __restrict__ jac, double* __restrict__ rhs_out,
            double* __restrict__ gscratch, int cv) {
  extern __shared__ __align__(16) uint8_t smem[];
  stage_image(smem, img, L.bytes);
  MechView m;
  m.bind(L, smem);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  WarpScratch s;
  if (!GJ) {
    const int sd = scratch_doubles(m.nsp, m.nrpad, JAC);
    s = carve(reinterpret_cast<double*>(smem + L.bytes) + wid * sd, m.nsp, m.nrpad, JAC);
  } else {
    const int sd = scratch_small_doubles(m.nsp, m.nrpad);
    const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid;
    s = carve2(reinterpret_cast<double*>(smem + L.bytes) + wid * sd,
               JAC ? gscratch + gw * scratch_jac_doubles(m.nsp, m.nrpad) : nullptr, m.nsp, m.nrpad);
  }
  const int ns = m.ns, nv = ns + 1;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t cell = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid; cell < n; cell += nwarps) {
    const double T = Tg[cell], p = pg[cell];
    double Yk[SPL];
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int k = lane + 32 * j;
      Yk[j] = 0.0;
      if (k < ns) Yk[j] = (layout == 1) ? Yg[(int64_t)k * n + cell] : Yg[cell * ns + k];
    }
    CellOutT<SPL> o;
    warp_kinetics<JAC, SPL>(m, s, lane, Yk, T, p, o, cv != 0);
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int k = lane + 32 * j;
      if (wdot && k < ns) {
        const double v = m.mw[k] * o.wmol[j];
        if (layout == 1) wdot[(int64_t)k * n + cell] = v;
        else wdot[cell * ns + k] = v;
      }
      if (rhs_out && k < nv) rhs_out[cell * nv + k] = o.f[j];
    }
    if (lane == 0) {
      if (cpo) cpo[cell] = o.cp_mass;
      if (ho) ho[cell] = o.h_mass;
    }
    if (JAC && jac) {
      // Fortran (nv, nv, N): column c of this cell is contiguous; lanes = rows.
      double* dst = jac + cell * (int64_t)nv * nv;
#pragma unroll
      for (int j = 0; j < SPL; ++j) {
        const int r = lane + 32 * j;
        if (r < nv)
          for (int c = 0; c < nv; ++c) dst[(int64_t)c * nv + r] = s.Jr[r * s.ldj + c];
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- thermo
// Mixture cp [J/kg/K] and h [J/kg] of N cells, one thread per cell
// (f_cp / H of Lib_ThermoTransport.f90:251-271, :40-52 on NASA-7 data).
__global__ void __launch_bounds__(SMALL_THREADS)
k_thermo(const uint8_t* __restrict__ img, ImageLayout L, int64_t n, int layout, const double* __restrict__ Tg,
         const double* __restrict__ Yg, double* __restrict__ cpo, double* __restrict__ ho) {
  extern __shared__ __align__(16) uint8_t smem[];
  stage_image(smem, img, L.bytes);
  MechView m;
  m.bind(L, smem);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double T = Tg[i], lnT = log(T), invT = 1.0 / T;
    double cpm = 0.0, hm = 0.0;
    for (int k = 0; k < m.ns; ++k) {
      const double y = (layout == 1) ? Yg[(int64_t)k * n + i] : Yg[i * m.ns + k];
      SpThermo th = nasa7(m, k, T, lnT, invT);
      cpm += y * th.cpR * m.invmw[k];
      hm += y * th.hRT * m.invmw[k];
    }
    if (cpo) cpo[i] = cpm * m.r_thermo;
    if (ho) ho[i] = hm * m.r_thermo * T;
  }
}

// ---------------------------------------------------------------- species thermo
// Species cp, h, s (at p_ref) and g = h - T s in mass units for N
// temperatures (cpi, H0i, S0i of Lib_ThermoTransport.f90:40-97, :233-248, from
// the polynomials): one thread per (cell, species), outputs cell-major (N, ns).
__global__ void k_species_thermo(const uint8_t* __restrict__ img, ImageLayout L, int64_t n,
                                 const double* __restrict__ Tg, double* __restrict__ cpo,
                                 double* __restrict__ ho, double* __restrict__ so, double* __restrict__ go) {
  extern __shared__ __align__(16) uint8_t smem[];
  stage_image(smem, img, L.bytes);
  MechView m;
  m.bind(L, smem);
  const int ns = m.ns;
  const int64_t total = n * ns;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = i / ns;
    const int k = (int)(i - cell * ns);
    const double T = Tg[cell], lnT = log(T), invT = 1.0 / T;
    const SpThermo th = nasa7(m, k, T, lnT, invT);
    const double rw = m.r_thermo * m.invmw[k];
    if (cpo) cpo[i] = th.cpR * rw;
    if (ho) ho[i] = th.hRT * rw * T;
    if (so) so[i] = th.sR * rw;
    if (go) go[i] = (th.hRT - th.sR) * rw * T;
  }
}

// ---------------------------------------------------------------- exp self-test
__global__ void k_exp_selftest(const uint8_t* __restrict__ img, ImageLayout L, int64_t n,
                               const double* __restrict__ x, double* __restrict__ y) {
  extern __shared__ __align__(16) uint8_t smem[];
  stage_image(smem, img, L.bytes);
  MechView m;
  m.bind(L, smem);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    y[2 * i] = fexp(x[i], m.exptab);
    y[2 * i + 1] = exp(x[i]);
  }
}

cudaError_t launch_exp_selftest(const uint8_t* img, const ImageLayout& L, int64_t n, const double* x, double* y,
                                cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = set_smem((const void*)k_exp_selftest, L.bytes);
  if (e != cudaSuccess) return e;
  k_exp_selftest<<<256, 256, L.bytes, st>>>(img, L, n, x, y);
  count_launch();
  return cudaGetLastError();
}

__global__ void k_log_selftest(const uint8_t* __restrict__ img, ImageLayout L, int64_t n,
                               const double* __restrict__ x, double* __restrict__ y) {
  extern __shared__ __align__(16) uint8_t smem[];
  stage_image(smem, img, L.bytes);
  MechView m;
  m.bind(L, smem);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    y[2 * i] = flog(x[i], m.logtab);
    y[2 * i + 1] = log(x[i]);
  }
}

cudaError_t launch_log_selftest(const uint8_t* img, const ImageLayout& L, int64_t n, const double* x, double* y,
                                cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = set_smem((const void*)k_log_selftest, L.bytes);
  if (e != cudaSuccess) return e;
  k_log_selftest<<<256, 256, L.bytes, st>>>(img, L, n, x, y);
  count_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------- FP64 probe
// Independent FMA chains: the FP64 pipe's throughput, the denominator of the
// FP64 roofline the benchmarks report.
__global__ void k_dfma_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
  double x4 = x0 + 4.0, x5 = x0 + 5.0, x6 = x0 + 6.0, x7 = x0 + 7.0;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

cudaError_t probe_fp64(double* tflops) {
  const int blocks = device_sms() * 8, threads = 256, iters = 2048;
  double* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double));
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_probe<<<blocks, threads>>>(buf, 64, 0.999, 1e-3);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_dfma_probe<<<blocks, threads>>>(buf, iters, 0.999, 1e-3);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  count_launch();
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return e;
}

// ---------------------------------------------------------------- launchers
// Device properties, cached per device (the current device of the calling
// thread); the cache entries are atomics, so concurrent first calls are safe.
constexpr int MAX_DEV_CACHE = 64;
static std::atomic<int> g_sms[MAX_DEV_CACHE];
static std::atomic<int> g_optin[MAX_DEV_CACHE];

static int cached_attr(std::atomic<int>* cache, cudaDeviceAttr attr, int fallback) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV_CACHE) dev = 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, attr, dev) != cudaSuccess || v <= 0) {
      (void)cudaGetLastError();
      v = fallback;
    }
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

int device_sms() { return cached_attr(g_sms, cudaDevAttrMultiProcessorCount, 1); }

size_t device_smem_optin() {
  return (size_t)cached_attr(g_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, 48 * 1024);
}

static int64_t grid_for(const void* fn, int threads, size_t smem, int64_t work_items) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
  if (per_sm < 1) per_sm = 1;
  int64_t full = (int64_t)device_sms() * per_sm;
  int64_t need = (work_items + threads - 1) / threads;
  if (need < 1) need = 1;
  return need < full ? need : full;
}

size_t small_smem(const ImageLayout& L) { return L.bytes + 3 * SMALL_NSMAX * SMALL_THREADS * sizeof(double); }
// Jacobian work area in global memory: 33-63 species, or a shared-memory
// layout too large for a block of 256 threads (the choice does not depend on
// the block size a caller tunes, so one kernel serves every block size).
static bool warp_gj(const ImageLayout& L, bool jac) {
  if (L.nsp > 32) return true;
  if (!jac) return false;
  return L.bytes + (WARP_THREADS / 32) * scratch_doubles(L.nsp, L.nrpad, true) * sizeof(double) > device_smem_optin();
}

static int warp_block(int threads) { return threads == 64 || threads == 128 ? threads : WARP_THREADS; }

size_t warp_smem(const ImageLayout& L, bool jac, int threads) {
  const int wpb = warp_block(threads) / 32;
  if (warp_gj(L, jac)) return L.bytes + wpb * scratch_small_doubles(L.nsp, L.nrpad) * sizeof(double);
  return L.bytes + wpb * scratch_doubles(L.nsp, L.nrpad, jac) * sizeof(double);
}

int warp_block_candidates(int* out) {
  out[0] = 64; out[1] = 128; out[2] = WARP_THREADS;
  return 3;
}

template <bool JAC>
static const void* warp_fn(const ImageLayout& L) {
  if (L.nsp > 32) return (const void*)k_wdot_warp<JAC, 2, true>;
  return warp_gj(L, JAC) ? (const void*)k_wdot_warp<JAC, 1, true> : (const void*)k_wdot_warp<JAC, 1, false>;
}

// Global Jacobian work area needed by the warp kernels (doubles), for a grid
// of full waves; 0 when it lives in shared memory.
// (enough for the resident warps of every block size)
int64_t warp_jac_scratch_doubles(const ImageLayout& L) {
  if (!warp_gj(L, true)) return 0;
  const void* fn = warp_fn<true>(L);
  int64_t most = 0;
  int cand[4];
  const int nc = warp_block_candidates(cand);
  for (int c = 0; c < nc; ++c) {
    const size_t sm = warp_smem(L, true, cand[c]);
    if (set_smem(fn, sm) != cudaSuccess) return 0;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, cand[c], sm);
    if (per_sm < 1) per_sm = 1;
    most = std::max(most, (int64_t)per_sm * device_sms() * (cand[c] / 32));
  }
  return most * scratch_jac_doubles(L.nsp, L.nrpad);
}

template <bool JAC>
static cudaError_t launch_warp(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                               const double* p, const double* Y, double* wdot, double* cp, double* h, double* jac,
                               double* rhs, double* gscratch, cudaStream_t st, int cv = 0, int threads = 0) {
  const int bt = warp_block(threads);
  size_t sm = warp_smem(L, JAC, bt);
  const void* fn = warp_fn<JAC>(L);
  cudaError_t e = set_smem(fn, sm);
  if (e != cudaSuccess) return e;
  const bool gj = warp_gj(L, JAC);
  if (gj && JAC && !gscratch) return cudaErrorInvalidValue;
  int64_t g = grid_for(fn, bt, sm, n * 32);
  if (L.nsp > 32)
    k_wdot_warp<JAC, 2, true><<<(unsigned)g, bt, sm, st>>>(img, L, n, layout, T, p, Y, wdot, cp, h, jac, rhs,
                                                            gscratch, cv);
  else if (gj)
    k_wdot_warp<JAC, 1, true><<<(unsigned)g, bt, sm, st>>>(img, L, n, layout, T, p, Y, wdot, cp, h, jac, rhs,
                                                            gscratch, cv);
  else
    k_wdot_warp<JAC, 1, false><<<(unsigned)g, bt, sm, st>>>(img, L, n, layout, T, p, Y, wdot, cp, h, jac, rhs,
                                                             nullptr, cv);
  count_launch();
  return cudaGetLastError();
}

bool use_small_kernel(const ImageLayout& L) { return L.ns <= SMALL_NSMAX && L.ns <= 8; }

cudaError_t launch_wdot(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                        const double* p, const double* Y, double* wdot, double* cp, double* h,
                        cudaStream_t st, int threads) {
  if (n <= 0) return cudaSuccess;
  if (use_small_kernel(L)) {
    size_t sm = small_smem(L);
    set_smem((const void*)k_wdot_small, sm);
    int64_t g = grid_for((const void*)k_wdot_small, SMALL_THREADS, sm, n);
    k_wdot_small<<<(unsigned)g, SMALL_THREADS, sm, st>>>(img, L, n, layout, T, p, Y, wdot, cp, h, 0, nullptr);
    count_launch();
    return cudaGetLastError();
  }
  return launch_warp<false>(img, L, n, layout, T, p, Y, wdot, cp, h, nullptr, nullptr, nullptr, st, 0, threads);
}

cudaError_t launch_thermo(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                          const double* Y, double* cp, double* h, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  size_t sm = L.bytes;
  set_smem((const void*)k_thermo, sm);
  int64_t g = grid_for((const void*)k_thermo, SMALL_THREADS, sm, n);
  k_thermo<<<(unsigned)g, SMALL_THREADS, sm, st>>>(img, L, n, layout, T, Y, cp, h);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_species_thermo(const uint8_t* img, const ImageLayout& L, int64_t n, const double* T, double* cp,
                                  double* h, double* s, double* g, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  size_t sm = L.bytes;
  set_smem((const void*)k_species_thermo, sm);
  const int64_t blocks = grid_for((const void*)k_species_thermo, SMALL_THREADS, sm, n * L.ns);
  k_species_thermo<<<(unsigned)blocks, SMALL_THREADS, sm, st>>>(img, L, n, T, cp, h, s, g);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_chemistry_source(const uint8_t* img, const ImageLayout& L, int64_t n, double* roi,
                                    const double* T, double* omegadot, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  size_t sm = small_smem(L);
  set_smem((const void*)k_wdot_small, sm);
  int64_t g = grid_for((const void*)k_wdot_small, SMALL_THREADS, sm, n);
  k_wdot_small<<<(unsigned)g, SMALL_THREADS, sm, st>>>(img, L, n, 0, T, nullptr, nullptr, omegadot, nullptr,
                                                         nullptr, 1, roi);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_wdot_jac(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                            const double* p, const double* Y, double* wdot, double* jac, double* gscratch,
                            cudaStream_t st, int cv, int threads) {
  if (n <= 0) return cudaSuccess;
  return launch_warp<true>(img, L, n, layout, T, p, Y, wdot, nullptr, nullptr, jac, nullptr, gscratch, st, cv,
                           threads);
}

cudaError_t launch_rhs(const uint8_t* img, const ImageLayout& L, int64_t n, const double* T, const double* p,
                       const double* Y, double* f, cudaStream_t st, int cv) {
  if (n <= 0) return cudaSuccess;
  return launch_warp<false>(img, L, n, 0, T, p, Y, nullptr, nullptr, nullptr, nullptr, f, nullptr, st, cv);
}

}  // namespace flint
