// flint_surrogate.cu -- learned reactor surrogate with a residual gate and an
// FP64 integrator fallback.
//
// A cell (T0, p, Y0, dt) is mapped by an MLP (flint_mlp.cu) to (dY, dT) over dt.
// The prediction is then made exactly conservative and checked:
//   * element conservation with non-negative mass fractions: dY is projected
//     onto the null space of the element matrix (mass fractions:
//     sum_k a_ek dY_k / W_k = 0; total mass follows) by least squares over the
//     species not clipped at zero, clipping negatives and repeating
//     (an active-set projection, at most 8 passes);
//   * energy conservation (adiabatic, constant p): T1 solves h(T1, Y1) = h(T0, Y0)
//     by Newton on the NASA-7 enthalpy, started from the network's T0 + dT;
//   (no clipping afterwards: a mass fraction below the gate's min_Y rejects
//   the cell, so accepted results conserve elements and enthalpy exactly)
// and the cell is accepted only if the residuals of the raw prediction are
// small: |T1(h) - (T0 + dT_net)| (energy residual), the element residual
// |B dY_net| (projection size), min Y1 (realizability), the input inside the
// training domain, and (two networks) the ensemble disagreement.  Rejected
// cells are compacted and re-solved by the BDF integrator (flint_reactor.cu)
// from their original state, so every result is either a gated surrogate
// step or an FP64 integrator step.
//
// Features (n_in = ns + 2): log10(max(Y_k, 1e-20)) of every species but the
// bath species, T, log10 p, log10 dt; targets (n_out = ns + 1): dY_k, dT.
// Both normalised by the training-set mean and standard deviation.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <cuda_bf16.h>

#include "flint_host.h"
#include "flint_mlp.h"
#include "flint_umma.h"

namespace flint {

constexpr int MAXL = 8;
constexpr int MAXS = 64;   // species of a surrogate mechanism (the reactor's limit, 63)
constexpr int NPASS = 8;   // active-set passes of the conservative projection

struct Net {
  int nl = 0;
  int dims[MAXL + 1] = {0};
  int64_t off_w[MAXL] = {0}, off_b[MAXL] = {0}, P = 0;
  float *w = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
  __nv_bfloat16* wb = nullptr;
  int64_t step = 0;
  // the fused tcgen05 inference forward (flint_umma.cu): packed BF16 hi/lo
  // weights, refreshed from w whenever w changed
  bool ufits = false, udirty = true;
  UmmaNet u{};
  uint8_t* upk = nullptr;
  float* ubias = nullptr;
  int64_t* uoff = nullptr;   // device: off_w[nl], off_b[nl]
};

struct Surrogate {
  const uint8_t* mimg;      // analytic mechanism image (device)
  ImageLayout L;
  unsigned int* counter;    // reactor counters (device)
  double* jsave;            // reactor scratch (device)
  int jslots;
  int ns, bath, n_in, n_out, nnets, H;
  Net net[2];
  float *xmean, *xstd, *ymean, *ystd;   // device, host copies below
  std::vector<float> hxm, hxs, hym, hys;
  double* G0;               // [ne][ne] B B^T (device)
  double* Bm;               // [ne][ns] element rows divided by W (device)
  int ne;
  // workspaces
  int64_t cap = 0;          // rows of the inference workspaces (A, yhat, yout2, xf)
  int64_t cap_tr = 0;       // rows of the training-only workspaces (Z, dz0, dz1)
  int64_t cap_fb = 0;       // cells of the fallback compaction buffers
  float* Z[MAXL] = {nullptr};
  float* A[MAXL] = {nullptr};   // FP32 activations (the forward GEMMs split them into BF16 hi + lo)
  float *dz0 = nullptr, *dz1 = nullptr, *yhat = nullptr, *xf = nullptr, *yout2 = nullptr;
  double* loss = nullptr;
  // fallback compaction
  int64_t* rej_idx = nullptr;
  unsigned long long* rej_count = nullptr;
  double *cT = nullptr, *cp = nullptr, *cY = nullptr, *cdt = nullptr;
  int *cst = nullptr, *cns = nullptr;
  int64_t last_accepted = 0, last_rejected = 0, last_fallback_steps = 0;
  int64_t last_n = 0;       // cells of the last advance (its rejected count stays on the device)
  int fwd_mode = 0;         // 0: fused tcgen05 forward where it fits, 1: per-layer mma.sync GEMMs
  int* uerr = nullptr;      // device word: a wait of the fused forward timed out
};

// ------------------------------------------------------------------ kernels
__global__ void k_features(int64_t n, int ns, int bath, const double* __restrict__ T, const double* __restrict__ p,
                           const double* __restrict__ Y, const double* __restrict__ dt,
                           const float* __restrict__ xm, const float* __restrict__ xs, float* __restrict__ X) {
  const int nin = ns + 2;
  // the logarithmic features in FP32, the precision the network takes them in
  // (a double log10 per species cost ~35 FP64-pipe slots on this GPU)
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float* x = X + i * nin;
    int c = 0;
    for (int k = 0; k < ns; ++k) {
      if (k == bath) continue;
      const double y = Y[i * ns + k];
      x[c] = (log10f((float)(y > 1e-20 ? y : 1e-20)) - xm[c]) / xs[c];
      ++c;
    }
    x[c] = (float)((T[i] - xm[c]) / xs[c]); ++c;
    x[c] = (log10f((float)p[i]) - xm[c]) / xs[c]; ++c;
    x[c] = (log10f((float)dt[i]) - xm[c]) / xs[c];
  }
}

__global__ void k_targets(int64_t n, int ns, const double* __restrict__ T0, const double* __restrict__ Y0,
                          const double* __restrict__ T1, const double* __restrict__ Y1, const float* __restrict__ ym,
                          const float* __restrict__ ys, float* __restrict__ Yt) {
  const int nout = ns + 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int k = 0; k < ns; ++k) Yt[i * nout + k] = (float)((Y1[i * ns + k] - Y0[i * ns + k] - ym[k]) / ys[k]);
    Yt[i * nout + ns] = (float)((T1[i] - T0[i] - ym[ns]) / ys[ns]);
  }
}

// The domain bounds of p and dt are given as log10 and compared as values
// (plo = 10^log10p_lo ...): the same test without two logarithms per cell.
struct GateParams {
  double max_dT_resid, max_elem_resid, min_Y, max_ens_dT, max_ens_dY;
  double Tlo, Thi, plo, phi, dtlo, dthi;
};

// Post-processing and gate, one thread per cell, POST_CELLS cells per block.
// The block stages the species part of the mechanism image (thermo only), the
// element rows B and G0 = B B^T, and works on chunks of POST_CELLS cells whose
// per-species arrays live in shared memory as [k][POST_CELLS] (a warp's 32
// lanes touch 32 consecutive doubles); the chunk's mass fractions and network
// outputs are read, and the accepted mass fractions written, by coalesced
// block-wide loops over the chunk's contiguous rows.  Accepted cells are
// written in place; rejected ones are listed for the fallback (their T, Y
// untouched).
constexpr int POST_CELLS = 64;

struct PostSmem {
  int head, n9;      // image bytes staged: [0, o_A) (species sections) and the NASA-9 block
  int oB, oG;        // B [ne][ns], G0 [ne][ne]
  int oY0, oD;       // [ns][POST_CELLS] each: Y0; the increment dY, Y1 after the projection
  int odT, oensT, oens, oacc;   // per cell
  int bytes;
};

__host__ __device__ inline PostSmem post_smem(const ImageLayout& L, int ne) {
  PostSmem S;
  auto up = [](int b) { return (b + 15) & ~15; };
  S.head = L.o_A;
  S.n9 = L.o_nasa9 >= 0 ? 8 * 32 * L.nsp : 0;
  S.oB = up(S.head + S.n9);
  S.oG = up(S.oB + 8 * (ne > 0 ? ne : 1) * L.ns);
  S.oY0 = up(S.oG + 8 * (ne > 0 ? ne * ne : 1));
  S.oD = S.oY0 + 8 * L.ns * POST_CELLS;
  S.odT = S.oD + 8 * L.ns * POST_CELLS;
  S.oensT = S.odT + 8 * POST_CELLS;
  S.oens = S.oensT + 8 * POST_CELLS;
  S.oacc = S.oens + 8 * POST_CELLS;
  S.bytes = S.oacc + 4 * POST_CELLS;
  return S;
}

__global__ void __launch_bounds__(POST_CELLS)
k_post(const uint8_t* __restrict__ img, ImageLayout L, int64_t n, int64_t base, double* __restrict__ T,
       const double* __restrict__ p, double* __restrict__ Y, const double* __restrict__ dt,
       const float* __restrict__ yn, const float* __restrict__ yn2, const float* __restrict__ ym,
       const float* __restrict__ ys, const double* __restrict__ G0, const double* __restrict__ Bm, int ne,
       GateParams gp, int* __restrict__ status, int* __restrict__ nsteps, int64_t* __restrict__ rej_idx,
       unsigned long long* __restrict__ rej_count, double* __restrict__ metrics) {
  extern __shared__ __align__(16) uint8_t smem[];
  const PostSmem S = post_smem(L, ne);
  const int t = threadIdx.x;
  {
    const int4* src = reinterpret_cast<const int4*>(img);
    int4* dst = reinterpret_cast<int4*>(smem);
    for (int i = t; i < S.head / 16; i += POST_CELLS) dst[i] = __ldg(src + i);
    if (S.n9) {
      const int4* s9 = reinterpret_cast<const int4*>(img + L.o_nasa9);
      int4* d9 = reinterpret_cast<int4*>(smem + S.head);
      for (int i = t; i < S.n9 / 16; i += POST_CELLS) d9[i] = __ldg(s9 + i);
    }
  }
  MechView m;
  m.bind(L, smem);   // only the species sections (and NASA-9, below) are staged
  m.nasa9 = S.n9 ? reinterpret_cast<const double*>(smem + S.head) : nullptr;
  const int ns = m.ns, nout = ns + 1;
  double* sB = reinterpret_cast<double*>(smem + S.oB);
  double* sG = reinterpret_cast<double*>(smem + S.oG);
  for (int i = t; i < ne * ns; i += POST_CELLS) sB[i] = Bm[i];
  for (int i = t; i < ne * ne; i += POST_CELLS) sG[i] = G0[i];
  double* sY0 = reinterpret_cast<double*>(smem + S.oY0);
  double* sD = reinterpret_cast<double*>(smem + S.oD);
  double* sdT = reinterpret_cast<double*>(smem + S.odT);
  double* sensT = reinterpret_cast<double*>(smem + S.oensT);
  unsigned long long* sens = reinterpret_cast<unsigned long long*>(smem + S.oens);
  int* sacc = reinterpret_cast<int*>(smem + S.oacc);
  __syncthreads();
  for (int64_t c0 = (int64_t)blockIdx.x * POST_CELLS; c0 < n; c0 += (int64_t)gridDim.x * POST_CELLS) {
    const int nc = (int)(n - c0 < POST_CELLS ? n - c0 : POST_CELLS);
    const int64_t cell0 = base + c0;
    // the chunk's rows: Y0 [nc][ns] and the network outputs [nc][nout] (dY, dT),
    // de-normalised and (two networks) averaged, with the ensemble spreads
    for (int idx = t; idx < nc * ns; idx += POST_CELLS) {
      const int c = idx / ns, k = idx - c * ns;
      sY0[k * POST_CELLS + c] = Y[cell0 * ns + idx];
    }
    sens[t] = 0ull;
    __syncthreads();
    for (int idx = t; idx < nc * nout; idx += POST_CELLS) {
      const int c = idx / nout, k = idx - c * nout;
      const int64_t o = c0 * nout + idx;
      // in FP32, like the network's outputs (relative rounding 6e-8 of the
      // increment, far below the targets; the projection and the enthalpy
      // Newton then work in FP64)
      float df = fmaf(ys[k], yn[o], ym[k]);
      float sf = 0.0f;
      if (yn2) {
        const float d2 = fmaf(ys[k], yn2[o], ym[k]);
        sf = fabsf(d2 - df);
        df = 0.5f * (df + d2);
      }
      const double d = (double)df, spread = (double)sf;
      if (k < ns) {
        sD[k * POST_CELLS + c] = d;
        if (yn2) atomicMax(&sens[c], (unsigned long long)absbits(spread));   // max of non-negative doubles
      } else {
        sdT[c] = d;
        sensT[c] = spread;
      }
    }
    __syncthreads();
    if (t < nc) {
      const int64_t i = c0 + t, cell = cell0 + t;
      double* y0 = sY0 + t;    // species k at y0[k * POST_CELLS]
      double* dY = sD + t;
      const double T0 = T[cell], dti = dt[cell], pc = p[cell];
      bool ok = isfinite(T0) && isfinite(pc) && pc > 0.0 && isfinite(dti) && dti > 0.0;
      ok = ok && T0 >= gp.Tlo && T0 <= gp.Thi;
      ok = ok && pc >= gp.plo && pc <= gp.phi && dti >= gp.dtlo && dti <= gp.dthi;
      const double dTn = sdT[t], ensT = yn2 ? sensT[t] : 0.0;
      const double ens = yn2 ? __longlong_as_double((long long)sens[t]) : 0.0;
      // element residual of the raw prediction
      double er = 0.0;
      for (int e = 0; e < ne; ++e) {
        double s = 0.0;
        for (int k = 0; k < ns; ++k) s += sB[e * ns + k] * dY[k * POST_CELLS];
        er = fmax(er, fabs(s));
      }
      // conservative, non-negative mass fractions: project dY onto element
      // conservation over the free species, clip negatives to zero (they leave
      // the free set), repeat (active-set least-squares, at most NPASS passes;
      // the last pass clips nothing, so a result still negative there is
      // rejected).  dY holds the increment Y1 - Y0 throughout; G over the free
      // species is G0 less the clipped species' terms.
      unsigned long long fixed = 0ull;   // bit k: species k clipped at zero
      double clipped = 0.0;
      bool clean = false;
      for (int pass = 0; pass < NPASS && !clean; ++pass) {
        double r[8], G[8][8], lam[8];
        for (int e = 0; e < ne; ++e) {
          double se = 0.0;
          for (int k = 0; k < ns; ++k) se += sB[e * ns + k] * dY[k * POST_CELLS];
          r[e] = se;
          for (int f = 0; f < ne; ++f) {
            double g = sG[e * ne + f];
            for (unsigned long long fx = fixed; fx; fx &= fx - 1) {
              const int k = __ffsll((long long)fx) - 1;
              g -= sB[e * ns + k] * sB[f * ns + k];
            }
            G[e][f] = g;
          }
        }
        // solve G lam = r (Gauss-Jordan, partial pivoting; empty rows get lam = 0)
        for (int e = 0; e < ne; ++e) lam[e] = r[e];
        int live[8];
        for (int c = 0; c < ne; ++c) {
          int pr = c; double best = fabs(G[c][c]);
          for (int q = c + 1; q < ne; ++q) if (fabs(G[q][c]) > best) { best = fabs(G[q][c]); pr = q; }
          live[c] = best > 1e-300;
          if (!live[c]) continue;
          if (pr != c) {
            for (int f = 0; f < ne; ++f) { double tt = G[c][f]; G[c][f] = G[pr][f]; G[pr][f] = tt; }
            double tt = lam[c]; lam[c] = lam[pr]; lam[pr] = tt;
          }
          const double inv = 1.0 / G[c][c];
          for (int f = 0; f < ne; ++f) G[c][f] *= inv;
          lam[c] *= inv;
          for (int q = 0; q < ne; ++q) {
            if (q == c) continue;
            const double fq = G[q][c];
            for (int f = 0; f < ne; ++f) G[q][f] -= fq * G[c][f];
            lam[q] -= fq * lam[c];
          }
        }
        for (int e = 0; e < ne; ++e) if (!live[e]) lam[e] = 0.0;
        clean = true;
        for (int k = 0; k < ns; ++k) {
          if ((fixed >> k) & 1ull) continue;
          double corr = 0.0;
          for (int e = 0; e < ne; ++e) corr += sB[e * ns + k] * lam[e];
          const double d = dY[k * POST_CELLS] - corr;
          const double yk = y0[k * POST_CELLS];
          if (yk + d < 0.0 && pass < NPASS - 1) {
            clipped += -(yk + d);
            dY[k * POST_CELLS] = -yk;    // Y1 = 0
            fixed |= 1ull << k;
            clean = false;
          } else {
            dY[k * POST_CELLS] = d;
          }
        }
      }
      // dY -> Y1 (in place) and its minimum
      double ymin = 1.0;
      double* y1 = dY;
      for (int k = 0; k < ns; ++k) {
        const double v = y0[k * POST_CELLS] + dY[k * POST_CELLS];
        y1[k * POST_CELLS] = v;
        ymin = fmin(ymin, v);
      }
      // realizability measure reported to the gate: clipped mass (negative) or
      // the most negative mass fraction left
      const double yreal = fmin(-clipped, ymin);
      // energy: h(T1, Y1) = h(T0, Y0), Newton from the network's temperature
      double h0 = 0.0;
      {
        // ln T enters only the NASA-9 enthalpy (NASA-7's h needs no log)
        const double lnT = m.nasa9 ? log(T0) : 0.0, invT = 1.0 / T0;
        for (int k = 0; k < ns; ++k) h0 += y0[k * POST_CELLS] * nasa7(m, k, T0, lnT, invT).hRT * m.invmw[k];
        h0 *= T0;
      }
      double T1 = T0 + dTn;
      bool conv = isfinite(T1) && T1 > 200.0 && T1 < 6000.0;
      for (int it = 0; it < 8 && conv; ++it) {
        const double lnT = m.nasa9 ? log(T1) : 0.0, invT = 1.0 / T1;
        double h = 0.0, cpm = 0.0;
        for (int k = 0; k < ns; ++k) {
          SpThermo th = nasa7(m, k, T1, lnT, invT);
          const double yw = y1[k * POST_CELLS] * m.invmw[k];
          h += yw * th.hRT;
          cpm += yw * th.cpR;
        }
        const double dT = (h * T1 - h0) / cpm;
        T1 -= dT;
        if (!(T1 > 200.0 && T1 < 6000.0)) conv = false;
        // quadratic convergence: after a correction below 1e-6 T1 the next one
        // would be below 1e-7 K (|d2h/dT2| / (2 cp) < 1e-3 / K, T1 < 6000 K)
        if (fabs(dT) < 1e-6 * T1) break;
      }
      const double dTres = conv ? fabs(T1 - (T0 + dTn)) : 1e300;
      int accept;
      if (metrics) {
        // evaluation mode: every cell takes the surrogate result, the gate
        // quantities are reported instead of applied
        double* mt = metrics + i * 6;
        mt[0] = dTres; mt[1] = er; mt[2] = yreal; mt[3] = ensT; mt[4] = ens;
        mt[5] = (ok && ymin >= 0.0) ? 1.0 : 0.0;   // the gate's fixed conditions
        T[cell] = conv ? T1 : T0 + dTn;
        accept = 1;
      } else {
        ok = ok && conv && dTres <= gp.max_dT_resid && er <= gp.max_elem_resid && yreal >= gp.min_Y && ymin >= 0.0;
        if (yn2) ok = ok && ensT <= gp.max_ens_dT && ens <= gp.max_ens_dY;
        accept = ok ? 1 : 0;
        if (ok) {
          T[cell] = T1;
          if (status) status[cell] = FLINT_CELL_OK;
          if (nsteps) nsteps[cell] = 0;
        } else {
          unsigned long long slot = atomicAdd(rej_count, 1ull);
          rej_idx[slot] = cell;
        }
      }
      sacc[t] = accept;
    }
    __syncthreads();
    // the accepted cells' mass fractions, written back row by row
    for (int idx = t; idx < nc * ns; idx += POST_CELLS) {
      const int c = idx / ns, k = idx - c * ns;
      if (sacc[c]) Y[cell0 * ns + idx] = sD[k * POST_CELLS + c];
    }
    __syncthreads();
  }
}

__global__ void k_gather(const unsigned long long* __restrict__ count, const int64_t* __restrict__ idx, int ns, const double* __restrict__ T,
                         const double* __restrict__ p, const double* __restrict__ Y, const double* __restrict__ dt,
                         double* __restrict__ cT, double* __restrict__ cp, double* __restrict__ cY, double* __restrict__ cdt) {
  const int64_t m = (int64_t)*count;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx[i];
    cT[i] = T[c]; cp[i] = p[c]; cdt[i] = dt[c];
    for (int k = 0; k < ns; ++k) cY[i * ns + k] = Y[c * ns + k];
  }
}

__global__ void k_scatter(const unsigned long long* __restrict__ count, const int64_t* __restrict__ idx, int ns, double* __restrict__ T,
                          double* __restrict__ Y, const double* __restrict__ cT, const double* __restrict__ cY,
                          const int* __restrict__ cst, const int* __restrict__ cns, int* __restrict__ status,
                          int* __restrict__ nsteps) {
  const int64_t m = (int64_t)*count;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx[i];
    T[c] = cT[i];
    for (int k = 0; k < ns; ++k) Y[c * ns + k] = cY[i * ns + k];
    if (status) status[c] = cst[i] == FLINT_CELL_OK ? FLINT_CELL_SURROGATE_REJECTED : cst[i];
    if (nsteps) nsteps[c] = cns[i];
  }
}

static int blocks_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  int64_t cap = (int64_t)device_sms() * 8;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

// ------------------------------------------------------------------ host side
static cudaError_t net_forward(Surrogate* s, Net& nt, int64_t n, const float* X, float* out, bool keep,
                               cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (!keep && s->fwd_mode == 0 && nt.ufits) {
    if (nt.udirty) {
      e = umma_pack(nt.u, nt.w, nt.uoff, nt.uoff + nt.nl, nt.upk, nt.ubias, st);
      if (e) return e;
      nt.udirty = false;
    }
    return launch_mlp_umma(nt.u, nt.upk, nt.ubias, n, X, out, s->uerr, st);
  }
  for (int l = 0; l < nt.nl && !e; ++l) {
    GemmArgs g{};
    g.M = (int)n; g.N = nt.dims[l + 1]; g.K = nt.dims[l];
    if (l == 0) { g.A = X; g.a_bf16 = 0; } else { g.A = s->A[l - 1]; g.a_bf16 = 0; }
    g.sa_m = g.K; g.sa_k = 1;
    g.B = nt.w + nt.off_w[l]; g.b_bf16 = 0; g.sb_k = 1; g.sb_n = g.K;
    g.split = 1;
    g.bias = nt.w + nt.off_b[l];
    if (l < nt.nl - 1) {
      g.epi = EPI_BIAS_GELU;
      g.C = keep ? s->Z[l] : nullptr; g.ldc = g.N;
      g.Cf = s->A[l]; g.ldcf = g.N;
    } else {
      g.epi = EPI_BIAS;
      g.C = out; g.ldc = g.N;
    }
    e = launch_gemm(g, st);
  }
  return e;
}

static int alloc_ws(Surrogate* s, int64_t cap, bool train) {
  auto fr = [](void* p) { if (p) cudaFree(p); };
  cudaError_t e = cudaSuccess;
  const int nh = s->net[0].nl - 1;
  if (cap > s->cap) {
    for (int l = 0; l < MAXL; ++l) { fr(s->A[l]); s->A[l] = nullptr; }
    fr(s->yhat); fr(s->xf); fr(s->yout2);
    s->yhat = s->xf = s->yout2 = nullptr;
    s->cap = 0;
    for (int l = 0; l < nh && !e; ++l) e = cudaMalloc(&s->A[l], cap * s->H * sizeof(float));
    if (!e) e = cudaMalloc(&s->yhat, cap * s->n_out * sizeof(float));
    if (!e) e = cudaMalloc(&s->yout2, cap * s->n_out * sizeof(float));
    if (!e) e = cudaMalloc(&s->xf, cap * s->n_in * sizeof(float));
    if (e) return FLINT_ERR_NOMEM;
    s->cap = cap;
  }
  if (train && cap > s->cap_tr) {
    for (int l = 0; l < MAXL; ++l) { fr(s->Z[l]); s->Z[l] = nullptr; }
    fr(s->dz0); fr(s->dz1);
    s->dz0 = s->dz1 = nullptr;
    s->cap_tr = 0;
    const int W = std::max(s->H, std::max(s->n_in, s->n_out));
    for (int l = 0; l < nh && !e; ++l) e = cudaMalloc(&s->Z[l], cap * s->H * sizeof(float));
    if (!e) e = cudaMalloc(&s->dz0, cap * W * sizeof(float));
    if (!e) e = cudaMalloc(&s->dz1, cap * W * sizeof(float));
    if (e) return FLINT_ERR_NOMEM;
    s->cap_tr = cap;
  }
  return 0;
}

// Compaction buffers of the fallback: room for every cell of a call.
static int alloc_fb(Surrogate* s, int64_t n) {
  if (n <= s->cap_fb) return 0;
  auto fr = [](void* p) { if (p) cudaFree(p); };
  fr(s->rej_idx); fr(s->cT); fr(s->cp); fr(s->cY); fr(s->cdt); fr(s->cst); fr(s->cns);
  s->rej_idx = nullptr; s->cT = s->cp = s->cY = s->cdt = nullptr; s->cst = s->cns = nullptr;
  s->cap_fb = 0;
  cudaError_t e = cudaMalloc(&s->rej_idx, n * sizeof(int64_t));
  if (!e) e = cudaMalloc(&s->cT, n * sizeof(double));
  if (!e) e = cudaMalloc(&s->cp, n * sizeof(double));
  if (!e) e = cudaMalloc(&s->cdt, n * sizeof(double));
  if (!e) e = cudaMalloc(&s->cY, n * s->ns * sizeof(double));
  if (!e) e = cudaMalloc(&s->cst, n * sizeof(int));
  if (!e) e = cudaMalloc(&s->cns, n * sizeof(int));
  if (e) return FLINT_ERR_NOMEM;
  s->cap_fb = n;
  return 0;
}

static void net_free(Net& nt) {
  cudaFree(nt.w); cudaFree(nt.g); cudaFree(nt.m1); cudaFree(nt.m2); cudaFree(nt.wb);
  cudaFree(nt.upk); cudaFree(nt.ubias); cudaFree(nt.uoff);
  nt = Net();
}

void surrogate_free(Surrogate* s) {
  if (!s) return;
  for (int i = 0; i < 2; ++i) net_free(s->net[i]);
  auto fr = [](void* p) { if (p) cudaFree(p); };
  for (int l = 0; l < MAXL; ++l) { fr(s->Z[l]); fr(s->A[l]); }
  fr(s->dz0); fr(s->dz1); fr(s->yhat); fr(s->xf); fr(s->yout2); fr(s->rej_idx); fr(s->rej_count);
  fr(s->cT); fr(s->cp); fr(s->cY); fr(s->cdt); fr(s->cst); fr(s->cns); fr(s->loss);
  fr(s->xmean); fr(s->xstd); fr(s->ymean); fr(s->ystd); fr(s->G0); fr(s->Bm); fr(s->uerr);
  delete s;
}

// Net layout: dims, then per layer W[dims[l+1]][dims[l]] followed by b[dims[l+1]].
static int net_init(Net& nt, int nl, const int* dims, const float* w0) {
  nt.nl = nl;
  int64_t off = 0;
  for (int l = 0; l <= nl; ++l) nt.dims[l] = dims[l];
  for (int l = 0; l < nl; ++l) {
    nt.off_w[l] = off; off += (int64_t)dims[l + 1] * dims[l];
    nt.off_b[l] = off; off += dims[l + 1];
  }
  nt.P = off;
  cudaError_t e = cudaMalloc(&nt.w, off * sizeof(float));
  if (!e) e = cudaMalloc(&nt.g, off * sizeof(float));
  if (!e) e = cudaMalloc(&nt.m1, off * sizeof(float));
  if (!e) e = cudaMalloc(&nt.m2, off * sizeof(float));
  if (!e) e = cudaMalloc(&nt.wb, off * sizeof(__nv_bfloat16));
  if (!e) e = cudaMemcpy(nt.w, w0, off * sizeof(float), cudaMemcpyHostToDevice);
  if (!e) e = cudaMemset(nt.m1, 0, off * sizeof(float));
  if (!e) e = cudaMemset(nt.m2, 0, off * sizeof(float));
  if (!e) e = launch_to_bf16(nt.w, nt.wb, off, nullptr);
  nt.ufits = umma_fits(nl, dims);
  if (!e && nt.ufits) {
    const int64_t bytes = umma_describe(nl, dims, &nt.u);
    std::vector<int64_t> offs(2 * nl);
    for (int l = 0; l < nl; ++l) { offs[l] = nt.off_w[l]; offs[nl + l] = nt.off_b[l]; }
    e = cudaMalloc(&nt.upk, bytes);
    if (!e) e = cudaMalloc(&nt.ubias, (size_t)nl * 256 * sizeof(float));
    if (!e) e = cudaMalloc(&nt.uoff, offs.size() * sizeof(int64_t));
    if (!e) e = cudaMemcpy(nt.uoff, offs.data(), offs.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
    nt.udirty = true;
  }
  if (!e) e = cudaDeviceSynchronize();
  return e ? FLINT_ERR_CUDA : 0;
}

int surrogate_create(const uint8_t* mimg, const ImageLayout& L, unsigned int* counter, const flint_surrogate_desc* d,
                     Surrogate** out, std::string& err) {
  if (d->n_layers < 2 || d->n_layers > MAXL) { err = "n_layers out of range"; return FLINT_ERR_ARG; }
  if (L.ns > MAXS - 1 || L.ns < 2) { err = "surrogate supports 2..63 species"; return FLINT_ERR_MECH; }
  if (d->bath < 0 || d->bath >= L.ns) { err = "bath species index"; return FLINT_ERR_ARG; }
  if (d->n_nets < 1 || d->n_nets > 2) { err = "n_nets must be 1 or 2"; return FLINT_ERR_ARG; }
  if (d->n_elements < 0 || d->n_elements > 8) { err = "n_elements must be 0..8"; return FLINT_ERR_ARG; }
  if (!d->weights || !d->x_mean || !d->x_std || !d->y_mean || !d->y_std || !d->elem) { err = "NULL array"; return FLINT_ERR_ARG; }
  auto* s = new Surrogate();
  s->mimg = mimg; s->L = L; s->counter = counter; s->jsave = nullptr; s->jslots = 0;
  s->ns = L.ns; s->bath = d->bath; s->n_in = L.ns + 2; s->n_out = L.ns + 1; s->H = d->hidden;
  s->nnets = d->n_nets; s->ne = d->n_elements;
  std::vector<int> dims(d->n_layers + 1);
  dims[0] = s->n_in;
  for (int l = 1; l < d->n_layers; ++l) dims[l] = d->hidden;
  dims[d->n_layers] = s->n_out;
  int64_t P = 0;
  for (int l = 0; l < d->n_layers; ++l) P += (int64_t)dims[l + 1] * dims[l] + dims[l + 1];
  for (int i = 0; i < s->nnets; ++i) {
    if (net_init(s->net[i], d->n_layers, dims.data(), d->weights + i * P)) {
      surrogate_free(s); err = "weight buffers"; return FLINT_ERR_NOMEM;
    }
  }
  s->hxm.assign(d->x_mean, d->x_mean + s->n_in); s->hxs.assign(d->x_std, d->x_std + s->n_in);
  s->hym.assign(d->y_mean, d->y_mean + s->n_out); s->hys.assign(d->y_std, d->y_std + s->n_out);
  // element rows B[e][k] = a_ek / W_k and G0 = B B^T (the projection's normal
  // matrix over all species; the gate subtracts the clipped species' terms)
  const int ns = s->ns, ne = s->ne;
  std::vector<double> Bm((size_t)ne * ns), BBt((size_t)ne * ne, 0.0);
  std::vector<double> W(ns);
  cudaMemcpy(W.data(), mimg + L.o_mw, ns * sizeof(double), cudaMemcpyDeviceToHost);
  for (int e = 0; e < ne; ++e)
    for (int k = 0; k < ns; ++k) Bm[e * ns + k] = d->elem[e * ns + k] / W[k];
  for (int a = 0; a < ne; ++a)
    for (int b = 0; b < ne; ++b)
      for (int k = 0; k < ns; ++k) BBt[a * ne + b] += Bm[a * ns + k] * Bm[b * ns + k];
  cudaError_t e = cudaMalloc(&s->xmean, s->n_in * 4);
  if (!e) e = cudaMalloc(&s->xstd, s->n_in * 4);
  if (!e) e = cudaMalloc(&s->ymean, s->n_out * 4);
  if (!e) e = cudaMalloc(&s->ystd, s->n_out * 4);
  if (!e) e = cudaMalloc(&s->G0, std::max(ne * ne, 1) * 8);
  if (!e) e = cudaMalloc(&s->Bm, std::max(ne, 1) * ns * 8);
  if (!e) e = cudaMalloc(&s->loss, 8);
  if (!e) e = cudaMalloc(&s->rej_count, 8);
  if (!e) e = cudaMalloc(&s->uerr, sizeof(int));
  if (!e) e = cudaMemset(s->uerr, 0, sizeof(int));
  if (!e) e = cudaMemcpy(s->xmean, d->x_mean, s->n_in * 4, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(s->xstd, d->x_std, s->n_in * 4, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(s->ymean, d->y_mean, s->n_out * 4, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(s->ystd, d->y_std, s->n_out * 4, cudaMemcpyHostToDevice);
  if (!e && ne) e = cudaMemcpy(s->G0, BBt.data(), ne * ne * 8, cudaMemcpyHostToDevice);
  if (!e && ne) e = cudaMemcpy(s->Bm, Bm.data(), ne * ns * 8, cudaMemcpyHostToDevice);
  if (e) { surrogate_free(s); err = cudaGetErrorString(e); return FLINT_ERR_CUDA; }
  *out = s;
  return 0;
}

int surrogate_features(Surrogate* s, int64_t n, const double* T, const double* p, const double* Y, const double* dt,
                       float* X, cudaStream_t st) {
  if (n <= 0) return 0;
  k_features<<<blocks_for(n, 256), 256, 0, st>>>(n, s->ns, s->bath, T, p, Y, dt, s->xmean, s->xstd, X);
  count_launch();
  return cudaGetLastError() ? FLINT_ERR_CUDA : 0;
}

int surrogate_targets(Surrogate* s, int64_t n, const double* T0, const double* Y0, const double* T1, const double* Y1,
                      float* Yt, cudaStream_t st) {
  if (n <= 0) return 0;
  k_targets<<<blocks_for(n, 256), 256, 0, st>>>(n, s->ns, T0, Y0, T1, Y1, s->ymean, s->ystd, Yt);
  count_launch();
  return cudaGetLastError() ? FLINT_ERR_CUDA : 0;
}

int surrogate_predict(Surrogate* s, int net, int64_t n, const float* X, float* Yn, cudaStream_t st) {
  if (net < 0 || net >= s->nnets) return FLINT_ERR_ARG;
  if (n <= 0) return 0;
  if (alloc_ws(s, std::min<int64_t>(n, 262144), false)) return FLINT_ERR_NOMEM;
  for (int64_t b = 0; b < n; b += s->cap) {
    const int64_t m = std::min<int64_t>(s->cap, n - b);
    if (net_forward(s, s->net[net], m, X + b * s->n_in, Yn + b * s->n_out, false, st)) return FLINT_ERR_CUDA;
  }
  return 0;
}

int surrogate_train_step(Surrogate* s, int net, int64_t n, const float* X, const float* Yt, float lr, double* loss_out,
                         cudaStream_t st) {
  if (net < 0 || net >= s->nnets || n <= 0) return FLINT_ERR_ARG;
  if (alloc_ws(s, n, true)) return FLINT_ERR_NOMEM;
  Net& nt = s->net[net];
  if (net_forward(s, nt, n, X, s->yhat, true, st)) return FLINT_ERR_CUDA;
  if (cudaMemsetAsync(s->loss, 0, 8, st)) return FLINT_ERR_CUDA;
  const int nl = nt.nl;
  float* dz = s->dz0;
  float* dzn = s->dz1;
  if (launch_mse(s->yhat, Yt, n * s->n_out, 1.0f / (float)(n * s->n_out), dz, s->loss, st)) return FLINT_ERR_CUDA;
  for (int l = nl - 1; l >= 0; --l) {
    const int N = nt.dims[l + 1], K = nt.dims[l];
    GemmArgs g{};
    g.M = N; g.N = K; g.K = (int)n;
    g.A = dz; g.a_bf16 = 0; g.sa_m = 1; g.sa_k = N;
    if (l == 0) { g.B = X; g.b_bf16 = 0; } else { g.B = s->A[l - 1]; g.b_bf16 = 0; }
    g.sb_k = K; g.sb_n = 1;
    g.C = nt.g + nt.off_w[l]; g.ldc = K; g.epi = EPI_STORE;
    if (launch_gemm(g, st)) return FLINT_ERR_CUDA;
    if (launch_colsum(dz, (int)n, N, N, nt.g + nt.off_b[l], 0, st)) return FLINT_ERR_CUDA;
    if (l > 0) {
      GemmArgs h{};
      h.M = (int)n; h.N = K; h.K = N;
      h.A = dz; h.a_bf16 = 0; h.sa_m = N; h.sa_k = 1;
      h.B = nt.wb + nt.off_w[l]; h.b_bf16 = 1; h.sb_k = K; h.sb_n = 1;
      h.C = dzn; h.ldc = K; h.epi = EPI_GELU_BWD; h.Zprev = s->Z[l - 1]; h.ldz = K;
      if (launch_gemm(h, st)) return FLINT_ERR_CUDA;
      std::swap(dz, dzn);
    }
  }
  nt.step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - powf(b1, (float)nt.step), bc2 = 1.f - powf(b2, (float)nt.step);
  if (launch_adam(nt.w, nt.g, nt.m1, nt.m2, nt.wb, nt.P, lr, b1, b2, 1e-8f, bc1, bc2, 0.f, st)) return FLINT_ERR_CUDA;
  nt.udirty = true;
  if (loss_out) {
    if (cudaMemcpyAsync(loss_out, s->loss, 8, cudaMemcpyDeviceToHost, st)) return FLINT_ERR_CUDA;
    if (cudaStreamSynchronize(st)) return FLINT_ERR_CUDA;
  }
  return 0;
}

int surrogate_state(Surrogate* s, int net, float* host, int64_t* step, int get) {
  if (net < 0 || net >= s->nnets) return FLINT_ERR_ARG;
  Net& nt = s->net[net];
  const int64_t P = nt.P;
  cudaError_t e;
  if (get) {
    e = cudaMemcpy(host, nt.w, P * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(host + P, nt.m1, P * 4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(host + 2 * P, nt.m2, P * 4, cudaMemcpyDeviceToHost);
    if (step) *step = nt.step;
  } else {
    e = cudaMemcpy(nt.w, host, P * 4, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(nt.m1, host + P, P * 4, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(nt.m2, host + 2 * P, P * 4, cudaMemcpyHostToDevice);
    if (!e) e = launch_to_bf16(nt.w, nt.wb, P, nullptr);
    if (!e) e = cudaDeviceSynchronize();
    nt.udirty = true;
    if (step) nt.step = *step;
  }
  return e ? FLINT_ERR_CUDA : 0;
}

int64_t surrogate_nparams(Surrogate* s) { return s->net[0].P; }

int surrogate_advance(Surrogate* s, int64_t n, double* T, const double* p, double* Y, const double* dt,
                      const flint_reactor_opts& o, const flint_surrogate_gate* gate, int* status, int* nsteps,
                      double* jsave, int jslots, double* metrics, bool want_counts, cudaStream_t st,
                      int reactor_layout) {
  s->last_accepted = s->last_rejected = 0;
  s->last_n = 0;
  if (n <= 0) return 0;
  // inference in chunks of up to 1,048,576 cells; the rejected cells of all
  // chunks are listed on the device and re-solved by one reactor launch whose
  // cell count is read on the device (no host round trip before it)
  const int64_t CH = 1048576;
  if (alloc_ws(s, std::min<int64_t>(n, CH), false)) return FLINT_ERR_NOMEM;
  if (!metrics && alloc_fb(s, n)) return FLINT_ERR_NOMEM;
  GateParams gp;
  gp.max_dT_resid = gate->max_dT_resid; gp.max_elem_resid = gate->max_elem_resid; gp.min_Y = gate->min_Y;
  gp.max_ens_dT = gate->max_ens_dT; gp.max_ens_dY = gate->max_ens_dY;
  gp.Tlo = gate->T_lo; gp.Thi = gate->T_hi;
  gp.plo = std::pow(10.0, gate->log10p_lo); gp.phi = std::pow(10.0, gate->log10p_hi);
  gp.dtlo = std::pow(10.0, gate->log10dt_lo); gp.dthi = std::pow(10.0, gate->log10dt_hi);
  const size_t psm = (size_t)post_smem(s->L, s->ne).bytes;
  if (set_smem((const void*)k_post, psm)) return FLINT_ERR_CUDA;
  if (cudaMemsetAsync(s->rej_count, 0, 8, st)) return FLINT_ERR_CUDA;
  for (int64_t b = 0; b < n; b += s->cap) {
    const int64_t m = std::min<int64_t>(s->cap, n - b);
    {
      NvtxRange r("surrogate.features");
      if (surrogate_features(s, m, T + b, p + b, Y + b * s->ns, dt + b, s->xf, st)) return FLINT_ERR_CUDA;
    }
    {
      NvtxRange r("surrogate.network");
      if (net_forward(s, s->net[0], m, s->xf, s->yhat, false, st)) return FLINT_ERR_CUDA;
      if (s->nnets > 1 && net_forward(s, s->net[1], m, s->xf, s->yout2, false, st)) return FLINT_ERR_CUDA;
    }
    NvtxRange r("surrogate.gate");
    k_post<<<blocks_for(m, POST_CELLS), POST_CELLS, psm, st>>>(
        s->mimg, s->L, m, b, T, p, Y, dt, s->yhat, s->nnets > 1 ? s->yout2 : nullptr, s->ymean, s->ystd, s->G0,
        s->Bm, s->ne, gp, status, nsteps, s->rej_idx, s->rej_count, metrics ? metrics + b * 6 : nullptr);
    count_launch();
    if (cudaGetLastError()) return FLINT_ERR_CUDA;
  }
  if (metrics) return 0;
  {
    NvtxRange r("surrogate.fallback");
    k_gather<<<blocks_for(n, 256), 256, 0, st>>>(s->rej_count, s->rej_idx, s->ns, T, p, Y, dt, s->cT, s->cp, s->cY,
                                                  s->cdt);
    count_launch();
    cudaError_t e = launch_reactor(s->mimg, s->L, n, s->cT, s->cp, s->cY, s->cdt, o, s->cst, s->cns, s->counter,
                                   jsave, jslots, st, s->rej_count, reactor_layout);
    if (e) return FLINT_ERR_CUDA;
    k_scatter<<<blocks_for(n, 256), 256, 0, st>>>(s->rej_count, s->rej_idx, s->ns, T, Y, s->cT, s->cY, s->cst,
                                                   s->cns, status, nsteps);
    count_launch();
    if (cudaGetLastError()) return FLINT_ERR_CUDA;
  }
  s->last_accepted = s->last_rejected = -1;
  s->last_n = n;
  if (!want_counts) return 0;   // stays asynchronous on st (and capturable in a CUDA graph)
  unsigned long long nrej = 0;
  if (cudaMemcpyAsync(&nrej, s->rej_count, 8, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st))
    return FLINT_ERR_CUDA;
  s->last_rejected = (int64_t)nrej;
  s->last_accepted = n - (int64_t)nrej;
  return 0;
}

int surrogate_set_forward(Surrogate* s, int mode) {
  if (mode != 0 && mode != 1) return FLINT_ERR_ARG;
  s->fwd_mode = mode;
  return 0;
}

int surrogate_forward_kind(Surrogate* s) { return s->fwd_mode == 0 && s->net[0].ufits ? 0 : 1; }

// The fused forward's error word (waits for the device); 0 when no wait of it timed out.
int surrogate_check(Surrogate* s, int* err) {
  if (cudaDeviceSynchronize() != cudaSuccess) return FLINT_ERR_CUDA;
  return cudaMemcpy(err, s->uerr, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : FLINT_ERR_CUDA;
}

void surrogate_counts(Surrogate* s, int64_t* acc, int64_t* rej) { *acc = s->last_accepted; *rej = s->last_rejected; }

// Counts of the last advance read from the device (waits for the device; for
// advances made without counts, e.g. replays of a captured graph).
int surrogate_read_counts(Surrogate* s, int64_t* acc, int64_t* rej) {
  unsigned long long nrej = 0;
  if (s->last_n > 0) {
    if (cudaDeviceSynchronize() || cudaMemcpy(&nrej, s->rej_count, 8, cudaMemcpyDeviceToHost)) return FLINT_ERR_CUDA;
  }
  *rej = (int64_t)nrej;
  *acc = s->last_n - (int64_t)nrej;
  return 0;
}

}  // namespace flint
