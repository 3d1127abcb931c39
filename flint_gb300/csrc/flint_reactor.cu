// flint_reactor.cu -- persistent batched 0D constant-pressure reactor (BDF/Newton).
//
// Replaces the run_odesolver loop a FLINT caller drives over rhs_native
// (src/test/Fortran/test-batchF.f90:81,103-108; src/lib/Lib_Chemistry_rhs.f90:15-52),
// with the analytic Jacobian of the constant-pressure system instead of
// finite differences.
//
// Execution model: one warp integrates one cell; component i of the state
// x = (Y_0..Y_{ns-1}, T) lives on lane i (ns + 1 <= 32).  The kernel is
// persistent (one wave of blocks) and warps fetch the next cell from a global
// atomic counter, so cells with very uneven step counts keep every warp busy.
// Every decision (step size, order, convergence) is made from warp-reduced
// norms that the xor-butterfly makes bit-identical on all lanes, so control
// flow stays warp-uniform.  All loops are bounded: max_steps accepted steps,
// at most 10 Newton failures and 7 error-test failures per step.
//
// Algorithm (identical to the oracle's bdf_cell): fixed-leading-coefficient
// Nordsieck BDF of order 1-5, modified Newton with a Jacobian/LU refresh when
// gamma moves by more than 30 %, every 20 steps or after a convergence
// failure with a stale matrix; step and order chosen every q+1 steps from the
// order q-1, q, q+1 error estimates; Newton converged in the weighted max norm;
// after an error-test failure with a stale Jacobian, a fresh one.  A cell whose
// integration fails is integrated again at order <= 2, then 1.  The Newton matrix I - gamma*J is factored
// in shared memory by a row-per-lane LU with partial pivoting that records the
// pivot order instead of swapping rows.  Step-size factors eta = (c*dsm)^(-1/(q+1))
// are heuristics and are evaluated in FP32 (the oracle does the same); every
// quantity of the solution itself stays FP64.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "flint_dev.cuh"
#include "flint_host.h"

namespace flint {

constexpr int REACTOR_THREADS = 256;
constexpr int MAX_DEVICES = 64;

// il1[q] = 1 / l_1 and Eq[q] = 1 / ((q + 1) l_1 + 1) of order q: per-order
// constants of every step, tabulated so that a step carries two fewer FP64
// divisions (each a dozen FP64-pipe instructions on this GPU).
struct BdfL { double l[6][6]; double il1[6]; double Eq[6]; };

// l^(q)_j = coefficient of x^j in prod_{i=1..q} (1 + x/i)  (Nordsieck BDF of order q).
static void bdf_coeffs(BdfL& B) {
  for (int q = 0; q < 6; ++q) {
    for (int j = 0; j < 6; ++j) B.l[q][j] = 0.0;
    B.il1[q] = 0.0; B.Eq[q] = 0.0;
  }
  for (int q = 1; q <= 5; ++q) {
    double* l = B.l[q];
    l[0] = 1.0;
    for (int i = 1; i <= q; ++i)
      for (int j = i; j >= 1; --j) l[j] += l[j - 1] / (double)i;
    B.il1[q] = 1.0 / l[1];
    B.Eq[q] = 1.0 / std::fma((double)(q + 1), l[1], 1.0);
  }
}

__constant__ BdfL c_bdf;

// Work counters of the last reactor launch (device side, summed per cell):
// [0] work-stealing cursor, [1] RHS evaluations, [2] Jacobian evaluations,
// [3] Newton iterations (LU solves), [4] accepted steps, [5] rejected attempts,
// [6] LU factorizations.
constexpr int NCOUNTERS = 7;
// Jacobian reuse (the CVODE policy): the Newton matrix I - gamma*J is rebuilt
// and factored when gamma moved by more than DGMAX or MSBP steps passed; the
// Jacobian itself is re-evaluated only every MSBJ steps or after a Newton
// failure with a stale Jacobian.  Between evaluations the last Jacobian is kept
// in a per-warp slot of global scratch (one slot per resident warp).
constexpr double DGMAX = 0.3;
constexpr int MSBP = 20;
constexpr int MSBJ = 50;
constexpr int JSLOT = 32 * 32;   // doubles per saved-Jacobian slot of up to 31 species

// Component k = lane + 32 j of the state lives in slot j (SPL slots per lane).
// inv_nv = 1 / nv, formed once per cell (a division per norm is a dozen
// FP64-pipe instructions).
template <int SPL>
__device__ inline double wrms(const double (&v)[SPL], const double (&w)[SPL], int lane, int nv, double inv_nv) {
  double t = 0.0;
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const double a = (lane + 32 * j < nv) ? v[j] * w[j] : 0.0;
    t += a * a;
  }
  return sqrt(warp_sum(t) * inv_nv);
}

// Weighted max norm (the Newton convergence test), the maximum taken on the
// bit patterns; the butterfly leaves the same value on every lane.  A NaN
// component makes the norm NaN (the iteration then counts as diverged).
template <int SPL>
__device__ inline double wmax(const double (&v)[SPL], const double (&w)[SPL], int lane, int nv) {
  long long t = 0;
#pragma unroll
  for (int j = 0; j < SPL; ++j)
    if (lane + 32 * j < nv) t = max(t, absbits(v[j] * w[j]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t = max(t, __shfl_xor_sync(FULL, t, o));
  return __longlong_as_double(t);
}

// LU of the rows (row r = lane + 32 j) held at A[r*ld ...], partial pivoting by
// the largest |a| (lowest row on ties; compared as bit patterns, see absbits);
// the pivot order goes to piv[step] and each row remembers its step in mystep
// (rows are not swapped).  Stored: L's multipliers; U with unit diagonal (each
// pivot row's entries right of the pivot divided by the pivot, by the lanes in
// parallel) and in the diagonal's place the pivot's reciprocal.  A solve then
// scales once per lane and has no per-column multiply or division (an FP64
// division is a dozen FP64-pipe instructions on this GPU, and a uniform
// per-column multiply costs a whole warp instruction for one value).
template <int SPL>
__device__ inline void warp_lu(double* A, int ld, int nv, int lane, int* piv, int (&mystep)[SPL]) {
#pragma unroll
  for (int j = 0; j < SPL; ++j) mystep[j] = (lane + 32 * j < nv) ? -1 : 1 << 20;
  for (int k = 0; k < nv; ++k) {
    long long cand = -1;
    int who = lane;
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int r = lane + 32 * j;
      if (r < nv && mystep[j] < 0) {
        const long long v = absbits(A[r * ld + k]);
        if (v > cand) { cand = v; who = r; }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long oc = __shfl_xor_sync(FULL, cand, o);
      const int ow = __shfl_xor_sync(FULL, who, o);
      if (oc > cand || (oc == cand && ow < who)) { cand = oc; who = ow; }
    }
#pragma unroll
    for (int j = 0; j < SPL; ++j)
      if (lane + 32 * j == who) mystep[j] = k;
    if (lane == 0) piv[k] = who;
    double* prow = A + who * ld;
    const double inv = 1.0 / prow[k];
    __syncwarp();
    // U row of the pivot: entries right of the pivot scaled to a unit diagonal;
    // the pivot's reciprocal in the diagonal's place
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int c = lane + 32 * j;
      if (c > k && c < nv) prow[c] *= inv;
    }
    if (lane == (who & 31)) prow[k] = inv;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int r = lane + 32 * j;
      if (r < nv && mystep[j] < 0) {
        double* row = A + r * ld;
        const double a = row[k];
        row[k] = a * inv;
        for (int c = k + 1; c < nv; ++c) row[c] -= a * prow[c];
      }
    }
    __syncwarp();
  }
}

// Solve (LU) x = b; component r = lane + 32 j of b in slot j in, x out.
template <int SPL>
__device__ inline void warp_lu_solve(const double* A, int ld, int nv, int lane, const int* piv,
                                     const int (&mystep)[SPL], double (&b)[SPL]) {
  // forward: y_k = b_{piv[k]}; rows pivoted later subtract L * y_k
  for (int k = 0; k < nv; ++k) {
    const int pk = piv[k];
    const double src = (SPL == 1 || (pk >> 5) == 0) ? b[0] : b[SPL - 1];
    const double yk = __shfl_sync(FULL, src, pk & 31);
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int r = lane + 32 * j;
      if (r < nv && mystep[j] > k) b[j] -= A[r * ld + k] * yk;
    }
  }
  // backward by columns on the unit-diagonal U: each row's y first divided by
  // its pivot (the stored reciprocal), then x_c = y_{piv[c]}
  double x[SPL];
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    x[j] = 0.0;
    const int r = lane + 32 * j;
    if (r < nv) b[j] *= A[r * ld + mystep[j]];
  }
  for (int c = nv - 1; c >= 0; --c) {
    const int pc = piv[c];
    const double src = (SPL == 1 || (pc >> 5) == 0) ? b[0] : b[SPL - 1];
    const double xc = __shfl_sync(FULL, src, pc & 31);
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int r = lane + 32 * j;
      if (r < nv && mystep[j] < c) b[j] -= A[r * ld + c] * xc;
      if (r == c) x[j] = xc;
    }
  }
#pragma unroll
  for (int j = 0; j < SPL; ++j) b[j] = x[j];
}

// Newton matrix refresh: the Jacobian evaluation (when asked for; it also
// refreshes the saved copy Jg) or its reload from Jg, M = I - gamma J, and the
// LU factorization.  The pivot order goes to pivs[0 .. 32 SPL) and each row's
// pivot step to pivs[32 SPL + row].  Inlined: an out-of-line version (to keep
// the Newton loop's code compact) measured 3 % slower on the 31-species
// workload and equal on the 54-species one.
template <int SPL>
__device__ __forceinline__ void refresh_newton_matrix(MechView m, WarpScratch s, int lane, double p, bool cv,
                                                   double gamma, int eval_J, double ya, double yb, double* Jg,
                                                   int* pivs) {
  constexpr int JW = 32 * SPL;
  const int ns = m.ns, nv = ns + 1, ld = s.ldj;
  const int Tslot = ns >> 5, Tlane = ns & 31;
  if (eval_J) {
    const double Tv = __shfl_sync(FULL, (SPL == 1 || Tslot == 0) ? ya : yb, Tlane);
    double yk[SPL];
    yk[0] = (lane < ns) ? ya : 0.0;
    if (SPL > 1) yk[SPL - 1] = (lane + 32 < ns) ? yb : 0.0;
    CellOutT<SPL> co;
    warp_kinetics<true, SPL>(m, s, lane, yk, Tv, p, co, cv);
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int r = lane + 32 * j;
      if (r < nv) {
        const double* row = s.Jr + r * ld;
        for (int c = 0; c < nv; ++c) Jg[c * JW + r] = row[c];
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int r = lane + 32 * j;
      if (r < nv) {
        double* row = s.Jr + r * ld;
        for (int c = 0; c < nv; ++c) row[c] = Jg[c * JW + r];
      }
    }
  }
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int r = lane + 32 * j;
    if (r < nv) {
      double* row = s.Jr + r * ld;
      for (int c = 0; c < nv; ++c) row[c] = (c == r ? 1.0 : 0.0) - gamma * row[c];
    }
  }
  __syncwarp();
  int mystep[SPL];
  warp_lu<SPL>(s.Jr, ld, nv, lane, pivs, mystep);
#pragma unroll
  for (int j = 0; j < SPL; ++j) pivs[32 * SPL + lane + 32 * j] = mystep[j];
  __syncwarp();
}

// Layout choice: the Newton matrix and the Jacobian work area live in shared
// memory (SPL = 1 and the block fits), or in the warp's global slot (GJ).
static int spl_of(const ImageLayout& L) { return L.nsp / 32; }

static size_t reactor_smem_spl1(const ImageLayout& L) {
  return L.bytes + (REACTOR_THREADS / 32) * (scratch_doubles(L.nsp, L.nrpad, true) * sizeof(double) + 64 * sizeof(int));
}

// layout: REACTOR_LAYOUT_AUTO picks shared memory whenever the block fits;
// REACTOR_LAYOUT_SHARED / _GLOBAL force one (the autotuner times both).
// REACTOR_LAYOUT_GLOBAL2B: global slots, two blocks of 8 warps per SM (16
// resident warps) from a build capped at 128 registers per thread.
static bool reactor_gj(const ImageLayout& L, int layout = REACTOR_LAYOUT_AUTO) {
  if (spl_of(L) > 1 || reactor_smem_spl1(L) > device_smem_optin()) return true;
  return layout == REACTOR_LAYOUT_GLOBAL || layout == REACTOR_LAYOUT_GLOBAL4 || layout == REACTOR_LAYOUT_GLOBAL2B;
}

// Threads per block: 8 warps, or 4 in the GLOBAL4 layout (half the resident
// warps, twice the L1 per warp for the global Newton matrices).
static int reactor_threads(int layout) { return layout == REACTOR_LAYOUT_GLOBAL4 ? 128 : REACTOR_THREADS; }

// Doubles per resident-warp slot of the reactor's global scratch: the saved
// Jacobian (32*SPL)^2, and in GJ layout the Jacobian work area too.
static int64_t reactor_slot_doubles_of(const ImageLayout& L, int layout = REACTOR_LAYOUT_AUTO) {
  const int spl = spl_of(L);
  return (int64_t)(32 * spl) * (32 * spl) + (reactor_gj(L, layout) ? scratch_jac_doubles(L.nsp, L.nrpad) : 0);
}

template <int SPL, bool GJ, int MINB = 1>
__global__ void __launch_bounds__(REACTOR_THREADS, MINB)
k_reactor(const uint8_t* __restrict__ img, ImageLayout L, int64_t n, double* __restrict__ Tg,
          const double* __restrict__ pg, double* __restrict__ Yg, const double* __restrict__ dtg,
          flint_reactor_opts o, int* __restrict__ status_g, int* __restrict__ nsteps_g,
          unsigned long long* __restrict__ counter, double* __restrict__ jsave, int64_t slot_doubles,
          const unsigned long long* __restrict__ n_dev) {
  extern __shared__ __align__(16) uint8_t smem[];
  if (n_dev) n = min(n, (int64_t)*n_dev);   // cell count produced on the device
  stage_image(smem, img, L.bytes);
  MechView m;
  m.bind(L, smem);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid;
  double* Jg = jsave + slot * slot_doubles;
  constexpr int JW = 32 * SPL;   // row stride of the saved Jacobian
  WarpScratch s;
  int* pivs;
  if (!GJ) {
    const int sd = scratch_doubles(m.nsp, m.nrpad, true);
    double* wbase = reinterpret_cast<double*>(smem + L.bytes) + wid * sd;
    s = carve(wbase, m.nsp, m.nrpad, true);
    pivs = reinterpret_cast<int*>(reinterpret_cast<double*>(smem + L.bytes) + (blockDim.x >> 5) * sd) + wid * 64;
  } else {
    const int sd = scratch_small_doubles(m.nsp, m.nrpad);
    double* wbase = reinterpret_cast<double*>(smem + L.bytes) + wid * sd;
    s = carve2(wbase, Jg + JW * JW, m.nsp, m.nrpad);
    pivs = reinterpret_cast<int*>(reinterpret_cast<double*>(smem + L.bytes) + (blockDim.x >> 5) * sd) + wid * 64 * SPL;
  }
  const int ns = m.ns, nv = ns + 1;
  const double inv_nv = 1.0 / nv;
  const int ld = s.ldj;
  const BdfL& B = c_bdf;
  unsigned long long n_rhs = 0, n_jac = 0, n_newt = 0, n_rej = 0, n_lu = 0;

  while (true) {
    unsigned long long c0 = 0;
    if (lane == 0) c0 = atomicAdd(counter, 1ull);
    const int64_t cell = (int64_t)__shfl_sync(FULL, c0, 0);
    if (cell >= n) break;

    const double p = pg[cell], tout = dtg[cell];
    double y[SPL];
    int bad = 0;
#pragma unroll
    for (int j = 0; j < SPL; ++j) {
      const int k = lane + 32 * j;
      y[j] = 0.0;
      if (k < ns) y[j] = Yg[cell * ns + k];
      else if (k == ns) y[j] = Tg[cell];
      if (k < nv && !isfinite(y[j])) bad = 1;
    }
    const double T0 = Tg[cell];
    bad |= !(isfinite(T0) && isfinite(p) && p > 0.0 && isfinite(tout) && tout >= 0.0);
    bad = __any_sync(FULL, bad);
    // constant volume: the kinetics take the density, fixed at its initial
    // value p / (R T sum Y/W)
    const bool cv = o.constant_volume != 0;
    double pr = p;
    if (cv) {
      double yw = 0.0;
#pragma unroll
      for (int j = 0; j < SPL; ++j)
        if (lane + 32 * j < ns) yw += y[j] * m.invmw[lane + 32 * j];
      pr = p / (m.r_eos * T0 * warp_sum(yw));
    }
    int status = FLINT_CELL_OK, nst = 0;
    if (bad) status = FLINT_CELL_NAN_INPUT;
    else if (T0 < o.tmin || T0 > o.tmax) status = FLINT_CELL_T_OUT_OF_RANGE;

    if (status == FLINT_CELL_OK && tout > 0.0) {
      double z[6][SPL], zs[6][SPL], e[SPL], eprev[SPL], ewt[SPL], f[SPL];
      int nst_total = 0;
      // attempt 0 with the caller's options; a cell that fails the error test
      // or Newton is integrated again from its initial state at order <= 2
      // with atol / 100 (BDF1-2 are A-stable, orders 3-5 are not), then at
      // order 1.  nsteps counts the steps of every attempt.
      for (int att = 0; att < 3; ++att) {
      const int qmax = att == 0 ? o.max_order : (att == 1 ? min(o.max_order, 2) : 1);
      const double atol = att == 1 ? o.atol * 1e-2 : o.atol;
      status = FLINT_CELL_OK;
      nst = 0;
#pragma unroll
      for (int jj = 0; jj < 6; ++jj)
#pragma unroll
        for (int j = 0; j < SPL; ++j) { z[jj][j] = 0.0; zs[jj][j] = 0.0; }
#pragma unroll
      for (int j = 0; j < SPL; ++j) { e[j] = 0.0; eprev[j] = 0.0; }
      CellOutT<SPL> co;
      const int Tslot = ns >> 5, Tlane = ns & 31;
      auto rhs = [&](const double (&yv)[SPL], double (&fo)[SPL]) {
        ++n_rhs;
        const double Tv = __shfl_sync(FULL, (SPL == 1 || Tslot == 0) ? yv[0] : yv[SPL - 1], Tlane);
        double yk[SPL];
#pragma unroll
        for (int j = 0; j < SPL; ++j) yk[j] = (lane + 32 * j < ns) ? yv[j] : 0.0;
        warp_kinetics<false, SPL>(m, s, lane, yk, Tv, pr, co, cv);
        __syncwarp();
#pragma unroll
        for (int j = 0; j < SPL; ++j) fo[j] = co.f[j];
      };
#pragma unroll
      for (int j = 0; j < SPL; ++j) z[0][j] = y[j];
      rhs(y, f);
#pragma unroll
      for (int j = 0; j < SPL; ++j) ewt[j] = (lane + 32 * j < nv) ? 1.0 / (o.rtol * fabs(y[j]) + atol) : 0.0;
      const double fn = wrms<SPL>(f, ewt, lane, nv, inv_nv);
      double h = (fn * tout > 1.0) ? 1.0 / fn : tout;
#pragma unroll
      for (int j = 0; j < SPL; ++j) z[1][j] = h * f[j];
      int q = 1;
      double t = 0.0;
      int ialth = 2, have_J = 0, jfresh = 0, nstJ = 0, nstP = 0, have_eprev = 0, last = 0;
      double gammaJ = 0.0, crate = 1.0, etamax = 1.0e4;
      int mystep[SPL];
#pragma unroll
      for (int j = 0; j < SPL; ++j) mystep[j] = 0;

      while (t < tout) {
        if (nst >= o.max_steps) { status = FLINT_CELL_MAX_STEPS; break; }
        last = 0;
        if (t + h >= tout) {
          const double eta = (tout - t) / h;
          double r = 1.0;
#pragma unroll
          for (int jj = 1; jj <= 5; ++jj) if (jj <= q) { r *= eta; for (int j = 0; j < SPL; ++j) z[jj][j] *= r; }
          h = tout - t;
          ialth = q + 1; have_eprev = 0; last = 1;
        }
#pragma unroll
        for (int j = 0; j < SPL; ++j) ewt[j] = (lane + 32 * j < nv) ? 1.0 / (o.rtol * fabs(z[0][j]) + atol) : 0.0;
        int ncf = 0, nef = 0, need_J = 0, accepted = 0;
        double dsm = 0.0;
        // the first Newton iterate of a step is judged with a rate of at least
        // 0.3: a small rate carried over from the last step would accept it unchecked
        if (crate < 0.3) crate = 0.3;
        while (!accepted) {
          if (h < 1e-300 || t + h == t) { status = FLINT_CELL_ERRTEST_FAIL; break; }
#pragma unroll
          for (int jj = 0; jj < 6; ++jj)
#pragma unroll
            for (int j = 0; j < SPL; ++j) zs[jj][j] = z[jj][j];
          // predict: z <- z * Pascal
#pragma unroll
          for (int k = 0; k < 5; ++k)
#pragma unroll
            for (int jj = 4; jj >= 0; --jj)
              if (k < q && jj >= k && jj <= q - 1)
#pragma unroll
                for (int j = 0; j < SPL; ++j) z[jj][j] += z[jj + 1][j];
          const double l1 = B.l[q][1];
          const double gamma = h / l1;
          double ypred[SPL];
#pragma unroll
          for (int j = 0; j < SPL; ++j) ypred[j] = z[0][j];
          // gamma / gammaJ once per attempt: the refresh test and the Newton
          // correction scale share it (1 after a refresh)
          double gamrat = 1.0;
          bool refresh = !have_J || need_J || nst >= nstP + MSBP;
          if (!refresh) {
            gamrat = gamma / gammaJ;
            refresh = fabs(gamrat - 1.0) > DGMAX;
          }
          if (refresh) {
            const int eval_J = (!have_J || need_J || nst >= nstJ + MSBJ) ? 1 : 0;
            if (eval_J) {
              ++n_jac;
              have_J = 1; jfresh = 1; nstJ = nst; need_J = 0;
            }
            refresh_newton_matrix<SPL>(m, s, lane, pr, cv, gamma, eval_J, ypred[0], ypred[SPL - 1], Jg, pivs);
#pragma unroll
            for (int j = 0; j < SPL; ++j) mystep[j] = pivs[32 * SPL + lane + 32 * j];
            ++n_lu;
            gammaJ = gamma; nstP = nst; crate = 1.0;
            gamrat = 1.0;
          }
          double yv[SPL];
#pragma unroll
          for (int j = 0; j < SPL; ++j) { e[j] = 0.0; yv[j] = ypred[j]; }
          int conv = 0;
          double delp = 0.0;
          const double Eq = B.Eq[q];
          const double il1 = B.il1[q];
          const double sc = gamrat != 1.0 ? 2.0 / (1.0 + gamrat) : 1.0;
          for (int mi = 0; mi < 3; ++mi) {
            ++n_newt;
            rhs(yv, f);
            double bv[SPL];
#pragma unroll
            for (int j = 0; j < SPL; ++j) bv[j] = (lane + 32 * j < nv) ? gamma * f[j] - z[1][j] * il1 - e[j] : 0.0;
            warp_lu_solve<SPL>(s.Jr, ld, nv, lane, pivs, mystep, bv);
            if (gamrat != 1.0) {
#pragma unroll
              for (int j = 0; j < SPL; ++j) bv[j] *= sc;
            }
            const double del = wmax<SPL>(bv, ewt, lane, nv);
#pragma unroll
            for (int j = 0; j < SPL; ++j) { e[j] += bv[j]; yv[j] = ypred[j] + e[j]; }
            if (mi > 0) { const double r = del / delp; crate = (0.3 * crate > r) ? 0.3 * crate : r; }
            const double dcon = del * (crate < 1.0 ? crate : 1.0) * Eq * 10.0;   // test constant 0.1
            if (dcon <= 1.0) { conv = 1; break; }
            if (mi > 0 && !(del <= 2.0 * delp)) break;
            delp = del;
          }
          if (!conv) {
#pragma unroll
            for (int jj = 0; jj < 6; ++jj)
#pragma unroll
              for (int j = 0; j < SPL; ++j) z[jj][j] = zs[jj][j];
            ++ncf;
            ++n_rej;
            if (ncf >= 10) { status = FLINT_CELL_NEWTON_FAIL; break; }
            if (!jfresh) { need_J = 1; continue; }
            const double eta = 0.25;
            double r = 1.0;
#pragma unroll
            for (int jj = 1; jj <= 5; ++jj) if (jj <= q) { r *= eta; for (int j = 0; j < SPL; ++j) z[jj][j] *= r; }
            h *= eta; ialth = q + 1; have_eprev = 0; need_J = 1; last = 0;
            continue;
          }
          dsm = Eq * wrms<SPL>(e, ewt, lane, nv, inv_nv);
          if (!(dsm <= 1.0)) {
#pragma unroll
            for (int jj = 0; jj < 6; ++jj)
#pragma unroll
              for (int j = 0; j < SPL; ++j) z[jj][j] = zs[jj][j];
            ++nef;
            ++n_rej;
            if (nef >= 7) { status = FLINT_CELL_ERRTEST_FAIL; break; }
            double eta;
            if (nef >= 3) {
              eta = 0.1;
              if (q > 1) q = 1;
            } else {
              eta = 1.0 / ((double)powf((float)(1.2 * dsm), 1.0f / (float)(q + 1)) + 1e-6);
              if (eta > 0.9) eta = 0.9;
              if (eta < 0.1) eta = 0.1;
            }
            double r = 1.0;
#pragma unroll
            for (int jj = 1; jj <= 5; ++jj) if (jj <= q) { r *= eta; for (int j = 0; j < SPL; ++j) z[jj][j] *= r; }
            h *= eta; ialth = q + 1; have_eprev = 0; last = 0;
            if (!jfresh) need_J = 1;   // retry with a Jacobian of this state
            continue;
          }
          accepted = 1;
        }
        if (status != FLINT_CELL_OK) break;
        t += h;
        ++nst;
        jfresh = 0;
#pragma unroll
        for (int jj = 0; jj <= 5; ++jj) if (jj <= q) for (int j = 0; j < SPL; ++j) z[jj][j] += B.l[q][jj] * e[j];
        if (last || t >= tout) { t = tout; break; }
        --ialth;
        double eta = 1.0;
        if (ialth <= 0) {
          const double l1 = B.l[q][1];
          const double etaq = 1.0 / ((double)powf((float)(1.2 * dsm), 1.0f / (float)(q + 1)) + 1.2e-6);
          double etadn = 0.0, etaup = 0.0;
          if (q > 1) {
            double fact = 1.0;
            for (int i = 2; i <= q; ++i) fact *= i;
            double zq[SPL];
#pragma unroll
            for (int j = 0; j < SPL; ++j) {
              zq[j] = 0.0;
#pragma unroll
              for (int jj = 2; jj <= 5; ++jj) if (jj == q) zq[j] = z[jj][j];
            }
            const double ddn = wrms<SPL>(zq, ewt, lane, nv, inv_nv) * fact / ((double)q * B.l[q - 1][1]);
            etadn = 1.0 / ((double)powf((float)(1.3 * ddn), 1.0f / (float)q) + 1.3e-6);
          }
          if (q < qmax && have_eprev) {
            const double Kq = 1.0 + 1.0 / ((double)(q + 1) * l1);
            double de[SPL];
#pragma unroll
            for (int j = 0; j < SPL; ++j) de[j] = e[j] - eprev[j];
            const double dup = wrms<SPL>(de, ewt, lane, nv, inv_nv) / (Kq * (double)(q + 2) * B.l[q + 1][1]);
            etaup = 1.0 / ((double)powf((float)(1.4 * dup), 1.0f / (float)(q + 2)) + 1.4e-6);
          }
          int newq = q;
          eta = etaq;
          if (etaup > eta && etaup >= etadn) { eta = etaup; newq = q + 1; }
          else if (etadn > eta) { eta = etadn; newq = q - 1; }
          if (newq == q + 1) {
            const double fct = B.l[q][q] / (double)(q + 1);
#pragma unroll
            for (int jj = 2; jj <= 5; ++jj) if (jj == q + 1) for (int j = 0; j < SPL; ++j) z[jj][j] = e[j] * fct;
          }
          if (eta < 1.1 && newq == q) {
            eta = 1.0;
            ialth = 3;
          } else {
            q = newq;
            if (eta > etamax) eta = etamax;
            ialth = q + 1;
          }
          have_eprev = 0;
          etamax = 10.0;
        } else if (ialth == 1 && q < qmax) {
#pragma unroll
          for (int j = 0; j < SPL; ++j) eprev[j] = e[j];
          have_eprev = 1;
        }
        if (eta != 1.0) {
          double r = 1.0;
#pragma unroll
          for (int jj = 1; jj <= 5; ++jj) if (jj <= q) { r *= eta; for (int j = 0; j < SPL; ++j) z[jj][j] *= r; }
          h *= eta;
        }
      }
      nst_total += nst;
      if (status != FLINT_CELL_ERRTEST_FAIL && status != FLINT_CELL_NEWTON_FAIL) break;
      }  // attempts
      nst = nst_total;
      if (lane == 0) atomicAdd(counter + 4, (unsigned long long)nst);
#pragma unroll
      for (int j = 0; j < SPL; ++j) {
        const int k = lane + 32 * j;
        if (k < ns) Yg[cell * ns + k] = z[0][j];
        else if (k == ns) Tg[cell] = z[0][j];
      }
    }
    if (lane == 0) {
      if (status_g) status_g[cell] = status;
      if (nsteps_g) nsteps_g[cell] = nst;
    }
    __syncwarp();
  }
  if (lane == 0) {
    atomicAdd(counter + 1, n_rhs);
    atomicAdd(counter + 2, n_jac);
    atomicAdd(counter + 3, n_newt);
    atomicAdd(counter + 5, n_rej);
    atomicAdd(counter + 6, n_lu);
  }
}

size_t reactor_smem(const ImageLayout& L, int layout = REACTOR_LAYOUT_AUTO) {
  if (!reactor_gj(L, layout)) return reactor_smem_spl1(L);
  return L.bytes + (reactor_threads(layout) / 32) *
                       (scratch_small_doubles(L.nsp, L.nrpad) * sizeof(double) + 64 * spl_of(L) * sizeof(int));
}

static const void* reactor_fn(const ImageLayout& L, int layout = REACTOR_LAYOUT_AUTO) {
  const bool two = layout == REACTOR_LAYOUT_GLOBAL2B;
  if (spl_of(L) > 1) return two ? (const void*)k_reactor<2, true, 2> : (const void*)k_reactor<2, true>;
  if (two) return (const void*)k_reactor<1, true, 2>;
  return reactor_gj(L, layout) ? (const void*)k_reactor<1, true> : (const void*)k_reactor<1, false>;
}

static int slots_of(const ImageLayout& L, int layout) {
  size_t sm = reactor_smem(L, layout);
  const void* fn = reactor_fn(L, layout);
  if (set_smem(fn, sm) != cudaSuccess) return 0;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, reactor_threads(layout), sm);
  return per_sm * device_sms() * (reactor_threads(layout) / 32);
}

// Resident-warp slots and bytes per slot that serve every layout.
int reactor_slots(const ImageLayout& L) {
  if (spl_of(L) < 1 || spl_of(L) > 2) return 0;
  return std::max(std::max(slots_of(L, REACTOR_LAYOUT_AUTO), slots_of(L, REACTOR_LAYOUT_GLOBAL2B)),
                  std::max(slots_of(L, REACTOR_LAYOUT_GLOBAL), slots_of(L, REACTOR_LAYOUT_GLOBAL4)));
}

size_t reactor_slot_bytes(const ImageLayout& L) {
  return (size_t)std::max(reactor_slot_doubles_of(L, REACTOR_LAYOUT_AUTO), reactor_slot_doubles_of(L, REACTOR_LAYOUT_GLOBAL)) *
         sizeof(double);
}

int reactor_layout_candidates(const ImageLayout& L, int* out) {
  int k = 0;
  if (spl_of(L) == 1 && reactor_smem_spl1(L) <= device_smem_optin()) out[k++] = REACTOR_LAYOUT_SHARED;
  out[k++] = REACTOR_LAYOUT_GLOBAL;
  out[k++] = REACTOR_LAYOUT_GLOBAL4;
  out[k++] = REACTOR_LAYOUT_GLOBAL2B;
  return k;
}

// The BDF coefficient table lives in __constant__ memory, one copy per device,
// uploaded by the first launch on that device (with it current).
static cudaError_t ensure_bdf_table() {
  static std::mutex bdf_mu;
  static bool bdf_ready[MAX_DEVICES] = {false};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(bdf_mu);
  if (!bdf_ready[dev]) {
    BdfL B;
    bdf_coeffs(B);
    e = cudaMemcpyToSymbol(c_bdf, &B, sizeof(B));
    if (e != cudaSuccess) return e;
    bdf_ready[dev] = true;
  }
  return cudaSuccess;
}

cudaError_t launch_reactor(const uint8_t* img, const ImageLayout& L, int64_t n, double* T, const double* p,
                           double* Y, const double* dt, const flint_reactor_opts& o, int* status, int* nsteps,
                           unsigned int* work_counter, double* jsave, int slots, cudaStream_t st,
                           const unsigned long long* n_dev, int layout) {
  if (n <= 0) return cudaSuccess;
  if (spl_of(L) < 1 || spl_of(L) > 2) return cudaErrorInvalidValue;
  NvtxRange nvtx("reactor.advance");
  size_t sm = reactor_smem(L, layout);
  const void* fn = reactor_fn(L, layout);
  cudaError_t e = set_smem(fn, sm);
  if (e != cudaSuccess) return e;
  const int threads = reactor_threads(layout), wpb = threads / 32;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, sm);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t warps_needed = n;
  int64_t blocks = (warps_needed + wpb - 1) / wpb;
  int64_t full = (int64_t)device_sms() * per_sm;
  if (blocks > full) blocks = full;
  if (blocks * wpb > slots) blocks = slots / wpb;
  if (blocks < 1) return cudaErrorInvalidValue;
  e = ensure_bdf_table();
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(work_counter, 0, NCOUNTERS * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  const int64_t sd = reactor_slot_doubles_of(L, layout);
  unsigned long long* wc = reinterpret_cast<unsigned long long*>(work_counter);
  if (layout == REACTOR_LAYOUT_GLOBAL2B && spl_of(L) > 1)
    k_reactor<2, true, 2><<<(unsigned)blocks, threads, sm, st>>>(img, L, n, T, p, Y, dt, o, status, nsteps, wc,
                                                                          jsave, sd, n_dev);
  else if (layout == REACTOR_LAYOUT_GLOBAL2B)
    k_reactor<1, true, 2><<<(unsigned)blocks, threads, sm, st>>>(img, L, n, T, p, Y, dt, o, status, nsteps, wc,
                                                                          jsave, sd, n_dev);
  else if (spl_of(L) > 1)
    k_reactor<2, true><<<(unsigned)blocks, threads, sm, st>>>(img, L, n, T, p, Y, dt, o, status, nsteps, wc,
                                                                       jsave, sd, n_dev);
  else if (reactor_gj(L, layout))
    k_reactor<1, true><<<(unsigned)blocks, threads, sm, st>>>(img, L, n, T, p, Y, dt, o, status, nsteps, wc,
                                                                       jsave, sd, n_dev);
  else
    k_reactor<1, false><<<(unsigned)blocks, threads, sm, st>>>(img, L, n, T, p, Y, dt, o, status, nsteps, wc,
                                                                        jsave, sd, n_dev);
  count_launch();
  return cudaGetLastError();
}


// ------------------------------------------------------- allocation-free entry
// Some callers cannot let a library call cudaMalloc: CFD solvers that reserve
// their whole device-memory budget for their own pool at start-up (a later
// allocation by a library fails or fragments that pool) and codes whose
// certification or real-time rules forbid device allocation after
// initialisation.  flint_reactor_advance_noalloc serves them: the reactor's
// scratch (its work-stealing and statistics counters and one saved-Jacobian
// slot per resident warp) lives in this file-scope device array instead of
// memory allocated by the handle.  Every GPU that loads the library holds it
// until the process exits.  With CUDA's lazy module loading (the default) the
// driver gives the array device memory only when this file's module is first
// used on a device; the n = 0 call (launch_reactor_noalloc_prepare) does that
// and every other one-time step, so a caller makes it before its own pool
// takes the device memory and before any stream capture.
constexpr int NOALLOC_SLOTS = 1280;                  // saved-Jacobian slots of 32 x 32 FP64
constexpr size_t NOALLOC_COUNTER_BYTES = 256;        // counters, zeroed by every call
constexpr size_t NOALLOC_BYTES = NOALLOC_COUNTER_BYTES + (size_t)NOALLOC_SLOTS * JSLOT * sizeof(double);
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Host-side address of g_noalloc_scratch on each device: the symbol's name is
// only a host stand-in, the kernel needs the device address, looked up once
// per device (with that device current) by cudaGetSymbolAddress.
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[MAX_DEVICES] = {nullptr};

static cudaError_t noalloc_scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = ptr;
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

size_t reactor_noalloc_bytes() { return NOALLOC_BYTES; }
// Only the shared-memory layout keeps a warp's scratch within one 32 x 32
// slot; the entry point always runs it (a layout chosen by
// flint_reactor_autotune applies to flint_reactor_advance only).
bool reactor_noalloc_fits(const ImageLayout& L) { return reactor_slot_doubles_of(L) <= JSLOT; }
int reactor_noalloc_slots() { return NOALLOC_SLOTS; }

// One-time set-up on the current device, without a launch: module load (and
// with it the static array's device memory), the array's address, the BDF
// table and the kernel's shared-memory attribute.
cudaError_t launch_reactor_noalloc_prepare(const ImageLayout& L) {
  if (!reactor_noalloc_fits(L)) return cudaErrorInvalidValue;
  void* base = nullptr;
  cudaError_t e = noalloc_scratch_address(&base);
  if (e != cudaSuccess) return e;
  e = ensure_bdf_table();
  if (e != cudaSuccess) return e;
  return set_smem(reactor_fn(L), reactor_smem(L));
}

cudaError_t launch_reactor_noalloc(const uint8_t* img, const ImageLayout& L, int64_t n, double* T, const double* p,
                                   double* Y, const double* dt, const flint_reactor_opts& o, int* status,
                                   int* nsteps, cudaStream_t st) {
  if (!reactor_noalloc_fits(L)) return cudaErrorInvalidValue;
  if (n <= 0) return launch_reactor_noalloc_prepare(L);
  void* base = nullptr;
  cudaError_t e = noalloc_scratch_address(&base);
  if (e != cudaSuccess) return e;
  unsigned int* counters = reinterpret_cast<unsigned int*>(base);
  double* jsave = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + NOALLOC_COUNTER_BYTES);
  // launch_reactor zeroes the counters on `st` and caps the grid to the slots
  return launch_reactor(img, L, n, T, p, Y, dt, o, status, nsteps, counters, jsave, NOALLOC_SLOTS, st);
}

}  // namespace flint
