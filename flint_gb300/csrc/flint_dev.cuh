// flint_dev.cuh -- device-side mechanism image and warp-per-cell kinetics.
//
// One warp owns one cell.  Species-parallel work (thermo, production sums,
// Jacobian rows) maps species k to lane k (k + 32 for the second row block);
// reaction-parallel work (rate constants, rates of progress) maps reaction r
// to lane r % 32 in rounds of 32.  The mechanism image is staged once per
// block in shared memory as structure-of-arrays so that the 32 lanes of a
// round read 32 consecutive words (no bank conflicts).
//
// Math follows FLINT's chemistry path (paths within the FLINT project):
//   rates of progress, third body, species sums  src/lib/Lib_Chemistry_wdot.f90:96-220
//   Lindemann / Troe blending, f_F              src/lib/Lib_Chemistry_falloff.f90:12-80
//   reverse rate kb = kf / kc                   src/lib/Lib_Chemistry_falloff.f90:31,56
// with kf, kc, Fcent evaluated from the Arrhenius / NASA-7 / Troe parameters
// the reference's tables were generated from (Kc = exp(-dG/RT)(p_ref/RT)^dnu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace flint {

constexpr int WARP = 32;
constexpr int MAXSIDE = 3;
constexpr unsigned FULL = 0xffffffffu;

// Reaction code word: bits 0-1 type, bit 2 reversible, bits 8-15 third-body
// row, bits 16-27 order codes of the 3 reactant slots (4 bits each) and
// bits 28-31 unused.  Order code: 0 absent, 1..3 integral power, 4 general pow.
__host__ __device__ inline int rx_type(uint32_t w) { return w & 3; }
__host__ __device__ inline bool rx_rev(uint32_t w) { return (w >> 2) & 1; }
__host__ __device__ inline int rx_tbrow(uint32_t w) { return (w >> 8) & 0xff; }
__host__ __device__ inline int rx_ordcode(uint32_t w, int s) { return (w >> (16 + 4 * s)) & 0xf; }

// Offsets (in bytes) of each section of the packed image.  All sections are
// 16-byte aligned; the image is copied to shared memory with 16-byte loads.
struct ImageLayout {
  int ns, nr, nrpad, nsp;        // nsp = species padded to a multiple of 32
  int ntb;                       // rows of third-body efficiencies
  int nlist;                     // CSR entries (species -> reactions)
  int bytes;                     // total image size
  double r_eos, r_thermo, lnpref_rth;   // ln(p_ref / r_thermo)
  double inv_r_eos;                     // 1 / r_eos
  // species
  int o_mw, o_invmw, o_nasa;     // nasa: [16][nsp] : low a0..a6, high a0..a6, tmid, unused
  int o_nasah;                   // [16][nsp]: low a1/2, a2/3, a3/4, a4/5, a2/2, a3/3, a4/4, 0; high the same
                                 // (the h and s polynomials' coefficients, divided once on the host)
  // reactions (nrpad each)
  int o_A, o_b, o_E, o_A0, o_b0, o_E0, o_tr;   // tr: [4][nrpad] = a, 1/T3, 1/T1, T2
  // falloff: the image stores the low-pressure limit relative to the high-
  // pressure one, k0/kinf = A0r T^b0r exp(-E0r/T) with A0r = A0/A, b0r = b0-b,
  // E0r = (Ea0-Ea)/R, so Pr = (k0/kinf) M costs one exp and no division.
  int o_rnu, o_rord, o_pnu;      // [3][nrpad]
  int o_rsp, o_psp;              // int32 [3][nrpad]
  int o_code;                    // uint32 [nrpad]
  int o_pcode;                   // uint32 [nrpad]: product order codes, 4 bits per slot
  int o_dnu;                     // double [nrpad]
  // third-body rows, sparse: M_t = tbd[t] * sum_k c_k + sum over e in
  // [tbp[t], tbp[t+1]) of tbv[e] * c[tbs[e]], tbd[t] the row's most common
  // efficiency and tbv the others minus tbd[t]
  int o_tbd;                     // double [ntb]
  int o_tbp;                     // int32 [ntb+1]
  int o_tbs;                     // int32 [ntbl]
  int o_tbv;                     // double [ntbl]
  int o_cstart;                  // int32 [nsp+1]
  int o_lr;                      // int32 [nlist]
  int o_lnu;                     // double [nlist]
  int o_exptab;                  // double [256]: 2^(j/256)
  int nfall;                     // falloff reactions (the last nfall after sorting; <= 16)
  int o_nasa9;                   // NASA-9 thermo [32][nsp] (nranges, T0..T3, 3 x 9 coefficients); -1 = none
  int o_logtab;                  // double [129][3]: c_j ~ 1/(1 + j/128), -ln c_j as hi + lo (flog)
};

struct MechView {
  int ns, nr, nrpad, nsp, ntb;
  double r_eos, r_thermo, lnpref_rth, inv_r_eos;
  const double *mw, *invmw, *nasa, *nasah;
  const double *A, *b, *E, *A0, *b0, *E0, *tr;
  const double *rnu, *rord, *pnu, *dnu;
  const int *rsp, *psp, *cstart, *lr;
  const uint32_t* code;
  const uint32_t* pcode;
  const double *tbd, *tbv, *lnu, *exptab;
  const int *tbp, *tbs;
  const double* nasa9;   // null: NASA-7 (nasa)
  const double* logtab;
  int nfall;

  __host__ __device__ void bind(const ImageLayout& L, const uint8_t* base) {
    ns = L.ns; nr = L.nr; nrpad = L.nrpad; nsp = L.nsp; ntb = L.ntb; nfall = L.nfall;
    exptab = (const double*)(base + L.o_exptab);
    r_eos = L.r_eos; r_thermo = L.r_thermo; lnpref_rth = L.lnpref_rth; inv_r_eos = L.inv_r_eos;
    mw = (const double*)(base + L.o_mw); invmw = (const double*)(base + L.o_invmw);
    nasa = (const double*)(base + L.o_nasa);
    nasah = (const double*)(base + L.o_nasah);
    A = (const double*)(base + L.o_A); b = (const double*)(base + L.o_b); E = (const double*)(base + L.o_E);
    A0 = (const double*)(base + L.o_A0); b0 = (const double*)(base + L.o_b0); E0 = (const double*)(base + L.o_E0);
    tr = (const double*)(base + L.o_tr);
    rnu = (const double*)(base + L.o_rnu); rord = (const double*)(base + L.o_rord);
    pnu = (const double*)(base + L.o_pnu); dnu = (const double*)(base + L.o_dnu);
    rsp = (const int*)(base + L.o_rsp); psp = (const int*)(base + L.o_psp);
    code = (const uint32_t*)(base + L.o_code);
    pcode = (const uint32_t*)(base + L.o_pcode);
    tbd = (const double*)(base + L.o_tbd); tbv = (const double*)(base + L.o_tbv);
    tbp = (const int*)(base + L.o_tbp); tbs = (const int*)(base + L.o_tbs);
    cstart = (const int*)(base + L.o_cstart); lr = (const int*)(base + L.o_lr);
    lnu = (const double*)(base + L.o_lnu);
    nasa9 = L.o_nasa9 >= 0 ? (const double*)(base + L.o_nasa9) : nullptr;
    logtab = (const double*)(base + L.o_logtab);
  }
};

// Third-body concentration of efficiency row t (sparse form, see o_tbd):
// M = sum_k eff_k c_k with ctot = sum_k c_k.
__device__ __forceinline__ double tb_conc(const MechView& m, int t, double ctot, const double* c) {
  double M = m.tbd[t] * ctot;
  for (int e = m.tbp[t]; e < m.tbp[t + 1]; ++e) M = fma(m.tbv[e], c[m.tbs[e]], M);
  return M;
}

// Copy the image (global) into shared memory; whole block participates.
__device__ inline void stage_image(uint8_t* smem, const uint8_t* __restrict__ g, int bytes) {
  const int4* src = reinterpret_cast<const int4*>(g);
  int4* dst = reinterpret_cast<int4*>(smem);
  for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) dst[i] = __ldg(src + i);
  __syncthreads();
}

// exp(x) by Tang's table-driven method (P. T. P. Tang, ACM TOMS 15(2), 1989):
// x = (256 m + j) ln2/256 + r with |r| <= ln2/512, exp(x) = 2^m 2^(j/256)
// exp(r), exp(r) - 1 by its degree-4 Taylor polynomial (truncation < 4e-17
// relative).  ln2/256 is split into a 32-bit head and a tail (the classic
// fdlibm split of ln2) so that n*head is exact.  2^(j/256) comes from the
// 256-entry table staged with the mechanism.  9 FP64 operations (the CUDA
// library's exp measured ~18 FP64-pipe slots per value on this GPU); |x| >= 700,
// NaN and Inf take the library path (the range test compares the high word as
// an integer, so it costs no FP64-pipe slot: |x| < 700 exactly when it is below
// 0x4085E000, the high word of 700.0).  Accuracy is tested against CUDA's exp
// (tests/test_gpu_parity.py).
__device__ __forceinline__ double fexp(double x, const double* __restrict__ tab) {
  if ((__double2hiint(x) & 0x7fffffff) >= 0x4085E000) return exp(x);
  const double SHIFT = 6755399441055744.0;               // 1.5 * 2^52
  const double INV_L = 369.3299304675746;                // 256 / ln2
  const double L_HI = 0.00270760617331689;               // 0x1.62e42fee00000p-9
  const double L_LO = 7.453964567463233e-13;             // 0x1.a39ef35793c76p-41
  double kd = fma(x, INV_L, SHIFT);
  const int k = __double2loint(kd);
  kd -= SHIFT;
  double r = fma(kd, -L_HI, x);
  r = fma(kd, -L_LO, r);
  const double p = r * fma(r, fma(r, fma(r, 1.0 / 24.0, 1.0 / 6.0), 0.5), 1.0);
  const double t = tab[k & 255];
  const double res = fma(t, p, t);
  return __hiloint2double(__double2hiint(res) + (k >> 8) * 1048576, __double2loint(res));
}

// ln x by a 129-point table (the table-driven method of P. T. P. Tang, ACM
// TOMS 16(4), 1990): x = 2^m y with y in [1, 2), j = round(128 (y - 1)),
// c_j ~ 1 / (1 + j/128) with -ln c_j tabulated as hi + lo, r = y c_j - 1 by
// one FMA (|r| <= 2^-8 plus rounding), and
//   ln x = m ln2 + (-ln c_j) + ln(1 + r),
// ln(1 + r) by its Taylor polynomial to r^7 (the first omitted term is below
// 2^-66).  ln2 is split into a 32-bit head and a tail (the fdlibm split) so
// that m * head is exact.  14 FP64 operations, where the CUDA library's log
// measured about 33 FP64-pipe slots per value on this GPU.  Zero, subnormal,
// negative, inf and NaN arguments take the library path (the test is on the
// integer high word).  Checked against CUDA's log in tests/test_gpu_parity.py.
__device__ __forceinline__ double flog(double x, const double* __restrict__ tab) {
  const int hi = __double2hiint(x);
  if (hi < 0x00100000 || hi >= 0x7ff00000) return log(x);
  const int mh = hi & 0x000fffff;
  const int j = (mh + 0x1000) >> 13;                       // 0..128
  const double y = __hiloint2double(mh | 0x3ff00000, __double2loint(x));
  const double* t = tab + 3 * j;
  const double r = fma(y, t[0], -1.0);
  double q = fma(r, 1.0 / 7.0, -1.0 / 6.0);
  q = fma(r, q, 0.2);
  q = fma(r, q, -0.25);
  q = fma(r, q, 1.0 / 3.0);
  q = fma(r, q, -0.5);
  const double l1p = fma(r * r, q, r);                      // ln(1 + r)
  const double dm = (double)((hi >> 20) - 1023);
  const double LN2_HI = 6.93147180369123816490e-01;         // 0x1.62e42fee00000p-1
  const double LN2_LO = 1.90821492927058770002e-10;         // 0x1.a39ef35793c76p-33
  return fma(dm, LN2_HI, t[1]) + (fma(dm, LN2_LO, t[2]) + l1p);
}

constexpr double INV_LN10 = 0.43429448190325182765;       // 1 / ln 10

__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;   // identical on every lane (xor butterfly)
}

__device__ inline double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
  return v;
}

// Bit pattern of |x|: for non-negative doubles the integer order of the bit
// patterns is the numeric order, so maxima and pivot searches can run on the
// integer pipe instead of as FP64 compares (NaN, 0x7ff8..., sorts above +inf).
__device__ __forceinline__ long long absbits(double x) { return __double_as_longlong(x) & 0x7fffffffffffffffLL; }

// NASA-7 thermo of species k at T (lane-local).
struct SpThermo { double cpR, hRT, sR, dcpR; };

// NASA-9 thermo of species k at T: range r holds (a1..a7, b1, b2);
// cp/R = a1/T^2 + a2/T + a3 + a4 T + ... + a7 T^4 and its h, s integrals.
static __device__ __noinline__ SpThermo nasa9(const MechView& m, int k, double T, double lnT, double invT) {
  const int S = m.nsp;
  const double* c = m.nasa9 + k;
  const int nr = (int)c[0];
  int r = 0;
  if (nr > 1 && T > c[2 * S]) r = 1;
  if (nr > 2 && T > c[3 * S]) r = 2;
  const double* a = c + (5 + 9 * r) * S;
  const double a1 = a[0], a2 = a[S], a3 = a[2 * S], a4 = a[3 * S], a5 = a[4 * S], a6 = a[5 * S], a7 = a[6 * S];
  const double b1 = a[7 * S], b2 = a[8 * S];
  const double iT2 = invT * invT;
  SpThermo t;
  t.cpR = a1 * iT2 + a2 * invT + a3 + T * (a4 + T * (a5 + T * (a6 + T * a7)));
  t.hRT = -a1 * iT2 + a2 * lnT * invT + a3 + T * (a4 * 0.5 + T * (a5 * (1.0 / 3.0) + T * (a6 * 0.25 + T * a7 * 0.2))) +
          b1 * invT;
  t.sR = -0.5 * a1 * iT2 - a2 * invT + a3 * lnT + T * (a4 + T * (a5 * 0.5 + T * (a6 * (1.0 / 3.0) + T * a7 * 0.25))) +
         b2;
  t.dcpR = -2.0 * a1 * iT2 * invT - a2 * iT2 + a4 + T * (2.0 * a5 + T * (3.0 * a6 + T * 4.0 * a7));
  return t;
}

__device__ inline SpThermo nasa7(const MechView& m, int k, double T, double lnT, double invT) {
  if (m.nasa9) return nasa9(m, k, T, lnT, invT);   // warp-uniform: a property of the mechanism
  const int S = m.nsp;
  const double tmid = m.nasa[14 * S + k];
  const bool lo = T <= tmid;
  const double* a = m.nasa + (lo ? 0 : 7 * S) + k;
  const double* c = m.nasah + (lo ? 0 : 8 * S) + k;   // a1/2, a2/3, a3/4, a4/5, a2/2, a3/3, a4/4
  double a0 = a[0], a1 = a[S], a2 = a[2 * S], a3 = a[3 * S], a4 = a[4 * S], a5 = a[5 * S], a6 = a[6 * S];
  SpThermo t;
  t.cpR = fma(T, fma(T, fma(T, fma(T, a4, a3), a2), a1), a0);
  t.hRT = fma(a5, invT, fma(T, fma(T, fma(T, fma(T, c[3 * S], c[2 * S]), c[S]), c[0]), a0));
  t.sR = fma(a0, lnT, fma(T, fma(T, fma(T, fma(T, c[6 * S], c[5 * S]), c[4 * S]), a1), a6));
  t.dcpR = a1 + T * (2.0 * a2 + T * (3.0 * a3 + T * 4.0 * a4));
  return t;
}

// c^ord by order code (1..3 integral, 4 general) with the derivative d(c^ord)/dc.
__device__ inline double powc(double c, int code, double ord, double* d, const double* tab, const double* ltab) {
  switch (code) {
    case 1: *d = 1.0; return c;
    case 2: *d = 2.0 * c; return c * c;
    case 3: *d = 3.0 * c * c; return c * c * c;
    case 4: {
      double cc = c > 0.0 ? c : 0.0;
      if (cc > 0.0) {
        double pw = fexp(ord * flog(cc, ltab), tab);
        *d = ord * pw / cc;
        return pw;
      }
      *d = 0.0;
      return 0.0;
    }
    default: *d = 0.0; return 1.0;
  }
}

// Per-warp scratch (doubles) used by the kinetics.
struct WarpScratch {
  double* c;      // [nsp]
  double* hRT;    // [nsp]
  double* gRT;    // [nsp]
  double* q;      // [nrpad] rates of progress
  double* fo;     // [8][32] falloff pre-pass values (aliases Jr in Jacobian mode)
  // Jacobian mode only
  double* dq;     // [8][nrpad]: 6 sparse partials (3 reactant, 3 product slots), tb coef, dq/dT
  double* Jr;     // [n][ldj] rows (species rows then T row), ldj = nsp+1 (odd stride)
  int ldj;
};

// Per-warp scratch in two parts.  The small part (shared memory): c, hRT, gRT
// [nsp each], q [nrpad] and the falloff pre-pass area [8][32].  The Jacobian
// part: dq [8][nrpad] and the rows Jr [(nsp+1)^2] -- in shared memory for up to
// 31 species, in a per-warp slot of global memory (L2-resident) for 32-63.
// The falloff pre-pass of a Jacobian evaluation uses Jr (written only after the
// rates of progress are done).
__host__ __device__ inline int scratch_small_doubles(int nsp, int nrpad) {
  return (3 * nsp + nrpad + 8 * 32 + 1) & ~1;   // keep 16-byte alignment
}
__host__ __device__ inline int scratch_jac_doubles(int nsp, int nrpad) {
  return (8 * nrpad + (nsp + 1) * (nsp + 1) + 1) & ~1;
}
// One block of scratch per warp.  With the Jacobian, the derivative rows dq
// start where the falloff scratch fo starts: fo is used only by the kernel
// calls without the Jacobian (in the Jacobian call it lives in Jr), and dq only
// inside a Jacobian call, so the two may share (8 nrpad >= 256 doubles).
__host__ __device__ inline int scratch_doubles(int nsp, int nrpad, bool jac) {
  return jac ? ((3 * nsp + nrpad + 8 * nrpad + (nsp + 1) * (nsp + 1) + 1) & ~1) : scratch_small_doubles(nsp, nrpad);
}

__device__ inline WarpScratch carve2(double* small, double* jacbuf, int nsp, int nrpad) {
  WarpScratch s;
  s.c = small; s.hRT = small + nsp; s.gRT = small + 2 * nsp; s.q = small + 3 * nsp;
  s.fo = s.q + nrpad;
  s.ldj = nsp + 1;
  s.dq = jacbuf;
  s.Jr = jacbuf ? jacbuf + 8 * nrpad : nullptr;
  return s;
}

// Both parts contiguous in one buffer (shared memory, up to 31 species).
__device__ inline WarpScratch carve(double* p, int nsp, int nrpad, bool jac) {
  return carve2(p, jac ? p + 3 * nsp + nrpad : nullptr, nsp, nrpad);
}

// Cell-level results held per lane: lane k (< ns) gets species k, the T-row
// quantities are uniform across the warp.
// SPL = species per lane: component k = lane + 32 j lives in slot j.
template <int SPL>
struct CellOutT {
  double wmol[SPL];   // component k < ns: molar production (kmol/m^3/s)
  double cpR[SPL];    // component k < ns: cp_k / R
  double f[SPL];      // component k < ns: dY_k/dt; k == ns: dT/dt
  double fT;          // dT/dt (uniform)
  double rho;         // uniform
  double cp_mass, h_mass;   // uniform: mixture cp [J/kg/K], h [J/kg]
};
using CellOut = CellOutT<1>;

// Troe / Lindemann effective forward coefficient with its derivatives.
struct Falloff { double keff, dlnkeff, dkeff_dM; };

__device__ inline Falloff falloff_eval(const MechView& m, int r, int type, double kinf, double dlnkinf,
                                       double M, double T, double lnT, double invT) {
  const double* tab = m.exptab;
  double kratio = m.A0[r] * fexp(m.b0[r] * lnT - m.E0[r] * invT, tab);
  double dlnPr = (m.b0[r] + m.E0[r] * invT) * invT;
  double Pr = kratio * M;
  double F = 1.0, G = 0.0, dlnF_T = 0.0;
  if (type == 3) {
    const int P = m.nrpad;
    double a = m.tr[r], iT3 = m.tr[P + r], iT1 = m.tr[2 * P + r], T2 = m.tr[3 * P + r];   // 1/T3, 1/T1
    double e3 = fexp(-T * iT3, tab), e1 = fexp(-T * iT1, tab);
    double Fc = (1.0 - a) * e3 + a * e1;
    double dFc = -(1.0 - a) * iT3 * e3 - a * iT1 * e1;
    if (T2 != 0.0) {
      double e2 = fexp(-T2 * invT, tab);
      Fc += e2;
      dFc += T2 * invT * invT * e2;
    }
    double logFc = flog(Fc, m.logtab) * INV_LN10;
    double cc = -0.4 - 0.67 * logFc;
    double nn = 0.75 - 1.27 * logFc;
    double x = flog(Pr > 1e-300 ? Pr : 1e-300, m.logtab) * INV_LN10 + cc;
    double den = nn - 0.14 * x;
    double f1 = x / den;
    double opf = 1.0 + f1 * f1;
    F = fexp(2.302585092994045684 * (logFc / opf), tab);
    double Aq = 2.0 * logFc * f1 / (opf * opf * den * den);
    G = -Aq * nn;
    dlnF_T = (1.0 / opf + Aq * (0.67 * nn - 1.27 * x)) * dFc / Fc;
  }
  double opr = 1.0 + Pr;
  Falloff o;
  o.keff = kinf * (Pr / opr) * F;
  o.dlnkeff = dlnkinf + dlnPr / opr + G * dlnPr + dlnF_T;
  o.dkeff_dM = kinf * F / opr * (1.0 / opr + G) * kratio;
  return o;
}

// Warp-cooperative kinetics of one cell.  Component k = lane + 32 j (slot j
// of SPL) supplies Y_k (0 beyond ns).  Computes c, thermo, rates of progress,
// molar production, the reactor RHS and (JAC) the Jacobian rows in s.Jr:
//   s.Jr[i*ldj + j] = d f_i / d x_j,  x = (Y_0..Y_{ns-1}, T), f = (dY/dt, dT/dt).
// cv = false: constant pressure, pr = p (rho follows from p, T, Y);
//   dT/dt = -sum_k h_k wdot_k / (rho cp).
// cv = true: constant volume, pr = rho (fixed); the energy equation of
//   rhs_native (Lib_Chemistry_rhs.f90:43-50), dT/dt = -sum_k u_k wdot_k /
//   (rho cv) with u_k = h_k - R T and cv = cp - R per mole, and c depends on Y
//   only (dc_k/dY_k = rho/W_k, dc/dT = 0).  The flag is warp-uniform.
template <bool JAC, int SPL>
__device__ void warp_kinetics(const MechView& m, const WarpScratch& s, int lane, const double (&Yk)[SPL],
                              double T, double pr, CellOutT<SPL>& out, bool cv = false) {
  const double p = pr;
  const int ns = m.ns, nsp = m.nsp, nrpad = m.nrpad;
  const double lnT = flog(T, m.logtab);
  const double lnC0 = m.lnpref_rth - lnT;        // ln(p_ref / (R T))
  // mixture molar mass and density
  double yw = 0.0;
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int k = lane + 32 * j;
    if (k < ns) yw += Yk[j] * m.invmw[k];
  }
  double sumYW = warp_sum(yw);
  // 1/T, 1/sumYW and 1/p from one reciprocal (the warp would otherwise pay
  // for three)
  const double rr = 1.0 / (T * sumYW * p);
  const double invT = rr * sumYW * p;
  double wbar = rr * T * p;
  const double invp = rr * T * sumYW;           // cv: 1 / rho
  double rho = cv ? pr : p * m.inv_r_eos * invT * wbar;   // p / (R T sum Y/W)
  const double ctot = rho * sumYW;                 // sum_k c_k
  // species-parallel: concentrations and thermo, species k = lane + 32 j
  double my_cpR[SPL], my_hRT[SPL], my_dcpR[SPL], my_c[SPL];
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int k = lane + 32 * j;
    double ck = 0.0, hr = 0.0, gr = 0.0;
    my_cpR[j] = 0.0; my_hRT[j] = 0.0; my_dcpR[j] = 0.0; my_c[j] = 0.0;
    if (k < ns) {
      ck = rho * Yk[j] * m.invmw[k];
      SpThermo th = nasa7(m, k, T, lnT, invT);
      hr = th.hRT; gr = th.hRT - th.sR;
      my_cpR[j] = th.cpR; my_hRT[j] = th.hRT; my_dcpR[j] = th.dcpR; my_c[j] = ck;
    }
    if (k < nsp) { s.c[k] = ck; s.hRT[k] = hr; s.gRT[k] = gr; }
  }
  __syncwarp();
  const double* tab = m.exptab;
  // ---- falloff pre-pass: the last nfall reactions (<= 16) -----------------
  // The transcendentals of all falloff reactions are spread over the lanes:
  // pass 1 evaluates k_inf, k_0 and the three Fcent exponentials of every
  // falloff reaction (5 jobs each), pass 2 forms M, Pr and Fcent on lane i,
  // pass 3 takes log10 of Fcent (lane i) and Pr (lane nfall + i) together,
  // pass 4 blends (Lindemann / Troe, Lib_Chemistry_falloff.f90:12-80).
  const int NF = m.nfall, f0 = m.nr - NF;
  double* fo = JAC ? s.Jr : s.fo;     // [8][32]
  if (NF > 0) {
    for (int jb = lane; jb < 5 * NF; jb += WARP) {
      const int i = jb / 5, kind = jb - 5 * i, r = f0 + i;
      const int P = m.nrpad;
      double arg = 0.0, pre = 1.0;
      const bool troe = rx_type(m.code[r]) == 3;
      switch (kind) {
        case 0: arg = m.b[r] * lnT - m.E[r] * invT; pre = m.A[r]; break;
        case 1: arg = m.b0[r] * lnT - m.E0[r] * invT; pre = m.A0[r]; break;   // k0 / kinf
        case 2: arg = troe ? -T * m.tr[P + r] : 0.0; break;       // tr rows 1, 2 hold 1/T3, 1/T1
        case 3: arg = troe ? -T * m.tr[2 * P + r] : 0.0; break;
        default: {
          const double T2 = m.tr[3 * P + r];
          arg = (troe && T2 != 0.0) ? -T2 * invT : 0.0;
          pre = (troe && T2 != 0.0) ? 1.0 : 0.0;
        }
      }
      fo[kind * WARP + i] = pre * fexp(arg, tab);
    }
    __syncwarp();
    double Pr = 1.0, Fc = 1.0, dFc = 0.0, kinf = 0.0, kratio = 0.0, dlnkinf = 0.0, dlnPr = 0.0;
    bool troe = false;
    if (lane < NF) {
      const int r = f0 + lane, P = m.nrpad;
      const uint32_t w = m.code[r];
      troe = rx_type(w) == 3;
      const double M = tb_conc(m, rx_tbrow(w), ctot, s.c);
      kinf = fo[lane];
      kratio = fo[WARP + lane];
      Pr = kratio * M;
      if (JAC) {
        dlnkinf = (m.b[r] + m.E[r] * invT) * invT;
        dlnPr = (m.b0[r] + m.E0[r] * invT) * invT;
      }
      if (troe) {
        const double a = m.tr[r];
        const double e3 = fo[2 * WARP + lane], e1 = fo[3 * WARP + lane], e2 = fo[4 * WARP + lane];
        Fc = (1.0 - a) * e3 + a * e1 + e2;
        if (JAC) {
          const double iT3 = m.tr[P + r], iT1 = m.tr[2 * P + r], T2 = m.tr[3 * P + r];
          dFc = -(1.0 - a) * iT3 * e3 - a * iT1 * e1 + (T2 != 0.0 ? T2 * invT * invT * e2 : 0.0);
        }
      }
    }
    const double Pr_src = __shfl_sync(FULL, Pr, lane >= NF && lane < 2 * NF ? lane - NF : 0);
    double lg_in = lane < NF ? Fc : (lane < 2 * NF ? Pr_src : 1.0);
    lg_in = lg_in > 1e-300 ? lg_in : 1e-300;
    const double lg = flog(lg_in, m.logtab) * INV_LN10;
    const double logPr = __shfl_sync(FULL, lg, lane < NF ? lane + NF : 0);
    // one division per lane for the blend (an FP64 division is a dozen pipe
    // instructions): with Q = den^2 + x^2, 1/(den (1 + Pr) Q) yields 1/den,
    // 1/(1 + Pr) and 1/Q, and 1/(1 + f1^2) = den^2 / Q
    double Fb = 1.0, G = 0.0, dlnF_T = 0.0, fexp_arg = 0.0;
    double iopf = 1.0, x = 0.0, nn = 0.0, logFc = 0.0, den = 1.0, iden = 1.0, f1 = 0.0;
    double iopr = 1.0;
    if (lane < NF && troe) {
      logFc = lg;
      const double cc = -0.4 - 0.67 * logFc;
      nn = 0.75 - 1.27 * logFc;
      x = logPr + cc;
      den = nn - 0.14 * x;
      const double opr = 1.0 + Pr;
      const double Q = fma(den, den, x * x);
      const double dQ = den * Q;
      const double rr = 1.0 / (dQ * opr);
      iden = rr * opr * Q;
      iopr = rr * dQ;
      f1 = x * iden;
      iopf = den * den * (rr * opr * den);
      fexp_arg = 2.302585092994045684 * (logFc * iopf);
    } else if (lane < NF) {
      iopr = 1.0 / (1.0 + Pr);
    }
    Fb = fexp(fexp_arg, tab);
    if (lane < NF) {
      if (!troe) Fb = 1.0;
      fo[5 * WARP + lane] = kinf * (Pr * iopr) * Fb;
      if (JAC) {
        if (troe) {
          const double Aq = 2.0 * logFc * f1 * (iopf * iopf) * (iden * iden);
          G = -Aq * nn;
          dlnF_T = (iopf + Aq * (0.67 * nn - 1.27 * x)) * dFc / Fc;
        }
        fo[6 * WARP + lane] = dlnkinf + dlnPr * iopr + G * dlnPr + dlnF_T;
        fo[7 * WARP + lane] = kinf * Fb * iopr * (iopr + G) * kratio;
      }
    }
    __syncwarp();
  }
  // ---- reaction-parallel: rates of progress --------------------------------
  for (int r = lane; r < nrpad; r += WARP) {
    double q = 0.0;
    if (r < m.nr) {
      const uint32_t w = m.code[r];
      const int type = rx_type(w);
      const bool rev = rx_rev(w);
      double kf = m.A[r] * fexp(m.b[r] * lnT - m.E[r] * invT, tab);
      double dlnkf = (m.b[r] + m.E[r] * invT) * invT;
      double pwf[MAXSIDE], dpf[MAXSIDE], pwr[MAXSIDE], dpr[MAXSIDE];
      double Pf = 1.0, Pr = 0.0;
#pragma unroll
      for (int sl = 0; sl < MAXSIDE; ++sl) {
        int sp = m.rsp[sl * nrpad + r];
        int oc = rx_ordcode(w, sl);
        if (sp >= 0) pwf[sl] = powc(s.c[sp], oc, m.rord[sl * nrpad + r], &dpf[sl], tab, m.logtab);
        else { pwf[sl] = 1.0; dpf[sl] = 0.0; }
        Pf *= pwf[sl];
      }
      double invKc = 0.0, dlnKc = 0.0;
      if (rev) {
        double dG = 0.0, dH = 0.0;
        Pr = 1.0;
#pragma unroll
        for (int sl = 0; sl < MAXSIDE; ++sl) {
          int sp = m.psp[sl * nrpad + r];
          if (sp >= 0) {
            double nu = m.pnu[sl * nrpad + r];
            dG += nu * s.gRT[sp];
            if (JAC) dH += nu * s.hRT[sp];
            pwr[sl] = powc(s.c[sp], (m.pcode[r] >> (4 * sl)) & 0xf, nu, &dpr[sl], tab, m.logtab);
          } else { pwr[sl] = 1.0; dpr[sl] = 0.0; }
          Pr *= pwr[sl];
          int sq = m.rsp[sl * nrpad + r];
          if (sq >= 0) {
            double nu = m.rnu[sl * nrpad + r];
            dG -= nu * s.gRT[sq];
            if (JAC) dH -= nu * s.hRT[sq];
          }
        }
        const double dn = m.dnu[r];
        // 1/Kc = exp(dG - dnu ln(p_ref/RT))
        invKc = fexp(dG - dn * lnC0, tab);
        dlnKc = (dH - dn) * invT;
      }
      double Mfac = 1.0, keff = kf, dlnkeff = dlnkf, dkdM = 0.0;
      if (type == 1) {
        Mfac = tb_conc(m, rx_tbrow(w), ctot, s.c);
      } else if (type >= 2) {
        const int i = r - f0;
        keff = fo[5 * WARP + i]; dlnkeff = fo[6 * WARP + i]; dkdM = fo[7 * WARP + i];
      }
      double fwd = Mfac * keff * Pf;
      double rvs = rev ? Mfac * keff * invKc * Pr : 0.0;
      q = fwd - rvs;
      if (JAC) {
        // sparse partials by slot: reactant slots 0..2, product slots 3..5
        const double kM = Mfac * keff;
#pragma unroll
        for (int sl = 0; sl < MAXSIDE; ++sl) {
          double d = dpf[sl];
#pragma unroll
          for (int u = 0; u < MAXSIDE; ++u) if (u != sl) d *= pwf[u];
          s.dq[sl * nrpad + r] = kM * d;
          double e = 0.0;
          if (rev) {
            e = dpr[sl];
#pragma unroll
            for (int u = 0; u < MAXSIDE; ++u) if (u != sl) e *= pwr[u];
            e = -kM * invKc * e;
          }
          s.dq[(3 + sl) * nrpad + r] = e;
        }
        double tb = 0.0;
        if (type == 1) tb = keff * (Pf - (rev ? invKc * Pr : 0.0));
        else if (type >= 2) tb = dkdM * (Pf - (rev ? invKc * Pr : 0.0));
        s.dq[6 * nrpad + r] = tb;
        s.dq[7 * nrpad + r] = fwd * dlnkeff - rvs * (dlnkeff - dlnKc);
      }
    }
    s.q[r] = q;
  }
  __syncwarp();
  // species-parallel: production rates (each lane sums its species' reaction lists)
  const double cvone = cv ? 1.0 : 0.0;
  double wm[SPL];
  double Ql = 0.0, Dl = 0.0, cpl = 0.0, hl = 0.0;
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int k = lane + 32 * j;
    wm[j] = 0.0;
    if (k < ns) {
      for (int e = m.cstart[k]; e < m.cstart[k + 1]; ++e) wm[j] += m.lnu[e] * s.q[m.lr[e]];
      if (cv) {
        Ql += (my_hRT[j] - 1.0) * wm[j];     // u_k / RT = h_k / RT - 1
        Dl += my_c[j] * (my_cpR[j] - 1.0);   // cv_k / R = cp_k / R - 1
      } else {
        Ql += my_hRT[j] * wm[j];
        Dl += my_c[j] * my_cpR[j];
      }
      cpl += Yk[j] * my_cpR[j] * m.invmw[k];
      hl += Yk[j] * my_hRT[j] * m.invmw[k];
    }
  }
  const double Q = warp_sum(Ql);
  const double D = warp_sum(Dl);
  const double invD = 1.0 / D;
  const double fT = -T * Q * invD;
  const double irho = cv ? invp : m.r_eos * T * sumYW * invp;   // 1 / rho
  out.rho = rho;
  out.fT = fT;
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int k = lane + 32 * j;
    out.wmol[j] = wm[j];
    out.cpR[j] = my_cpR[j];
    out.f[j] = (k < ns) ? m.mw[k] * wm[j] * irho : (k == ns ? fT : 0.0);
  }
  // mixture cp and h (mass)
  out.cp_mass = warp_sum(cpl) * m.r_thermo;
  out.h_mass = warp_sum(hl) * m.r_thermo * T;
  if (!JAC) return;

  // ---- Jacobian in concentration space: row k = species k ------------------
  const int ld = s.ldj;
  double JT[SPL];
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int k = lane + 32 * j;
    JT[j] = 0.0;
    if (k < ns) {
      double* Jrow = s.Jr + k * ld;
      for (int jj = 0; jj < ns; ++jj) Jrow[jj] = 0.0;
      double tball = 0.0;   // third-body terms common to every column
      for (int e = m.cstart[k]; e < m.cstart[k + 1]; ++e) {
        const int r = m.lr[e];
        const double nu = m.lnu[e];
#pragma unroll
        for (int sl = 0; sl < MAXSIDE; ++sl) {
          int sp = m.rsp[sl * nrpad + r];
          if (sp >= 0) Jrow[sp] += nu * s.dq[sl * nrpad + r];
          int sq = m.psp[sl * nrpad + r];
          if (sq >= 0) Jrow[sq] += nu * s.dq[(3 + sl) * nrpad + r];
        }
        const uint32_t w = m.code[r];
        if (rx_type(w) != 0) {
          const double t = nu * s.dq[6 * nrpad + r];
          const int row = rx_tbrow(w);
          tball = fma(t, m.tbd[row], tball);
          for (int q = m.tbp[row]; q < m.tbp[row + 1]; ++q) Jrow[m.tbs[q]] += t * m.tbv[q];
        }
        JT[j] += nu * s.dq[7 * nrpad + r];
      }
      if (tball != 0.0)
        for (int jj = 0; jj < ns; ++jj) Jrow[jj] += tball;
    }
  }
  __syncwarp();
  // S_k = sum_j c_j Jc[k][j] (row k); HJ_m = sum_k hRT_k Jc[k][m] (column m)
  double Sk[SPL], HJ[SPL];
  double HSl = 0.0, dQTl = 0.0, dDTl = 0.0;
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int k = lane + 32 * j;
    Sk[j] = 0.0; HJ[j] = 0.0;
    if (k < ns) {
      const double* Jrow = s.Jr + k * ld;
      if (cv) {
        // rho fixed: no dependence of c on T or through rho on Y (Sk = 0)
        for (int kk = 0; kk < ns; ++kk) HJ[j] += (s.hRT[kk] - 1.0) * s.Jr[kk * ld + k];
        dQTl += (my_cpR[j] - my_hRT[j]) * invT * wm[j] + (my_hRT[j] - 1.0) * JT[j];
        dDTl += my_c[j] * my_dcpR[j];
      } else {
        for (int jj = 0; jj < ns; ++jj) Sk[j] += s.c[jj] * Jrow[jj];
        for (int kk = 0; kk < ns; ++kk) HJ[j] += s.hRT[kk] * s.Jr[kk * ld + k];
        HSl += my_hRT[j] * Sk[j];
        dQTl += (my_cpR[j] - my_hRT[j]) * invT * wm[j] + my_hRT[j] * (JT[j] - Sk[j] * invT);
        dDTl += my_c[j] * (my_dcpR[j] - my_cpR[j] * invT);
      }
    }
  }
  const double HS = warp_sum(HSl);
  __syncwarp();
  const double wr = cv ? 0.0 : wbar * irho;
  const double dQT = warp_sum(dQTl), dDT = warp_sum(dDTl);
  const double QD = Q * invD, TD = T * invD;
  const double JTT = -QD - TD * (dQT - QD * dDT);
  double JTm[SPL];
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int k = lane + 32 * j;
    JTm[j] = 0.0;
    if (k < ns) {
      const double rw = rho * m.invmw[k], ww = cv ? 0.0 : wbar * m.invmw[k];
      const double dQ = rw * HJ[j] - ww * HS;
      const double dD = rw * (my_cpR[j] - cvone) - ww * D;
      JTm[j] = -TD * (dQ - QD * dD);
      // species row k in (Y, T) variables
      const double tk = Sk[j] - wm[j];
      const double Wk = m.mw[k];
      double* Jrow = s.Jr + k * ld;
      for (int jj = 0; jj < ns; ++jj) Jrow[jj] = Wk * m.invmw[jj] * (Jrow[jj] - wr * tk);
      Jrow[ns] = (Wk * irho) * (cv ? JT[j] : JT[j] - tk * invT);
    }
  }
  __syncwarp();
  // T row (row ns)
  double* JrowT = s.Jr + ns * ld;
#pragma unroll
  for (int j = 0; j < SPL; ++j) {
    const int k = lane + 32 * j;
    if (k < ns) JrowT[k] = JTm[j];
  }
  if (lane == 0) JrowT[ns] = JTT;
  __syncwarp();
}

}  // namespace flint
