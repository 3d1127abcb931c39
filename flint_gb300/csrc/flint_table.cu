// flint_table.cu -- the reference's tabulated path on the GPU.
//
// FLINT's `general` source term (src/lib/Lib_Chemistry_wdot.f90:96-220) and
// `rhs_native` (src/lib/Lib_Chemistry_rhs.f90:15-52) over a batch of cells,
// on FLINT's own 1-K tables (kf/kb, falloff k_inf/k_0/k_c/F_cent, cp and h),
// interpolated as comp_ch_tabT / f_tabT_expr do (a + (b - a) * Tdiff,
// Lib_Chemistry_data.f90:36-48, Lib_ThermoTransport.f90:531-542).
//
// Layout: the Fortran tables tab(T, reaction) are transposed once at handle
// creation to tab[row][reaction] so that the 32 lanes of a reaction round read
// 32 consecutive doubles of one row (coalesced; the whole table set stays in
// L2).  Stoichiometry is compacted to sparse lists (up to 4 species per side)
// staged in shared memory with the third-body rows and the species CSR lists.
// One warp per cell; reactions on lanes, species sums per lane.
#include <cmath>
#include <string>
#include <vector>
#include <algorithm>

#include "flint_host.h"

namespace flint {

constexpr int TSIDE = 4;
constexpr int TABLE_THREADS = 256;

struct TableLayout {
  int ns, nsp, nr, nrpad, ntb, nlist, bytes;
  int nra, nrt, nrl;           // Arrhenius, Troe, Lindemann counts (reference order)
  int ti1, nrow_r, tmin, tmax, nrow_t;
  double runiv;
  int o_wm, o_ri, o_kind, o_tb, o_rsp, o_rex, o_psp, o_pex, o_eff, o_cstart, o_lr, o_lnu;
  // global tables (doubles offsets into the table buffer)
  size_t g_k1, g_k2, g_k3, g_k4, g_cp, g_h;
  // transport (when given): species viscosity and conductivity [row][nsp],
  // and Wilke's species-pair factors (W_i/W_j)^(1/4) and sqrt(8 (1 + W_i/W_j)) [ns][ns]
  int has_tr;
  size_t g_mu, g_kt, g_p4, g_s8;
};

struct TableView {
  int ns, nsp, nr, nrpad, ntb;
  const double *wm, *ri, *rex, *pex, *eff, *lnu;
  const int *kind, *tb, *rsp, *psp, *cstart, *lr;
  __device__ void bind(const TableLayout& L, const uint8_t* b) {
    ns = L.ns; nsp = L.nsp; nr = L.nr; nrpad = L.nrpad; ntb = L.ntb;
    wm = (const double*)(b + L.o_wm); ri = (const double*)(b + L.o_ri);
    kind = (const int*)(b + L.o_kind); tb = (const int*)(b + L.o_tb);
    rsp = (const int*)(b + L.o_rsp); rex = (const double*)(b + L.o_rex);
    psp = (const int*)(b + L.o_psp); pex = (const double*)(b + L.o_pex);
    eff = (const double*)(b + L.o_eff);
    cstart = (const int*)(b + L.o_cstart); lr = (const int*)(b + L.o_lr); lnu = (const double*)(b + L.o_lnu);
  }
};

static int rupT(int x, int m) { return (x + m - 1) / m * m; }

// Pack the Fortran-layout tables into the device image and transposed tables.
int table_pack(const flint_table_desc* d, TableLayout& L, std::vector<uint8_t>& img, std::vector<double>& tabs,
               std::string& err) {
  const int ns = d->ns;
  if (ns < 1 || ns > 31) { err = "tabulated path supports 1..31 species"; return FLINT_ERR_MECH; }
  if (d->nr_arrh < 0 || d->nr_troe < 0 || d->nr_lind < 0) { err = "negative reaction count"; return FLINT_ERR_ARG; }
  const int nra = d->nr_arrh, nrt = d->nr_troe, nrl = d->nr_lind, nr = nra + nrt + nrl;
  if (d->ti2 <= d->ti1 || d->tmax <= d->tmin) { err = "table row range"; return FLINT_ERR_ARG; }
  if (!d->wm || !d->cp_tab || !d->h_tab) { err = "NULL thermo array"; return FLINT_ERR_ARG; }
  if (nra && (!d->kf_tab || !d->kb_tab || !d->ni1_arrh || !d->ni2_arrh || !d->eps_arrh)) { err = "NULL Arrhenius array"; return FLINT_ERR_ARG; }
  if (nrt && (!d->kinf_troe || !d->k0_troe || !d->kc_troe || !d->fcent_troe || !d->ni1_troe || !d->ni2_troe || !d->eps_troe)) { err = "NULL Troe array"; return FLINT_ERR_ARG; }
  if (nrl && (!d->kinf_lind || !d->k0_lind || !d->kc_lind || !d->ni1_lind || !d->ni2_lind || !d->eps_lind)) { err = "NULL Lindemann array"; return FLINT_ERR_ARG; }
  L = TableLayout{};
  L.ns = ns; L.nsp = rupT(ns, 32); L.nr = nr; L.nrpad = rupT(std::max(nr, 1), 32);
  L.nra = nra; L.nrt = nrt; L.nrl = nrl;
  L.ti1 = d->ti1; L.nrow_r = d->ti2 - d->ti1 + 1; L.tmin = d->tmin; L.tmax = d->tmax; L.nrow_t = d->tmax - d->tmin + 1;
  L.runiv = d->runiv;
  const int S = L.nsp, P = L.nrpad;
  std::vector<int> kind(P, 0), tbrow(P, -1), rsp(TSIDE * P, -1), psp(TSIDE * P, -1);
  std::vector<double> rex(TSIDE * P, 0.0), pex(TSIDE * P, 0.0), effs;
  std::vector<std::vector<std::pair<int, double>>> lists(ns);
  int ntb = 0;
  for (int r = 0; r < nr; ++r) {
    int k = r < nra ? 0 : (r < nra + nrt ? 1 : 2);
    int j = k == 0 ? r : (k == 1 ? r - nra : r - nra - nrt);
    const double* n1 = (k == 0 ? d->ni1_arrh : k == 1 ? d->ni1_troe : d->ni1_lind) + (size_t)j * (ns + 1);
    const double* n2 = (k == 0 ? d->ni2_arrh : k == 1 ? d->ni2_troe : d->ni2_lind) + (size_t)j * (ns + 1);
    const double* ep = (k == 0 ? d->eps_arrh : k == 1 ? d->eps_troe : d->eps_lind) + (size_t)j * (ns + 1);
    kind[r] = k;
    int a = 0, b = 0;
    for (int s = 0; s < ns; ++s) {
      if (n1[s] != 0.0) {
        if (a == TSIDE) { err = "a tabulated reaction has more than 4 reactant species"; return FLINT_ERR_MECH; }
        rsp[a * P + r] = s; rex[a * P + r] = n1[s]; ++a;
      }
      if (n2[s] != 0.0) {
        if (b == TSIDE) { err = "a tabulated reaction has more than 4 product species"; return FLINT_ERR_MECH; }
        psp[b * P + r] = s; pex[b * P + r] = n2[s]; ++b;
      }
      double dn = n2[s] - n1[s];
      if (dn != 0.0) lists[s].push_back({r, dn});
    }
    if (n1[ns] > 0.0) {
      tbrow[r] = ntb++;
      for (int s = 0; s < S; ++s) effs.push_back(s < ns ? ep[s] : 0.0);
    }
  }
  L.ntb = std::max(ntb, 1);
  if (effs.empty()) effs.assign(S, 0.0);
  int nlist = 0;
  for (auto& l : lists) nlist += (int)l.size();
  L.nlist = nlist;
  int off = 0;
  auto sec = [&](int bytes) { int o = off; off = rupT(off + bytes, 16); return o; };
  L.o_wm = sec(8 * S); L.o_ri = sec(8 * S); L.o_kind = sec(4 * P); L.o_tb = sec(4 * P);
  L.o_rsp = sec(4 * TSIDE * P); L.o_rex = sec(8 * TSIDE * P); L.o_psp = sec(4 * TSIDE * P); L.o_pex = sec(8 * TSIDE * P);
  L.o_eff = sec(8 * L.ntb * S); L.o_cstart = sec(4 * (S + 1)); L.o_lr = sec(4 * std::max(nlist, 1));
  L.o_lnu = sec(8 * std::max(nlist, 1));
  L.bytes = off;
  img.assign(off, 0);
  auto D = [&](int o) { return reinterpret_cast<double*>(img.data() + o); };
  auto I = [&](int o) { return reinterpret_cast<int*>(img.data() + o); };
  for (int s = 0; s < ns; ++s) { D(L.o_wm)[s] = d->wm[s]; D(L.o_ri)[s] = d->runiv / d->wm[s]; }
  for (int r = 0; r < P; ++r) { I(L.o_kind)[r] = kind[r]; I(L.o_tb)[r] = tbrow[r]; }
  for (int i = 0; i < TSIDE * P; ++i) {
    I(L.o_rsp)[i] = rsp[i]; D(L.o_rex)[i] = rex[i]; I(L.o_psp)[i] = psp[i]; D(L.o_pex)[i] = pex[i];
  }
  std::copy(effs.begin(), effs.end(), D(L.o_eff));
  int e = 0;
  for (int s = 0; s < S; ++s) {
    I(L.o_cstart)[s] = e;
    if (s < ns) for (auto& pr : lists[s]) { I(L.o_lr)[e] = pr.first; D(L.o_lnu)[e] = pr.second; ++e; }
  }
  I(L.o_cstart)[S] = e;
  // transposed tables: rate tables [row][reaction], thermo tables [row][species]
  const size_t RR = (size_t)L.nrow_r * P, TT = (size_t)L.nrow_t * S;
  L.g_k1 = 0; L.g_k2 = RR; L.g_k3 = 2 * RR; L.g_k4 = 3 * RR; L.g_cp = 4 * RR; L.g_h = 4 * RR + TT;
  L.has_tr = (d->mi_tab && d->k_tab) ? 1 : 0;
  const size_t PP = (size_t)ns * ns;
  L.g_mu = 4 * RR + 2 * TT; L.g_kt = L.g_mu + TT; L.g_p4 = L.g_kt + TT; L.g_s8 = L.g_p4 + PP;
  tabs.assign(L.has_tr ? L.g_s8 + PP : 4 * RR + 2 * TT, 0.0);
  auto put = [&](size_t base, const double* src, int nrj, int r0) {
    for (int j = 0; j < nrj; ++j)
      for (int row = 0; row < L.nrow_r; ++row) tabs[base + (size_t)row * P + r0 + j] = src[(size_t)j * L.nrow_r + row];
  };
  if (nra) { put(L.g_k1, d->kf_tab, nra, 0); put(L.g_k2, d->kb_tab, nra, 0); }
  if (nrt) {
    put(L.g_k1, d->kinf_troe, nrt, nra); put(L.g_k2, d->k0_troe, nrt, nra);
    put(L.g_k3, d->kc_troe, nrt, nra); put(L.g_k4, d->fcent_troe, nrt, nra);
  }
  if (nrl) { put(L.g_k1, d->kinf_lind, nrl, nra + nrt); put(L.g_k2, d->k0_lind, nrl, nra + nrt); put(L.g_k3, d->kc_lind, nrl, nra + nrt); }
  for (int s = 0; s < ns; ++s)
    for (int row = 0; row < L.nrow_t; ++row) {
      tabs[L.g_cp + (size_t)row * S + s] = d->cp_tab[(size_t)s * L.nrow_t + row];
      tabs[L.g_h + (size_t)row * S + s] = d->h_tab[(size_t)s * L.nrow_t + row];
      if (L.has_tr) {
        tabs[L.g_mu + (size_t)row * S + s] = d->mi_tab[(size_t)s * L.nrow_t + row];
        tabs[L.g_kt + (size_t)row * S + s] = d->k_tab[(size_t)s * L.nrow_t + row];
      }
    }
  if (L.has_tr) {
    // T-independent parts of co_fiij, evaluated once on the host as the
    // reference evaluates them per call: Mi_Mj**0.25d0 and dsqrt(8*(1+Mi_Mj))
    for (int i = 0; i < ns; ++i)
      for (int j = 0; j < ns; ++j) {
        const double MiMj = d->wm[i] / d->wm[j];
        tabs[L.g_p4 + (size_t)i * ns + j] = std::pow(MiMj, 0.25);
        tabs[L.g_s8 + (size_t)i * ns + j] = std::sqrt(8.0 * (1.0 + MiMj));
      }
  }
  return FLINT_OK;
}

// The general loop is evaluated in the reference's operation order with
// uncontracted IEEE operations (__dmul_rn / __dadd_rn are never fused into
// FMA), so the Arrhenius path reproduces a -ffp-contract=off build of the
// Fortran bit for bit.
__device__ inline double lerp_rn(double a, double b, double Tdiff) {
  return __dadd_rn(a, __dmul_rn(__dsub_rn(b, a), Tdiff));
}

// Fortran x**n with integer n (nint of the stoichiometric entry).
__device__ inline double ipow(double x, int n) {
  double r = 1.0;
  int m = n < 0 ? -n : n;
  for (int i = 0; i < m; ++i) r = __dmul_rn(r, x);
  return n < 0 ? 1.0 / r : r;
}

// f_F (Lib_Chemistry_falloff.f90:61-80).
__device__ inline double troe_F(double Pr, double Fcent) {
  double logFcent = log10(Fcent);
  double logPr = log10(Pr);
  double c = -0.4 - 0.67 * logFcent;
  double n = 0.75 - 1.27 * logFcent;
  double f1 = (logPr + c) / (n - 0.14 * (logPr + c));
  return pow(10.0, logFcent / (1.0 + f1 * f1));
}

// RHS = 0: chemistry_source(roi, T) -> omegadot.  RHS = 1: rhs_native(Z) -> F.
template <int RHS>
__global__ void __launch_bounds__(TABLE_THREADS)
k_general_warp(const uint8_t* __restrict__ img, TableLayout L, const double* __restrict__ tabs, int64_t n,
               const double* __restrict__ roi_g, const double* __restrict__ Tg, double* __restrict__ out) {
  extern __shared__ __align__(16) uint8_t smem[];
  {
    const int4* src = reinterpret_cast<const int4*>(img);
    int4* dst = reinterpret_cast<int4*>(smem);
    for (int i = threadIdx.x; i < L.bytes / 16; i += blockDim.x) dst[i] = __ldg(src + i);
    __syncthreads();
  }
  TableView m;
  m.bind(L, smem);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double* coi = reinterpret_cast<double*>(smem + L.bytes) + wid * (L.nsp + L.nrpad);
  double* qn = coi + L.nsp;
  const int ns = m.ns, P = m.nrpad, nz = ns + 1;
  const double* K1 = tabs + L.g_k1;
  const double* K2 = tabs + L.g_k2;
  const double* K3 = tabs + L.g_k3;
  const double* K4 = tabs + L.g_k4;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t cell = (int64_t)blockIdx.x * (blockDim.x >> 5) + wid; cell < n; cell += nwarps) {
    double temp, rho_s = 0.0;
    if (RHS) {
      temp = roi_g[cell * nz + ns];
      if (temp < L.tmin || temp > L.tmax || isnan(temp)) {   // Lib_Chemistry_rhs.f90:31-34
        if (lane < nz) out[cell * nz + lane] = -1.0;
        continue;
      }
      if (lane < ns) { rho_s = roi_g[cell * nz + lane]; rho_s = rho_s > 0.0 ? rho_s : 0.0; }
    } else {
      temp = Tg[cell];
      if (lane < ns) rho_s = roi_g[cell * ns + lane];
    }
    if (lane < ns) coi[lane] = rho_s / m.wm[lane];
    __syncwarp();
    int Ti = (int)temp;
    const double Tdiff = temp - Ti;
    int row = Ti - L.ti1;
    row = row < 0 ? 0 : (row > L.nrow_r - 2 ? L.nrow_r - 2 : row);
    for (int r = lane; r < P; r += WARP) {
      double net = 0.0;
      if (r < m.nr) {
        const int k = m.kind[r], t = m.tb[r];
        double coM = 1.0;
        if (t >= 0) {
          coM = 0.0;
          const double* ep = m.eff + t * m.nsp;
          for (int s = 0; s < ns; ++s) coM = __dadd_rn(coM, __dmul_rn(coi[s], ep[s]));
        }
        double pf = 1.0, pr = 1.0;
#pragma unroll
        for (int u = 0; u < TSIDE; ++u) {
          const int a = m.rsp[u * P + r], b = m.psp[u * P + r];
          if (k == 0) {
            if (a >= 0) pf = __dmul_rn(pf, ipow(coi[a], (int)rint(m.rex[u * P + r])));
            if (b >= 0) pr = __dmul_rn(pr, ipow(coi[b], (int)rint(m.pex[u * P + r])));
          } else {
            if (a >= 0) pf = __dmul_rn(pf, pow(coi[a], m.rex[u * P + r]));
            if (b >= 0) pr = __dmul_rn(pr, pow(coi[b], m.pex[u * P + r]));
          }
        }
        const double* k1r = K1 + (size_t)row * P + r;
        const double* k2r = K2 + (size_t)row * P + r;
        double a1 = k1r[0], b1 = k1r[P];
        double a2 = k2r[0], b2 = k2r[P];
        double v1 = lerp_rn(a1, b1, Tdiff), v2 = lerp_rn(a2, b2, Tdiff);
        if (k == 0) {
          net = __dsub_rn(__dmul_rn(__dmul_rn(v1, pf), coM), __dmul_rn(__dmul_rn(v2, pr), coM));
        } else {
          const double* k3r = K3 + (size_t)row * P + r;
          double kc = lerp_rn(k3r[0], k3r[P], Tdiff);
          double Pr = __dmul_rn(v2, coM) / v1;
          double kk = __dmul_rn(v1, Pr / __dadd_rn(1.0, Pr));
          if (k == 1) {
            const double* k4r = K4 + (size_t)row * P + r;
            kk = __dmul_rn(kk, troe_F(Pr, lerp_rn(k4r[0], k4r[P], Tdiff)));
          }
          net = __dsub_rn(__dmul_rn(kk, pf), __dmul_rn(kk / kc, pr));
        }
      }
      qn[r] = net;
    }
    __syncwarp();
    double w = 0.0;
    if (lane < ns) {
      for (int e = m.cstart[lane]; e < m.cstart[lane + 1]; ++e)
        w = __dadd_rn(w, __dmul_rn(__dmul_rn(m.wm[lane], m.lnu[e]), qn[m.lr[e]]));
    }
    if (!RHS) {
      if (lane < ns) out[cell * ns + lane] = w;
    } else {
      // energy equation on the thermo tables (Lib_Chemistry_rhs.f90:43-50)
      int Tt = (int)temp;
      int trow = Tt - L.tmin;
      trow = trow < 0 ? 0 : (trow > L.nrow_t - 2 ? L.nrow_t - 2 : trow);
      const double Td = temp - Tt;
      double e_l = 0.0, c_l = 0.0;
      if (lane < ns) {
        const double* H = tabs + L.g_h + (size_t)trow * m.nsp + lane;
        const double* CP = tabs + L.g_cp + (size_t)trow * m.nsp + lane;
        double h = lerp_rn(H[0], H[m.nsp], Td);
        double cp = lerp_rn(CP[0], CP[m.nsp], Td);
        e_l = (h - m.ri[lane] * temp) * w;
        c_l = rho_s * (cp - m.ri[lane]);
      }
      const double eiroi = warp_sum(e_l), rho_cv = warp_sum(c_l);
      if (lane < ns) out[cell * nz + lane] = w;
      if (lane == ns) out[cell * nz + ns] = -eiroi / rho_cv;
    }
    __syncwarp();
  }
}

size_t table_smem(const TableLayout& L) {
  return L.bytes + (TABLE_THREADS / 32) * (size_t)(L.nsp + L.nrpad) * sizeof(double);
}

cudaError_t launch_general(const uint8_t* img, const TableLayout& L, const double* tabs, int64_t n, int rhs,
                           const double* roi, const double* T, double* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  size_t sm = table_smem(L);
  const void* fn = rhs ? (const void*)k_general_warp<1> : (const void*)k_general_warp<0>;
  cudaError_t e = set_smem(fn, sm);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, TABLE_THREADS, sm);
  if (per_sm < 1) per_sm = 1;
  int64_t blocks = (n + TABLE_THREADS / 32 - 1) / (TABLE_THREADS / 32);
  int64_t full = (int64_t)device_sms() * per_sm;
  if (blocks > full) blocks = full;
  if (rhs)
    k_general_warp<1><<<(unsigned)blocks, TABLE_THREADS, sm, st>>>(img, L, tabs, n, roi, T, out);
  else
    k_general_warp<0><<<(unsigned)blocks, TABLE_THREADS, sm, st>>>(img, L, tabs, n, roi, T, out);
  count_launch();
  return cudaGetLastError();
}

// ------------------------------------------------------------- cons2prim
// cons2prim (Lib_ThermoTransport.f90:129-165) over a batch: prim = (rho_s, u_d,
// p) from cons = (rho_s, rho u_d, rho E0) by the reference's Newton iteration on
// the static energy, with its helpers f_Rtot (:217-230), f_cp (:251-271), H
// (:40-54) and f_tab (:500-512) in their own operation order, uncontracted, so
// that the oracle's -ffp-contract=off restatement is matched bit for bit.  One
// thread per cell: every sum runs over the species in order, as the Fortran
// loops do.  norm2 is the scaled sum of squares gfortran evaluates.
struct C2PView {
  const double* cpt;   // [row][nsp]
  const double* ht;
  const double* ri;
  int ns, nsp, tmin, nrow;
  __device__ double lerp_row(const double* tab, double T, int s) const {
    const int Ti = (int)T;
    int row = Ti - tmin;
    row = row < 0 ? 0 : (row > nrow - 2 ? nrow - 2 : row);
    const double* a = tab + (size_t)row * nsp + s;
    return lerp_rn(a[0], a[nsp], __dsub_rn(T, (double)Ti));
  }
};

__device__ inline double sum_rn(const double* x, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s = __dadd_rn(s, x[i]);
  return s;
}

__device__ inline double rtot_rn(const C2PView& v, const double* r) {
  const double rho = sum_rn(r, v.ns);
  double res = 0.0;
  for (int s = 0; s < v.ns; ++s) res = __dadd_rn(res, __ddiv_rn(__dmul_rn(v.ri[s], r[s]), rho));
  return res;
}

__global__ void k_cons2prim(C2PView v, int64_t n, int np, const double* __restrict__ cons,
                            const double* __restrict__ Tg, double* __restrict__ prim, double* __restrict__ Tout) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double* c = cons + i * np;
    double* pr = prim + i * np;
    const int ns = v.ns, nui = ns, nuf = np - 2;
    const double Rgas = rtot_rn(v, c);
    const double rho = sum_rn(c, ns);
    for (int s = 0; s < ns; ++s) pr[s] = c[s];
    for (int d = nui; d <= nuf; ++d) pr[d] = __ddiv_rn(c[d], rho);
    double scale = 1.0, ssq = 0.0;
    for (int d = nui; d <= nuf; ++d) {
      const double x = pr[d];
      if (x != 0.0) {
        const double a = fabs(x);
        if (scale < a) {
          const double q = __ddiv_rn(scale, a);
          ssq = __dadd_rn(1.0, __dmul_rn(__dmul_rn(ssq, q), q));
          scale = a;
        } else {
          const double q = __ddiv_rn(a, scale);
          ssq = __dadd_rn(ssq, __dmul_rn(q, q));
        }
      }
    }
    const double vel = __dmul_rn(scale, __dsqrt_rn(ssq));
    const double energy = __dsub_rn(__ddiv_rn(c[np - 1], rho), __dmul_rn(__dmul_rn(0.5, vel), vel));
    double diff_en = 1.0e3, T = Tg[i];
    int it = 1;
    while (fabs(__ddiv_rn(diff_en, energy)) >= 1e-6 && it <= 20) {
      const double p_it = __dmul_rn(__dmul_rn(rho, Rgas), T);
      double cp = 0.0;
      for (int s = 0; s < ns; ++s) cp = __dadd_rn(cp, __dmul_rn(__ddiv_rn(c[s], rho), v.lerp_row(v.cpt, T, s)));
      const double cv = __dsub_rn(cp, Rgas);
      // E(p, rhoi) = H(p, rhoi) - p / sum(rhoi); H re-derives T = p / (Rtot rho)
      const double rho_h = sum_rn(c, ns), R_h = rtot_rn(v, c);
      const double Th = __ddiv_rn(p_it, __dmul_rn(R_h, rho_h));
      double h = 0.0;
      for (int s = 0; s < ns; ++s) h = __dadd_rn(h, __ddiv_rn(__dmul_rn(v.lerp_row(v.ht, Th, s), c[s]), rho_h));
      const double e_it = __dsub_rn(h, __ddiv_rn(p_it, sum_rn(c, ns)));
      diff_en = fabs(__dsub_rn(e_it, energy));
      T = __dadd_rn(T, __ddiv_rn(__dsub_rn(energy, e_it), cv));
      ++it;
    }
    pr[np - 1] = __dmul_rn(__dmul_rn(rho, Rgas), T);
    if (Tout) Tout[i] = T;
  }
}

// ------------------------------------------------------------- transport
// co_k_mi_lam_Wilke (Lib_ThermoTransport.f90:407-462) with f_molecularWeight
// (:200-214) and co_fiij (:350-362): warp per cell, species i on lane i.  Each
// lane forms its own Wilke denominator over j in order; the mixture sums run
// over the species in order through shuffles, so every sum has the Fortran
// loop's order and the result matches the oracle bit for bit (the
// T-independent pair factors are the host's pow / sqrt, as in the oracle).
struct TransView {
  const double *mu, *kt, *p4, *s8, *wm;
  int ns, nsp, tmin, nrow;
};

__device__ inline double ordered_sum(double v, int ns) {
  double acc = 0.0;
  for (int s = 0; s < ns; ++s) acc = __dadd_rn(acc, __shfl_sync(FULL, v, s));
  return acc;
}

__global__ void k_transport(TransView v, int64_t n, const double* __restrict__ rhoi, const double* __restrict__ Tg,
                            double* __restrict__ mu, double* __restrict__ lam) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int ns = v.ns;
  const bool act = lane < ns;
  for (int64_t cell = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cell < n; cell += nwarps) {
    const double T = Tg[cell];
    const double r = act ? rhoi[cell * ns + lane] : 0.0;
    const double W = act ? v.wm[lane] : 1.0;
    const double rho = ordered_sum(r, ns);
    const double Wmtot = __ddiv_rn(1.0, ordered_sum(act ? __ddiv_rn(__ddiv_rn(r, rho), W) : 0.0, ns));
    const double Xi = act ? __ddiv_rn(__dmul_rn(r, Wmtot), __dmul_rn(rho, W)) : 0.0;
    const int Ti = (int)T;
    int row = Ti - v.tmin;
    row = row < 0 ? 0 : (row > v.nrow - 2 ? v.nrow - 2 : row);
    const double Tdiff = __dsub_rn(T, (double)Ti);
    double mi = 0.0, ki = 0.0;
    if (act) {
      const double* a = v.mu + (size_t)row * v.nsp + lane;
      const double* b = v.kt + (size_t)row * v.nsp + lane;
      mi = lerp_rn(a[0], a[v.nsp], Tdiff);
      ki = lerp_rn(b[0], b[v.nsp], Tdiff);
    }
    double den = 0.0;
    for (int j = 0; j < ns; ++j) {
      const double mj = __shfl_sync(FULL, mi, j), Xj = __shfl_sync(FULL, Xi, j);
      if (act) {
        const double q = __dsqrt_rn(__ddiv_rn(mi, __dadd_rn(mj, 1e-20)));
        const double a = __dadd_rn(1.0, __ddiv_rn(q, v.p4[lane * ns + j]));
        const double fi = __ddiv_rn(__dmul_rn(a, a), v.s8[lane * ns + j]);
        den = __dadd_rn(den, __dmul_rn(Xj, fi));
      }
    }
    const double inv = act ? __ddiv_rn(1.0, den) : 0.0;
    const double mil = ordered_sum(act ? __dmul_rn(__dmul_rn(Xi, mi), inv) : 0.0, ns);
    const double kl = ordered_sum(act ? __dmul_rn(__dmul_rn(Xi, ki), inv) : 0.0, ns);
    if (lane == 0) { mu[cell] = mil; lam[cell] = kl; }
  }
}

// ------------------------------------------------------------ handle glue
struct TableHandle {
  TableLayout L;
  uint8_t* dimg = nullptr;
  double* dtabs = nullptr;
};

int table_create(const flint_table_desc* d, void** out, std::string& err) {
  TableLayout L;
  std::vector<uint8_t> img;
  std::vector<double> tabs;
  int rc = table_pack(d, L, img, tabs, err);
  if (rc) return rc;
  auto* th = new TableHandle();
  th->L = L;
  cudaError_t e = cudaMalloc(&th->dimg, img.size());
  if (!e) e = cudaMalloc(&th->dtabs, tabs.size() * sizeof(double));
  if (!e) e = cudaMemcpy(th->dimg, img.data(), img.size(), cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(th->dtabs, tabs.data(), tabs.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e) {
    cudaFree(th->dimg); cudaFree(th->dtabs);
    delete th;
    err = cudaGetErrorString(e);
    return FLINT_ERR_CUDA;
  }
  *out = th;
  return FLINT_OK;
}

void table_destroy(void* p) {
  auto* th = static_cast<TableHandle*>(p);
  if (!th) return;
  cudaFree(th->dimg);
  cudaFree(th->dtabs);
  delete th;
}

int table_ns(void* p) { return static_cast<TableHandle*>(p)->L.ns; }
int table_nr(void* p) { return static_cast<TableHandle*>(p)->L.nr; }

cudaError_t table_cons2prim(void* p, int64_t n, int np, const double* cons, const double* T, double* prim,
                            double* Tout, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  auto* th = static_cast<TableHandle*>(p);
  const TableLayout& L = th->L;
  C2PView v;
  v.cpt = th->dtabs + L.g_cp; v.ht = th->dtabs + L.g_h;
  v.ri = reinterpret_cast<const double*>(th->dimg + L.o_ri);
  v.ns = L.ns; v.nsp = L.nsp; v.tmin = L.tmin; v.nrow = L.nrow_t;
  int64_t blocks = (n + 127) / 128;
  const int64_t cap = (int64_t)device_sms() * 16;
  if (blocks > cap) blocks = cap;
  k_cons2prim<<<(unsigned)blocks, 128, 0, st>>>(v, n, np, cons, T, prim, Tout);
  count_launch();
  return cudaGetLastError();
}

int table_has_transport(void* p) { return static_cast<TableHandle*>(p)->L.has_tr; }

cudaError_t table_transport(void* p, int64_t n, const double* rhoi, const double* T, double* mu, double* lam,
                            cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  auto* th = static_cast<TableHandle*>(p);
  const TableLayout& L = th->L;
  TransView v;
  v.mu = th->dtabs + L.g_mu; v.kt = th->dtabs + L.g_kt; v.p4 = th->dtabs + L.g_p4; v.s8 = th->dtabs + L.g_s8;
  v.wm = reinterpret_cast<const double*>(th->dimg + L.o_wm);
  v.ns = L.ns; v.nsp = L.nsp; v.tmin = L.tmin; v.nrow = L.nrow_t;
  int64_t blocks = (n + 7) / 8;
  const int64_t cap = (int64_t)device_sms() * 8;
  if (blocks > cap) blocks = cap;
  k_transport<<<(unsigned)blocks, 256, 0, st>>>(v, n, rhoi, T, mu, lam);
  count_launch();
  return cudaGetLastError();
}

cudaError_t table_run(void* p, int64_t n, int rhs, const double* roi, const double* T, double* out, cudaStream_t st) {
  auto* th = static_cast<TableHandle*>(p);
  return launch_general(th->dimg, th->L, th->dtabs, n, rhs, roi, T, out, st);
}

}  // namespace flint
