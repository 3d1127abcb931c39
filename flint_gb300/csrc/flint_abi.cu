// flint_abi.cu -- the extern "C" boundary of include/flint_gpu.h.
//
// A handle (flint_mech_s) replaces FLINT's module globals (the tables and
// stoichiometry that read_idealgas_thermo / read_chemistry fill,
// Lib_ThermoTransport.f90:8-25, Lib_Chemistry_data.f90:4-32): it owns one
// packed, 16-byte-aligned device image of the mechanism that every kernel
// stages into shared memory.  Several handles may coexist (FLINT allows one
// mechanism per process).  No exception crosses the boundary: every entry
// point returns a status and records a message for flint_last_error().
#include <atomic>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "flint_host.h"

namespace flint {

static std::atomic<int64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static thread_local std::string g_err;

static int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
static int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

static int cuda_fail(cudaError_t e, const char* what) {
  return fail(FLINT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

static int rup(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace flint

using namespace flint;

struct flint_mech_s {
  void* table = nullptr;   // tabulated mechanism (flint_mech_create_tables)
  ImageLayout L;
  std::vector<uint8_t> himg;
  uint8_t* dimg = nullptr;
  unsigned int* dcounter = nullptr;
  int device = 0;
  // saved-Jacobian scratch of the reactor, one slot per resident warp
  double* djsave = nullptr;
  int jslots = 0;
  int rx_layout = 0;       // reactor layout chosen by flint_reactor_autotune (0: by size)
  int tuned_n = 0;         // layouts the last flint_reactor_autotune timed, and their times
  int tuned_layout[8] = {0};
  float tuned_ms[8] = {0.f};
  int wdot_threads = 0;    // threads per block of the source-term warp kernels (0: default)
  int jac_threads = 0;
  // Jacobian work area of the warp kernels for 32-63 species
  double* dwscratch = nullptr;
  // staging buffers of the *_host entry points (grow only)
  void* dstage = nullptr;
  size_t stage_bytes = 0;
};

namespace flint {

// Pack a mechanism description into the device image (see ImageLayout).
static int pack(const flint_mech_desc* d, ImageLayout& L, std::vector<uint8_t>& img) {
  const int ns = d->ns, nr = d->nr;
  if (ns < 1 || nr < 0) return fail(FLINT_ERR_ARG, "ns=%d nr=%d", ns, nr);
  if (ns > 63) return fail(FLINT_ERR_MECH, "ns=%d: the kernels support up to 63 species", ns);
  if (!d->mw || !d->nasa7 || (nr > 0 && (!d->rtype || !d->reversible || !d->arrh || !d->rsp || !d->rnu ||
                                         !d->rord || !d->psp || !d->pnu)))
    return fail(FLINT_ERR_ARG, "NULL array in mechanism description");
  for (int k = 0; k < ns; ++k)
    if (!(d->mw[k] > 0.0)) return fail(FLINT_ERR_MECH, "species %d: molar mass %g", k, d->mw[k]);
  // order reactions by type: elementary, three-body, Lindemann, Troe
  std::vector<int> order(nr);
  for (int r = 0; r < nr; ++r) order[r] = r;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return d->rtype[a] < d->rtype[b]; });
  int ntb = 0;
  for (int r = 0; r < nr; ++r) {
    int t = d->rtype[r];
    if (t < 0 || t > 3) return fail(FLINT_ERR_MECH, "reaction %d: type %d", r, t);
    if (t != 0) {
      if (!d->eff) return fail(FLINT_ERR_ARG, "third-body reactions need efficiencies");
      if (t >= 2 && (!d->arrh0 || (t == 3 && !d->troe))) return fail(FLINT_ERR_ARG, "falloff data missing");
    if (t >= 2 && !(d->arrh[3 * r] > 0.0)) return fail(FLINT_ERR_MECH, "reaction %d: falloff with A_inf <= 0", r);
      ++ntb;
    }
    for (int s = 0; s < 3; ++s) {
      int a = d->rsp[3 * r + s], b = d->psp[3 * r + s];
      if (a < -1 || a >= ns || b < -1 || b >= ns) return fail(FLINT_ERR_MECH, "reaction %d: species index", r);
      if (a >= 0 && (d->rnu[3 * r + s] < 0.0 || d->rord[3 * r + s] < 0.0))
        return fail(FLINT_ERR_MECH, "reaction %d: negative order", r);
    }
  }
  if (ntb > 255) return fail(FLINT_ERR_MECH, "more than 255 third-body/falloff reactions");
  int nfall = 0;
  for (int r = 0; r < nr; ++r) nfall += d->rtype[r] >= 2;
  if (nfall > 16) return fail(FLINT_ERR_MECH, "%d falloff reactions: the kernels support up to 16", nfall);
  L = ImageLayout{};
  L.ns = ns; L.nr = nr; L.nsp = rup(ns, 32); L.nrpad = rup(std::max(nr, 1), 32); L.ntb = std::max(ntb, 1);
  L.r_eos = d->r_eos; L.r_thermo = d->r_thermo; L.inv_r_eos = 1.0 / d->r_eos;
  L.lnpref_rth = std::log(d->p_ref / d->r_thermo);
  // CSR species -> (reaction, net nu)
  std::vector<std::vector<std::pair<int, double>>> lists(ns);
  for (int rr = 0; rr < nr; ++rr) {
    int r = order[rr];
    std::vector<double> net(ns, 0.0);
    for (int s = 0; s < 3; ++s) {
      if (d->rsp[3 * r + s] >= 0) net[d->rsp[3 * r + s]] -= d->rnu[3 * r + s];
      if (d->psp[3 * r + s] >= 0) net[d->psp[3 * r + s]] += d->pnu[3 * r + s];
    }
    for (int k = 0; k < ns; ++k)
      if (net[k] != 0.0) lists[k].push_back({rr, net[k]});
  }
  int nlist = 0;
  for (auto& l : lists) nlist += (int)l.size();
  L.nlist = nlist;
  // third-body rows in sparse form (ImageLayout::o_tbd): the row's most
  // common efficiency times the total concentration plus the exceptions
  std::vector<double> tbd, tbv;
  std::vector<int> tbp{0}, tbs;
  for (int rr = 0; rr < nr; ++rr) {
    const int r = order[rr];
    if (d->rtype[r] == 0) continue;
    const double* e = d->eff + (size_t)r * ns;
    double mode = e[0];
    int best = 0;
    for (int a = 0; a < ns; ++a) {
      int c = 0;
      for (int b = 0; b < ns; ++b) c += e[b] == e[a];
      if (c > best) { best = c; mode = e[a]; }
    }
    tbd.push_back(mode);
    for (int k = 0; k < ns; ++k)
      if (e[k] != mode) { tbs.push_back(k); tbv.push_back(e[k] - mode); }
    tbp.push_back((int)tbs.size());
  }
  const int ntbl = std::max((int)tbs.size(), 1);
  const int S = L.nsp, P = L.nrpad;
  int off = 0;
  auto sec = [&](int bytes) { int o = off; off = rup(off + bytes, 16); return o; };
  L.o_mw = sec(8 * S); L.o_invmw = sec(8 * S); L.o_nasa = sec(8 * 16 * S); L.o_nasah = sec(8 * 16 * S);
  L.o_A = sec(8 * P); L.o_b = sec(8 * P); L.o_E = sec(8 * P);
  L.o_A0 = sec(8 * P); L.o_b0 = sec(8 * P); L.o_E0 = sec(8 * P); L.o_tr = sec(8 * 4 * P);
  L.o_rnu = sec(8 * 3 * P); L.o_rord = sec(8 * 3 * P); L.o_pnu = sec(8 * 3 * P);
  L.o_rsp = sec(4 * 3 * P); L.o_psp = sec(4 * 3 * P); L.o_code = sec(4 * P); L.o_dnu = sec(8 * P);
  L.o_pcode = sec(4 * P);
  L.o_tbd = sec(8 * L.ntb); L.o_tbp = sec(4 * (L.ntb + 1)); L.o_tbs = sec(4 * ntbl); L.o_tbv = sec(8 * ntbl);
  L.o_cstart = sec(4 * (S + 1)); L.o_lr = sec(4 * std::max(nlist, 1)); L.o_lnu = sec(8 * std::max(nlist, 1));
  L.o_exptab = sec(8 * 256);
  L.o_nasa9 = d->nasa9 ? sec(8 * 32 * S) : -1;
  L.o_logtab = sec(8 * 3 * 129);
  L.nfall = nfall;
  L.bytes = off;
  img.assign(off, 0);
  auto D = [&](int o) { return reinterpret_cast<double*>(img.data() + o); };
  auto I = [&](int o) { return reinterpret_cast<int*>(img.data() + o); };
  for (int k = 0; k < ns; ++k) {
    D(L.o_mw)[k] = d->mw[k];
    D(L.o_invmw)[k] = 1.0 / d->mw[k];
    const double* c = d->nasa7 + 17 * k;
    for (int j = 0; j < 7; ++j) {
      D(L.o_nasa)[j * S + k] = c[3 + j];
      D(L.o_nasa)[(7 + j) * S + k] = c[10 + j];
    }
    D(L.o_nasa)[14 * S + k] = c[1];
    for (int r = 0; r < 2; ++r) {   // low (c[3..9]) and high (c[10..16]) range
      const double* a = c + 3 + 7 * r;
      double* h = D(L.o_nasah) + 8 * r * S + k;
      h[0] = a[1] / 2.0; h[S] = a[2] / 3.0; h[2 * S] = a[3] / 4.0; h[3 * S] = a[4] / 5.0;
      h[4 * S] = a[2] / 2.0; h[5 * S] = a[3] / 3.0; h[6 * S] = a[4] / 4.0; h[7 * S] = 0.0;
    }
    if (d->nasa9)
      for (int j = 0; j < 32; ++j) D(L.o_nasa9)[j * S + k] = d->nasa9[32 * k + j];
  }
  for (int i = 0; i < 3 * P; ++i) { I(L.o_rsp)[i] = -1; I(L.o_psp)[i] = -1; }
  std::copy(tbd.begin(), tbd.end(), D(L.o_tbd));
  std::copy(tbp.begin(), tbp.end(), I(L.o_tbp));
  std::copy(tbs.begin(), tbs.end(), I(L.o_tbs));
  std::copy(tbv.begin(), tbv.end(), D(L.o_tbv));
  int tb = 0;
  for (int rr = 0; rr < nr; ++rr) {
    int r = order[rr];
    int t = d->rtype[r];
    D(L.o_A)[rr] = d->arrh[3 * r]; D(L.o_b)[rr] = d->arrh[3 * r + 1]; D(L.o_E)[rr] = d->arrh[3 * r + 2];
    if (t >= 2) {  // low-pressure limit relative to the high-pressure one
      D(L.o_A0)[rr] = d->arrh0[3 * r] / d->arrh[3 * r];
      D(L.o_b0)[rr] = d->arrh0[3 * r + 1] - d->arrh[3 * r + 1];
      D(L.o_E0)[rr] = d->arrh0[3 * r + 2] - d->arrh[3 * r + 2];
    }
    if (t == 3) {
      // Troe a, 1/T3, 1/T1, T2: the kernels multiply by the reciprocals
      const double* tr = d->troe + 4 * r;
      D(L.o_tr)[rr] = tr[0];
      D(L.o_tr)[P + rr] = 1.0 / tr[1];
      D(L.o_tr)[2 * P + rr] = 1.0 / tr[2];
      D(L.o_tr)[3 * P + rr] = tr[3];
    }
    uint32_t w = (uint32_t)t | ((d->reversible[r] ? 1u : 0u) << 2);
    double dn = 0.0;
    for (int s = 0; s < 3; ++s) {
      int a = d->rsp[3 * r + s], b = d->psp[3 * r + s];
      I(L.o_rsp)[s * P + rr] = a; I(L.o_psp)[s * P + rr] = b;
      if (a >= 0) {
        double nu = d->rnu[3 * r + s], ord = d->rord[3 * r + s];
        D(L.o_rnu)[s * P + rr] = nu; D(L.o_rord)[s * P + rr] = ord;
        uint32_t oc = ord == 1.0 ? 1 : ord == 2.0 ? 2 : ord == 3.0 ? 3 : ord == 0.0 ? 0 : 4;
        w |= oc << (16 + 4 * s);
        dn -= nu;
      }
      if (b >= 0) {
        double nu = d->pnu[3 * r + s];
        D(L.o_pnu)[s * P + rr] = nu;
        dn += nu;
        uint32_t pc = nu == 1.0 ? 1 : nu == 2.0 ? 2 : nu == 3.0 ? 3 : nu == 0.0 ? 0 : 4;
        reinterpret_cast<uint32_t*>(img.data() + L.o_pcode)[rr] |= pc << (4 * s);
      }
    }
    if (t != 0) {
      w |= (uint32_t)tb << 8;
      ++tb;
    }
    reinterpret_cast<uint32_t*>(img.data() + L.o_code)[rr] = w;
    D(L.o_dnu)[rr] = dn;
  }
  int e = 0;
  for (int k = 0; k < S; ++k) {
    I(L.o_cstart)[k] = e;
    if (k < ns)
      for (auto& pr : lists[k]) { I(L.o_lr)[e] = pr.first; D(L.o_lnu)[e] = pr.second; ++e; }
  }
  I(L.o_cstart)[S] = e;
  // 2^(j/256), rounded from extended precision, for the table-driven exp
  for (int j = 0; j < 256; ++j) D(L.o_exptab)[j] = (double)exp2l((long double)j / 256.0L);
  // flog's table: c_j = 1/(1 + j/128) rounded to double, -ln c_j as hi + lo
  // (long double: at least 64 significant bits on either host)
  for (int j = 0; j <= 128; ++j) {
    const double c = (double)(1.0L / (1.0L + (long double)j / 128.0L));
    const long double l = -logl((long double)c);
    const double hi = (double)l;
    D(L.o_logtab)[3 * j] = c;
    D(L.o_logtab)[3 * j + 1] = hi;
    D(L.o_logtab)[3 * j + 2] = (double)(l - (long double)hi);
  }
  return FLINT_OK;
}

static int ensure_stage(flint_mech_s* h, size_t bytes) {
  if (bytes <= h->stage_bytes) return FLINT_OK;
  if (h->dstage) cudaFree(h->dstage);
  h->dstage = nullptr;
  h->stage_bytes = 0;
  cudaError_t e = cudaMalloc(&h->dstage, bytes);
  if (e != cudaSuccess) return fail(FLINT_ERR_NOMEM, "staging buffer of %zu bytes: %s", bytes, cudaGetErrorString(e));
  h->stage_bytes = bytes;
  return FLINT_OK;
}

}  // namespace flint

extern "C" {

static int ensure_jsave(flint_mech_t h);   // the reactor's per-warp scratch, allocated on first use

const char* flint_last_error(void) { return g_err.c_str(); }
const char* flint_version(void) { return "flint_gb300 0.1.0 sm_103a"; }
int64_t flint_kernel_launch_count(void) { return g_launches.load(); }

int flint_mech_create(const flint_mech_desc* desc, flint_mech_t* out) {
  if (!desc || !out) return fail(FLINT_ERR_ARG, "NULL argument");
  *out = nullptr;
  auto* h = new flint_mech_s();
  int rc = pack(desc, h->L, h->himg);
  if (rc != FLINT_OK) { delete h; return rc; }
  cudaGetDevice(&h->device);
  cudaError_t e = cudaMalloc(&h->dimg, h->himg.size());
  if (e != cudaSuccess) { delete h; return fail(FLINT_ERR_NOMEM, "device image: %s", cudaGetErrorString(e)); }
  e = cudaMemcpy(h->dimg, h->himg.data(), h->himg.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&h->dcounter, 256);
  if (e != cudaSuccess) {
    cudaFree(h->dimg);
    delete h;
    return cuda_fail(e, "flint_mech_create");
  }
  *out = h;
  return FLINT_OK;
}

int flint_mech_create_tables(const flint_table_desc* desc, flint_mech_t* out) {
  if (!desc || !out) return fail(FLINT_ERR_ARG, "NULL argument");
  *out = nullptr;
  auto* h = new flint_mech_s();
  std::string err;
  int rc = table_create(desc, &h->table, err);
  if (rc != FLINT_OK) { delete h; return fail(rc, "flint_mech_create_tables: %s", err.c_str()); }
  h->L = ImageLayout{};
  h->L.ns = table_ns(h->table);
  h->L.nr = table_nr(h->table);
  cudaGetDevice(&h->device);
  *out = h;
  return FLINT_OK;
}

int flint_rhs_native_batch(flint_mech_t h, int64_t n, const double* Z, double* F, void* stream) {
  if (!h) return fail(FLINT_ERR_ARG, "NULL handle");
  if (n < 0) return fail(FLINT_ERR_ARG, "negative cell count");
  if (!h->table) return fail(FLINT_ERR_MECH, "flint_rhs_native_batch needs a tabulated mechanism");
  if (n == 0) return FLINT_OK;
  if (!Z || !F) return fail(FLINT_ERR_ARG, "NULL array");
  cudaError_t e = table_run(h->table, n, 1, Z, nullptr, F, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_rhs_native_batch");
}

int flint_transport_batch(flint_mech_t h, int64_t n, const double* rhoi, const double* T, double* mu, double* lambda,
                          void* stream) {
  if (!h) return fail(FLINT_ERR_ARG, "NULL handle");
  if (n < 0) return fail(FLINT_ERR_ARG, "negative cell count");
  if (!h->table) return fail(FLINT_ERR_MECH, "flint_transport_batch needs a tabulated mechanism");
  if (!table_has_transport(h->table)) return fail(FLINT_ERR_MECH, "the handle was created without transport tables");
  if (n == 0) return FLINT_OK;
  if (!rhoi || !T || !mu || !lambda) return fail(FLINT_ERR_ARG, "NULL array");
  cudaError_t e = table_transport(h->table, n, rhoi, T, mu, lambda, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_transport_batch");
}

int flint_cons2prim_batch(flint_mech_t h, int64_t n, int ndim, const double* cons, const double* T, double* prim,
                          double* T_out, void* stream) {
  if (!h) return fail(FLINT_ERR_ARG, "NULL handle");
  if (n < 0) return fail(FLINT_ERR_ARG, "negative cell count");
  if (ndim < 0 || ndim > 3) return fail(FLINT_ERR_ARG, "ndim must be 0..3");
  if (!h->table) return fail(FLINT_ERR_MECH, "flint_cons2prim_batch needs a tabulated mechanism");
  if (n == 0) return FLINT_OK;
  if (!cons || !T || !prim) return fail(FLINT_ERR_ARG, "NULL array");
  const int np = table_ns(h->table) + ndim + 1;
  cudaError_t e = table_cons2prim(h->table, n, np, cons, T, prim, T_out, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_cons2prim_batch");
}

int flint_mech_destroy(flint_mech_t h) {
  if (!h) return FLINT_OK;
  if (h->table) table_destroy(h->table);
  if (h->dimg) cudaFree(h->dimg);
  if (h->dcounter) cudaFree(h->dcounter);
  if (h->dstage) cudaFree(h->dstage);
  if (h->djsave) cudaFree(h->djsave);
  if (h->dwscratch) cudaFree(h->dwscratch);
  delete h;
  return FLINT_OK;
}

int flint_tables_read(const char* folder, const char* prefix, flint_table_set_t* out) {
  if (!folder || !out) return fail(FLINT_ERR_ARG, "NULL argument");
  *out = nullptr;
  auto* t = new flint_table_set_s();
  std::string err;
  int rc = tables_read(folder, prefix, t, err);
  if (rc != FLINT_OK) { delete t; return fail(rc, "flint_tables_read(%s): %s", folder, err.c_str()); }
  *out = t;
  return FLINT_OK;
}

int flint_tables_desc(flint_table_set_t t, flint_table_desc* desc) {
  if (!t || !desc) return fail(FLINT_ERR_ARG, "NULL argument");
  tables_desc(t, desc);
  return FLINT_OK;
}

const char* flint_tables_species_name(flint_table_set_t t, int k) {
  if (!t || k < 0 || k >= t->ns) return nullptr;
  return t->names[k].c_str();
}

int flint_tables_free(flint_table_set_t t) {
  delete t;
  return FLINT_OK;
}

int flint_ir_parse(const void* blob, int64_t bytes, flint_ir_t* out) {
  if (!blob || !out) return fail(FLINT_ERR_ARG, "NULL argument");
  *out = nullptr;
  auto* ir = new flint_ir_s();
  std::string err;
  int rc = ir_parse(blob, bytes, ir, err);
  if (rc != FLINT_OK) { delete ir; return fail(rc, "flint_ir_parse: %s", err.c_str()); }
  *out = ir;
  return FLINT_OK;
}

int flint_ir_desc(flint_ir_t ir, flint_mech_desc* desc) {
  if (!ir || !desc) return fail(FLINT_ERR_ARG, "NULL argument");
  ir_desc(ir, desc);
  return FLINT_OK;
}

int flint_ir_free(flint_ir_t ir) {
  delete ir;
  return FLINT_OK;
}

int64_t flint_ir_bytes(int ns, int nr, int nasa9) {
  if (ns < 1 || nr < 0) return -1;
  return ir_bytes(ns, nr, nasa9 != 0);
}

int flint_mech_create_from_ir(const void* blob, int64_t bytes, flint_mech_t* out) {
  if (!out) return fail(FLINT_ERR_ARG, "NULL argument");
  *out = nullptr;
  flint_ir_t ir = nullptr;
  int rc = flint_ir_parse(blob, bytes, &ir);
  if (rc != FLINT_OK) return rc;
  flint_mech_desc d;
  ir_desc(ir, &d);
  rc = flint_mech_create(&d, out);
  delete ir;
  return rc;
}

int flint_mech_create_from_files(const char* folder, const char* prefix, flint_mech_t* out) {
  if (!out) return fail(FLINT_ERR_ARG, "NULL argument");
  *out = nullptr;
  flint_table_set_t t = nullptr;
  int rc = flint_tables_read(folder, prefix, &t);
  if (rc != FLINT_OK) return rc;
  flint_table_desc d;
  tables_desc(t, &d);
  rc = flint_mech_create_tables(&d, out);
  delete t;
  return rc;
}

int flint_mech_sizes(flint_mech_t h, int* ns, int* nr) {
  // (tabulated handles report their species and total reaction counts too)
  if (!h) return fail(FLINT_ERR_ARG, "NULL handle");
  if (ns) *ns = h->L.ns;
  if (nr) *nr = h->L.nr;
  return FLINT_OK;
}

static int check_common(flint_mech_t h, int64_t n, int layout) {
  if (!h) return fail(FLINT_ERR_ARG, "NULL handle");
  if (h->table) return fail(FLINT_ERR_MECH, "this entry point needs an analytic (NASA-7/Arrhenius) mechanism");
  if (n < 0) return fail(FLINT_ERR_ARG, "negative cell count");
  if (layout != FLINT_CELL_MAJOR && layout != FLINT_SPECIES_MAJOR) return fail(FLINT_ERR_ARG, "layout %d", layout);
  return FLINT_OK;
}

int flint_wdot_batch(flint_mech_t h, int64_t n, int layout, const double* T, const double* p, const double* Y,
                     double* wdot, double* cp, double* hm, void* stream) {
  int rc = check_common(h, n, layout);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !p || !Y || !wdot) return fail(FLINT_ERR_ARG, "NULL array");
  cudaError_t e = launch_wdot(h->dimg, h->L, n, layout, T, p, Y, wdot, cp, hm, (cudaStream_t)stream, h->wdot_threads);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_wdot_batch");
}

int flint_thermo_batch(flint_mech_t h, int64_t n, int layout, const double* T, const double* Y, double* cp,
                       double* hm, void* stream) {
  int rc = check_common(h, n, layout);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !Y) return fail(FLINT_ERR_ARG, "NULL array");
  cudaError_t e = launch_thermo(h->dimg, h->L, n, layout, T, Y, cp, hm, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_thermo_batch");
}

int flint_species_thermo_batch(flint_mech_t h, int64_t n, const double* T, double* cp, double* hs, double* s,
                               double* g, void* stream) {
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (n == 0 || (!cp && !hs && !s && !g)) return FLINT_OK;
  if (!T) return fail(FLINT_ERR_ARG, "NULL array");
  cudaError_t e = launch_species_thermo(h->dimg, h->L, n, T, cp, hs, s, g, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_species_thermo_batch");
}

int flint_chemistry_source_batch(flint_mech_t h, int64_t n, double* roi, const double* T, double* omegadot,
                                 void* stream) {
  if (h && h->table) {
    if (n < 0) return fail(FLINT_ERR_ARG, "negative cell count");
    if (n == 0) return FLINT_OK;
    if (!roi || !T || !omegadot) return fail(FLINT_ERR_ARG, "NULL array");
    cudaError_t e = table_run(h->table, n, 0, roi, T, omegadot, (cudaStream_t)stream);
    return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_chemistry_source_batch");
  }
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!roi || !T || !omegadot) return fail(FLINT_ERR_ARG, "NULL array");
  if (h->L.ns > 16) return fail(FLINT_ERR_MECH, "chemistry_source batch supports up to 16 species");
  cudaError_t e = launch_chemistry_source(h->dimg, h->L, n, roi, T, omegadot, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_chemistry_source_batch");
}

int flint_wdot_jac_batch(flint_mech_t h, int64_t n, int layout, const double* T, const double* p, const double* Y,
                         double* wdot, double* jac, void* stream) {
  int rc = check_common(h, n, layout);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !p || !Y || !jac) return fail(FLINT_ERR_ARG, "NULL array");
  const int64_t need = warp_jac_scratch_doubles(h->L);
  if (need > 0 && !h->dwscratch) {
    cudaError_t ea = cudaMalloc(&h->dwscratch, (size_t)need * sizeof(double));
    if (ea != cudaSuccess) { h->dwscratch = nullptr; return fail(FLINT_ERR_NOMEM, "Jacobian work area: %s", cudaGetErrorString(ea)); }
  }
  cudaError_t e = launch_wdot_jac(h->dimg, h->L, n, layout, T, p, Y, wdot, jac, h->dwscratch, (cudaStream_t)stream,
                                  0, h->jac_threads);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_wdot_jac_batch");
}

int flint_rhs_constp_batch(flint_mech_t h, int64_t n, const double* T, const double* p, const double* Y, double* f,
                           void* stream) {
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !p || !Y || !f) return fail(FLINT_ERR_ARG, "NULL array");
  cudaError_t e = launch_rhs(h->dimg, h->L, n, T, p, Y, f, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_rhs_constp_batch");
}

int flint_wdot_jac_constv_batch(flint_mech_t h, int64_t n, int layout, const double* T, const double* rho,
                                const double* Y, double* wdot, double* jac, void* stream) {
  int rc = check_common(h, n, layout);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !rho || !Y || !jac) return fail(FLINT_ERR_ARG, "NULL array");
  const int64_t need = warp_jac_scratch_doubles(h->L);
  if (need > 0 && !h->dwscratch) {
    cudaError_t ea = cudaMalloc(&h->dwscratch, (size_t)need * sizeof(double));
    if (ea != cudaSuccess) { h->dwscratch = nullptr; return fail(FLINT_ERR_NOMEM, "Jacobian work area: %s", cudaGetErrorString(ea)); }
  }
  cudaError_t e = launch_wdot_jac(h->dimg, h->L, n, layout, T, rho, Y, wdot, jac, h->dwscratch,
                                  (cudaStream_t)stream, 1);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_wdot_jac_constv_batch");
}

int flint_rhs_constv_batch(flint_mech_t h, int64_t n, const double* T, const double* rho, const double* Y, double* f,
                           void* stream) {
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !rho || !Y || !f) return fail(FLINT_ERR_ARG, "NULL array");
  cudaError_t e = launch_rhs(h->dimg, h->L, n, T, rho, Y, f, (cudaStream_t)stream, 1);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_rhs_constv_batch");
}

void flint_reactor_default_opts(flint_reactor_opts* o) {
  if (!o) return;
  o->rtol = 1e-8; o->atol = 1e-14; o->max_steps = 20000; o->max_order = 5;
  o->constant_volume = 0; o->reserved = 0; o->tmin = 200.0; o->tmax = 6000.0;
}

int flint_reactor_advance(flint_mech_t h, int64_t n, double* T, const double* p, double* Y, const double* dt,
                          const flint_reactor_opts* opts, int* status, int* nsteps, void* stream) {
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !p || !Y || !dt) return fail(FLINT_ERR_ARG, "NULL array");
  flint_reactor_opts o;
  if (opts) o = *opts; else flint_reactor_default_opts(&o);
  if (!(o.rtol > 0.0) || !(o.atol > 0.0) || o.max_steps < 1 || o.max_order < 1 || o.max_order > 5)
    return fail(FLINT_ERR_ARG, "reactor options out of range");
  rc = ensure_jsave(h);
  if (rc) return rc;
  cudaError_t e = launch_reactor(h->dimg, h->L, n, T, p, Y, dt, o, status, nsteps, h->dcounter, h->djsave,
                                 h->jslots, (cudaStream_t)stream, nullptr, h->rx_layout);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_reactor_advance");
}

int flint_reactor_autotune(flint_mech_t h, int64_t n, const double* T, const double* p, const double* Y,
                           const double* dt, const flint_reactor_opts* opts, int* layout_out, void* stream) {
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (!T || !p || !Y || !dt) return fail(FLINT_ERR_ARG, "NULL array");
  flint_reactor_opts o;
  if (opts) o = *opts; else flint_reactor_default_opts(&o);
  if (!(o.rtol > 0.0) || !(o.atol > 0.0) || o.max_steps < 1 || o.max_order < 1 || o.max_order > 5)
    return fail(FLINT_ERR_ARG, "reactor options out of range");
  rc = ensure_jsave(h);
  if (rc) return rc;
  h->rx_layout = REACTOR_LAYOUT_AUTO;
  h->tuned_n = 0;
  int cand[8];
  const int nc = reactor_layout_candidates(h->L, cand);
  if (n > 0) {
    // time the sample under each layout on private copies (the caller's arrays stay as they are)
    cudaStream_t st = (cudaStream_t)stream;
    const int ns = h->L.ns;
    double *Tc = nullptr, *Yc = nullptr;
    int *sc = nullptr, *nsc = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&Tc, n * sizeof(double));
    if (!e) e = cudaMalloc(&Yc, n * ns * sizeof(double));
    if (!e) e = cudaMalloc(&sc, n * sizeof(int));
    if (!e) e = cudaMalloc(&nsc, n * sizeof(int));
    if (!e) e = cudaEventCreate(&e0);
    if (!e) e = cudaEventCreate(&e1);
    float best = 0.f;
    for (int c = 0; c < nc && !e; ++c) {
      for (int rep = 0; rep < 2 && !e; ++rep) {   // the first run of each layout warms up
        e = cudaMemcpyAsync(Tc, T, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
        if (!e) e = cudaMemcpyAsync(Yc, Y, n * ns * sizeof(double), cudaMemcpyDeviceToDevice, st);
        if (!e) e = cudaEventRecord(e0, st);
        if (!e) e = launch_reactor(h->dimg, h->L, n, Tc, p, Yc, dt, o, sc, nsc, h->dcounter, h->djsave, h->jslots,
                                   st, nullptr, cand[c]);
        if (!e) e = cudaEventRecord(e1, st);
        if (!e) e = cudaEventSynchronize(e1);
      }
      float ms = 0.f;
      if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
      if (!e && c < 8) { h->tuned_layout[c] = cand[c]; h->tuned_ms[c] = ms; h->tuned_n = c + 1; }
      if (!e && (c == 0 || ms < best)) { best = ms; h->rx_layout = cand[c]; }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(Tc); cudaFree(Yc); cudaFree(sc); cudaFree(nsc);
    if (e) { h->rx_layout = REACTOR_LAYOUT_AUTO; return cuda_fail(e, "flint_reactor_autotune"); }
  }
  if (layout_out) *layout_out = h->rx_layout;
  return FLINT_OK;
}

int flint_reactor_autotune_times(flint_mech_t h, int* layouts, float* ms, int cap, int* count) {
  if (!h || cap < 0 || (cap > 0 && (!layouts || !ms)) || !count) return fail(FLINT_ERR_ARG, "NULL argument");
  *count = h->tuned_n;
  for (int i = 0; i < h->tuned_n && i < cap; ++i) { layouts[i] = h->tuned_layout[i]; ms[i] = h->tuned_ms[i]; }
  return FLINT_OK;
}

int flint_tuning_get(flint_mech_t h, flint_tuning* t) {
  if (!h || !t) return fail(FLINT_ERR_ARG, "NULL argument");
  t->reactor_layout = h->rx_layout;
  t->wdot_threads = h->wdot_threads;
  t->jac_threads = h->jac_threads;
  t->reserved = 0;
  return FLINT_OK;
}

int flint_tuning_set(flint_mech_t h, const flint_tuning* t) {
  if (!h || !t) return fail(FLINT_ERR_ARG, "NULL argument");
  if (h->table) return fail(FLINT_ERR_MECH, "this entry point needs an analytic (NASA-7/Arrhenius) mechanism");
  bool ok = t->reactor_layout == REACTOR_LAYOUT_AUTO;
  int cand[8];
  const int nc = reactor_layout_candidates(h->L, cand);
  for (int c = 0; c < nc; ++c) ok |= cand[c] == t->reactor_layout;
  if (!ok) return fail(FLINT_ERR_ARG, "reactor layout %d does not fit this mechanism on this device", t->reactor_layout);
  int bc[4];
  const int nb = warp_block_candidates(bc);
  for (int v : {t->wdot_threads, t->jac_threads}) {
    bool okb = v == 0;
    for (int c = 0; c < nb; ++c) okb |= bc[c] == v;
    if (!okb) return fail(FLINT_ERR_ARG, "%d threads per block: the source-term kernels take 0, 64, 128 or 256", v);
  }
  h->rx_layout = t->reactor_layout;
  h->wdot_threads = t->wdot_threads;
  h->jac_threads = t->jac_threads;
  return FLINT_OK;
}

int flint_wdot_autotune(flint_mech_t h, int64_t n, const double* T, const double* p, const double* Y,
                        flint_tuning* out, void* stream) {
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (n < 1 || !T || !p || !Y) return fail(FLINT_ERR_ARG, "flint_wdot_autotune needs a sample of cells");
  const int64_t need = warp_jac_scratch_doubles(h->L);
  if (need > 0 && !h->dwscratch) {
    cudaError_t ea = cudaMalloc(&h->dwscratch, (size_t)need * sizeof(double));
    if (ea != cudaSuccess) { h->dwscratch = nullptr; return fail(FLINT_ERR_NOMEM, "Jacobian work area: %s", cudaGetErrorString(ea)); }
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int ns = h->L.ns, nv = ns + 1;
  double *w = nullptr, *J = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&w, (size_t)n * ns * sizeof(double));
  if (!e) e = cudaMalloc(&J, (size_t)n * nv * nv * sizeof(double));
  if (!e) e = cudaEventCreate(&e0);
  if (!e) e = cudaEventCreate(&e1);
  int cand[4];
  const int nc = warp_block_candidates(cand);
  int best_w = 0, best_j = 0;
  float tw = 0.f, tj = 0.f;
  for (int jac = 0; jac < 2 && !e; ++jac) {
    if (!jac && use_small_kernel(h->L)) continue;   // the thread-per-cell kernel serves this mechanism
    for (int c = 0; c < nc && !e; ++c) {
      float ms = 0.f;
      for (int rep = 0; rep < 3 && !e; ++rep) {   // the first run of each block size warms up
        e = cudaEventRecord(e0, st);
        if (!e) e = jac ? launch_wdot_jac(h->dimg, h->L, n, FLINT_CELL_MAJOR, T, p, Y, w, J, h->dwscratch, st, 0, cand[c])
                        : launch_wdot(h->dimg, h->L, n, FLINT_CELL_MAJOR, T, p, Y, w, nullptr, nullptr, st, cand[c]);
        if (!e) e = cudaEventRecord(e1, st);
        if (!e) e = cudaEventSynchronize(e1);
        float one = 0.f;
        if (!e) e = cudaEventElapsedTime(&one, e0, e1);
        if (rep > 0) ms += one;
      }
      if (e) break;
      if (jac) { if (c == 0 || ms < tj) { tj = ms; best_j = cand[c]; } }
      else { if (c == 0 || ms < tw) { tw = ms; best_w = cand[c]; } }
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(w);
  cudaFree(J);
  if (e) return cuda_fail(e, "flint_wdot_autotune");
  h->wdot_threads = best_w;
  h->jac_threads = best_j;
  if (out) return flint_tuning_get(h, out);
  return FLINT_OK;
}

int flint_reactor_advance_noalloc(flint_mech_t h, int64_t n, double* T, const double* p, double* Y, const double* dt,
                                  const flint_reactor_opts* opts, int* status, int* nsteps, void* stream) {
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  // n == 0 is the warm-up: it advances nothing (the arrays may be NULL) and
  // does the one-time set-up on the current device
  if (n > 0 && (!T || !p || !Y || !dt)) return fail(FLINT_ERR_ARG, "NULL array");
  if ((int64_t)(h->L.ns + 1) * (h->L.ns + 1) > 32 * 32)
    return fail(FLINT_ERR_MECH, "flint_reactor_advance_noalloc: %d unknowns exceed the 32 x 32 Jacobian slots of its "
                                "static scratch (%zu bytes)", h->L.ns + 1, reactor_noalloc_bytes());
  if (!reactor_noalloc_fits(h->L))
    return fail(FLINT_ERR_MECH, "flint_reactor_advance_noalloc: this mechanism's Newton matrix does not fit shared "
                                "memory and needs more scratch per warp than the static array holds");
  flint_reactor_opts o;
  if (opts) o = *opts; else flint_reactor_default_opts(&o);
  if (!(o.rtol > 0.0) || !(o.atol > 0.0) || o.max_steps < 1 || o.max_order < 1 || o.max_order > 5)
    return fail(FLINT_ERR_ARG, "reactor options out of range");
  cudaError_t e = launch_reactor_noalloc(h->dimg, h->L, n, T, p, Y, dt, o, status, nsteps, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_reactor_advance_noalloc");
}

// ------------------------------------------------------------------ surrogate
struct flint_surrogate_s {
  flint_mech_t mech;
  flint::Surrogate* s;
};

static int ensure_jsave(flint_mech_t h) {
  if (h->djsave) return FLINT_OK;
  int slots = reactor_slots(h->L);
  if (slots < 1) return fail(FLINT_ERR_MECH, "reactor kernel does not fit this mechanism (shared memory)");
  cudaError_t ea = cudaMalloc(&h->djsave, (size_t)slots * reactor_slot_bytes(h->L));
  if (ea != cudaSuccess) { h->djsave = nullptr; return fail(FLINT_ERR_NOMEM, "reactor scratch: %s", cudaGetErrorString(ea)); }
  h->jslots = slots;
  return FLINT_OK;
}

int flint_surrogate_create(flint_mech_t mech, const flint_surrogate_desc* desc, flint_surrogate_t* out) {
  if (!mech || !desc || !out) return fail(FLINT_ERR_ARG, "NULL argument");
  if (mech->table) return fail(FLINT_ERR_MECH, "the surrogate needs an analytic mechanism");
  *out = nullptr;
  std::string err;
  flint::Surrogate* s = nullptr;
  int rc = surrogate_create(mech->dimg, mech->L, mech->dcounter, desc, &s, err);
  if (rc) return fail(rc, "flint_surrogate_create: %s", err.c_str());
  *out = new flint_surrogate_s{mech, s};
  return FLINT_OK;
}

int flint_surrogate_destroy(flint_surrogate_t s) {
  if (!s) return FLINT_OK;
  surrogate_free(s->s);
  delete s;
  return FLINT_OK;
}

int64_t flint_surrogate_nparams(flint_surrogate_t s) { return s ? surrogate_nparams(s->s) : 0; }

int flint_surrogate_features(flint_surrogate_t s, int64_t n, const double* T, const double* p, const double* Y,
                             const double* dt, float* X, void* stream) {
  if (!s || n < 0 || (n > 0 && (!T || !p || !Y || !dt || !X))) return fail(FLINT_ERR_ARG, "bad argument");
  int rc = surrogate_features(s->s, n, T, p, Y, dt, X, (cudaStream_t)stream);
  return rc ? fail(rc, "flint_surrogate_features failed") : FLINT_OK;
}

int flint_surrogate_targets(flint_surrogate_t s, int64_t n, const double* T0, const double* Y0, const double* T1,
                            const double* Y1, float* Yt, void* stream) {
  if (!s || n < 0 || (n > 0 && (!T0 || !Y0 || !T1 || !Y1 || !Yt))) return fail(FLINT_ERR_ARG, "bad argument");
  int rc = surrogate_targets(s->s, n, T0, Y0, T1, Y1, Yt, (cudaStream_t)stream);
  return rc ? fail(rc, "flint_surrogate_targets failed") : FLINT_OK;
}

int flint_surrogate_train_step(flint_surrogate_t s, int net, int64_t n, const float* X, const float* Yt, float lr,
                               double* loss, void* stream) {
  if (!s || n <= 0 || !X || !Yt) return fail(FLINT_ERR_ARG, "bad argument");
  int rc = surrogate_train_step(s->s, net, n, X, Yt, lr, loss, (cudaStream_t)stream);
  return rc ? fail(rc, "flint_surrogate_train_step failed") : FLINT_OK;
}

int flint_surrogate_predict(flint_surrogate_t s, int net, int64_t n, const float* X, float* Yn, void* stream) {
  if (!s || n < 0 || (n > 0 && (!X || !Yn))) return fail(FLINT_ERR_ARG, "bad argument");
  int rc = surrogate_predict(s->s, net, n, X, Yn, (cudaStream_t)stream);
  return rc ? fail(rc, "flint_surrogate_predict failed") : FLINT_OK;
}

int flint_surrogate_state(flint_surrogate_t s, int net, float* host, int64_t* step, int get) {
  if (!s || !host) return fail(FLINT_ERR_ARG, "bad argument");
  int rc = surrogate_state(s->s, net, host, step, get);
  return rc ? fail(rc, "flint_surrogate_state failed") : FLINT_OK;
}

int flint_surrogate_advance(flint_surrogate_t s, int64_t n, double* T, const double* p, double* Y, const double* dt,
                            const flint_reactor_opts* opts, const flint_surrogate_gate* gate, int* status,
                            int* nsteps, int64_t* counts, void* stream) {
  if (!s || !gate) return fail(FLINT_ERR_ARG, "NULL argument");
  int rc = check_common(s->mech, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !p || !Y || !dt) return fail(FLINT_ERR_ARG, "NULL array");
  flint_reactor_opts o;
  if (opts) o = *opts; else flint_reactor_default_opts(&o);
  if (!(o.rtol > 0.0) || !(o.atol > 0.0) || o.max_steps < 1 || o.max_order < 1 || o.max_order > 5)
    return fail(FLINT_ERR_ARG, "reactor options out of range");
  if (o.constant_volume)
    return fail(FLINT_ERR_ARG, "the surrogate advances at constant pressure (its projection and gate conserve enthalpy)");
  rc = ensure_jsave(s->mech);
  if (rc) return rc;
  rc = surrogate_advance(s->s, n, T, p, Y, dt, o, gate, status, nsteps, s->mech->djsave, s->mech->jslots,
                         nullptr, counts != nullptr, (cudaStream_t)stream, s->mech->rx_layout);
  if (rc) return fail(rc, "flint_surrogate_advance failed: %s", cudaGetErrorString(cudaGetLastError()));
  if (counts) surrogate_counts(s->s, &counts[0], &counts[1]);
  return FLINT_OK;
}

int flint_surrogate_counts(flint_surrogate_t s, int64_t* counts) {
  if (!s || !counts) return fail(FLINT_ERR_ARG, "NULL argument");
  int rc = surrogate_read_counts(s->s, &counts[0], &counts[1]);
  return rc ? fail(rc, "flint_surrogate_counts: %s", cudaGetErrorString(cudaGetLastError())) : FLINT_OK;
}

int flint_surrogate_set_forward(flint_surrogate_t s, int mode, int* kind) {
  if (!s) return fail(FLINT_ERR_ARG, "NULL handle");
  if (surrogate_set_forward(s->s, mode)) return fail(FLINT_ERR_ARG, "forward mode %d (0 fused tcgen05, 1 mma.sync)", mode);
  if (kind) *kind = surrogate_forward_kind(s->s);
  return FLINT_OK;
}

int flint_surrogate_check(flint_surrogate_t s, int* err) {
  if (!s || !err) return fail(FLINT_ERR_ARG, "NULL argument");
  int rc = surrogate_check(s->s, err);
  return rc ? cuda_fail(cudaGetLastError(), "flint_surrogate_check") : FLINT_OK;
}

int flint_surrogate_evaluate(flint_surrogate_t s, int64_t n, double* T, const double* p, double* Y,
                             const double* dt, const flint_surrogate_gate* gate, double* metrics, void* stream) {
  if (!s || !gate || !metrics) return fail(FLINT_ERR_ARG, "NULL argument");
  int rc = check_common(s->mech, n, FLINT_CELL_MAJOR);
  if (rc) return rc;
  if (n == 0) return FLINT_OK;
  if (!T || !p || !Y || !dt) return fail(FLINT_ERR_ARG, "NULL array");
  flint_reactor_opts o;
  flint_reactor_default_opts(&o);
  rc = surrogate_advance(s->s, n, T, p, Y, dt, o, gate, nullptr, nullptr, nullptr, 0, metrics, false,
                         (cudaStream_t)stream);
  return rc ? fail(rc, "flint_surrogate_evaluate failed") : FLINT_OK;
}

int flint_reactor_stats(flint_mech_t h, int64_t out[6]) {
  if (!h || !out) return fail(FLINT_ERR_ARG, "NULL argument");
  unsigned long long c[7];
  cudaError_t e = cudaMemcpy(c, h->dcounter, sizeof c, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "flint_reactor_stats");
  for (int i = 0; i < 6; ++i) out[i] = (int64_t)c[i + 1];
  return FLINT_OK;
}

int flint_selftest_exp(flint_mech_t h, int64_t n, const double* x, double* y, void* stream) {
  if (!h || n < 0 || (n > 0 && (!x || !y))) return fail(FLINT_ERR_ARG, "bad argument");
  cudaError_t e = launch_exp_selftest(h->dimg, h->L, n, x, y, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_selftest_exp");
}

int flint_selftest_log(flint_mech_t h, int64_t n, const double* x, double* y, void* stream) {
  if (!h || n < 0 || (n > 0 && (!x || !y))) return fail(FLINT_ERR_ARG, "bad argument");
  cudaError_t e = launch_log_selftest(h->dimg, h->L, n, x, y, (cudaStream_t)stream);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_selftest_log");
}

int flint_probe_fp64_peak(double* tflops) {
  if (!tflops) return fail(FLINT_ERR_ARG, "NULL argument");
  cudaError_t e = probe_fp64(tflops);
  return e == cudaSuccess ? FLINT_OK : cuda_fail(e, "flint_probe_fp64_peak");
}

// ------------------------------------------------------------------ host forms
int flint_wdot_batch_host(flint_mech_t h, int64_t n, int layout, const double* T, const double* p, const double* Y,
                          double* wdot, double* cp, double* hm) {
  int rc = check_common(h, n, layout);
  if (rc || n == 0) return rc;
  const int ns = h->L.ns;
  size_t nb = (size_t)n * 8;
  rc = ensure_stage(h, nb * (4 + 2 * ns));
  if (rc) return rc;
  double* dT = (double*)h->dstage;
  double* dp = dT + n;
  double* dY = dp + n;
  double* dw = dY + (size_t)n * ns;
  double* dcp = dw + (size_t)n * ns;
  double* dh = dcp + n;
  cudaError_t e = cudaMemcpy(dT, T, nb, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(dp, p, nb, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(dY, Y, nb * ns, cudaMemcpyHostToDevice);
  if (e) return cuda_fail(e, "H2D");
  rc = flint_wdot_batch(h, n, layout, dT, dp, dY, dw, cp ? dcp : nullptr, hm ? dh : nullptr, nullptr);
  if (rc) return rc;
  e = cudaMemcpy(wdot, dw, nb * ns, cudaMemcpyDeviceToHost);
  if (!e && cp) e = cudaMemcpy(cp, dcp, nb, cudaMemcpyDeviceToHost);
  if (!e && hm) e = cudaMemcpy(hm, dh, nb, cudaMemcpyDeviceToHost);
  return e ? cuda_fail(e, "D2H") : FLINT_OK;
}

int flint_wdot_jac_batch_host(flint_mech_t h, int64_t n, int layout, const double* T, const double* p,
                              const double* Y, double* wdot, double* jac) {
  int rc = check_common(h, n, layout);
  if (rc || n == 0) return rc;
  const int ns = h->L.ns, nv = ns + 1;
  size_t nb = (size_t)n * 8;
  rc = ensure_stage(h, nb * (2 + 2 * ns + nv * nv));
  if (rc) return rc;
  double* dT = (double*)h->dstage;
  double* dp = dT + n;
  double* dY = dp + n;
  double* dw = dY + (size_t)n * ns;
  double* dj = dw + (size_t)n * ns;
  cudaError_t e = cudaMemcpy(dT, T, nb, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(dp, p, nb, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(dY, Y, nb * ns, cudaMemcpyHostToDevice);
  if (e) return cuda_fail(e, "H2D");
  rc = flint_wdot_jac_batch(h, n, layout, dT, dp, dY, wdot ? dw : nullptr, dj, nullptr);
  if (rc) return rc;
  if (wdot) e = cudaMemcpy(wdot, dw, nb * ns, cudaMemcpyDeviceToHost);
  if (!e) e = cudaMemcpy(jac, dj, nb * nv * nv, cudaMemcpyDeviceToHost);
  return e ? cuda_fail(e, "D2H") : FLINT_OK;
}

int flint_reactor_advance_host(flint_mech_t h, int64_t n, double* T, const double* p, double* Y, const double* dt,
                               const flint_reactor_opts* opts, int* status, int* nsteps) {
  int rc = check_common(h, n, FLINT_CELL_MAJOR);
  if (rc || n == 0) return rc;
  const int ns = h->L.ns;
  size_t nb = (size_t)n * 8;
  rc = ensure_stage(h, nb * (3 + ns) + (size_t)n * 8);
  if (rc) return rc;
  double* dT = (double*)h->dstage;
  double* dp = dT + n;
  double* dY = dp + n;
  double* ddt = dY + (size_t)n * ns;
  int* dst = (int*)(ddt + n);
  int* dns = dst + n;
  cudaError_t e = cudaMemcpy(dT, T, nb, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(dp, p, nb, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(dY, Y, nb * ns, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(ddt, dt, nb, cudaMemcpyHostToDevice);
  if (e) return cuda_fail(e, "H2D");
  rc = flint_reactor_advance(h, n, dT, dp, dY, ddt, opts, dst, dns, nullptr);
  if (rc) return rc;
  e = cudaMemcpy(T, dT, nb, cudaMemcpyDeviceToHost);
  if (!e) e = cudaMemcpy(Y, dY, nb * ns, cudaMemcpyDeviceToHost);
  if (!e && status) e = cudaMemcpy(status, dst, (size_t)n * 4, cudaMemcpyDeviceToHost);
  if (!e && nsteps) e = cudaMemcpy(nsteps, dns, (size_t)n * 4, cudaMemcpyDeviceToHost);
  return e ? cuda_fail(e, "D2H") : FLINT_OK;
}

}  // extern "C"
