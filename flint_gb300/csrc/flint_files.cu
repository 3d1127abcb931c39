// flint_files.cu -- native reader of FLINT's tabulated input files (host code).
//
// The C counterpart of read_idealgas_thermo (Load_ThermoTransport.f90:7-95),
// read_idealgas_transport (:129-174) and read_chemistry
// (Load_Chemistry.f90:7-164) for callers without FLINT's Fortran loaders: it
// parses phase.txt, thermo, chemistry-info.txt, chemistry-Arrhenius,
// chemistry-Troe, chemistry-Lindemann (each as Tecplot ASCII POINT zones,
// .dat, or else as SZL binary, .szplt) and (optional) transport.dat
// into arrays in the Fortran layout of
// flint_table_desc.  Where the reference prints [ERROR] and returns, or stops
// (a missing rate file), this returns an error code with the reason.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <fstream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include "flint_host.h"

namespace flint {

namespace {

struct Zone {
  std::string title;
  std::vector<std::vector<double>> rows;
};

bool read_lines(const std::string& path, std::vector<std::string>& lines) {
  std::ifstream f(path);
  if (!f) return false;
  std::string ln;
  while (std::getline(f, ln)) {
    if (!ln.empty() && ln.back() == '\r') ln.pop_back();
    lines.push_back(ln);
  }
  return true;
}

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// Tecplot ASCII POINT file: "ZONE T=..." opens a zone, numeric lines are rows
// (Fortran D exponents accepted).
bool read_zones(const std::string& path, std::vector<Zone>& zones) {
  std::vector<std::string> lines;
  if (!read_lines(path, lines)) return false;
  for (const std::string& raw : lines) {
    const std::string s = trim(raw);
    if (s.compare(0, 4, "ZONE") == 0) {
      Zone z;
      size_t q1 = s.find('"');
      size_t q2 = q1 == std::string::npos ? q1 : s.find('"', q1 + 1);
      z.title = (q1 != std::string::npos && q2 != std::string::npos) ? s.substr(q1 + 1, q2 - q1 - 1) : s;
      zones.push_back(z);
      continue;
    }
    if (s.empty() || zones.empty()) continue;
    const char c = s[0];
    if (!((c >= '0' && c <= '9') || c == '+' || c == '-' || c == '.')) continue;
    std::string t = s;
    for (char& ch : t)
      if (ch == 'D' || ch == 'd') ch = 'E';
    std::vector<double> row;
    const char* p = t.c_str();
    char* end = nullptr;
    while (true) {
      double v = std::strtod(p, &end);
      if (end == p) break;
      row.push_back(v);
      p = end;
    }
    zones.back().rows.push_back(row);
  }
  return true;
}

// SZL binary (.szplt): ordered one-dimensional zones of float32 or float64
// nodal variables, the form of FLINT's binary tables.  Layout: bytes 34-41 the
// byte-order mark 08 07 .. 01, bytes 42-49 the offset of the file header;
// a header is uint16 n, n uint16 tags, n uint64 values (counts or record
// offsets): 0x001 zones, 0x002 variables, 0x100 zone titles, 0x200 variable
// names (uint64 length, names ended by '\r'), 0x101 zone types ('o'), 0x102
// zone-header offsets, 0x107/0x108/0x109 I/J/K per zone, 0x301 value location
// (1 nodal), 0x302 data type (1 float32, 2 float64), 0x304 sharing zone (int32,
// -1 none) per zone and variable; a zone header's tag 0x600 is the offset of
// its variables' data offsets.  Every offset and length is checked against the
// file size; other forms (compressed FE zones, shared or cell-centred
// variables) are refused with a reason.
class SzlFile {
 public:
  explicit SzlFile(std::vector<unsigned char>&& d) : d_(std::move(d)) {}
  bool ok(uint64_t off, uint64_t len) const { return off <= d_.size() && len <= d_.size() - off; }
  template <class T>
  bool get(uint64_t off, T* out) const {
    if (!ok(off, sizeof(T))) return false;
    std::memcpy(out, d_.data() + off, sizeof(T));   // little-endian host (checked by the byte-order mark)
    return true;
  }
  bool tags(uint64_t off, std::vector<std::pair<uint16_t, uint64_t>>& out) const {
    uint16_t n = 0;
    if (!get(off, &n) || !ok(off + 2, 10ull * n)) return false;
    out.resize(n);
    for (uint16_t i = 0; i < n; ++i) {
      get(off + 2 + 2ull * i, &out[i].first);
      get(off + 2 + 2ull * n + 8ull * i, &out[i].second);
    }
    return true;
  }
  bool names(uint64_t off, size_t count, std::vector<std::string>& out) const {
    uint64_t len = 0;
    if (!get(off, &len) || !ok(off + 8, len)) return false;
    out.clear();
    std::string cur;
    for (uint64_t i = 0; i < len && out.size() < count; ++i) {
      const char c = (char)d_[off + 8 + i];
      if (c == '\r') { out.push_back(cur); cur.clear(); } else cur.push_back(c);
    }
    return out.size() == count;
  }
  const std::vector<unsigned char>& data() const { return d_; }

 private:
  std::vector<unsigned char> d_;
};

bool read_szplt(const std::string& path, std::vector<Zone>& zones, std::string& err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  const unsigned char bom[8] = {8, 7, 6, 5, 4, 3, 2, 1};
  if (buf.size() < 50 || std::memcmp(buf.data(), "#!SZPLT", 7) != 0 || std::memcmp(buf.data() + 34, bom, 8) != 0) {
    err = path + ": not a little-endian SZL file";
    return false;
  }
  uint16_t probe = 1;
  unsigned char first = 0;
  std::memcpy(&first, &probe, 1);
  if (first != 1) { err = path + ": SZL reader needs a little-endian host"; return false; }
  SzlFile F(std::move(buf));
  uint64_t hoff = 0;
  std::vector<std::pair<uint16_t, uint64_t>> hv;
  if (!F.get(42, &hoff) || !F.tags(hoff, hv)) { err = path + ": bad SZL file header"; return false; }
  auto tag = [&](uint16_t t, uint64_t* v) {
    for (auto& kv : hv)
      if (kv.first == t) { *v = kv.second; return true; }
    return false;
  };
  uint64_t nz = 0, nv = 0, o_zt = 0, o_vn = 0, o_ty = 0, o_zh = 0, o_i = 0, o_j = 0, o_k = 0, o_loc = 0, o_dt = 0,
           o_sh = 0;
  if (!tag(0x1, &nz) || !tag(0x2, &nv) || !tag(0x100, &o_zt) || !tag(0x200, &o_vn) || !tag(0x101, &o_ty) ||
      !tag(0x102, &o_zh) || !tag(0x107, &o_i) || !tag(0x108, &o_j) || !tag(0x109, &o_k) || !tag(0x301, &o_loc) ||
      !tag(0x302, &o_dt) || !tag(0x304, &o_sh) || nz < 1 || nv < 1 || nz > (1u << 20) || nv > 4096) {
    err = path + ": SZL file header lacks a record this reader needs";
    return false;
  }
  std::vector<std::string> zt, vn;
  if (!F.names(o_zt, nz, zt) || !F.names(o_vn, nv, vn)) { err = path + ": bad SZL zone or variable names"; return false; }
  if (!F.ok(o_ty, nz) || !F.ok(o_loc, nz * nv) || !F.ok(o_dt, nz * nv) || !F.ok(o_sh, 4 * nz * nv)) {
    err = path + ": SZL record past the end of the file";
    return false;
  }
  const std::vector<unsigned char>& d = F.data();
  for (uint64_t z = 0; z < nz; ++z) {
    uint64_t I = 0, J = 0, K = 0, zh = 0;
    if (!F.get(o_i + 8 * z, &I) || !F.get(o_j + 8 * z, &J) || !F.get(o_k + 8 * z, &K) || !F.get(o_zh + 8 * z, &zh)) {
      err = path + ": SZL zone record past the end of the file";
      return false;
    }
    if (d[o_ty + z] != 'o' || J != 1 || K != 1 || I < 1 || I > (1u << 28)) {
      err = path + ": zone " + std::to_string(z + 1) + " is not an ordered one-dimensional zone";
      return false;
    }
    std::vector<std::pair<uint16_t, uint64_t>> zv;
    uint64_t vtab = 0;
    bool have = F.tags(zh, zv);
    for (auto& kv : zv)
      if (kv.first == 0x600) vtab = kv.second;
    if (!have || vtab == 0 || !F.ok(vtab, 8 * nv)) { err = path + ": bad SZL zone header"; return false; }
    Zone Zn;
    Zn.title = zt[z];
    Zn.rows.assign(I, std::vector<double>(nv, 0.0));
    for (uint64_t v = 0; v < nv; ++v) {
      const uint64_t k = z * nv + v;
      int32_t sh = 0;
      F.get(o_sh + 4 * k, &sh);
      const unsigned dt = d[o_dt + k];
      if (d[o_loc + k] != 1 || sh != -1 || (dt != 1 && dt != 2)) {
        err = path + ": zone " + std::to_string(z + 1) + " variable " + vn[v] +
              ": only unshared nodal float32/float64 data is supported";
        return false;
      }
      uint64_t off = 0;
      F.get(vtab + 8 * v, &off);
      const uint64_t es = dt == 1 ? 4 : 8;
      if (!F.ok(off, I * es)) { err = path + ": SZL variable data past the end of the file"; return false; }
      for (uint64_t r = 0; r < I; ++r) {
        if (dt == 1) {
          float x;
          std::memcpy(&x, d.data() + off + 4 * r, 4);
          Zn.rows[r][v] = (double)x;
        } else {
          std::memcpy(&Zn.rows[r][v], d.data() + off + 8 * r, 8);
        }
      }
    }
    zones.push_back(std::move(Zn));
  }
  return true;
}

// A table by its base name: the ASCII base.dat, else the SZL binary
// base.szplt (the order of Load_Chemistry.f90:95-96 and
// Load_ThermoTransport.f90:57-60).  False with err empty: neither exists.
bool read_table(const std::string& base, std::vector<Zone>& zones, std::string& err) {
  err.clear();
  if (read_zones(base + ".dat", zones)) return true;
  zones.clear();
  return read_szplt(base + ".szplt", zones, err);
}

}  // namespace

int tables_read(const char* folder, const char* prefix, flint_table_set_s* t, std::string& err) {
  const std::string dir = std::string(folder ? folder : ".") + "/" + (prefix ? prefix : "");
  // phase.txt: header line, then "NAME MW" (Load_ThermoTransport.f90:37-51)
  std::vector<std::string> lines;
  if (!read_lines(dir + "phase.txt", lines)) { err = "phase.txt type file not found"; return FLINT_ERR_IO; }
  for (size_t i = 1; i < lines.size(); ++i) {
    std::istringstream is(lines[i]);
    std::string nm;
    double w;
    if (is >> nm >> w) { t->names.push_back(nm); t->wm.push_back(w); }
  }
  const int ns = (int)t->names.size();
  if (ns < 1) { err = "phase.txt lists no species"; return FLINT_ERR_IO; }
  t->ns = ns;
  // thermo.dat: one zone per species, rows T cp h s dcp (:57-85)
  std::vector<Zone> th;
  std::string why;
  if (!read_table(dir + "thermo", th, why)) { err = why.empty() ? "Reading thermo file" : why; return FLINT_ERR_IO; }
  if ((int)th.size() < ns || th[0].rows.empty()) { err = "thermo.dat has fewer zones than species"; return FLINT_ERR_IO; }
  const int rows = (int)th[0].rows.size();
  int tmin = (int)std::lround(th[0].rows[0][0]);
  const int tmax = tmin + rows - 1;
  const bool clone0 = tmin == 1;   // row 0 cloned from row 1, h(0) = 0 (:70, :80-85)
  if (clone0) tmin = 0;
  const int nrow = tmax - tmin + 1;
  t->tmin = tmin; t->tmax = tmax;
  t->cp.assign((size_t)ns * nrow, 0.0);
  t->h.assign((size_t)ns * nrow, 0.0);
  for (int s = 0; s < ns; ++s) {
    if ((int)th[s].rows.size() != rows) { err = "thermo.dat zones differ in length"; return FLINT_ERR_IO; }
    for (int r = 0; r < rows; ++r) {
      if (th[s].rows[r].size() < 3) { err = "thermo.dat row with fewer than 3 columns"; return FLINT_ERR_IO; }
      t->cp[(size_t)s * nrow + r + clone0] = th[s].rows[r][1];
      t->h[(size_t)s * nrow + r + clone0] = th[s].rows[r][2];
    }
    if (clone0) { t->cp[(size_t)s * nrow] = t->cp[(size_t)s * nrow + 1]; t->h[(size_t)s * nrow] = 0.0; }
  }
  // chemistry-info.txt: reaction kinds, then (ns+1) stoichiometry lines per
  // reaction "j NAME ni1 ni2 eps" (Load_Chemistry.f90:36-94)
  lines.clear();
  if (!read_lines(dir + "chemistry-info.txt", lines) || lines.size() < 8) {
    err = "chemistry-info.txt not found"; return FLINT_ERR_IO;
  }
  const int nrc = (lines[2].size() > 17) ? std::atoi(lines[2].substr(17, 4).c_str()) : 0;
  if (nrc < 0 || (int)lines.size() < 7 + nrc + 2 + nrc * (ns + 1)) { err = "chemistry-info.txt truncated"; return FLINT_ERR_IO; }
  std::vector<int> kind(nrc);
  for (int j = 0; j < nrc; ++j) {
    const std::string k = lines[7 + j];
    kind[j] = k.find("Troe") != std::string::npos ? 1 : (k.find("Lindemann") != std::string::npos ? 2 : 0);
    ++t->nr[kind[j]];
  }
  for (int j = 0; j < nrc; ++j) {
    for (int s = 0; s <= ns; ++s) {
      std::istringstream is(lines[7 + nrc + 2 + j * (ns + 1) + s]);
      int idx;
      std::string nm;
      double a, b, c;
      if (!(is >> idx >> nm >> a >> b >> c)) { err = "chemistry-info.txt: bad stoichiometry line"; return FLINT_ERR_IO; }
      t->ni1[kind[j]].push_back(a);
      t->ni2[kind[j]].push_back(b);
      t->eps[kind[j]].push_back(c);
    }
  }
  // rate tables: one zone per reaction of the kind
  std::vector<Zone> z;
  if (!read_table(dir + "chemistry-Arrhenius", z, why)) {
    err = why.empty() ? "chemistry-Arrhenius file not found" : why;
    return FLINT_ERR_IO;
  }
  if ((int)z.size() < t->nr[0] || z.empty() || z[0].rows.empty()) { err = "chemistry-Arrhenius.dat: too few zones"; return FLINT_ERR_IO; }
  const int rrows = (int)z[0].rows.size();
  t->ti1 = (int)std::lround(z[0].rows[0][0]);
  t->ti2 = t->ti1 + rrows - 1;
  auto take = [&](const std::vector<Zone>& zz, int nzone, int col, std::vector<double>& out) -> bool {
    for (int j = 0; j < nzone; ++j) {
      if ((int)zz[j].rows.size() != rrows) return false;
      for (int r = 0; r < rrows; ++r) {
        if ((int)zz[j].rows[r].size() <= col) return false;
        out.push_back(zz[j].rows[r][col]);
      }
    }
    return true;
  };
  if (!take(z, t->nr[0], 1, t->kf) || !take(z, t->nr[0], 2, t->kb)) { err = "chemistry-Arrhenius.dat: ragged zones"; return FLINT_ERR_IO; }
  if (t->nr[1]) {
    z.clear();
    if (!read_table(dir + "chemistry-Troe", z, why) || (int)z.size() < t->nr[1]) {
      err = why.empty() ? "chemistry-Troe file not found or short" : why;
      return FLINT_ERR_IO;
    }
    for (int c = 0; c < 4; ++c)
      if (!take(z, t->nr[1], 1 + c, t->ktroe[c])) { err = "chemistry-Troe.dat: ragged zones"; return FLINT_ERR_IO; }
  }
  if (t->nr[2]) {
    z.clear();
    if (!read_table(dir + "chemistry-Lindemann", z, why) || (int)z.size() < t->nr[2]) {
      err = why.empty() ? "chemistry-Lindemann file not found or short" : why;
      return FLINT_ERR_IO;
    }
    for (int c = 0; c < 3; ++c)
      if (!take(z, t->nr[2], 1 + c, t->klind[c])) { err = "chemistry-Lindemann.dat: ragged zones"; return FLINT_ERR_IO; }
  }
  // transport.dat (optional): rows T mu k on the thermo rows
  z.clear();
  if (read_zones(dir + "transport.dat", z) && (int)z.size() >= ns) {
    t->mu.assign((size_t)ns * nrow, 0.0);
    t->kt.assign((size_t)ns * nrow, 0.0);
    for (int s = 0; s < ns; ++s) {
      const int rs = (int)z[s].rows.size();
      const int off = nrow - rs;   // 1 when row 0 is cloned
      if (off < 0 || off > 1) { err = "transport.dat rows do not match thermo.dat"; return FLINT_ERR_IO; }
      for (int r = 0; r < rs; ++r) {
        if (z[s].rows[r].size() < 3) { err = "transport.dat row with fewer than 3 columns"; return FLINT_ERR_IO; }
        t->mu[(size_t)s * nrow + r + off] = z[s].rows[r][1];
        t->kt[(size_t)s * nrow + r + off] = z[s].rows[r][2];
      }
      if (off) { t->mu[(size_t)s * nrow] = t->mu[(size_t)s * nrow + 1]; t->kt[(size_t)s * nrow] = t->kt[(size_t)s * nrow + 1]; }
    }
  }
  return FLINT_OK;
}

void tables_desc(const flint_table_set_s* t, flint_table_desc* d) {
  std::memset(d, 0, sizeof(*d));
  auto P = [](const std::vector<double>& v) { return v.empty() ? nullptr : v.data(); };
  d->ns = t->ns;
  d->nr_arrh = t->nr[0]; d->nr_troe = t->nr[1]; d->nr_lind = t->nr[2];
  d->tmin = t->tmin; d->tmax = t->tmax; d->ti1 = t->ti1; d->ti2 = t->ti2;
  d->wm = P(t->wm); d->cp_tab = P(t->cp); d->h_tab = P(t->h);
  d->kf_tab = P(t->kf); d->kb_tab = P(t->kb);
  d->kinf_troe = P(t->ktroe[0]); d->k0_troe = P(t->ktroe[1]); d->kc_troe = P(t->ktroe[2]); d->fcent_troe = P(t->ktroe[3]);
  d->kinf_lind = P(t->klind[0]); d->k0_lind = P(t->klind[1]); d->kc_lind = P(t->klind[2]);
  d->ni1_arrh = P(t->ni1[0]); d->ni2_arrh = P(t->ni2[0]); d->eps_arrh = P(t->eps[0]);
  d->ni1_troe = P(t->ni1[1]); d->ni2_troe = P(t->ni2[1]); d->eps_troe = P(t->eps[1]);
  d->ni1_lind = P(t->ni1[2]); d->ni2_lind = P(t->ni2[2]); d->eps_lind = P(t->eps[2]);
  d->runiv = 8314.51;   // FLINT's Runiv (Lib_ThermoTransport.f90:13)
  d->mi_tab = P(t->mu); d->k_tab = P(t->kt);
}

}  // namespace flint
