// flint_files.cu -- native reader of FLINT's tabulated input files (host code).
//
// The C counterpart of read_idealgas_thermo (Load_ThermoTransport.f90:7-95),
// read_idealgas_transport (:129-174) and read_chemistry
// (Load_Chemistry.f90:7-164) for callers without FLINT's Fortran loaders: it
// parses phase.txt, thermo.dat, chemistry-info.txt, chemistry-Arrhenius.dat,
// chemistry-Troe.dat, chemistry-Lindemann.dat and (optional) transport.dat
// (Tecplot ASCII POINT zones) into arrays in the Fortran layout of
// flint_table_desc.  Where the reference prints [ERROR] and returns, or stops
// (a missing rate file), this returns an error code with the reason.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
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
  if (!read_zones(dir + "thermo.dat", th)) { err = "Reading thermo file"; return FLINT_ERR_IO; }
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
  if (!read_zones(dir + "chemistry-Arrhenius.dat", z)) { err = "chemistry-Arrhenius.dat not found"; return FLINT_ERR_IO; }
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
    if (!read_zones(dir + "chemistry-Troe.dat", z) || (int)z.size() < t->nr[1]) { err = "chemistry-Troe.dat not found or short"; return FLINT_ERR_IO; }
    for (int c = 0; c < 4; ++c)
      if (!take(z, t->nr[1], 1 + c, t->ktroe[c])) { err = "chemistry-Troe.dat: ragged zones"; return FLINT_ERR_IO; }
  }
  if (t->nr[2]) {
    z.clear();
    if (!read_zones(dir + "chemistry-Lindemann.dat", z) || (int)z.size() < t->nr[2]) { err = "chemistry-Lindemann.dat not found or short"; return FLINT_ERR_IO; }
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
