// flint_ir.cu -- the mechanism IR blob: one flat, versioned serialization of
// flint_mech_desc (host code).
//
// FLINT hands a mechanism to its kernels through module globals filled by its
// loaders (Load_Chemistry.f90:7-164) or compiled into a generated routine
// (utils/YTF.py:96-260).  The blob is this library's equivalent of that hand-
// over for callers that hold a mechanism as bytes (a file written by
// flint_gb300.mech, a message, a resource): the layout is documented in
// flint_gpu.h next to flint_mech_create_from_ir, and every size is checked
// against the blob's length before anything is read.
#include <cstring>
#include <string>
#include <vector>

#include "flint_host.h"

namespace flint {

namespace {

constexpr uint32_t IR_VERSION = 1;
constexpr int IR_HEADER = 48;
constexpr int IR_MAX_NS = 4096;
constexpr int IR_MAX_NR = 1 << 20;

struct Reader {
  const uint8_t* p;
  int64_t left;
  template <class T>
  void take(std::vector<T>& v, int64_t n) {
    v.resize((size_t)n);
    if (n) std::memcpy(v.data(), p, sizeof(T) * (size_t)n);
    p += sizeof(T) * n;
    left -= sizeof(T) * n;
  }
};

}  // namespace

int64_t ir_bytes(int ns, int nr, bool nasa9) {
  const int64_t d = 8, i = 4, S = ns, R = nr;
  return IR_HEADER + d * S * (1 + 17) + i * R * 2 + d * R * (3 + 3 + 4) + i * R * 3 + d * R * 3 * 2 +
         i * R * 3 + d * R * 3 + d * R * S + (nasa9 ? d * S * 32 : 0);
}

int ir_parse(const void* blob, int64_t bytes, flint_ir_s* ir, std::string& err) {
  if (bytes < IR_HEADER) { err = "blob shorter than the 48-byte header"; return FLINT_ERR_ARG; }
  const uint8_t* b = static_cast<const uint8_t*>(blob);
  if (std::memcmp(b, "FLIR", 4) != 0) { err = "bad magic (not a FLIR blob)"; return FLINT_ERR_ARG; }
  uint32_t version, flags, reserved;
  int32_t ns, nr;
  std::memcpy(&version, b + 4, 4);
  std::memcpy(&ns, b + 8, 4);
  std::memcpy(&nr, b + 12, 4);
  std::memcpy(&flags, b + 16, 4);
  std::memcpy(&reserved, b + 20, 4);
  if (version != IR_VERSION) { err = "unsupported IR version " + std::to_string(version); return FLINT_ERR_ARG; }
  if (ns < 1 || ns > IR_MAX_NS || nr < 0 || nr > IR_MAX_NR) {
    err = "species/reaction counts out of range (ns " + std::to_string(ns) + ", nr " + std::to_string(nr) + ")";
    return FLINT_ERR_ARG;
  }
  if ((flags & ~1u) != 0 || reserved != 0) { err = "unknown flags"; return FLINT_ERR_ARG; }
  const bool n9 = flags & 1u;
  const int64_t want = ir_bytes(ns, nr, n9);
  if (bytes != want) {
    err = "blob is " + std::to_string(bytes) + " bytes, the header's sizes need " + std::to_string(want);
    return FLINT_ERR_ARG;
  }
  ir->ns = ns; ir->nr = nr; ir->flags = (int)flags;
  std::memcpy(ir->consts, b + 24, 24);
  Reader r{b + IR_HEADER, bytes - IR_HEADER};
  r.take(ir->mw, ns);
  r.take(ir->nasa7, (int64_t)ns * 17);
  r.take(ir->rtype, nr);
  r.take(ir->reversible, nr);
  r.take(ir->arrh, (int64_t)nr * 3);
  r.take(ir->arrh0, (int64_t)nr * 3);
  r.take(ir->troe, (int64_t)nr * 4);
  r.take(ir->rsp, (int64_t)nr * 3);
  r.take(ir->rnu, (int64_t)nr * 3);
  r.take(ir->rord, (int64_t)nr * 3);
  r.take(ir->psp, (int64_t)nr * 3);
  r.take(ir->pnu, (int64_t)nr * 3);
  r.take(ir->eff, (int64_t)nr * ns);
  if (n9) r.take(ir->nasa9, (int64_t)ns * 32);
  return r.left == 0 ? FLINT_OK : (err = "internal size mismatch", FLINT_ERR_ARG);
}

void ir_desc(const flint_ir_s* ir, flint_mech_desc* d) {
  std::memset(d, 0, sizeof(*d));
  d->ns = ir->ns; d->nr = ir->nr;
  d->mw = ir->mw.data(); d->nasa7 = ir->nasa7.data();
  d->rtype = ir->rtype.data(); d->reversible = ir->reversible.data();
  d->arrh = ir->arrh.data(); d->arrh0 = ir->arrh0.data(); d->troe = ir->troe.data();
  d->rsp = ir->rsp.data(); d->rnu = ir->rnu.data(); d->rord = ir->rord.data();
  d->psp = ir->psp.data(); d->pnu = ir->pnu.data(); d->eff = ir->eff.data();
  d->r_eos = ir->consts[0]; d->r_thermo = ir->consts[1]; d->p_ref = ir->consts[2];
  d->nasa9 = ir->nasa9.empty() ? nullptr : ir->nasa9.data();
}

}  // namespace flint
