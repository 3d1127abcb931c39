"""CUDA backend of the mechanism code generator: one sm_103a kernel per mechanism.

FLINT's ``utils/YTF.py`` turns a Cantera YAML mechanism into a Fortran routine
(the ``Lib_ChemMech/*.f90`` family, e.g. ``WD.f90:6-47``) whose rate constants
and stoichiometry are literals.  This module is the device-code counterpart:
``emit(mech)`` writes a CUDA translation unit in which every species, reaction,
coefficient and efficiency of the mechanism is a compile-time constant, and
``GeneratedMechanism`` compiles it with nvcc into a shared library of its own
and launches it through a C entry point:

    ytf_<id>_wdot(n, T, p, Y, wdot, cp, h, stream)
        thread per cell, Fortran (ns, n) layout; wdot in kg/m^3/s,
        cp in J/kg/K, h in J/kg (either may be NULL)

The arithmetic is the analytic path's (NASA-7 thermo, Arrhenius, third body,
Lindemann / Troe falloff, reverse rates from Kc = exp(-dG/RT)(p_ref/RT)^dnu,
integer orders as products, other orders as exp(o ln c) on c > 0), so the oracle
that checks the data-driven kernels checks this one too.  Nothing is looked up
at run time: no mechanism image, no shared memory, no loops over reactions.
That suits mechanisms small enough for a thread to hold the cell (tens of
species); the warp-per-cell kernels serve the large ones.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess

from . import mech as mechmod
from .mech import TYPE_ELEMENTARY, TYPE_THREEBODY, TYPE_TROE

_HERE = os.path.dirname(os.path.abspath(__file__))
_GEN = os.path.join(_HERE, "_gen")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _d(x):
    """A double literal that round-trips exactly."""
    x = float(x)
    if x == 0.0:
        return "0.0"
    r = repr(x) if ("e" in repr(x) or "." in repr(x)) else repr(x) + ".0"
    return f"({r})" if x < 0 else r


def _ident(s):
    h = hashlib.sha1(s.encode()).hexdigest()[:12]
    return "m" + h


def _powexpr(c, order):
    """c^order as the analytic path forms it."""
    o = float(order)
    if o == int(o) and 0 <= o <= 4:
        n = int(o)
        if n == 0:
            return None
        return "*".join([c] * n)
    # c^o = exp(o ln c) for c > 0, 0 otherwise (pow on max(c, 0) of the analytic path)
    return f"({c} > 0.0 ? exp({_d(o)} * log({c})) : 0.0)"


def emit(m: mechmod.Mechanism, ident=None):
    """CUDA source of the per-mechanism kernel (returns (ident, source))."""
    ns = m.ns
    idx = {s.name: k for k, s in enumerate(m.species)}
    body = []
    w = body.append
    # --- thermo: every species' NASA-7 pieces at this T
    w("    const double T2 = t * t, T3 = T2 * t, T4 = T3 * t;")
    for k, s in enumerate(m.species):
        w(f"    double cpR{k}, hRT{k}, gRT{k};")
        w("    {")
        if s.nasa9:
            # NASA-9: pick the range, then the 9-coefficient forms
            rng = s.nasa9
            for i in range(9):
                expr = _d(rng[-1][2 + i])
                for r in reversed(rng[:-1]):
                    expr = f"(t <= {_d(r[1])} ? {_d(r[2 + i])} : {expr})"
                w(f"      const double c{i} = {expr};")
            w("      const double iT2 = invT * invT;")
            w(f"      cpR{k} = c0 * iT2 + c1 * invT + c2 + c3 * t + c4 * T2 + c5 * T3 + c6 * T4;")
            w(f"      hRT{k} = -c0 * iT2 + c1 * lnT * invT + c2 + c3 * t / 2.0 + c4 * T2 / 3.0 + c5 * T3 / 4.0"
              f" + c6 * T4 / 5.0 + c7 * invT;")
            w("      const double sR = -c0 * iT2 / 2.0 - c1 * invT + c2 * lnT + c3 * t + c4 * T2 / 2.0"
              " + c5 * T3 / 3.0 + c6 * T4 / 4.0 + c8;")
        else:
            lo, hi = s.low, s.high
            sel = [f"(t <= {_d(s.tmid)} ? {_d(a)} : {_d(b)})" for a, b in zip(lo, hi)]
            for i in range(7):
                w(f"      const double a{i} = {sel[i]};")
            w(f"      cpR{k} = a0 + a1 * t + a2 * T2 + a3 * T3 + a4 * T4;")
            w(f"      hRT{k} = a0 + a1 * t / 2.0 + a2 * T2 / 3.0 + a3 * T3 / 4.0 + a4 * T4 / 5.0 + a5 * invT;")
            w("      const double sR = a0 * lnT + a1 * t + a2 * T2 / 2.0 + a3 * T3 / 3.0 + a4 * T4 / 4.0 + a6;")
        w(f"      gRT{k} = hRT{k} - sR;")
        w("    }")
    # --- state
    w("    double sumYW = 0.0;")
    for k, s in enumerate(m.species):
        w(f"    const double y{k} = Y[i * {ns} + {k}];")
        w(f"    sumYW += y{k} / {_d(s.mw)};")
    w(f"    const double rho = pc / ({_d(m.r_eos)} * t * sumYW);")
    for k, s in enumerate(m.species):
        w(f"    const double c{k} = rho * y{k} / {_d(s.mw)};")
        w(f"    double w{k} = 0.0;")
    w(f"    const double lnPref = log({_d(m.p_ref)} / ({_d(m.r_thermo)} * t));")
    # --- reactions
    for j, r in enumerate(m.reactions):
        w(f"    {{  // {r.equation}")
        w(f"      const double kf = {_d(r.A)} * exp({_d(r.b)} * lnT - {_d(r.EaR)} * invT);")
        # forward product with orders
        rnames = list(r.reactants.keys()) + [k for k in r.orders if k not in r.reactants]
        fterms = [_powexpr(f"c{idx[nm]}", r.orders.get(nm, r.reactants.get(nm, 0.0))) for nm in rnames]
        fterms = [x for x in fterms if x]
        w(f"      const double Pf = {' * '.join(fterms) if fterms else '1.0'};")
        if r.reversible:
            pterms = [_powexpr(f"c{idx[nm]}", nu) for nm, nu in r.products.items()]
            pterms = [x for x in pterms if x]
            dG = []
            dnu = 0.0
            for nm, nu in r.products.items():
                dG.append(f"+ {_d(nu)} * gRT{idx[nm]}")
                dnu += nu
            for nm, nu in r.reactants.items():
                dG.append(f"- {_d(nu)} * gRT{idx[nm]}")
                dnu -= nu
            w(f"      const double dG = 0.0 {' '.join(dG)};")
            w(f"      const double invKc = exp(dG - {_d(dnu)} * lnPref);")
            w(f"      const double Pr = {' * '.join(pterms) if pterms else '1.0'};")
        if r.rtype != TYPE_ELEMENTARY:
            if r.collider is not None:
                w(f"      const double M = c{idx[r.collider]};")
            else:
                effs = {nm: e for nm, e in (r.efficiencies or {}).items()}
                terms = []
                for k, s in enumerate(m.species):
                    e = effs.get(s.name, r.default_eff)
                    if e == 0.0:
                        continue
                    terms.append(f"c{k}" if e == 1.0 else f"{_d(e)} * c{k}")
                w(f"      const double M = {' + '.join(terms) if terms else '0.0'};")
        if r.rtype in (TYPE_ELEMENTARY, TYPE_THREEBODY):
            w("      const double keff = kf;")
            mfac = "M * " if r.rtype == TYPE_THREEBODY else ""
        else:
            w(f"      const double k0 = {_d(r.A0)} * exp({_d(r.b0)} * lnT - {_d(r.EaR0)} * invT);")
            w("      const double Prd = k0 / kf * M;")
            if r.rtype == TYPE_TROE:
                a, T3, T1 = r.troe[0], r.troe[1], r.troe[2]
                T2 = r.troe[3] if len(r.troe) > 3 else 0.0
                fc = f"(1.0 - {_d(a)}) * exp(-t * {_d(1.0 / T3)}) + {_d(a)} * exp(-t * {_d(1.0 / T1)})"
                if T2 != 0.0:
                    fc += f" + exp(-{_d(T2)} * invT)"
                w(f"      const double logFc = log10({fc});")
                w("      const double cc = -0.4 - 0.67 * logFc;")
                w("      const double nn = 0.75 - 1.27 * logFc;")
                w("      const double x = log10(Prd > 1e-300 ? Prd : 1e-300) + cc;")
                w("      const double f1 = x / (nn - 0.14 * x);")
                w("      const double F = pow(10.0, logFc / (1.0 + f1 * f1));")
                w("      const double keff = kf * (Prd / (1.0 + Prd)) * F;")
            else:
                w("      const double keff = kf * (Prd / (1.0 + Prd));")
            mfac = ""
        if r.reversible:
            w(f"      const double q = {mfac}keff * Pf - {mfac}keff * invKc * Pr;")
        else:
            w(f"      const double q = {mfac}keff * Pf;")
        for nm, nu in r.reactants.items():
            w(f"      w{idx[nm]} -= {_d(nu)} * q;")
        for nm, nu in r.products.items():
            w(f"      w{idx[nm]} += {_d(nu)} * q;")
        w("    }")
    # --- outputs
    w("    if (wdot) {")
    for k, s in enumerate(m.species):
        w(f"      wdot[i * {ns} + {k}] = {_d(s.mw)} * w{k};")
    w("    }")
    w("    if (cp || h) {")
    cps = " + ".join(f"y{k} * cpR{k} / {_d(s.mw)}" for k, s in enumerate(m.species))
    hs = " + ".join(f"y{k} * hRT{k} / {_d(s.mw)}" for k, s in enumerate(m.species))
    w(f"      if (cp) cp[i] = ({cps}) * {_d(m.r_thermo)};")
    w(f"      if (h) h[i] = ({hs}) * {_d(m.r_thermo)} * t;")
    w("    }")
    src_body = "\n".join(body)
    ident = ident or _ident(m.to_json())
    src = f"""// Generated by flint_gb300.ytf_cuda from mechanism "{m.name}" ({ns} species,
// {m.nr} reactions).  Every coefficient is a literal; regenerate instead of editing.
#include <cstdint>
#include <cuda_runtime.h>

extern "C" __global__ void __launch_bounds__(128)
ytf_{ident}_kernel(int64_t n, const double* __restrict__ T, const double* __restrict__ p,
                   const double* __restrict__ Y, double* __restrict__ wdot,
                   double* __restrict__ cp, double* __restrict__ h) {{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {{
    const double t = T[i], pc = p[i];
    const double lnT = log(t), invT = 1.0 / t;
{src_body}
  }}
}}

extern "C" int ytf_{ident}_wdot(int64_t n, const double* T, const double* p, const double* Y, double* wdot,
                              double* cp, double* h, void* stream) {{
  if (n <= 0) return 0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  int64_t blocks = (n + 127) / 128;
  const int64_t cap = (int64_t)sms * 16;
  if (blocks > cap) blocks = cap;
  ytf_{ident}_kernel<<<(unsigned)blocks, 128, 0, (cudaStream_t)stream>>>(n, T, p, Y, wdot, cp, h);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}}

extern "C" int ytf_{ident}_species() {{ return {ns}; }}
"""
    return ident, src


def build(m: mechmod.Mechanism, outdir=None, quiet=True):
    """Emit and compile; returns the path of the shared library (cached by content)."""
    ident, src = emit(m)
    outdir = outdir or _GEN
    os.makedirs(outdir, exist_ok=True)
    cu = os.path.join(outdir, f"ytf_{ident}.cu")
    so = os.path.join(outdir, f"libytf_{ident}.so")
    if os.path.exists(so) and os.path.exists(cu) and open(cu).read() == src:
        return ident, so
    with open(cu, "w") as f:
        f.write(src)
    nvcc = os.environ.get("NVCC", "nvcc")
    cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-shared", "-Xcompiler", "-fPIC", "-o", so + ".tmp", cu]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {cu}:\n{r.stderr}")
    os.replace(so + ".tmp", so)
    return ident, so


class GeneratedMechanism:
    """A mechanism compiled to its own kernel; wdot/cp/h on device arrays."""

    def __init__(self, m: mechmod.Mechanism):
        self.mech = m
        self.ident, self.path = build(m)
        self.L = C.CDLL(self.path)
        fn = getattr(self.L, f"ytf_{self.ident}_wdot")
        fn.argtypes = [C.c_int64] + [C.c_void_p] * 7
        fn.restype = C.c_int
        self._fn = fn

    def wdot(self, T, p, Y, wdot=None, cp=None, h=None, stream=None):
        """Device tensors (torch, float64, Y cell-major (n, ns)); returns (wdot, cp, h)."""
        import torch
        n = T.shape[0]
        if wdot is None:
            wdot = torch.empty_like(Y)
        if cp is None:
            cp = torch.empty_like(T)
        if h is None:
            h = torch.empty_like(T)
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        ptr = lambda t: C.c_void_p(t.data_ptr() if t is not None else 0)   # noqa: E731
        rc = self._fn(n, ptr(T), ptr(p), ptr(Y), ptr(wdot), ptr(cp), ptr(h), C.c_void_p(st))
        if rc != 0:
            raise RuntimeError(f"generated kernel ytf_{self.ident} failed to launch")
        return wdot, cp, h
