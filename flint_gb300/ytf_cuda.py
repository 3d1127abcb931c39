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
    ytf_<id>_wdot_jac(n, T, p, Y, wdot, jac, stream)
        thread per cell; wdot (may be NULL) and the constant-pressure Jacobian
        d(dY/dt, dT/dt)/d(Y, T), Fortran (ns+1, ns+1, n), as
        flint_wdot_jac_batch gives it, with the sparsity of every reaction
        fixed at generation time

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


def _thermo_lines(m, w):
    """Per-species cpR, hRT, gRT and dcpR at t, as generated statements."""
    w("    const double T2 = t * t, T3 = T2 * t, T4 = T3 * t;")
    for k, s in enumerate(m.species):
        w(f"    double cpR{k}, hRT{k}, gRT{k}, dcpR{k};")
        w("    {")
        if s.nasa9:
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
            w(f"      dcpR{k} = -2.0 * c0 * iT2 * invT - c1 * iT2 + c3 + 2.0 * c4 * t + 3.0 * c5 * T2"
              " + 4.0 * c6 * T3;")
        else:
            sel = [f"(t <= {_d(s.tmid)} ? {_d(a)} : {_d(b)})" for a, b in zip(s.low, s.high)]
            for i in range(7):
                w(f"      const double a{i} = {sel[i]};")
            w(f"      cpR{k} = a0 + a1 * t + a2 * T2 + a3 * T3 + a4 * T4;")
            w(f"      hRT{k} = a0 + a1 * t / 2.0 + a2 * T2 / 3.0 + a3 * T3 / 4.0 + a4 * T4 / 5.0 + a5 * invT;")
            w("      const double sR = a0 * lnT + a1 * t + a2 * T2 / 2.0 + a3 * T3 / 3.0 + a4 * T4 / 4.0 + a6;")
            w(f"      dcpR{k} = a1 + 2.0 * a2 * t + 3.0 * a3 * T2 + 4.0 * a4 * T3;")
        w(f"      gRT{k} = hRT{k} - sR;")
        w("    }")


def _pow_and_derivative(c, order, pw, dpw):
    """Statements setting pw = c^order and dpw = d pw / d c, as the analytic path forms them."""
    o = float(order)
    if o == int(o) and 1 <= o <= 4:
        n = int(o)
        return [f"const double {pw} = {'*'.join([c] * n)};",
                f"const double {dpw} = {'1.0' if n == 1 else _d(n) + ' * ' + '*'.join([c] * (n - 1))};"]
    return [f"const double {pw} = {c} > 0.0 ? exp({_d(o)} * log({c})) : 0.0;",
            f"const double {dpw} = {c} > 0.0 ? {_d(o)} * {pw} / {c} : 0.0;"]


def emit_jac(m: mechmod.Mechanism, ident):
    """CUDA source of the per-mechanism wdot + Jacobian kernel (thread per cell).

    The Jacobian is that of the data-driven kernels (flint_wdot_jac_batch):
    d(dY/dt, dT/dt)/d(Y, T) of the constant-pressure reactor, written to
    jac[cell][col][row] (Fortran (ns+1, ns+1, n)).  The sparsity is fixed at
    generation time: each reaction adds its partial derivatives only to the
    rows of its own species and the columns of the species it depends on, and
    a third body's dependence on the concentrations only where its efficiency
    is non-zero.  The concentration Jacobian is dense ns x ns in the thread's
    local memory, which suits mechanisms of up to a few tens of species."""
    ns, nv = m.ns, m.ns + 1
    idx = {s.name: k for k, s in enumerate(m.species)}
    mw = [_d(s.mw) for s in m.species]
    body = []
    w = body.append
    _thermo_lines(m, w)
    w("    double sumYW = 0.0;")
    for k, s in enumerate(m.species):
        w(f"    const double y{k} = Y[i * {ns} + {k}];")
        w(f"    sumYW += y{k} / {mw[k]};")
    w(f"    const double rho = pc / ({_d(m.r_eos)} * t * sumYW);")
    w("    const double wbar = 1.0 / sumYW;")
    for k in range(ns):
        w(f"    const double c{k} = rho * y{k} / {mw[k]};")
        w(f"    double w{k} = 0.0, JT{k} = 0.0;")
    w(f"    double Jc[{ns * ns}];   // Jc[j * {ns} + k] = d wmol_k / d c_j")
    w(f"    for (int e = 0; e < {ns * ns}; ++e) Jc[e] = 0.0;")
    w(f"    const double lnPref = log({_d(m.p_ref)} / ({_d(m.r_thermo)} * t));")
    for r in m.reactions:
        w(f"    {{  // {r.equation}")
        w(f"      const double kf = {_d(r.A)} * exp({_d(r.b)} * lnT - {_d(r.EaR)} * invT);")
        w(f"      const double dlnkf = ({_d(r.b)} + {_d(r.EaR)} * invT) * invT;")
        rnames = list(r.reactants.keys()) + [k for k in r.orders if k not in r.reactants]
        fw = [(idx[nm], r.orders.get(nm, r.reactants.get(nm, 0.0))) for nm in rnames]
        fw = [(k, o) for k, o in fw if float(o) != 0.0]
        for a, (k, o) in enumerate(fw):
            for ln in _pow_and_derivative(f"c{k}", o, f"pf{a}", f"dpf{a}"):
                w("      " + ln)
        w(f"      const double Pf = {' * '.join(f'pf{a}' for a in range(len(fw))) or '1.0'};")
        bw = []
        if r.reversible:
            bw = [(idx[nm], nu) for nm, nu in r.products.items()]
            for a, (k, nu) in enumerate(bw):
                for ln in _pow_and_derivative(f"c{k}", nu, f"pr{a}", f"dpr{a}"):
                    w("      " + ln)
            w(f"      const double Pr = {' * '.join(f'pr{a}' for a in range(len(bw))) or '1.0'};")
            dG, dH, dnu = [], [], 0.0
            for nm, nu in r.products.items():
                dG.append(f"+ {_d(nu)} * gRT{idx[nm]}")
                dH.append(f"+ {_d(nu)} * hRT{idx[nm]}")
                dnu += nu
            for nm, nu in r.reactants.items():
                dG.append(f"- {_d(nu)} * gRT{idx[nm]}")
                dH.append(f"- {_d(nu)} * hRT{idx[nm]}")
                dnu -= nu
            w(f"      const double invKc = exp(0.0 {' '.join(dG)} - {_d(dnu)} * lnPref);")
            w(f"      const double dlnKc = (0.0 {' '.join(dH)} - {_d(dnu)}) * invT;")
        else:
            w("      const double Pr = 0.0, invKc = 0.0, dlnKc = 0.0;")
        effs = None
        if r.rtype != TYPE_ELEMENTARY:
            if r.collider is not None:
                effs = {idx[r.collider]: 1.0}
            else:
                given = dict(r.efficiencies or {})
                effs = {k: given.get(s.name, r.default_eff) for k, s in enumerate(m.species)}
                effs = {k: e for k, e in effs.items() if e != 0.0}
            terms = [f"c{k}" if e == 1.0 else f"{_d(e)} * c{k}" for k, e in effs.items()]
            w(f"      const double M = {' + '.join(terms) if terms else '0.0'};")
        if r.rtype == TYPE_ELEMENTARY:
            w("      const double Mfac = 1.0, keff = kf, dlnkeff = dlnkf, dkdM = 0.0;")
        elif r.rtype == TYPE_THREEBODY:
            w("      const double Mfac = M, keff = kf, dlnkeff = dlnkf, dkdM = 0.0;")
        else:
            w(f"      const double k0 = {_d(r.A0)} * exp({_d(r.b0)} * lnT - {_d(r.EaR0)} * invT);")
            w(f"      const double dlnk0 = ({_d(r.b0)} + {_d(r.EaR0)} * invT) * invT;")
            w("      const double kratio = k0 / kf;")
            w("      const double Prd = kratio * M;")
            if r.rtype == TYPE_TROE:
                a, T3, T1 = r.troe[0], r.troe[1], r.troe[2]
                T2 = r.troe[3] if len(r.troe) > 3 else 0.0
                w(f"      const double e3 = exp(-t * {_d(1.0 / T3)}), e1 = exp(-t * {_d(1.0 / T1)});")
                fc = f"(1.0 - {_d(a)}) * e3 + {_d(a)} * e1"
                dfc = f"-(1.0 - {_d(a)}) * {_d(1.0 / T3)} * e3 - {_d(a)} * {_d(1.0 / T1)} * e1"
                if T2 != 0.0:
                    w(f"      const double e2 = exp(-{_d(T2)} * invT);")
                    fc += " + e2"
                    dfc += f" + {_d(T2)} * invT * invT * e2"
                w(f"      const double Fc = {fc}, dFc = {dfc};")
                w("      const double logFc = log10(Fc);")
                w("      const double cc = -0.4 - 0.67 * logFc, nn = 0.75 - 1.27 * logFc;")
                w("      const double x = log10(Prd > 1e-300 ? Prd : 1e-300) + cc;")
                w("      const double den = nn - 0.14 * x, f1 = x / den, opf = 1.0 + f1 * f1;")
                w("      const double F = pow(10.0, logFc / opf);")
                w("      const double Aq = 2.0 * logFc * f1 / (opf * opf * den * den);")
                w("      const double G = -Aq * nn;")
                w("      const double dlnF_T = (1.0 / opf + Aq * (0.67 * nn - 1.27 * x)) * dFc / Fc;")
            else:
                w("      const double F = 1.0, G = 0.0, dlnF_T = 0.0;")
            w("      const double opr = 1.0 + Prd;")
            w("      const double Mfac = 1.0, keff = kf * (Prd / opr) * F;")
            w("      const double dlnPr = dlnk0 - dlnkf;")
            w("      const double dlnkeff = dlnkf + dlnPr / opr + G * dlnPr + dlnF_T;")
            w("      const double dkdM = kf * F / opr * (1.0 / opr + G) * kratio;")
        w("      const double fwd = Mfac * keff * Pf;")
        w(f"      const double rvs = {'Mfac * keff * invKc * Pr' if r.reversible else '0.0'};")
        w("      const double q = fwd - rvs;")
        w("      const double kM = Mfac * keff;")
        net = {}
        for nm, nu in r.products.items():
            net[idx[nm]] = net.get(idx[nm], 0.0) + nu
        for nm, nu in r.reactants.items():
            net[idx[nm]] = net.get(idx[nm], 0.0) - nu
        net = {k: v for k, v in net.items() if v != 0.0}
        for k, nu in net.items():
            w(f"      w{k} += {_d(nu)} * q;")
        w("      const double dqdT = fwd * dlnkeff - rvs * (dlnkeff - dlnKc);")
        for k, nu in net.items():
            w(f"      JT{k} += {_d(nu)} * dqdT;")
        # d q / d c_j through the concentration products
        dq = {}
        for a, (j_, _) in enumerate(fw):
            others = "".join(f" * pf{b}" for b in range(len(fw)) if b != a)
            dq.setdefault(j_, []).append(f"kM * dpf{a}{others}")
        for a, (j_, _) in enumerate(bw):
            others = "".join(f" * pr{b}" for b in range(len(bw)) if b != a)
            dq.setdefault(j_, []).append(f"- kM * invKc * dpr{a}{others}")
        for j_, terms in dq.items():
            w(f"      {{ const double d = {' '.join(terms)};")
            for k, nu in net.items():
                w(f"        Jc[{j_ * ns + k}] += {_d(nu)} * d;")
            w("      }")
        # d q / d c_j through the third body
        if effs and net:
            tb = "keff" if r.rtype == TYPE_THREEBODY else "dkdM"
            w(f"      {{ const double g = {tb} * (Pf - invKc * Pr);")
            for k, nu in net.items():
                w(f"        const double g{k} = {_d(nu)} * g;")
            for j_, e in effs.items():
                for k in net:
                    w(f"        Jc[{j_ * ns + k}] += {'' if e == 1.0 else _d(e) + ' * '}g{k};")
            w("      }")
        w("    }")
    # Y, T variables and the energy row, as the data-driven kernel forms them
    w(f"    const double cv[{ns}] = {{{', '.join(f'c{k}' for k in range(ns))}}};")
    w(f"    const double hv[{ns}] = {{{', '.join(f'hRT{k}' for k in range(ns))}}};")
    w(f"    const double iw[{ns}] = {{{', '.join('1.0 / ' + mw[k] for k in range(ns))}}};")
    w("    double Q = 0.0, D = 0.0, HS = 0.0, dQT = 0.0, dDT = 0.0;")
    for k in range(ns):
        w(f"    double S{k} = 0.0;")
        w(f"    for (int j = 0; j < {ns}; ++j) S{k} += cv[j] * Jc[j * {ns} + {k}];")
    for k in range(ns):
        w(f"    Q += hRT{k} * w{k};")
        w(f"    D += c{k} * cpR{k};")
        w(f"    HS += hRT{k} * S{k};")
        w(f"    dQT += (cpR{k} - hRT{k}) * invT * w{k} + hRT{k} * (JT{k} - S{k} * invT);")
        w(f"    dDT += c{k} * (dcpR{k} - cpR{k} * invT);")
    w("    const double wr = wbar / rho, invD = 1.0 / D, QD = Q * invD, TD = t * invD;")
    w(f"    double* J = jac + i * (int64_t){nv * nv};")
    for k in range(ns):
        w(f"    {{ const double tk = S{k} - w{k};")
        w(f"      for (int j = 0; j < {ns}; ++j) J[j * {nv} + {k}] = {mw[k]} * iw[j] * (Jc[j * {ns} + {k}] - wr * tk);")
        w(f"      J[{ns * nv + k}] = ({mw[k]} / rho) * (JT{k} - tk * invT); }}")
    for j_ in range(ns):
        w("    { double HJ = 0.0;")
        w(f"      for (int k = 0; k < {ns}; ++k) HJ += hv[k] * Jc[{j_ * ns} + k];")
        w(f"      const double dQ = (rho / {mw[j_]}) * HJ - (wbar / {mw[j_]}) * HS;")
        w(f"      const double dD = (rho / {mw[j_]}) * cpR{j_} - (wbar / {mw[j_]}) * D;")
        w(f"      J[{j_ * nv + ns}] = -TD * (dQ - QD * dD); }}")
    w(f"    J[{ns * nv + ns}] = -QD - TD * (dQT - QD * dDT);")
    w("    if (wdot) {")
    for k in range(ns):
        w(f"      wdot[i * {ns} + {k}] = {mw[k]} * w{k};")
    w("    }")
    body_src = "\n".join(body)
    return f"""
extern "C" __global__ void __launch_bounds__(64)
ytf_{ident}_jac_kernel(int64_t n, const double* __restrict__ T, const double* __restrict__ p,
                       const double* __restrict__ Y, double* __restrict__ wdot, double* __restrict__ jac) {{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {{
    const double t = T[i], pc = p[i];
    const double lnT = log(t), invT = 1.0 / t;
{body_src}
  }}
}}

extern "C" int ytf_{ident}_wdot_jac(int64_t n, const double* T, const double* p, const double* Y, double* wdot,
                                  double* jac, void* stream) {{
  if (n <= 0) return 0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  int64_t blocks = (n + 63) / 64;
  const int64_t cap = (int64_t)sms * 32;
  if (blocks > cap) blocks = cap;
  ytf_{ident}_jac_kernel<<<(unsigned)blocks, 64, 0, (cudaStream_t)stream>>>(n, T, p, Y, wdot, jac);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}}
"""


def build(m: mechmod.Mechanism, outdir=None, quiet=True):
    """Emit and compile; returns the path of the shared library (cached by content)."""
    ident, src = emit(m)
    src += emit_jac(m, ident)
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
        fj = getattr(self.L, f"ytf_{self.ident}_wdot_jac")
        fj.argtypes = [C.c_int64] + [C.c_void_p] * 6
        fj.restype = C.c_int
        self._fnj = fj

    def wdot_jac(self, T, p, Y, wdot=None, jac=None, stream=None):
        """wdot and the constant-pressure Jacobian jac[cell, col, row] (device tensors,
        Y cell-major); the same quantities as Chemistry.wdot_jac."""
        import torch
        n, nv = T.shape[0], self.mech.ns + 1
        if jac is None:
            jac = torch.empty((n, nv, nv), dtype=torch.float64, device=T.device)
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        ptr = lambda t: C.c_void_p(t.data_ptr() if t is not None else 0)   # noqa: E731
        rc = self._fnj(n, ptr(T), ptr(p), ptr(Y), ptr(wdot), ptr(jac), C.c_void_p(st))
        if rc != 0:
            raise RuntimeError(f"generated kernel ytf_{self.ident}_jac failed to launch")
        return wdot, jac

    def wdot(self, T, p, Y, wdot=None, cp=None, h=None, stream=None, alloc=True):
        """Device tensors (torch, float64, Y cell-major (n, ns)); returns (wdot, cp, h).
        With alloc=False a cp or h left None is not computed."""
        import torch
        n = T.shape[0]
        if wdot is None:
            wdot = torch.empty_like(Y)
        if cp is None and alloc:
            cp = torch.empty_like(T)
        if h is None and alloc:
            h = torch.empty_like(T)
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        ptr = lambda t: C.c_void_p(t.data_ptr() if t is not None else 0)   # noqa: E731
        rc = self._fn(n, ptr(T), ptr(p), ptr(Y), ptr(wdot), ptr(cp), ptr(h), C.c_void_p(st))
        if rc != 0:
            raise RuntimeError(f"generated kernel ytf_{self.ident} failed to launch")
        return wdot, cp, h
