"""The reference's generated Fortran mechanism routines, evaluated in NumPy.

tests/golden/fortran_forms.json holds each src/lib/Lib_ChemMech/*.f90 routine
that utils/YTF.py writes (parsed by tests/golden/make_golden.py): per reaction
its rate source, the species of the concentration factors of prodf and prodb,
whether the third body M multiplies them and M's terms; per species the
omegadot terms.  ``omegadot`` below executes that routine's arithmetic on a
batch of cells, in its order:

    coi = roi / Wm
    prodf(r) = kf(r) * coi(a) * coi(b) ... [* M]      (f_kf or k(1) of f_k_troe / f_k_lindemann)
    prodb(r) = kb(r) * coi(c) ... [* M]               (f_kb or k(2))
    omegadot(k) = Wm(k) * sum_r (nu''_kr - nu'_kr) * (prodf(r) - prodb(r))

with the rate constants supplied by the caller (the reference reads them from
its tables; the tests take the oracle's analytic values, which the golden
tables pin, or the tables themselves).  f_k_troe / f_k_lindemann follow
src/lib/Lib_Chemistry_falloff.f90:12-80.
"""
import json
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load_forms():
    with open(os.path.join(GOLD, "fortran_forms.json")) as f:
        return json.load(f)


def troe_rates(kinf, k0, kc, fcent, M):
    """k(1), k(2) of f_k_troe (Lib_Chemistry_falloff.f90:37-60, f_F :62-80)."""
    Pr = k0 * M / kinf
    logF = np.log10(fcent)
    logPr = np.log10(Pr)
    c = -0.4 - 0.67 * logF
    n = 0.75 - 1.27 * logF
    f1 = (logPr + c) / (n - 0.14 * (logPr + c))
    F = 10.0 ** (logF / (1.0 + f1 * f1))
    k1 = kinf * (Pr / (1.0 + Pr)) * F
    return k1, k1 / kc


def lindemann_rates(kinf, k0, kc, M):
    """k(1), k(2) of f_k_lindemann (Lib_Chemistry_falloff.f90:12-34)."""
    Pr = k0 * M / kinf
    k1 = kinf * (Pr / (1.0 + Pr))
    return k1, k1 / kc


def omegadot(form, W, roi, rates):
    """The routine's omegadot for cells roi (n, ns) [kg/m^3] and per-reaction
    rate data rates[r] = dict(kf=..., kb=...) (arrays over cells) for "arrh"
    reactions or dict(kinf=, k0=, kc=, fcent=) for "troe" / "lind" ones.
    Returns (omegadot (n, ns), scale (n, ns)): the scale is the sum of the
    absolute values of the terms of each species sum, for error bars."""
    W = np.asarray(W, dtype=np.float64)
    coi = roi / W[None, :]
    n, ns = roi.shape
    R = len(form["reactions"])
    pf = np.zeros((R, n))
    pb = np.zeros((R, n))
    for r, fr in enumerate(form["reactions"]):
        M = None
        if fr.get("M") is not None:
            if fr["M"] == "sum":
                M = coi.sum(axis=1)
            else:
                M = np.zeros(n)
                for k, e in fr["M"].items():
                    M = M + coi[:, int(k)] * e
        d = rates[r]
        if fr["kind"] == "arrh":
            kf, kb = d["kf"], d["kb"]
        elif fr["kind"] == "troe":
            kf, kb = troe_rates(d["kinf"], d["k0"], d["kc"], d["fcent"], M)
        else:
            kf, kb = lindemann_rates(d["kinf"], d["k0"], d["kc"], M)
        f = kf * np.ones(n)
        for k in fr["fwd"]:
            f = f * coi[:, k]
        b = kb * np.ones(n)
        for k in fr["bwd"]:
            b = b * coi[:, k]
        if fr.get("Mf"):
            f = f * M
        if fr.get("Mb"):
            b = b * M
        pf[r], pb[r] = f, b
    w = np.zeros((n, ns))
    sc = np.zeros((n, ns))
    for k, terms in enumerate(form["omegadot"]):
        for r, nip, nir in terms:
            w[:, k] += (nip - nir) * (pf[r] - pb[r])
            sc[:, k] += abs(nip - nir) * (np.abs(pf[r]) + np.abs(pb[r]))
        w[:, k] *= W[k]
        sc[:, k] *= W[k]
    return w, sc


def analytic_rates(orc, mech, T):
    """Per-reaction rate data of the routine from the oracle's analytic rate
    constants at each cell's T: kf, kb = kf / Kc (0 when irreversible); for
    falloff k_inf, k_0, Kc, F_cent."""
    cols = [orc.rate_constants(t) for t in T]
    kf = np.array([c[0] for c in cols]).T
    Kc = np.array([c[1] for c in cols]).T
    k0 = np.array([c[2] for c in cols]).T
    fc = np.array([c[3] for c in cols]).T
    out = []
    for r, rx in enumerate(mech.reactions):
        if rx.rtype >= 2:
            out.append({"kinf": kf[r], "k0": k0[r], "kc": Kc[r] if rx.reversible else np.full(len(T), np.inf),
                        "fcent": fc[r] if rx.rtype == 3 else np.ones(len(T))})
        else:
            out.append({"kf": kf[r], "kb": kf[r] / Kc[r] if rx.reversible else np.zeros(len(T))})
    return out
