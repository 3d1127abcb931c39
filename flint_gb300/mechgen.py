"""Seeded synthetic mechanisms and state generators for the benchmark workloads.

* ``c1``  -- 2-step CH4/air (6 species, 2 irreversible reactions with
  non-integer orders, NASA-7), data/mech_c1.json, built from the reference's
  WD.yaml reactions 1-2 by tests/golden/make_golden.py.
* ``c2``  -- 31 species / 160 reversible reactions (12 third-body, 6 Troe),
  species compositions from the in-tree C/H/O/N species (TSR-Rich-31 list,
  N2 as bath), element-balanced reactions sampled from the enumeration of
  1-2 <=> 1-2 species combinations, A = 10^U(6,14) SI, b ~ U(-2,2),
  Ea ~ U(0,60) kcal/mol, third-body efficiencies U(0.5,12), NASA-7 fitted as
  two quartics (continuous at Tmid = 1000 K) to a smooth random cp(T).
* ``c5``  -- 54 species / 320 reactions (20 third-body, 12 Troe), same recipe.

The generated mechanisms are committed (data/mech_c2.json, data/mech_c5.json)
so every machine uses bit-identical coefficients; ``python -m
flint_gb300.mechgen`` regenerates them.

State generators use numpy's PCG64 with seed = 1000 + config number.
"""
from __future__ import annotations

import itertools
import json
import math
import os

import numpy as np

from . import data_path
from .mech import (Mechanism, Reaction, Species, P_ATM, R_CAL, TYPE_ELEMENTARY,
                   TYPE_THREEBODY, TYPE_TROE, ATOMIC_WEIGHTS)

# Extra C/H/O/N formulas for the 54-species pool beyond the in-tree ones.
_EXTRA = [("NO", {"N": 1, "O": 1}), ("NO2", {"N": 1, "O": 2}), ("N2O", {"N": 2, "O": 1}),
          ("NH3", {"N": 1, "H": 3}), ("NH2", {"N": 1, "H": 2}), ("NH", {"N": 1, "H": 1}),
          ("N", {"N": 1}), ("HCN", {"H": 1, "C": 1, "N": 1}), ("CN", {"C": 1, "N": 1}),
          ("HNO", {"H": 1, "N": 1, "O": 1}), ("NCO", {"N": 1, "C": 1, "O": 1}),
          ("HNCO", {"H": 1, "N": 1, "C": 1, "O": 1}), ("C3H8", {"C": 3, "H": 8}),
          ("C3H6", {"C": 3, "H": 6}), ("N2H2", {"N": 2, "H": 2})]


def _natoms(comp):
    return sum(comp.values())


def _fit_nasa7(rng, comp):
    """Two NASA-7 quartics fitted to a smooth random cp(T), continuous at 1000 K."""
    na = _natoms(comp)
    cp0 = 2.5 if na == 1 else (3.0 + 0.9 * (na - 1)) * rng.uniform(0.85, 1.1)
    cpinf = 2.5 if na == 1 else (3.0 + 1.55 * (na - 1)) * rng.uniform(0.95, 1.1)
    Tc, w = rng.uniform(700.0, 1500.0), rng.uniform(300.0, 700.0)

    def cp(T):
        return cp0 + (cpinf - cp0) * 0.5 * (1.0 + np.tanh((T - Tc) / w))

    tlow, tmid, thigh = 200.0, 1000.0, 6000.0
    Tl = np.linspace(tlow, tmid, 81)
    Th = np.linspace(tmid, thigh, 251)
    Al = np.vstack([Tl ** i for i in range(5)]).T
    Ah = np.vstack([Th ** i for i in range(5)]).T
    lo = np.linalg.lstsq(Al, cp(Tl), rcond=None)[0]
    hi = np.linalg.lstsq(Ah, cp(Th), rcond=None)[0]
    # continuity of cp at Tmid
    cl = sum(lo[i] * tmid ** i for i in range(5))
    ch = sum(hi[i] * tmid ** i for i in range(5))
    hi[0] += cl - ch
    hf_R = rng.uniform(-8000.0, 8000.0)          # h(298.15)/R  [K]
    s_R = 20.0 + 2.0 * na + rng.uniform(-3.0, 3.0)  # s(298.15)/R

    def hpoly(a, T):  # h/R without a6
        return a[0] * T + a[1] * T ** 2 / 2 + a[2] * T ** 3 / 3 + a[3] * T ** 4 / 4 + a[4] * T ** 5 / 5

    def spoly(a, T):  # s/R without a7
        return a[0] * math.log(T) + a[1] * T + a[2] * T ** 2 / 2 + a[3] * T ** 3 / 3 + a[4] * T ** 4 / 4

    T0 = 298.15
    a6l = hf_R - hpoly(lo, T0)
    a7l = s_R - spoly(lo, T0)
    a6h = hpoly(lo, tmid) + a6l - hpoly(hi, tmid)
    a7h = spoly(lo, tmid) + a7l - spoly(hi, tmid)
    low = [float(x) for x in lo] + [float(a6l), float(a7l)]
    high = [float(x) for x in hi] + [float(a6h), float(a7h)]
    return tlow, tmid, thigh, low, high


def _balanced_combos(names, comps, elements):
    """All element-balanced (reactants, products) with 1-2 species per side."""
    vec = {n: np.array([comps[n].get(e, 0) for e in elements]) for n in names}
    sides = [(a,) for a in names] + list(itertools.combinations_with_replacement(names, 2))
    bykey = {}
    for s in sides:
        v = sum(vec[x] for x in s)
        bykey.setdefault(tuple(int(t) for t in v), []).append(s)
    out = []
    for key, group in bykey.items():
        for i in range(len(group)):
            for j in range(i + 1, len(group)):
                a, b = group[i], group[j]
                if set(a) & set(b):
                    continue
                out.append((a, b))
    out.sort()
    return out


def synthetic(ns, nr, n3b, ntroe, seed, name):
    """Build a seeded synthetic reversible mechanism (see module docstring)."""
    rng = np.random.default_rng(seed)
    with open(data_path("chon_species.json")) as f:
        pool = [(s["name"], s["composition"]) for s in json.load(f)["species"]]
    names_pool = [n for n, _ in pool if n != "N2"]
    comps = dict(pool)
    for n, c in _EXTRA:
        if n not in comps:
            names_pool.append(n)
            comps[n] = c
    # reactive species: largest-first excluded until ns-1 remain, N2 last (bath)
    reactive = names_pool[: ns - 1] if ns - 1 <= len(names_pool) else None
    if reactive is None:
        raise ValueError("species pool too small")
    if ns - 1 < len(names_pool) and "IC3H7CO" in reactive:
        reactive = [n for n in names_pool if n != "IC3H7CO"][: ns - 1]
    names = reactive + ["N2"]
    comps["N2"] = {"N": 2}
    elements = ["C", "H", "O", "N"]
    species = []
    for n in names:
        tl, tm, th, low, high = _fit_nasa7(rng, comps[n])
        mw = sum(ATOMIC_WEIGHTS[e] * k for e, k in comps[n].items())
        species.append(Species(n, float(mw), dict(comps[n]), tl, tm, th, low, high))
    combos = _balanced_combos(reactive, comps, elements)
    uni_bi = [c for c in combos if (len(c[0]) == 1) != (len(c[1]) == 1)]
    # pick falloff/third-body among 1 <=> 2 combos, the rest among all
    perm = rng.permutation(len(uni_bi))
    chosen, used = [], set()
    for idx in perm:
        c = uni_bi[idx]
        if c in used:
            continue
        chosen.append(("tb" if len(chosen) < n3b else "troe", c))
        used.add(c)
        if len(chosen) == n3b + ntroe:
            break
    perm = rng.permutation(len(combos))
    for idx in perm:
        if len(chosen) == nr:
            break
        c = combos[idx]
        if c in used:
            continue
        chosen.append(("el", c))
        used.add(c)
    if len(chosen) < nr:
        raise ValueError("not enough balanced combinations")
    # element-balanced sides; order reactions: elementary, three-body, Troe
    chosen.sort(key=lambda t: {"el": 0, "tb": 1, "troe": 2}[t[0]])
    reactions = []
    kcal = 1000.0 / R_CAL
    for kind, (a, b) in chosen:
        if rng.uniform() < 0.5:
            a, b = b, a
        reac, prod = {}, {}
        for x in a:
            reac[x] = reac.get(x, 0.0) + 1.0
        for x in b:
            prod[x] = prod.get(x, 0.0) + 1.0
        eq = " + ".join(a) + " <=> " + " + ".join(b)
        A = 10.0 ** rng.uniform(6.0, 14.0)
        beta = rng.uniform(-2.0, 2.0)
        EaR = rng.uniform(0.0, 60.0) * kcal
        if kind == "el":
            reactions.append(Reaction(eq, TYPE_ELEMENTARY, reac, prod, {}, True, A, beta, EaR))
            continue
        effs = {}
        for k in rng.choice(len(names), size=min(6, len(names)), replace=False):
            effs[names[int(k)]] = float(rng.uniform(0.5, 12.0))
        if kind == "tb":
            reactions.append(Reaction(eq.replace(" <=> ", " + M <=> ") + " + M", TYPE_THREEBODY, reac, prod, {},
                                      True, A, beta, EaR, efficiencies=effs))
        else:
            A0 = A * 10.0 ** rng.uniform(1.0, 4.0)
            b0 = beta - rng.uniform(0.0, 2.0)
            E0 = EaR * rng.uniform(0.0, 0.8)
            troe = [float(rng.uniform(0.3, 0.9)), float(10 ** rng.uniform(1.5, 3.0)),
                    float(10 ** rng.uniform(2.5, 3.7)),
                    float(10 ** rng.uniform(3.0, 4.0)) if rng.uniform() < 0.5 else 0.0]
            eqf = " + ".join(a) + " (+M) <=> " + " + ".join(b) + " (+M)"
            reactions.append(Reaction(eqf, TYPE_TROE, reac, prod, {}, True, A, beta, EaR, A0, b0, E0, troe,
                                      efficiencies=effs))
    return Mechanism(name, species, reactions, elements)


def load(config):
    """Mechanism of a benchmark configuration: 'c1', 'c2' or 'c5'."""
    return Mechanism.load(data_path(f"mech_{config}.json"))


# --------------------------------------------------------------------- states
def c1_states(n, seed=1001):
    """T~U(300,2500) K, p~U(1,20) atm, Y = (1-c) Y_unburnt(phi) + c Y_burnt(phi)."""
    mech = load("c1")
    rng = np.random.default_rng(seed)
    T = rng.uniform(300.0, 2500.0, n)
    p = rng.uniform(1.0, 20.0, n) * P_ATM
    phi = rng.uniform(0.5, 2.0, n)
    c = rng.uniform(0.0, 1.0, n)
    names = [s.name for s in mech.species]
    W = np.array([s.mw for s in mech.species])
    iCH4, iO2, iCO, iCO2, iH2O, iN2 = (names.index(k) for k in ("CH4", "O2", "CO", "CO2", "H2O", "N2"))
    o2 = 2.0 / phi
    Xu = np.zeros((n, 6))
    Xu[:, iCH4] = 1.0; Xu[:, iO2] = o2; Xu[:, iN2] = 3.76 * o2
    x = np.minimum(1.0, o2 / 1.5)          # CH4 burnt to CO + 2 H2O
    o2l = o2 - 1.5 * x
    y = np.minimum(x, 2.0 * o2l)           # CO burnt to CO2
    Xb = np.zeros((n, 6))
    Xb[:, iCH4] = 1.0 - x; Xb[:, iCO] = x - y; Xb[:, iCO2] = y; Xb[:, iH2O] = 2.0 * x
    Xb[:, iO2] = o2l - 0.5 * y; Xb[:, iN2] = 3.76 * o2
    Yu = Xu * W; Yu /= Yu.sum(1, keepdims=True)
    Yb = Xb * W; Yb /= Yb.sum(1, keepdims=True)
    Y = (1.0 - c)[:, None] * Yu + c[:, None] * Yb
    Y = np.clip(Y, 0.0, None)
    return T, p, np.ascontiguousarray(Y)


def c2_states(n, mech=None, seed=1002, alpha=0.3):
    """T~U(800,2800) K, p~U(1,40) atm, Y~Dirichlet(alpha) over the species."""
    mech = mech or load("c2")
    rng = np.random.default_rng(seed)
    T = rng.uniform(800.0, 2800.0, n)
    p = rng.uniform(1.0, 40.0, n) * P_ATM
    Y = rng.dirichlet(np.full(mech.ns, alpha), size=n)
    return T, p, np.ascontiguousarray(Y)


def fuel_air_states(n, mech, seed, T0=(900.0, 1600.0), patm=(1.0, 20.0), phi=(0.5, 2.0),
                    log10dt=(-6.0, -4.0), fuel="CH4"):
    """Reactor initial states: fuel + air (O2:N2 = 1:3.76) at equivalence ratio phi."""
    rng = np.random.default_rng(seed)
    names = [s.name for s in mech.species]
    W = np.array([s.mw for s in mech.species])
    comp = mech.species[names.index(fuel)].composition
    o2_st = comp.get("C", 0) + comp.get("H", 0) / 4.0 - comp.get("O", 0) / 2.0
    T = rng.uniform(T0[0], T0[1], n)
    p = rng.uniform(patm[0], patm[1], n) * P_ATM
    ph = rng.uniform(phi[0], phi[1], n)
    dt = 10.0 ** rng.uniform(log10dt[0], log10dt[1], n)
    X = np.zeros((n, mech.ns))
    X[:, names.index(fuel)] = 1.0
    X[:, names.index("O2")] = o2_st / ph
    X[:, names.index("N2")] = 3.76 * o2_st / ph
    Y = X * W
    Y /= Y.sum(1, keepdims=True)
    return T, p, np.ascontiguousarray(Y), dt


def c3_states(n, mech=None, seed=1003, log10dt=(-6.0, -4.0)):
    mech = mech or load("c2")
    return fuel_air_states(n, mech, seed, log10dt=log10dt)


def c5_states(n, mech=None, seed=1005, log10dt=(-7.0, -4.0)):
    mech = mech or load("c5")
    return fuel_air_states(n, mech, seed, T0=(900.0, 2000.0), patm=(1.0, 40.0), phi=(0.4, 3.0),
                           log10dt=log10dt)


def main():
    for cfg, (ns, nr, n3b, ntroe, seed) in {"c2": (31, 160, 12, 6, 2002), "c5": (54, 320, 20, 12, 2005)}.items():
        m = synthetic(ns, nr, n3b, ntroe, seed, f"synthetic-{ns}sp-{nr}r")
        with open(data_path(f"mech_{cfg}.json"), "w") as f:
            f.write(m.to_json())
        print(cfg, m.ns, m.nr, sum(r.rtype == 1 for r in m.reactions), sum(r.rtype == 3 for r in m.reactions))


if __name__ == "__main__":
    main()
