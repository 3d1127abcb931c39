"""Parity with the reference's generated Fortran mechanism routines.

FLINT's chemistry_source dispatches a named mechanism to its routine in
src/lib/Lib_ChemMech/ (Lib_Chemistry_wdot.f90:24-91), written by
utils/YTF.py.  Mechanism.ytf_form() restates YTF's emission rules on the
mechanism IR; these tests hold it to the ten generated routines of the tree
(tests/golden/fortran_forms.json):

* structure, reaction by reaction: the rate source and its table row, the
  concentration factors of prodf and prodb (stoichiometric coefficients,
  truncated, custom orders unused), the third body (efficiencies as printed,
  zeros of three-body reactions dropped, falloff efficiencies defaulting to 1,
  termolecular reactions with a species on both sides read as three-body with
  that collider) and every omegadot coefficient;
* arithmetic: the routine evaluated in NumPy (tests/fortran_forms.py) with the
  oracle's rate constants equals the oracle's wdot of ytf_form() to 1e-12 of
  the sum of the absolute terms (the GPU test does the same for the kernels).
"""
import os

import numpy as np
import pytest

from flint_gb300 import mechgen
from flint_gb300.mech import Mechanism
from oracle.oracle import Oracle

import fortran_forms as FF

FORMS = FF.load_forms()


def _mech(form):
    return Mechanism.load(os.path.join(FF.GOLD, form["mechanism"])).ytf_form()


@pytest.mark.parametrize("name", sorted(FORMS))
def test_structure_matches_the_routine(name):
    form = FORMS[name]
    m = _mech(form)
    names = [s.name for s in m.species]
    ns = len(names)
    assert len(form["reactions"]) == m.nr
    count = {"arrh": 0, "troe": 0, "lind": 0}
    for i, (fr, r) in enumerate(zip(form["reactions"], m.reactions)):
        kind = {0: "arrh", 1: "arrh", 2: "lind", 3: "troe"}[r.rtype]
        count[kind] += 1
        assert (fr["kind"], fr["table_index"]) == (kind, count[kind]), (i, r.equation)
        fwd = sorted(sum([[names.index(k)] * int(v) for k, v in r.orders.items()], []))
        bwd = sorted(sum([[names.index(k)] * int(v) for k, v in r.products.items()], []))
        assert (fr["fwd"], fr["bwd"]) == (fwd, bwd), (i, r.equation)
        assert bool(fr.get("Mf")) == bool(fr.get("Mb")) == (r.rtype == 1), (i, r.equation)
        if r.rtype != 0:
            M = fr["M"]
            got = {k: 1.0 for k in range(ns)} if M == "sum" else {int(k): v for k, v in M.items()}
            if r.collider is not None:
                want = {names.index(r.collider): 1.0}
            else:
                want = {k: (r.efficiencies or {}).get(names[k], r.default_eff) for k in range(ns)}
                if r.rtype == 1:
                    want = {k: v for k, v in want.items() if v != 0.0}
            assert got == want, (i, r.equation)
    # omegadot(k) = Wm(k) * sum_r (nu'' - nu') (prodf - prodb)
    for k, terms in enumerate(form["omegadot"]):
        got = {r: nip - nir for r, nip, nir in terms}
        want = {}
        for r, rx in enumerate(m.reactions):
            if names[k] in rx.reactants or names[k] in rx.products:
                want[r] = rx.products.get(names[k], 0.0) - rx.reactants.get(names[k], 0.0)
        assert got == want, (name, names[k])


@pytest.mark.parametrize("name", sorted(FORMS))
def test_routine_arithmetic_equals_the_oracle(name):
    form = FORMS[name]
    m = _mech(form)
    orc = Oracle(m)
    T, p, Y = mechgen.c2_states(64, m, seed=71)
    T = np.clip(T, 800.0, 2800.0)
    W = np.array([s.mw for s in m.species])
    rho = p / (m.r_eos * T * (Y / W).sum(1))
    w_ref, sc = FF.omegadot(form, W, rho[:, None] * Y, FF.analytic_rates(orc, m, T))
    w_o, _, _, _ = orc.wdot_batch(T, p, Y)
    err = np.abs(w_o.reshape(w_ref.shape) - w_ref) / (sc + 1e-300)
    assert err.max() < 1e-12, (name, err.max())


def test_troyes_routine_on_its_tables_equals_the_general_loop():
    """troyes.f90 on the reference's own Troyes tables (its .szplt files, with
    the reference's lerp a + (b - a) Tdiff) against FLINT's general loop on the
    same tables (the oracle's restatement of Lib_Chemistry_wdot.f90:96-220)."""
    from oracle.oracle import TableOracle
    from test_szl import troyes_tables
    t = troyes_tables()
    form = FORMS["troyes"]
    rng = np.random.default_rng(5)
    n = 256
    T = rng.uniform(300.0, 2990.0, n)
    Y = rng.dirichlet(np.full(t["ns"], 0.4), n)
    roi = rng.uniform(0.05, 20.0, n)[:, None] * Y
    Ti = T.astype(np.int64)
    Td = T - Ti

    def lerp(tab, j):
        a, b = tab[j, Ti - t["ti1"]], tab[j, Ti + 1 - t["ti1"]]
        return a + (b - a) * Td

    rates = [{"kf": lerp(t["kf_tab"], fr["table_index"] - 1), "kb": lerp(t["kb_tab"], fr["table_index"] - 1)}
             for fr in form["reactions"]]
    w_ref, sc = FF.omegadot(form, t["wm"], roi, rates)
    w_gen = TableOracle(t).general(roi, T)
    assert np.max(np.abs(w_gen - w_ref) / (sc + 1e-300)) < 1e-13
