"""The gate calibration search (host logic): the accepted set it returns holds
no out-of-tolerance cell, its thresholds reproduce that set, and on small
synthetic data no threshold combination on the same candidate grids accepts
more (brute force)."""
import itertools

import numpy as np

from flint_gb300.surrogate import DEFAULT_GATE, search_gate


def synthetic(n=3000, seed=0):
    rng = np.random.default_rng(seed)
    M = np.zeros((n, 6))
    M[:, 0] = rng.exponential(0.05, n)          # energy residual
    M[:, 1] = rng.uniform(0, 1e-6, n)           # element residual
    M[:, 2] = -rng.uniform(0, 1e-6, n)          # realizability
    M[:, 3] = rng.exponential(0.05, n)          # ensemble dT spread
    M[:, 4] = rng.exponential(2e-5, n)          # ensemble dY spread
    M[:, 5] = 1.0
    T0 = rng.uniform(900, 2000, n)
    ld = rng.uniform(-7, -4, n)
    # errors grow with the spreads, the dt and the start temperature
    eY = 0.5 * M[:, 4] * rng.uniform(0.2, 2.0, n) * (1 + 3 * (ld > -4.5)) * (1 + (T0 > 1900))
    eT = 0.5 * M[:, 3] * rng.uniform(0.2, 2.0, n)
    return M, eT, eY, T0, ld


def accepted(M, T0, ld, g):
    return ((M[:, 5] > 0) & (M[:, 1] <= DEFAULT_GATE["max_elem_resid"]) & (M[:, 2] >= DEFAULT_GATE["min_Y"])
            & (M[:, 0] <= g["max_dT_resid"]) & (M[:, 3] <= g["max_ens_dT"]) & (M[:, 4] <= g["max_ens_dY"])
            & (ld <= g["log10dt_hi"]) & (T0 <= g["T_hi"]))


def test_search_is_safe_and_consistent():
    M, eT, eY, T0, ld = synthetic()
    for margin in (0.5, 0.8):
        frac, g, mT, mY = search_gate(M, eT, eY, T0, ld, DEFAULT_GATE, 2, margin=margin)
        acc = accepted(M, T0, ld, g)
        assert acc.mean() == frac and frac > 0.3
        assert (eY[acc] <= margin * 1e-4).all() and (eT[acc] <= margin * 1.0).all()
        assert mY == eY[acc].max() and mT == eT[acc].max()


def test_search_beats_brute_force_on_its_grids():
    M, eT, eY, T0, ld = synthetic(600, 3)
    frac, g, _, _ = search_gate(M, eT, eY, T0, ld, DEFAULT_GATE, 2, margin=0.5)
    good = (eT <= 0.5) & (eY <= 0.5e-4)
    best = 0
    q = np.linspace(0.0, 1.0, 21)
    for dth, Th in itertools.product(np.quantile(ld, [0.7, 0.8, 0.9, 1.0]), np.quantile(T0, [0.85, 0.95, 1.0])):
        for a, b, c in itertools.product(np.quantile(M[:, 0], q), np.quantile(M[:, 3], q), np.quantile(M[:, 4], q)):
            acc = ((M[:, 0] <= a) & (M[:, 3] <= b) & (M[:, 4] <= c) & (ld <= dth) & (T0 <= Th))
            if acc.any() and good[acc].all():
                best = max(best, acc.mean())
    assert frac >= best
