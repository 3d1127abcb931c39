"""Wilke mixture viscosity and conductivity (co_k_mi_lam_Wilke,
Lib_ThermoTransport.f90:407-462) on tabulated species values.

No transport table ships with the reference's tests, so the species tables
here are smooth synthetic ones on the 2-step mechanism's thermo grid.  CPU:
the oracle against a pure-Python restatement (same operation order: bit for
bit) and the single-species limit (Wilke's rule returns the species' own
value).  GPU: the batched kernel against the oracle, bit for bit."""
import copy
import math

import numpy as np
import pytest

from flint_gb300 import mechgen, tables
from oracle.oracle import TableOracle


@pytest.fixture(scope="module")
def tab():
    m = copy.deepcopy(mechgen.load("c1"))
    t = tables.generate(m, 200, 4000)
    T = np.arange(t["tmin"], t["tmax"] + 1, dtype=np.float64)
    rng = np.random.default_rng(5)
    a = rng.uniform(1.0e-5, 3.0e-5, m.ns)
    b = rng.uniform(0.01, 0.05, m.ns)
    t["mi_tab"] = np.array([ai * (T / 300.0) ** 0.7 for ai in a])
    t["k_tab"] = np.array([bi * (T / 300.0) ** 0.8 for bi in b])
    return m, t


def _lerp(tab, tmin, nrow, T, s):
    Ti = int(T)
    row = min(max(Ti - tmin, 0), nrow - 2)
    a, b = float(tab[s][row]), float(tab[s][row + 1])
    return a + (b - a) * (T - Ti)


def py_wilke(t, r, T):
    ns, W = t["ns"], [float(w) for w in t["wm"]]
    nrow = t["tmax"] - t["tmin"] + 1

    def ssum(x):
        s = 0.0
        for v in x:
            s = s + v
        return s

    rho = ssum(r)
    acc = 0.0
    for s in range(ns):
        acc = acc + r[s] / rho / W[s]
    Wmtot = 1.0 / acc
    X = [r[s] * Wmtot / (rho * W[s]) for s in range(ns)]
    mi = [_lerp(t["mi_tab"], t["tmin"], nrow, T, s) for s in range(ns)]
    ki = [_lerp(t["k_tab"], t["tmin"], nrow, T, s) for s in range(ns)]
    den = []
    for i in range(ns):
        d = 0.0
        for j in range(ns):
            MiMj = W[i] / W[j]
            a = 1.0 + math.sqrt(mi[i] / (mi[j] + 1e-20)) / MiMj ** 0.25
            d = d + X[j] * (a * a / math.sqrt(8.0 * (1.0 + MiMj)))
        den.append(d)
    mu = lam = 0.0
    for s in range(ns):
        inv = 1.0 / den[s]
        mu = mu + X[s] * mi[s] * inv
        lam = lam + X[s] * ki[s] * inv
    return mu, lam


def _cells(m, t, n, seed):
    T, p, Y = mechgen.c1_states(n, seed=seed)
    W = np.array([s.mw for s in m.species])
    rho = p / (t["runiv"] * T * (Y / W).sum(1))
    return rho[:, None] * Y, T


def test_oracle_matches_python_restatement(tab):
    m, t = tab
    rhoi, T = _cells(m, t, 50, 3)
    mu, lam = TableOracle(t).transport(rhoi, T)
    for i in range(len(T)):
        assert (mu[i], lam[i]) == py_wilke(t, [float(x) for x in rhoi[i]], float(T[i]))


def test_single_species_limit(tab):
    m, t = tab
    n = m.ns
    rhoi = np.eye(n) * 0.7
    T = np.full(n, 1234.5)
    mu, lam = TableOracle(t).transport(rhoi, T)
    nrow = t["tmax"] - t["tmin"] + 1
    for s in range(n):
        assert mu[s] == pytest.approx(_lerp(t["mi_tab"], t["tmin"], nrow, 1234.5, s), rel=1e-15)
        assert lam[s] == pytest.approx(_lerp(t["k_tab"], t["tmin"], nrow, 1234.5, s), rel=1e-15)


@pytest.mark.gpu
def test_gpu_bit_exact(tab):
    torch = pytest.importorskip("torch")
    m, t = tab
    rhoi, T = _cells(m, t, 5000, 4)
    mu_o, lam_o = TableOracle(t).transport(rhoi, T)
    gpu = tables.Tables(t)
    mu, lam = gpu.transport(torch.from_numpy(rhoi).cuda(), torch.from_numpy(T).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(mu.cpu().numpy(), mu_o)
    assert np.array_equal(lam.cpu().numpy(), lam_o)
