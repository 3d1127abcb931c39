"""cons2prim (Lib_ThermoTransport.f90:129-165) on tabulated thermo.

CPU: the oracle against a second, pure-Python restatement of the reference's
iteration (the same sequential sums and operation order, so the two agree bit
for bit), and a prim -> cons -> prim round trip.  GPU: the batched kernel
against the oracle, bit for bit (both uncontracted, in the reference's order)."""
import copy
import math

import numpy as np
import pytest

from flint_gb300 import mechgen, tables
from oracle.oracle import TableOracle


@pytest.fixture(scope="module")
def tab():
    m = copy.deepcopy(mechgen.load("c1"))
    return m, tables.generate(m, 200, 4000)


def _lerp(t, name, T, s):
    tmin, tmax = t["tmin"], t["tmax"]
    Ti = int(T)
    row = min(max(Ti - tmin, 0), tmax - tmin - 1)
    col = t[name][:, s] if t[name].shape[0] == tmax - tmin + 1 else t[name][s]
    a, b = float(col[row]), float(col[row + 1])
    return a + (b - a) * (T - Ti)


def py_cons2prim(t, cons, T):
    """The reference's cons2prim, restated with Python floats."""
    ns = t["ns"]
    W = [float(x) for x in t["wm"]]
    R = [t["runiv"] / w for w in W]
    np_ = len(cons)
    r = [float(x) for x in cons[:ns]]

    def ssum(x):
        s = 0.0
        for v in x:
            s = s + v
        return s

    def rtot(r):
        rho = ssum(r); res = 0.0
        for s in range(ns):
            res = res + R[s] * r[s] / rho
        return res

    Rgas = rtot(r); rho = ssum(r)
    u = [float(c) / rho for c in cons[ns:np_ - 1]]
    scale, ssq = 1.0, 0.0
    for x in u:
        if x != 0.0:
            a = abs(x)
            if scale < a:
                v = scale / a; ssq = 1.0 + ssq * v * v; scale = a
            else:
                v = a / scale; ssq = ssq + v * v
    vel = scale * math.sqrt(ssq)
    energy = float(cons[-1]) / rho - 0.5 * vel * vel
    diff, Ti, it = 1.0e3, float(T), 1
    while abs(diff / energy) >= 1e-6 and it <= 20:
        p = rho * Rgas * Ti
        cp = 0.0
        for s in range(ns):
            cp = cp + r[s] / rho * _lerp(t, "cp_tab", Ti, s)
        cv = cp - Rgas
        rho_h = ssum(r); Rh = rtot(r); Th = p / (Rh * rho_h)
        h = 0.0
        for s in range(ns):
            h = h + _lerp(t, "h_tab", Th, s) * r[s] / rho_h
        e_it = h - p / ssum(r)
        diff = abs(e_it - energy)
        Ti = Ti + (energy - e_it) / cv
        it += 1
    return r + u + [rho * Rgas * Ti], Ti


def _cells(m, t, n, ndim, seed):
    """Conservative states from primitive (rho_i, u, T) with the table's e(T)."""
    rng = np.random.default_rng(seed)
    T, p, Y = mechgen.c1_states(n, seed=seed)
    W = np.array([s.mw for s in m.species])
    rho = p / (t["runiv"] * T * (Y / W).sum(1))
    u = rng.uniform(-400, 400, size=(n, ndim))
    e = np.zeros(n)
    for i in range(n):
        R = sum(t["runiv"] / W[s] * Y[i, s] for s in range(m.ns))
        h = sum(_lerp(t, "h_tab", T[i], s) * Y[i, s] for s in range(m.ns))
        e[i] = h - R * T[i]
    cons = np.hstack([rho[:, None] * Y, rho[:, None] * u, (rho * (e + 0.5 * (u ** 2).sum(1)))[:, None]])
    Tguess = T * rng.uniform(0.8, 1.2, size=n)
    return cons, Tguess, T, p


def test_oracle_matches_python_restatement(tab):
    m, t = tab
    cons, Tg, _, _ = _cells(m, t, 40, 3, 5)
    prim, Tout = TableOracle(t).cons2prim(cons, Tg)
    for i in range(len(Tg)):
        ref, Tr = py_cons2prim(t, cons[i], Tg[i])
        assert list(prim[i]) == ref and Tout[i] == Tr


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_round_trip(tab, ndim):
    m, t = tab
    cons, Tg, T, p = _cells(m, t, 200, ndim, 6 + ndim)
    prim, Tout = TableOracle(t).cons2prim(cons, Tg)
    assert np.max(np.abs(Tout - T) / T) < 1e-5
    assert np.max(np.abs(prim[:, -1] - p) / p) < 1e-5
    np.testing.assert_array_equal(prim[:, :m.ns], cons[:, :m.ns])


@pytest.mark.gpu
@pytest.mark.parametrize("ndim", [0, 3])
def test_gpu_bit_exact(tab, ndim):
    torch = pytest.importorskip("torch")
    m, t = tab
    cons, Tg, _, _ = _cells(m, t, 3000, max(ndim, 1), 11)
    if ndim == 0:
        cons = np.hstack([cons[:, :m.ns], cons[:, -1:]])
    prim_o, T_o = TableOracle(t).cons2prim(cons, Tg)
    gpu = tables.Tables(t)
    prim, Tout = gpu.cons2prim(torch.from_numpy(cons).cuda(), torch.from_numpy(Tg).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(prim.cpu().numpy(), prim_o)
    assert np.array_equal(Tout.cpu().numpy(), T_o)
