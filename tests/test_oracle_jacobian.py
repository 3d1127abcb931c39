"""The oracle's analytic Jacobian against central differences of its own RHS.

Covers elementary, third-body, Lindemann and Troe reactions (Pelucchi) and the
constant-pressure energy equation.  Complex-step is unavailable through the C
oracle, so a Richardson-extrapolated central difference is the reference.
"""
import os

import numpy as np
import pytest

from flint_gb300.mech import Mechanism
from oracle.oracle import Oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def fd_jac(orc, T, p, Y):
    n = orc.ns + 1
    x0 = np.concatenate([Y, [T]])
    J = np.zeros((n, n))
    for j in range(n):
        h = 1e-4 * max(abs(x0[j]), 1e-3 if j < n - 1 else 1.0)

        def f(hh):
            x = x0.copy(); x[j] += hh
            return orc.rhs(x[-1], p, x[:-1])
        d1 = (f(h) - f(-h)) / (2 * h)
        d2 = (f(h / 2) - f(-h / 2)) / h
        J[:, j] = (4 * d2 - d1) / 3
    return J


@pytest.mark.parametrize("T,p", [(900.0, 101325.0), (1500.0, 5e5), (2400.0, 2e6)])
def test_jacobian_vs_fd_pelucchi(T, p):
    orc = Oracle(Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json")))
    rng = np.random.default_rng(7)
    Y = rng.dirichlet(np.full(orc.ns, 0.5))
    Y = 0.98 * Y + 0.02 / orc.ns
    f, J, Js = orc.jac(T, p, Y)
    np.testing.assert_allclose(f, orc.rhs(T, p, Y), rtol=1e-13, atol=0)
    Jfd = fd_jac(orc, T, p, Y)
    scale = np.maximum(Js, 1e-300)
    err = np.abs(J - Jfd) / (scale + np.abs(Jfd))
    assert err.max() < 1e-6, (err.max(), np.unravel_index(err.argmax(), err.shape))
    assert np.all(Js >= np.abs(J) * (1 - 1e-12))


def test_jacobian_vs_fd_c1():
    from flint_gb300 import data_path
    orc = Oracle(Mechanism.load(data_path("mech_c1.json")))
    # C1 has fractional orders: keep every concentration well above zero
    Y = np.array([0.05, 0.2, 0.02, 0.03, 0.05, 0.65])
    f, J, Js = orc.jac(1600.0, 3e5, Y)
    Jfd = fd_jac(orc, 1600.0, 3e5, Y)
    err = np.abs(J - Jfd) / (Js + np.abs(Jfd) + 1e-300)
    assert err.max() < 1e-6, err.max()
