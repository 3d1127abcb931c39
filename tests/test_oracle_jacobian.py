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


def fd_jac_constv(orc, T, rho, Y):
    """At fixed density the rates are low-order polynomials in each c_j (rational
    through falloff M): a 1 % step on the species columns keeps the Richardson
    central difference accurate and clear of the round-off in wdot's large
    opposing terms, which a 1e-4 step does not for the small entries."""
    n = orc.ns + 1
    x0 = np.concatenate([Y, [T]])
    J = np.zeros((n, n))
    steps = np.zeros(n)
    for j in range(n):
        h = 1e-2 * max(abs(x0[j]), 1e-3) if j < n - 1 else 1e-4 * abs(x0[j])
        steps[j] = h

        def f(hh):
            x = x0.copy(); x[j] += hh
            return orc.rhs_constv(x[-1], rho, x[:-1])
        d1 = (f(h) - f(-h)) / (2 * h)
        d2 = (f(h / 2) - f(-h / 2)) / h
        J[:, j] = (4 * d2 - d1) / 3
    return J, steps


@pytest.mark.parametrize("T,rho", [(900.0, 0.4), (1500.0, 1.2), (2400.0, 3.0)])
def test_constv_jacobian_vs_fd_pelucchi(T, rho):
    """The constant-volume system (rhs_native's, Lib_Chemistry_rhs.f90:15-52)
    with the analytic mechanism: Jacobian at fixed density against central
    differences of its own RHS; Troe, Lindemann and third-body reactions."""
    orc = Oracle(Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json")))
    rng = np.random.default_rng(9)
    Y = rng.dirichlet(np.full(orc.ns, 0.5))
    Y = 0.98 * Y + 0.02 / orc.ns
    f, J, Js = orc.jac_constv(T, rho, Y)
    np.testing.assert_allclose(f, orc.rhs_constv(T, rho, Y), rtol=1e-13, atol=0)
    Jfd, steps = fd_jac_constv(orc, T, rho, Y)
    # round-off floor of a difference quotient: a row's f is a sum of terms as
    # large as its term scale (wscale / rho for the species rows), so the
    # quotient carries an error of ~1e-13 of that scale over the step
    W = np.array([s.mw for s in orc.mech.species])
    p_eq = rho * orc.mech.r_eos * T * (Y / W).sum()
    _, ws, _, _ = orc.wdot_batch(np.array([T]), np.array([p_eq]), Y[None, :], nthreads=1)
    fs = np.concatenate([ws / rho, [abs(f[-1])]])
    noise = 1e-13 * fs[:, None] / steps[None, :]
    excess = np.abs(J - Jfd) - (1e-6 * (Js + np.abs(Jfd)) + noise)
    assert excess.max() <= 0.0, np.unravel_index(excess.argmax(), excess.shape)
    resolved = noise < 1e-6 * (Js + np.abs(Jfd))
    assert resolved.mean() > 0.5          # most entries are held to 1e-6 itself
    assert np.all(Js >= np.abs(J) * (1 - 1e-12))


def test_constv_and_constp_share_species_rates():
    """At the density the constant-pressure state implies, both systems give the
    same dY/dt; dT/dt differs by the ratio of (sum u wdot)/(rho cv) to
    (sum h wdot)/(rho cp), recomputed here from the NASA-7 thermo."""
    mech = Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json"))
    orc = Oracle(mech)
    rng = np.random.default_rng(4)
    Y = rng.dirichlet(np.full(orc.ns, 0.5))
    T, p = 1700.0, 3e5
    W = np.array([s.mw for s in mech.species])
    rho = p / (mech.r_eos * T * (Y / W).sum())
    fp, fv = orc.rhs(T, p, Y), orc.rhs_constv(T, rho, Y)
    np.testing.assert_allclose(fv[:-1], fp[:-1], rtol=1e-12, atol=1e-300)
    cpR = np.zeros(orc.ns); hRT = np.zeros(orc.ns)
    for k, sp in enumerate(mech.species):
        a = sp.low if T < sp.tmid else sp.high
        cpR[k] = a[0] + a[1] * T + a[2] * T ** 2 + a[3] * T ** 3 + a[4] * T ** 4
        hRT[k] = a[0] + a[1] * T / 2 + a[2] * T ** 2 / 3 + a[3] * T ** 3 / 4 + a[4] * T ** 4 / 5 + a[5] / T
    wmol = fp[:-1] * rho / W
    c = rho * Y / W
    Tp = -T * (hRT * wmol).sum() / (c * cpR).sum()
    Tv = -T * ((hRT - 1.0) * wmol).sum() / (c * (cpR - 1.0)).sum()
    np.testing.assert_allclose([fp[-1], fv[-1]], [Tp, Tv], rtol=1e-10)
