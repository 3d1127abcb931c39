"""The oracle's constant-pressure BDF reactor on the CPU: against SciPy's BDF at
tight tolerances (an independent integrator of the same right-hand side), on the
54-species scale-up mechanism against its own rtol = 1e-12 solution, and the
per-cell status codes."""
import numpy as np
import pytest

from flint_gb300 import mechgen
from flint_gb300.native import reactor_opts
from oracle.oracle import Oracle


def test_reactor_vs_scipy_bdf_c3():
    integrate = pytest.importorskip("scipy.integrate")
    mech = mechgen.load("c2")
    T, p, Y, dt = mechgen.c3_states(12, mech, seed=77)
    orc = Oracle(mech)
    T1, Y1, st, nst = orc.reactor_advance(T, p, Y, dt, reactor_opts(), nthreads=1)
    assert (st == 0).all()
    ns = mech.ns
    for i in range(len(T)):
        def f(t, y):
            return orc.rhs(y[ns], p[i], y[:ns])

        def jac(t, y):
            return orc.jac(y[ns], p[i], y[:ns])[1]

        y0 = np.concatenate([Y[i], [T[i]]])
        sol = integrate.solve_ivp(f, (0.0, dt[i]), y0, method="BDF", jac=jac, rtol=1e-11, atol=1e-17)
        assert sol.status == 0
        assert abs(T1[i] - sol.y[ns, -1]) / sol.y[ns, -1] < 1e-5
        assert np.abs(Y1[i] - sol.y[:ns, -1]).max() < 1e-6


def test_reactor_c5_all_cells_converge():
    """54 species / 320 reactions: stiff oscillatory modes defeat BDF orders 3-5 on
    a few cells; the order <= 2 retry must bring every cell home, accurately."""
    mech = mechgen.load("c5")
    T, p, Y, dt = mechgen.c5_states(160, mech, seed=51)
    orc = Oracle(mech)
    T1, Y1, st, nst = orc.reactor_advance(T, p, Y, dt, reactor_opts())
    Tx, Yx, stx, _ = orc.reactor_advance(T, p, Y, dt, reactor_opts(rtol=1e-12, atol=1e-18, max_steps=400000))
    assert (st == 0).all() and (stx == 0).all()
    assert np.max(np.abs(T1 - Tx) / Tx) < 1e-5
    assert np.abs(Y1 - Yx).max() < 1e-6


def test_reactor_status_codes_cpu():
    mech = mechgen.load("c2")
    T, p, Y, dt = mechgen.c3_states(5, mech, seed=3)
    T = T.copy(); p = p.copy(); Y = Y.copy(); dt = dt.copy()
    T[0] = np.nan                 # NaN input
    T[1] = 7000.0                 # above tmax
    dt[2] = 0.0                   # nothing to do
    p[3] = -1.0                   # non-positive pressure
    Y0 = Y.copy()
    T1, Y1, st, nst = orc_run(mech, T, p, Y, dt)
    assert list(st[:4]) == [2, 1, 0, 2]
    assert np.array_equal(Y1[2], Y0[2]) and nst[2] == 0
    _, _, st5, nst5 = orc_run(mech, T[4:], p[4:], Y[4:], dt[4:], max_steps=5)
    assert st5[0] == 3 and nst5[0] == 5


def orc_run(mech, T, p, Y, dt, **kw):
    return Oracle(mech).reactor_advance(T, p, Y, dt, reactor_opts(**kw))


def _u_mass(mech, T, Y):
    """Mixture internal energy per kg, sum_k Y_k/W_k R (h_k/RT - 1) T (NASA-7)."""
    W = np.array([s.mw for s in mech.species])
    hRT = np.zeros(mech.ns)
    for k, sp in enumerate(mech.species):
        a = sp.low if T < sp.tmid else sp.high
        hRT[k] = a[0] + a[1] * T / 2 + a[2] * T ** 2 / 3 + a[3] * T ** 3 / 4 + a[4] * T ** 4 / 5 + a[5] / T
    return (Y / W * (hRT - 1.0)).sum() * mech.r_thermo * T


def test_constv_reactor_vs_scipy_and_energy():
    """Constant volume (opts.constant_volume = 1): the oracle's BDF against
    SciPy's BDF on the same constant-volume RHS, the density held at the initial
    state's, and the mixture internal energy conserved (the adiabatic rigid
    vessel of rhs_native, Lib_Chemistry_rhs.f90:43-50)."""
    integrate = pytest.importorskip("scipy.integrate")
    mech = mechgen.load("c2")
    T, p, Y, dt = mechgen.c3_states(8, mech, seed=78)
    orc = Oracle(mech)
    T1, Y1, st, nst = orc.reactor_advance(T, p, Y, dt, reactor_opts(constant_volume=True), nthreads=1)
    assert (st == 0).all()
    ns = mech.ns
    W = np.array([s.mw for s in mech.species])
    for i in range(len(T)):
        rho = p[i] / (mech.r_eos * T[i] * (Y[i] / W).sum())

        def f(t, y):
            return orc.rhs_constv(y[ns], rho, y[:ns])

        def jac(t, y):
            return orc.jac_constv(y[ns], rho, y[:ns])[1]

        y0 = np.concatenate([Y[i], [T[i]]])
        sol = integrate.solve_ivp(f, (0.0, dt[i]), y0, method="BDF", jac=jac, rtol=1e-11, atol=1e-17)
        assert sol.status == 0
        assert abs(T1[i] - sol.y[ns, -1]) / sol.y[ns, -1] < 1e-5
        assert np.abs(Y1[i] - sol.y[:ns, -1]).max() < 1e-6
        u0, u1 = _u_mass(mech, T[i], Y[i]), _u_mass(mech, T1[i], Y1[i])
        assert abs(u1 - u0) <= 1e-6 * (abs(u0) + mech.r_thermo * T[i] * (Y[i] / W).sum())
    # the option changes the system: the same cells at constant pressure end elsewhere
    Tp, _, stp, _ = orc.reactor_advance(T, p, Y, dt, reactor_opts(), nthreads=1)
    assert (stp == 0).all() and np.abs(T1 - Tp).max() > 1.0
