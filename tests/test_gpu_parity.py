"""GPU parity: the CUDA library through the C-ABI against the FP64 oracle.

Tolerances: net production rates and Jacobian entries agree with the oracle to
1e-12 relative to the absolute sum of their terms (the scale the oracle
accumulates); mixture cp and h to 1e-13 relative.  The reactor is compared by
its own tolerance: both the GPU and the oracle run against a
tighter-tolerance oracle solution.
"""
import os

import numpy as np
import pytest

from flint_gb300 import mechgen
from flint_gb300.api import Chemistry, CELL_MAJOR, SPECIES_MAJOR
from flint_gb300.mech import Mechanism
from oracle.oracle import Oracle
from flint_gb300.native import reactor_opts

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

RTOL_WDOT = 1e-12


def cuda(*arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def wdot_err(w, w_ref, scale):
    return np.max(np.abs(w - w_ref) / (scale + 1e-300)) if w.size else 0.0


@pytest.fixture(scope="module")
def c1():
    return Chemistry.from_config("c1")


@pytest.fixture(scope="module")
def c2():
    return Chemistry.from_config("c2")


@pytest.mark.parametrize("n", [65536, 1, 33, 1000])
def test_c1_wdot_cp_h(c1, n):
    orc = Oracle(c1.mech)
    T, p, Y = mechgen.c1_states(n)
    w_o, ws_o, cp_o, h_o = orc.wdot_batch(T, p, Y)
    Tt, pt, Yt = cuda(T, p, Y)
    cp, h = torch.empty_like(Tt), torch.empty_like(Tt)
    w, _, _ = c1.wdot(Tt, pt, Yt, cp=cp, h=h)
    torch.cuda.synchronize()
    assert wdot_err(w.cpu().numpy().ravel(), w_o, ws_o) < RTOL_WDOT
    np.testing.assert_allclose(cp.cpu().numpy(), cp_o, rtol=1e-13)
    hs = np.abs(h_o) + cp_o * T
    assert np.max(np.abs(h.cpu().numpy() - h_o) / hs) < 1e-13


@pytest.mark.parametrize("layout", [CELL_MAJOR, SPECIES_MAJOR])
def test_thermo_batch(c2, layout):
    """flint_thermo_batch: mixture cp and h (f_cp / H on NASA-7) against the oracle."""
    orc = Oracle(c2.mech)
    T, p, Y = mechgen.c2_states(5000, c2.mech, seed=13)
    _, _, cp_o, h_o = orc.wdot_batch(T, p, Y)
    Tt, Yt = cuda(T, Y if layout == CELL_MAJOR else Y.T.copy())
    cp, h = torch.empty_like(Tt), torch.empty_like(Tt)
    c2.thermo(Tt, Yt, layout=layout, cp=cp, h=h)
    torch.cuda.synchronize()
    np.testing.assert_allclose(cp.cpu().numpy(), cp_o, rtol=1e-13)
    assert np.max(np.abs(h.cpu().numpy() - h_o) / (np.abs(h_o) + cp_o * T)) < 1e-13


def test_c1_species_major_layout(c1):
    orc = Oracle(c1.mech)
    T, p, Y = mechgen.c1_states(4099, seed=77)
    w_o, ws_o, _, _ = orc.wdot_batch(T, p, Y)
    Tt, pt, Ys = cuda(T, p, Y.T.copy())
    w, _, _ = c1.wdot(Tt, pt, Ys, layout=SPECIES_MAJOR)
    torch.cuda.synchronize()
    assert wdot_err(w.cpu().numpy().T.ravel(), w_o, ws_o) < RTOL_WDOT


def test_c1_host_path(c1):
    orc = Oracle(c1.mech)
    T, p, Y = mechgen.c1_states(2048, seed=5)
    w_o, ws_o, cp_o, _ = orc.wdot_batch(T, p, Y)
    w, cp, _ = c1.wdot(T, p, Y)
    assert wdot_err(w.ravel(), w_o, ws_o) < RTOL_WDOT
    np.testing.assert_allclose(cp, cp_o, rtol=1e-13)


def test_c1_chemistry_source_clamps(c1):
    """chemistry_source(roi, T): negative partial densities clamp to 0 in place."""
    T, p, Y = mechgen.c1_states(512, seed=9)
    orc = Oracle(c1.mech)
    W = np.array([s.mw for s in c1.mech.species])
    rho = p / (c1.mech.r_eos * T * (Y / W).sum(1))
    roi = rho[:, None] * Y
    roi[::7, 1] = -1e-3  # negative O2 partial density
    roi_t, Tt = cuda(roi, T)
    w = c1.chemistry_source(roi_t, Tt)
    torch.cuda.synchronize()
    roi_c = np.clip(roi, 0, None)
    assert (roi_t.cpu().numpy() >= 0).all()
    rho_c = roi_c.sum(1)
    Yc = roi_c / rho_c[:, None]
    pc = rho_c * c1.mech.r_eos * T * (Yc / W).sum(1)
    w_o, ws_o, _, _ = orc.wdot_batch(T, pc, Yc)
    assert wdot_err(w.cpu().numpy().ravel(), w_o, ws_o) < 1e-11


@pytest.mark.parametrize("cfg", ["c2", "pelucchi", "c5"])
def test_wdot_and_jacobian(cfg):
    if cfg == "pelucchi":
        import os
        mech = Mechanism.load(os.path.join(os.path.dirname(__file__), "golden", "mech_pelucchi.json"))
        T, p, Y = mechgen.c2_states(1500, mech, seed=11)
    elif cfg == "c5":
        mech = mechgen.load("c5")            # 54 species: two species per lane
        T, p, Y = mechgen.c2_states(1200, mech, seed=12)
    else:
        mech = mechgen.load("c2")
        T, p, Y = mechgen.c2_states(3000, mech)
    chem = Chemistry(mech)
    orc = Oracle(mech)
    w_o, ws_o, _, _ = orc.wdot_batch(T, p, Y)
    _, J_o, Js_o = orc.wdot_jac_batch(T, p, Y)
    Tt, pt, Yt = cuda(T, p, Y)
    w, _, _ = chem.wdot(Tt, pt, Yt)
    w2 = torch.empty_like(Yt)
    _, J = chem.wdot_jac(Tt, pt, Yt, wdot=w2)
    torch.cuda.synchronize()
    assert wdot_err(w.cpu().numpy().ravel(), w_o, ws_o) < RTOL_WDOT
    assert wdot_err(w2.cpu().numpy().ravel(), w_o, ws_o) < RTOL_WDOT
    Jg = J.cpu().numpy().ravel()
    err = np.abs(Jg - J_o) / (Js_o + 1e-300)
    assert err.max() < RTOL_WDOT, err.max()


def test_table_driven_exp_vs_cuda(c2):
    """The kernels' exp (Tang's table method) within 2 ulp of CUDA's exp."""
    import ctypes as C
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-700, 700, 400000), rng.uniform(-2, 2, 100000),
                        [0.0, -0.0, 1e-300, -1e-20, 699.9, -699.9, 700.0, -745.0, 710.0, np.inf, -np.inf, np.nan]])
    xt = torch.from_numpy(x).cuda()
    y = torch.empty(2 * x.size, dtype=torch.float64, device="cuda")
    rc = c2.L.flint_selftest_exp(c2.h, x.size, C.c_void_p(xt.data_ptr()), C.c_void_p(y.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    yy = y.cpu().numpy().reshape(-1, 2)
    fin = np.isfinite(yy[:, 1]) & (yy[:, 1] > 0)
    rel = np.abs(yy[fin, 0] / yy[fin, 1] - 1.0)
    assert rel.max() < 4.5e-16, rel.max()
    same = ~fin
    np.testing.assert_array_equal(np.isnan(yy[same, 0]), np.isnan(yy[same, 1]))
    np.testing.assert_array_equal(yy[same & ~np.isnan(yy[:, 1]), 0], yy[same & ~np.isnan(yy[:, 1]), 1])


def test_table_driven_log_vs_cuda(c2):
    """The kernels' ln (Tang's table method) within 2 ulp of CUDA's log, and
    within 2e-17 absolutely near x = 1; zero, subnormal, negative, inf and NaN
    arguments take CUDA's log itself."""
    import ctypes as C
    rng = np.random.default_rng(2)
    x = np.concatenate([10.0 ** rng.uniform(-307, 307, 300000), rng.uniform(200.0, 6000.0, 100000),
                        rng.uniform(0.98, 1.02, 100000), 1.0 + rng.uniform(-1e-6, 1e-6, 20000),
                        2.0 ** np.arange(-1022, 1024, 1.0), np.nextafter(2.0 ** np.arange(-1021, 1024, 1.0), 0.0),
                        [1.0, 2.0, 0.5, 0.0, -0.0, -1.0, 5e-324, 1e-310, np.inf, -np.inf, np.nan,
                         np.finfo(float).max, np.finfo(float).tiny]])
    xt = torch.from_numpy(x).cuda()
    y = torch.empty(2 * x.size, dtype=torch.float64, device="cuda")
    rc = c2.L.flint_selftest_log(c2.h, x.size, C.c_void_p(xt.data_ptr()), C.c_void_p(y.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    yy = y.cpu().numpy().reshape(-1, 2)
    fin = np.isfinite(yy[:, 1])
    err = np.abs(yy[fin, 0] - yy[fin, 1])
    assert (err <= np.maximum(2 * np.spacing(np.abs(yy[fin, 1])), 2e-17)).all(), err.max()
    same = ~fin
    np.testing.assert_array_equal(np.isnan(yy[same, 0]), np.isnan(yy[same, 1]))
    np.testing.assert_array_equal(yy[same & ~np.isnan(yy[:, 1]), 0], yy[same & ~np.isnan(yy[:, 1]), 1])


def test_empty_batch(c2):
    Tt = torch.empty(0, dtype=torch.float64, device="cuda")
    Yt = torch.empty((0, c2.ns), dtype=torch.float64, device="cuda")
    w, _, _ = c2.wdot(Tt, Tt, Yt)
    torch.cuda.synchronize()
    assert w.shape == (0, c2.ns)


def _reactor_case(n, seed=3):
    mech = mechgen.load("c2")
    T, p, Y, dt = mechgen.c3_states(n, mech, seed=seed)
    return mech, T, p, Y, dt


def test_reactor_vs_oracle():
    mech, T, p, Y, dt = _reactor_case(384)
    chem = Chemistry(mech)
    orc = Oracle(mech)
    opts = reactor_opts()
    T_o, Y_o, st_o, ns_o = orc.reactor_advance(T, p, Y, dt, opts)
    T_x, Y_x, st_x, _ = orc.reactor_advance(T, p, Y, dt, reactor_opts(rtol=1e-12, atol=1e-18, max_steps=400000))
    Tt, pt, Yt, dtt = cuda(T, p, Y, dt)
    st, nst = chem.reactor_advance(Tt, pt, Yt, dtt)
    torch.cuda.synchronize()
    st, nst = st.cpu().numpy(), nst.cpu().numpy()
    Tg, Yg = Tt.cpu().numpy(), Yt.cpu().numpy()
    assert (st == 0).all() and (st_o == 0).all() and (st_x == 0).all()
    # same algorithm: adaptive step sequences diverge by roundoff cell by cell,
    # but the total work agrees
    assert abs(nst.sum() / ns_o.sum() - 1.0) < 0.05
    # both close to the tight solution: the local tolerances rtol=1e-8,
    # atol=1e-14 accumulate over ~650 steps into a global error of ~1e-8 in Y
    # and ~1e-4 K in T; the bounds leave a factor ~50 of margin
    for Tv, Yv in ((Tg, Yg), (T_o, Y_o)):
        errT = np.abs(Tv - T_x) / np.abs(T_x)
        errY = np.abs(Yv - Y_x)
        assert errT.max() < 1e-5 and errY.max() < 1e-6, (errT.max(), errY.max())
    # GPU and oracle agree to the integrator tolerance
    assert np.max(np.abs(Tg - T_o) / T_o) < 1e-6
    assert np.max(np.abs(Yg - Y_o)) < 1e-6


def test_reactor_status_codes():
    mech, T, p, Y, dt = _reactor_case(8, seed=4)
    T[1] = np.nan            # NaN input
    T[2] = 7000.0            # out of range
    dt[3] = 0.0              # nothing to do
    p[4] = -1.0              # bad pressure
    chem = Chemistry(mech)
    Tt, pt, Yt, dtt = cuda(T, p, Y, dt)
    Y3 = Y[3].copy()
    st, nst = chem.reactor_advance(Tt, pt, Yt, dtt)
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    assert st[1] == 2 and st[2] == 1 and st[3] == 0 and st[4] == 2
    assert np.array_equal(Yt.cpu().numpy()[3], Y3)
    # bounded work: a tiny step limit reports MAX_STEPS
    mech, T, p, Y, dt = _reactor_case(4, seed=5)
    Tt, pt, Yt, dtt = cuda(T, p, Y, dt)
    st, nst = chem.reactor_advance(Tt, pt, Yt, dtt, max_steps=5)
    torch.cuda.synchronize()
    assert (st.cpu().numpy() == 3).all() and (nst.cpu().numpy() == 5).all()


def test_reactor_real_mechanism_pelucchi():
    """Reactor on the reference's Pelucchi mechanism (25 species: third-body,
    Lindemann and Troe falloff, Cl chemistry): GPU vs oracle vs a tight oracle run."""
    import os
    mech = Mechanism.load(os.path.join(os.path.dirname(__file__), "golden", "mech_pelucchi.json"))
    names = [s.name for s in mech.species]
    rng = np.random.default_rng(17)
    n = 256
    X = np.zeros((n, mech.ns))
    phi = rng.uniform(0.5, 2.0, n)
    X[:, names.index("H2")] = 2.0 * phi
    X[:, names.index("O2")] = 1.0
    X[:, names.index("N2")] = 3.76
    X[:, names.index("HCL")] = rng.uniform(0.0, 0.5, n)
    X[:, names.index("CO")] = rng.uniform(0.0, 0.3, n)
    W = np.array([s.mw for s in mech.species])
    Y = X * W
    Y /= Y.sum(1, keepdims=True)
    T = rng.uniform(1100.0, 1600.0, n)
    p = rng.uniform(1.0, 10.0, n) * 101325.0
    dt = 10.0 ** rng.uniform(-6.0, -4.5, n)
    orc = Oracle(mech)
    T_o, Y_o, st_o, ns_o = orc.reactor_advance(T, p, Y, dt, reactor_opts())
    T_x, Y_x, st_x, _ = orc.reactor_advance(T, p, Y, dt, reactor_opts(rtol=1e-12, atol=1e-18, max_steps=400000))
    chem = Chemistry(mech)
    Tt, pt, Yt, dtt = cuda(T, p, Y, dt)
    st, nst = chem.reactor_advance(Tt, pt, Yt, dtt)
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    assert (st == 0).all() and (st_o == 0).all() and (st_x == 0).all()
    Tg, Yg = Tt.cpu().numpy(), Yt.cpu().numpy()
    # many cells ignite within dt (T rises by up to ~1500 K): the ignition
    # delay amplifies the local tolerance into a global error of ~5e-6 in T
    # and ~2e-6 in Y, and a cell caught in the middle of its ignition front at
    # the end of dt (cell 125: 1170 K -> 1490 K) reaches 5.1e-5 in T and
    # 2.2e-5 in Y, in the oracle and the GPU alike; the bounds here are
    # therefore 10-20x looser than for the non-igniting synthetic cases
    for Tv, Yv in ((Tg, Yg), (T_o, Y_o)):
        assert np.max(np.abs(Tv - T_x) / T_x) < 1e-4 and np.abs(Yv - Y_x).max() < 5e-5
    assert abs(nst.cpu().numpy().sum() / ns_o.sum() - 1.0) < 0.05


def test_reactor_c5_54_species():
    """The 54-species / 320-reaction scale-up mechanism (55 unknowns: two per lane,
    the Newton matrix in a global per-warp slot)."""
    mech = mechgen.load("c5")
    T, p, Y, dt = mechgen.c5_states(160, mech, seed=51)
    orc = Oracle(mech)
    T_o, Y_o, st_o, ns_o = orc.reactor_advance(T, p, Y, dt, reactor_opts())
    T_x, Y_x, st_x, _ = orc.reactor_advance(T, p, Y, dt, reactor_opts(rtol=1e-12, atol=1e-18, max_steps=400000))
    chem = Chemistry(mech)
    Tt, pt, Yt, dtt = cuda(T, p, Y, dt)
    st, nst = chem.reactor_advance(Tt, pt, Yt, dtt)
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    assert (st == 0).all() and (st_o == 0).all() and (st_x == 0).all()
    Tg, Yg = Tt.cpu().numpy(), Yt.cpu().numpy()
    for Tv, Yv in ((Tg, Yg), (T_o, Y_o)):
        assert np.max(np.abs(Tv - T_x) / T_x) < 1e-5 and np.abs(Yv - Y_x).max() < 1e-6
    assert abs(nst.cpu().numpy().sum() / ns_o.sum() - 1.0) < 0.05


INTREE = ["ecker", "smooke", "troyes", "tsr_cdf_13", "tsr_gp_24", "tsr_rich_31", "zk", "coria", "wd", "cross"]


@pytest.mark.parametrize("name", INTREE)
def test_intree_mechanisms_wdot_jacobian_generated(name):
    """The reference's own mechanisms (test/*/INPUT/*.yaml, as IR; WD and Cross
    with NASA-9 thermo): data-driven wdot, cp, h and Jacobian, and the generated
    per-mechanism kernel."""
    import os
    from flint_gb300.ytf_cuda import GeneratedMechanism
    mech = Mechanism.load(os.path.join(os.path.dirname(__file__), "golden", f"mech_{name}.json"))
    T, p, Y = mechgen.c2_states(1000, mech, seed=31)
    T = np.clip(T, 300.0, 3400.0)
    orc = Oracle(mech)
    w_o, ws_o, cp_o, h_o = orc.wdot_batch(T, p, Y)
    _, J_o, Js_o = orc.wdot_jac_batch(T, p, Y)
    chem = Chemistry(mech)
    Tt, pt, Yt = cuda(T, p, Y)
    cp, h = torch.empty_like(Tt), torch.empty_like(Tt)
    w, _, _ = chem.wdot(Tt, pt, Yt, cp=cp, h=h)
    _, J = chem.wdot_jac(Tt, pt, Yt)
    wg, cpg, hg = GeneratedMechanism(mech).wdot(Tt, pt, Yt)
    torch.cuda.synchronize()
    assert wdot_err(w.cpu().numpy().ravel(), w_o, ws_o) < RTOL_WDOT
    np.testing.assert_allclose(cp.cpu().numpy(), cp_o, rtol=1e-13)
    hs = np.abs(h_o) + cp_o * T
    assert np.max(np.abs(h.cpu().numpy() - h_o) / hs) < 1e-13
    assert wdot_err(wg.cpu().numpy().ravel(), w_o, ws_o) < RTOL_WDOT
    np.testing.assert_allclose(cpg.cpu().numpy(), cp_o, rtol=1e-13)
    err = np.abs(J.cpu().numpy().ravel() - J_o) / (Js_o + 1e-300)
    assert err.max() < RTOL_WDOT, err.max()


def test_reactor_tsr_rich_31():
    """A real 31-species / 197-reaction mechanism (TSR-Rich-31, 12 Troe) in the reactor."""
    import os
    mech = Mechanism.load(os.path.join(os.path.dirname(__file__), "golden", "mech_tsr_rich_31.json"))
    T, p, Y, dt = tsr_rich_states(mech, 96, 71)
    orc = Oracle(mech)
    T_o, Y_o, st_o, ns_o = orc.reactor_advance(T, p, Y, dt, reactor_opts())
    T_x, Y_x, st_x, _ = orc.reactor_advance(T, p, Y, dt, reactor_opts(rtol=1e-12, atol=1e-18, max_steps=400000))
    chem = Chemistry(mech)
    Tt, pt, Yt, dtt = cuda(T, p, Y, dt)
    st, nst = chem.reactor_advance(Tt, pt, Yt, dtt)
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    assert (st == 0).all() and (st_o == 0).all() and (st_x == 0).all()
    Tg, Yg = Tt.cpu().numpy(), Yt.cpu().numpy()
    for Tv, Yv in ((Tg, Yg), (T_o, Y_o)):
        assert np.max(np.abs(Tv - T_x) / T_x) < 5e-5 and np.abs(Yv - Y_x).max() < 2e-5
    assert abs(nst.cpu().numpy().sum() / ns_o.sum() - 1.0) < 0.05


def tsr_rich_states(mech, n, seed):
    """CH4/O2 at phi 0.5-2 diluted by 30-50 % CO2 and H2O (the mechanism has no N2)."""
    rng = np.random.default_rng(seed)
    names = [sp.name for sp in mech.species]
    X = np.zeros((n, mech.ns))
    phi = rng.uniform(0.5, 2.0, n)
    dil = rng.uniform(0.3, 0.5, n)
    X[:, names.index("CH4")] = phi / (phi + 2.0) * (1 - dil)
    X[:, names.index("O2")] = 2.0 / (phi + 2.0) * (1 - dil)
    X[:, names.index("CO2")] = 0.5 * dil
    X[:, names.index("H2O")] = 0.5 * dil
    W = np.array([sp.mw for sp in mech.species])
    Y = X * W
    Y /= Y.sum(1, keepdims=True)
    T = rng.uniform(1300.0, 1900.0, n)
    p = rng.uniform(1.0, 20.0, n) * 101325.0
    dt = 10.0 ** rng.uniform(-5.0, -3.0, n)
    return T, p, Y, dt


@pytest.mark.parametrize("cfg", ["c2", "c5"])
def test_reactor_autotune(cfg):
    """The autotuner times the shared-memory and global-slot layouts and keeps
    the fastest; every layout computes the same numbers."""
    mech = mechgen.load(cfg)
    states = mechgen.c5_states if cfg == "c5" else mechgen.c3_states
    T, p, Y, dt = states(256, mech, seed=91)
    chem = Chemistry(mech)
    Tt, pt, Yt, dtt = cuda(T, p, Y, dt)
    Ta, Ya = Tt.clone(), Yt.clone()
    sa, na = chem.reactor_advance(Ta, pt, Ya, dtt)
    lay = chem.reactor_autotune(Tt, pt, Yt, dtt)
    torch.cuda.synchronize()
    assert np.array_equal(Tt.cpu().numpy(), T) and np.array_equal(Yt.cpu().numpy(), Y)   # inputs untouched
    assert lay in ((1, 2, 3) if cfg == "c2" else (2, 3))
    sb, nb = chem.reactor_advance(Tt, pt, Yt, dtt)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(Tt.cpu().numpy(), Ta.cpu().numpy())
    np.testing.assert_array_equal(Yt.cpu().numpy(), Ya.cpu().numpy())
    np.testing.assert_array_equal(nb.cpu().numpy(), na.cpu().numpy())


@pytest.mark.parametrize("name", ["pelucchi", "c5"])
def test_handle_from_ir_blob_matches_descriptor(name):
    """flint_mech_create_from_ir (the mechanism as one IR byte string) gives a
    handle whose wdot, cp, h and Jacobian equal, bit for bit, those of the
    handle built from the same mechanism's descriptor."""
    mech = (mechgen.load(name) if name == "c5" else
            Mechanism.load(os.path.join(os.path.dirname(__file__), "golden", f"mech_{name}.json")))
    a, b = Chemistry(mech), Chemistry.from_ir(mech.to_ir())
    assert (b.ns, b.nr) == (mech.ns, mech.nr)
    T, p, Y = mechgen.c2_states(777, mech, seed=41)
    Tt, pt, Yt = cuda(np.clip(T, 300.0, 3400.0), p, Y)
    outs = []
    for chem in (a, b):
        cp, h = torch.empty_like(Tt), torch.empty_like(Tt)
        w, _, _ = chem.wdot(Tt, pt, Yt, cp=cp, h=h)
        _, J = chem.wdot_jac(Tt, pt, Yt)
        outs.append((w, cp, h, J))
    torch.cuda.synchronize()
    for x, y in zip(*outs):
        assert torch.equal(x, y)


@pytest.mark.parametrize("cfg", ["pelucchi", "c5"])
def test_constv_rhs_and_jacobian(cfg):
    """Constant volume (rhs_native's system with the analytic mechanism): the
    RHS and the fixed-density Jacobian against the oracle, to 1e-12 of the
    oracle's term scale, on one (Pelucchi: Troe, Lindemann) and two (54
    species) species per lane."""
    if cfg == "c5":
        mech = mechgen.load("c5")
    else:
        mech = Mechanism.load(os.path.join(os.path.dirname(__file__), "golden", "mech_pelucchi.json"))
    T, p, Y = mechgen.c2_states(1100, mech, seed=17)
    W = np.array([s.mw for s in mech.species])
    rho = p / (mech.r_eos * T * (Y / W).sum(1))
    orc = Oracle(mech)
    f_o, J_o, Js_o = orc.jac_constv_batch(T, rho, Y)
    chem = Chemistry(mech)
    Tt, rt, Yt = cuda(T, rho, Y)
    f = chem.rhs_constv(Tt, rt, Yt)
    _, J = chem.wdot_jac_constv(Tt, rt, Yt)
    torch.cuda.synchronize()
    nv = mech.ns + 1
    Jg = J.cpu().numpy().ravel()
    assert (np.abs(Jg - J_o) / (Js_o + 1e-300)).max() < RTOL_WDOT
    # f's term scales: wscale / rho for dY/dt, T x the scale of d(dT/dt)/dT
    # (which bounds sum |u_k wdot_k| / (rho cv)) for dT/dt
    _, ws_o, _, _ = orc.wdot_batch(T, p, Y)
    fsT = T * Js_o.reshape(len(T), nv, nv)[:, mech.ns, mech.ns]
    fs = np.concatenate([ws_o.reshape(-1, mech.ns) / rho[:, None], fsT[:, None]], axis=1)
    assert (np.abs(f.cpu().numpy() - f_o) / (fs + 1e-300)).max() < RTOL_WDOT
    # at the density the pressure implies, dY/dt equals the constant-pressure one
    fp = torch.empty((len(T), nv), dtype=torch.float64, device="cuda")
    pt = cuda(p)[0]
    assert chem.L.flint_rhs_constp_batch(chem.h, len(T), Tt.data_ptr(), pt.data_ptr(), Yt.data_ptr(),
                                         fp.data_ptr(), None) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(f.cpu().numpy()[:, :-1], fp.cpu().numpy()[:, :-1], rtol=1e-11,
                               atol=1e-12 * fs[:, :-1].max())


def test_constv_reactor_vs_oracle():
    """opts.constant_volume = 1: the GPU reactor and the oracle's, both against
    a tight-tolerance oracle solution, and the mixture internal energy held."""
    mech, T, p, Y, dt = _reactor_case(256, seed=8)
    chem = Chemistry(mech)
    orc = Oracle(mech)
    T_o, Y_o, st_o, ns_o = orc.reactor_advance(T, p, Y, dt, reactor_opts(constant_volume=True))
    T_x, Y_x, st_x, _ = orc.reactor_advance(T, p, Y, dt, reactor_opts(rtol=1e-12, atol=1e-18, max_steps=400000,
                                                                       constant_volume=True))
    Tt, pt, Yt, dtt = cuda(T, p, Y, dt)
    st, nst = chem.reactor_advance(Tt, pt, Yt, dtt, constant_volume=True)
    torch.cuda.synchronize()
    st, nst = st.cpu().numpy(), nst.cpu().numpy()
    Tg, Yg = Tt.cpu().numpy(), Yt.cpu().numpy()
    assert (st == 0).all() and (st_o == 0).all() and (st_x == 0).all()
    assert abs(nst.sum() / ns_o.sum() - 1.0) < 0.05
    for Tv, Yv in ((Tg, Yg), (T_o, Y_o)):
        assert np.max(np.abs(Tv - T_x) / T_x) < 1e-5 and np.abs(Yv - Y_x).max() < 1e-6
    assert np.max(np.abs(Tg - T_o) / T_o) < 1e-6 and np.max(np.abs(Yg - Y_o)) < 1e-6
    # internal energy per kg, sum_k Y_k/W_k R T (h_k/RT - 1), before and after
    W = np.array([s.mw for s in mech.species])

    def u_mass(Tc, Yc):
        hRT = np.zeros((len(Tc), mech.ns))
        for k, sp in enumerate(mech.species):
            lo = Tc < sp.tmid
            for sel, a in ((lo, sp.low), (~lo, sp.high)):
                t = Tc[sel]
                hRT[sel, k] = a[0] + a[1] * t / 2 + a[2] * t ** 2 / 3 + a[3] * t ** 3 / 4 + a[4] * t ** 4 / 5 + a[5] / t
        return (Yc / W * (hRT - 1.0)).sum(1) * mech.r_thermo * Tc
    u0, u1 = u_mass(T, Y), u_mass(Tg, Yg)
    scale = np.abs(u0) + mech.r_thermo * T * (Y / W).sum(1)
    assert np.max(np.abs(u1 - u0) / scale) < 1e-6
    # constant pressure on the same cells ends elsewhere (the option takes effect)
    Tt2, Yt2 = cuda(T, Y)
    chem.reactor_advance(Tt2, pt, Yt2, dtt)
    torch.cuda.synchronize()
    assert np.abs(Tt2.cpu().numpy() - Tg).max() > 1.0
