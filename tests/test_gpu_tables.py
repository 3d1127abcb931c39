"""GPU parity of FLINT's tabulated path (general loop, rhs_native) through the C-ABI.

The Arrhenius part is evaluated in the reference's operation order with
uncontracted IEEE operations, so it matches the oracle bit for bit; falloff
reactions call log10/pow, where the CUDA and C libraries differ by an ulp, and
are held to 1e-12 of the cell's largest production rate."""
import copy
import os

import numpy as np
import pytest

from flint_gb300 import mechgen, tables
from flint_gb300.mech import Mechanism
from oracle.oracle import TableOracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def cuda(*arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def _states(mech, n, seed):
    T, p, Y = mechgen.c2_states(n, mech, seed=seed)
    T = np.clip(T, 300.0, 2990.0)
    W = np.array([s.mw for s in mech.species])
    rho = p / (mech.r_eos * T * (Y / W).sum(1))
    return T, rho[:, None] * Y


def test_general_elementary_bit_exact():
    m = copy.deepcopy(mechgen.load("c2"))
    m.reactions = [r for r in m.reactions if r.rtype == 0]
    t = tables.generate(m, 1, 3000)
    T, roi = _states(m, 4099, 21)
    ref = TableOracle(t).general(roi, T)
    gpu = tables.Tables(t)
    roi_t, T_t = cuda(roi, T)
    w = gpu.chemistry_source(roi_t, T_t)
    torch.cuda.synchronize()
    assert np.array_equal(w.cpu().numpy(), ref)


def test_general_with_falloff():
    m = Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json"))
    t = tables.generate(m, 1, 3000)
    T, roi = _states(m, 3001, 22)
    ref = TableOracle(t).general(roi, T)
    gpu = tables.Tables(t)
    roi_t, T_t = cuda(roi, T)
    w = gpu.chemistry_source(roi_t, T_t).cpu().numpy()
    scale = np.abs(ref).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(w - ref) / scale) < 1e-12


def test_rhs_native():
    m = Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json"))
    t = tables.generate(m, 200, 3000)
    T, roi = _states(m, 2049, 23)
    T[::97] = 150.0          # below the table: F = -1
    T[1::101] = np.nan       # NaN: F = -1
    roi[::13, 3] = -1e-4     # negative partial density: clamped to 0
    Z = np.hstack([roi, T[:, None]])
    ref = TableOracle(t).rhs_native(Z)
    gpu = tables.Tables(t)
    (Zt,) = cuda(Z)
    F = gpu.rhs_native(Zt).cpu().numpy()
    bad = (T < 200.0) | np.isnan(T)
    assert np.all(F[bad] == -1.0) and np.all(ref[bad] == -1.0)
    scale = np.abs(ref[~bad, :-1]).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(F[~bad, :-1] - ref[~bad, :-1]) / scale) < 1e-12
    np.testing.assert_allclose(F[~bad, -1], ref[~bad, -1], rtol=1e-11)


def test_handle_from_files_matches_handle_from_arrays(tmp_path):
    """flint_mech_create_from_files parses the files itself; its handle gives the
    same general-loop and rhs_native output as one built from the Python reader's
    arrays of the same files, bit for bit."""
    m = Mechanism.load(os.path.join(GOLD, "mech_pelucchi.json"))
    tables.write_folder(tables.generate(m, 1, 3000), str(tmp_path))
    a = tables.Tables.from_files(str(tmp_path))
    b = tables.Tables(tables.read_folder(str(tmp_path)))
    assert a.ns == b.ns == m.ns
    T, roi = _states(m, 2053, 24)
    roi_t, T_t = cuda(roi, T)
    assert torch.equal(a.chemistry_source(roi_t.clone(), T_t), b.chemistry_source(roi_t.clone(), T_t))
    Z = torch.cat([roi_t, T_t[:, None]], dim=1).contiguous()
    assert torch.equal(a.rhs_native(Z), b.rhs_native(Z))


def test_general_and_rhs_native_on_the_reference_troyes_tables():
    """FLINT's general loop and rhs_native on the Troyes tables the reference
    ships only as SZL binaries (chemistry-Arrhenius.szplt, thermo.szplt, read by
    the library's reader when the fixture was made; rows 280-3000 K): 17
    elementary and three-body reactions, so bit for bit with the oracle."""
    from test_szl import troyes_tables
    t = troyes_tables()
    rng = np.random.default_rng(31)
    n = 5003
    T = rng.uniform(300.0, 2990.0, n)
    Y = rng.dirichlet(np.full(t["ns"], 0.4), n)
    rho = rng.uniform(0.05, 20.0, n)
    roi = rho[:, None] * Y
    orc = TableOracle(t)
    ref = orc.general(roi, T)
    gpu = tables.Tables(t)
    roi_t, T_t = cuda(roi, T)
    w = gpu.chemistry_source(roi_t, T_t)
    torch.cuda.synchronize()
    assert np.array_equal(w.cpu().numpy(), ref)
    # rhs_native at the bars of test_rhs_native: 1e-12 of the cell's largest
    # species term, 1e-11 relative on dT/dt
    Z = np.hstack([roi, T[:, None]])
    F_ref = orc.rhs_native(Z)
    F = gpu.rhs_native(cuda(Z)[0]).cpu().numpy()
    scale = np.abs(F_ref[:, :-1]).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(F[:, :-1] - F_ref[:, :-1]) / scale) < 1e-12
    np.testing.assert_allclose(F[:, -1], F_ref[:, -1], rtol=1e-11)
