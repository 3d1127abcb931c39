"""The CUDA backend of the mechanism generator: emitted sources compile for
sm_103a here (no GPU needed); on the GPU the generated kernels -- wdot, cp, h
and wdot + the constant-pressure Jacobian -- match the oracle with the
tolerances of the data-driven kernels."""
import os

import numpy as np
import pytest

from flint_gb300 import mechgen, ytf_cuda
from flint_gb300.mech import Mechanism

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _mechs():
    return {"c1": mechgen.load("c1"), "pelucchi": Mechanism.load(os.path.join(GOLDEN, "mech_pelucchi.json"))}


@pytest.mark.parametrize("name", ["c1", "pelucchi"])
def test_emitted_source_compiles(name, tmp_path):
    m = _mechs()[name]
    ident, so = ytf_cuda.build(m, outdir=str(tmp_path))
    assert os.path.getsize(so) > 0
    src = open(os.path.join(str(tmp_path), f"ytf_{ident}.cu")).read()
    assert f"ytf_{ident}_wdot" in src and f"ytf_{ident}_wdot_jac" in src
    assert src.count("{  //") == 2 * m.nr   # one block per reaction in each kernel


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "pelucchi"])
def test_generated_kernel_vs_oracle(name):
    torch = pytest.importorskip("torch")
    from oracle.oracle import Oracle
    m = _mechs()[name]
    g = ytf_cuda.GeneratedMechanism(m)
    if name == "c1":
        T, p, Y = mechgen.c1_states(20000)
    else:
        T, p, Y = mechgen.c2_states(20000, m, seed=21)
    w_o, ws_o, cp_o, h_o = Oracle(m).wdot_batch(T, p, Y)
    Tt, pt, Yt = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (T, p, Y))
    w, cp, h = g.wdot(Tt, pt, Yt)
    torch.cuda.synchronize()
    err = np.max(np.abs(w.cpu().numpy().ravel() - w_o) / (ws_o + 1e-300))
    assert err < 1e-12, err
    np.testing.assert_allclose(cp.cpu().numpy(), cp_o, rtol=1e-13)
    hs = np.abs(h_o) + cp_o * T
    assert np.max(np.abs(h.cpu().numpy() - h_o) / hs) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "troyes", "pelucchi", "c2"])
def test_generated_jacobian_vs_oracle(name):
    """wdot + d(dY/dt, dT/dt)/d(Y, T) of the generated thread-per-cell kernel
    against the oracle at the 1e-12 bar of the data-driven Jacobian kernel."""
    torch = pytest.importorskip("torch")
    from oracle.oracle import Oracle
    if name in ("c1", "c2"):
        m = mechgen.load(name)
    else:
        m = Mechanism.load(os.path.join(GOLDEN, f"mech_{name}.json"))
    g = ytf_cuda.GeneratedMechanism(m)
    T, p, Y = (mechgen.c1_states(3000) if name == "c1" else mechgen.c2_states(3000, m, seed=23))
    T = np.clip(T, 300.0, 2800.0)
    w_o, ws_o, _, _ = Oracle(m).wdot_batch(T, p, Y)
    _, J_o, Js_o = Oracle(m).wdot_jac_batch(T, p, Y)
    Tt, pt, Yt = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (T, p, Y))
    w = torch.empty_like(Yt)
    _, J = g.wdot_jac(Tt, pt, Yt, wdot=w)
    torch.cuda.synchronize()
    assert np.max(np.abs(w.cpu().numpy().ravel() - w_o) / (ws_o + 1e-300)) < 1e-12
    err = np.abs(J.cpu().numpy().ravel() - J_o) / (Js_o + 1e-300)
    assert err.max() < 1e-12, err.max()
