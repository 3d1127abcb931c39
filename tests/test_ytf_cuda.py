"""The CUDA backend of the mechanism generator: emitted sources compile for
sm_103a here (no GPU needed); on the GPU the generated kernels match the oracle
with the tolerances of the data-driven kernels."""
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
    assert f"ytf_{ident}_wdot" in src and src.count("{  //") == m.nr   # one block per reaction


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
