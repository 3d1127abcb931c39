"""The fused Blackwell inference forward of the surrogate MLP (flint_umma.cu).

tcgen05.mma with the accumulator in tensor memory, all five layers of a
128-cell tile on one SM, split-BF16 operands.  Checked against:

* the NumPy restatement of the split-BF16 / FP32 arithmetic
  (test_gpu_surrogate.np_forward_backward) to 1e-4 of the output scale, the
  bar of the per-layer path, and far closer than single-BF16 operands;
* the per-layer mma.sync path on the same network and inputs (the two
  accumulate in different orders: 1e-5 of the output scale);
* the shipped checkpoint: both paths give the same gated advance on 16,384
  cells (accepted set and results within the surrogate's own tolerance).

Cell counts that are not multiples of the 128-cell tile check the tail tile,
and the 54-species network (56 inputs, 55 outputs) the padded widths.  Every
call's bounded waits must have completed (the error word stays 0).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _net(cfg, seed):
    from flint_gb300.api import Chemistry
    from flint_gb300.surrogate import Surrogate
    chem = Chemistry.from_config(cfg)
    ns = chem.ns
    stats = {"x_mean": np.zeros(ns + 2, np.float32), "x_std": np.ones(ns + 2, np.float32),
             "y_mean": np.zeros(ns + 1, np.float32), "y_std": np.ones(ns + 1, np.float32),
             "bath": chem.mech.index("N2"), "domain": {}}
    return chem, Surrogate(chem, stats, n_nets=1, hidden=256, n_layers=5, seed=seed)


@pytest.mark.parametrize("cfg,n", [("c2", 1000), ("c2", 128), ("c5", 777)])
def test_fused_forward_matches_numpy_and_per_layer_path(cfg, n):
    from test_gpu_surrogate import bf16, np_forward_backward
    chem, sur = _net(cfg, seed=11)
    rng = np.random.default_rng(17)
    X = rng.normal(size=(n, sur.n_in)).astype(np.float32)
    w0, _ = sur.get_state()
    w0 = w0[:sur.P]
    y_np, _ = np_forward_backward(w0, sur.dims, X, np.zeros((n, sur.n_out), np.float32))
    Xd = torch.from_numpy(X).cuda()
    assert sur.set_forward(0) == 0            # the fused kernel serves this network
    y_fused = sur.predict(Xd).cpu().numpy()
    assert sur.check() == 0
    assert sur.set_forward(1) == 1
    y_layer = sur.predict(Xd).cpu().numpy()
    scale = np.abs(y_np).max()
    err = np.abs(y_fused - y_np).max() / scale
    assert err < 1e-4, err
    y_b, _ = np_forward_backward(w0, sur.dims, X, np.zeros((n, sur.n_out), np.float32), rnd=bf16)
    assert err < 0.1 * np.abs(y_b - y_np).max() / scale
    assert np.abs(y_fused - y_layer).max() / scale < 1e-5


def test_fused_forward_follows_training():
    """After a training step the packed weights are refreshed: the fused and
    per-layer forwards agree on the updated network."""
    chem, sur = _net("c2", seed=12)
    rng = np.random.default_rng(19)
    X = torch.from_numpy(rng.normal(size=(4096, sur.n_in)).astype(np.float32)).cuda()
    T = torch.from_numpy(rng.normal(size=(4096, sur.n_out)).astype(np.float32)).cuda()
    sur.set_forward(0)
    y0 = sur.predict(X).clone()
    sur.train_step(X, T, 1e-3)
    y1 = sur.predict(X)
    sur.set_forward(1)
    y2 = sur.predict(X)
    torch.cuda.synchronize()
    scale = float(y2.abs().max())
    assert float((y1 - y0).abs().max()) > 1e-3 * scale      # the weights did change
    assert float((y1 - y2).abs().max()) < 1e-5 * scale
    assert sur.check() == 0


def test_shipped_checkpoint_same_advance():
    from flint_gb300 import mechgen
    from flint_gb300.api import Chemistry
    from flint_gb300.surrogate import Surrogate
    chem = Chemistry.from_config("c2")
    sur = Surrogate.load(chem, os.path.join(REPO, "flint_gb300", "data", "surrogate_c3.bin"), weights_only=True)
    T0, p, Y0, dt = mechgen.c3_states(16384, chem.mech, seed=9002)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()   # noqa: E731
    out = {}
    for mode in (0, 1):
        sur.set_forward(mode)
        T, Y = d(T0), d(Y0)
        st, _, (acc, rej) = sur.advance(T, d(p), Y, d(dt))
        out[mode] = (T.cpu().numpy(), Y.cpu().numpy(), st.cpu().numpy(), acc)
    assert sur.check() == 0
    (Ta, Ya, sa, na), (Tb, Yb, sb, nb) = out[0], out[1]
    same = sa == sb
    assert same.mean() > 0.999, same.mean()      # a cell at the gate's edge may flip
    assert abs(na - nb) <= 16
    both = same & (sa == 0)
    # the two forwards differ by ~1e-5 of the outputs' normalisation spread
    # (about 100 K for dT): far inside 1 % of the surrogate's targets
    assert np.abs(Ta - Tb)[both].max() < 1e-2 and np.abs(Ya - Yb)[both].max() < 1e-6
