"""The shipped surrogate on cells it has never seen: accuracy and gain.

The benchmark's network (flint_gb300/data/surrogate_c3.bin, the 31-species
mechanism) advances 65,536 reactor cells drawn with a seed used neither in
training (5000 + seed), nor in calibration (6000 + seed), nor by the benchmark
(1004).  Every cell is judged by the plain FP64 integrator, a 4,096-cell sample
also by the FP64 CPU oracle, against the targets max |dT| <= 1 K and
max |dY| <= 1e-4; and the gated surrogate + fallback must be at least 5x
faster than the plain integrator on the same cells (CUDA events, both warmed
up), which is what the network gains over the method without it.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CKPT = os.path.join(REPO, "flint_gb300", "data", "surrogate_c3.bin")
N = 65536
N_ORACLE = 4096
SEED = 9001
TARGET_DT, TARGET_DY = 1.0, 1e-4


def _timed(fn):
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    out = fn()
    e1.record(s)
    e1.synchronize()
    return out, e0.elapsed_time(e1) / 1e3


def test_shipped_surrogate_on_fresh_cells():
    from flint_gb300 import mechgen
    from flint_gb300.api import Chemistry
    from flint_gb300.native import reactor_opts
    from flint_gb300.surrogate import Surrogate
    from oracle.oracle import Oracle

    chem = Chemistry.from_config("c2")
    sur = Surrogate.load(chem, CKPT, weights_only=True)
    T0, p, Y0, dt = mechgen.c3_states(N, chem.mech, seed=SEED)
    dev = torch.device("cuda")
    T0d, Y0d = torch.from_numpy(T0).to(dev), torch.from_numpy(Y0).to(dev)
    pd, dtd = torch.from_numpy(p).to(dev), torch.from_numpy(dt).to(dev)

    # warm both paths up on a slice (module load, buffers sized, BDF table)
    m = 2048
    Tw, Yw = T0d[:m].clone(), Y0d[:m].clone()
    chem.reactor_advance(Tw, pd[:m], Yw, dtd[:m])
    Tw, Yw = T0d.clone(), Y0d.clone()
    sur.advance(Tw, pd, Yw, dtd)
    torch.cuda.synchronize()

    Tp, Yp = T0d.clone(), Y0d.clone()
    (stp, _), t_plain = _timed(lambda: chem.reactor_advance(Tp, pd, Yp, dtd))
    stp = stp.cpu().numpy()
    ok = stp == 0                               # cells the integrator itself finished
    assert ok.mean() > 0.999, np.unique(stp, return_counts=True)
    Ts, Ys = T0d.clone(), Y0d.clone()
    (sts, _, (acc, rej)), t_sur = _timed(lambda: sur.advance(Ts, pd, Ys, dtd))
    assert acc + rej == N
    sts = sts.cpu().numpy()
    # accepted (0), or re-solved by the integrator (6, or the integrator's own failure code)
    assert ((sts == 0) | (sts == 6) | (sts == stp)).all()

    # every cell against the FP64 GPU integrator
    eT = (Ts - Tp).abs().cpu().numpy()[ok]
    eY = (Ys - Yp).abs().amax(dim=1).cpu().numpy()[ok]
    assert eT.max() <= TARGET_DT, eT.max()
    assert eY.max() <= TARGET_DY, eY.max()
    # the re-solved cells are the integrator's own result
    rejected = (sts == 6)[ok]
    assert eT[rejected].max(initial=0.0) == 0.0 and eY[rejected].max(initial=0.0) == 0.0

    # a sample against the FP64 CPU oracle
    To, Yo, so, _ = Oracle(chem.mech).reactor_advance(T0[:N_ORACLE], p[:N_ORACLE], Y0[:N_ORACLE],
                                                       dt[:N_ORACLE], reactor_opts())
    good = so == 0
    assert good.mean() > 0.999
    eTo = np.abs(Ts[:N_ORACLE].cpu().numpy() - To)[good].max()
    eYo = np.abs(Ys[:N_ORACLE].cpu().numpy() - Yo)[good].max()
    assert eTo <= TARGET_DT, eTo
    assert eYo <= TARGET_DY, eYo

    speedup = t_plain / t_sur
    print(f"\nsurrogate on {N} fresh cells: {acc} accepted, {rej} re-solved; max |dT| {eT.max():.3g} K, "
          f"max |dY| {eY.max():.3g} (integrator), {eTo:.3g} K / {eYo:.3g} (oracle, {N_ORACLE} cells); "
          f"plain {t_plain * 1e3:.1f} ms, surrogate {t_sur * 1e3:.1f} ms: {speedup:.1f}x")
    assert speedup >= 5.0, speedup
