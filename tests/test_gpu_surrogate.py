"""The learned surrogate: MLP forward and gradients against a NumPy oracle of
the same split-BF16 / BF16 / FP32 arithmetic, training, checkpoint resume, and the gated
surrogate + fallback advance (conservation, status codes, fallback = integrator)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def bf16(x):
    """Round float32 to bfloat16 (nearest, ties to even), returned as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(0.7978845608028654 * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    u = 0.7978845608028654 * (x + 0.044715 * x ** 3)
    t = np.tanh(u)
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * 0.7978845608028654 * (1 + 3 * 0.044715 * x * x)


def np_forward_backward(w, dims, X, T, rnd=None):
    """NumPy oracle of the device arithmetic, FP64 accumulation, FP32 storage.

    Forward: FP32 operands (the device splits each into a BF16 hi + lo pair,
    about 16 significant bits); ``rnd=bf16`` gives plain single-BF16 operands
    instead, for comparison.  Backward: BF16 operands (weights, activations
    and back-propagated errors rounded once)."""
    rnd = rnd or (lambda x: np.asarray(x, np.float32))
    Ws, bs, o = [], [], 0
    for i in range(len(dims) - 1):
        Ws.append(w[o:o + dims[i + 1] * dims[i]].reshape(dims[i + 1], dims[i])); o += dims[i + 1] * dims[i]
        bs.append(w[o:o + dims[i + 1]]); o += dims[i + 1]
    a, ins, zs = X.astype(np.float32), [], []
    for l in range(len(Ws)):
        ins.append(bf16(a))
        z = (rnd(a).astype(np.float64) @ rnd(Ws[l]).T.astype(np.float64) + bs[l]).astype(np.float32)
        zs.append(z)
        a = gelu(z).astype(np.float32) if l < len(Ws) - 1 else z
    y = a
    g = (2.0 * (y - T) / y.size).astype(np.float32)
    grads = [None] * len(Ws)
    for l in range(len(Ws) - 1, -1, -1):
        gw = bf16(g).T.astype(np.float64) @ ins[l].astype(np.float64)
        gb = g.sum(0)
        grads[l] = (gw, gb)
        if l > 0:
            dA = bf16(g).astype(np.float64) @ bf16(Ws[l]).astype(np.float64)
            g = (dA * gelu_grad(zs[l - 1])).astype(np.float32)
    return y, grads


def small_surrogate(seed=0, n_nets=1, hidden=64, n_layers=3, dy_scale=1.0):
    from flint_gb300.api import Chemistry
    from flint_gb300.surrogate import Surrogate
    chem = Chemistry.from_config("c2")
    ns = chem.ns
    ys = np.full(ns + 1, dy_scale, np.float32)
    ys[-1] = 1.0
    stats = {"x_mean": np.zeros(ns + 2, np.float32), "x_std": np.ones(ns + 2, np.float32),
             "y_mean": np.zeros(ns + 1, np.float32), "y_std": ys,
             "bath": chem.mech.index("N2"), "domain": {}}
    return chem, Surrogate(chem, stats, n_nets=n_nets, hidden=hidden, n_layers=n_layers, seed=seed)


def test_mlp_forward_and_gradient_vs_numpy():
    chem, sur = small_surrogate(hidden=64, n_layers=3)
    rng = np.random.default_rng(3)
    n = 300
    X = rng.normal(size=(n, sur.n_in)).astype(np.float32)
    Tt = rng.normal(size=(n, sur.n_out)).astype(np.float32)
    w0, _ = sur.get_state()
    w0 = w0[:sur.P]
    y_np, grads = np_forward_backward(w0, sur.dims, X, Tt)
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(Tt).cuda()
    y = sur.predict(Xd).cpu().numpy()
    err = np.abs(y - y_np).max() / np.abs(y_np).max()
    assert err < 1e-4, err
    # the split operands beat single-BF16 operands by more than an order of magnitude
    y_b, _ = np_forward_backward(w0, sur.dims, X, Tt, rnd=bf16)
    assert err < 0.1 * np.abs(y_b - y_np).max() / np.abs(y_np).max()
    loss = sur.train_step(Xd, Td, 1e-7, want_loss=True)
    assert abs(loss - float(((y_np - Tt) ** 2).mean())) < 1e-3 * loss
    st, step = sur.get_state()
    assert step == 1
    m1 = st[sur.P:2 * sur.P] / 0.1          # first Adam moment after one step = 0.1 * gradient
    o = 0
    for l, (gw, gb) in enumerate(grads):
        nw = gw.size
        gpu_w = m1[o:o + nw].reshape(gw.shape); o += nw
        gpu_b = m1[o:o + gb.size]; o += gb.size
        assert np.linalg.norm(gpu_w - gw) / np.linalg.norm(gw) < 1e-2, l
        assert np.linalg.norm(gpu_b - gb) / np.linalg.norm(gb) < 1e-3, l


def test_training_reduces_loss():
    chem, sur = small_surrogate(seed=1, hidden=64, n_layers=3)
    rng = np.random.default_rng(5)
    X = rng.normal(size=(8192, sur.n_in)).astype(np.float32)
    A = rng.normal(size=(sur.n_in, sur.n_out)).astype(np.float32) / np.sqrt(sur.n_in)
    Tt = np.tanh(X @ A).astype(np.float32)
    from flint_gb300.surrogate import train
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(Tt).cuda()
    l0 = float(((sur.predict(Xd) - Td) ** 2).mean())
    train(sur, Xd, Td, 600, batch=512, lr=3e-3, log_every=10000)
    l1 = float(((sur.predict(Xd) - Td) ** 2).mean())
    assert l1 < 0.1 * l0, (l0, l1)


def test_checkpoint_resume_equals_continuous(tmp_path):
    from flint_gb300.surrogate import Surrogate, train
    rng = np.random.default_rng(9)
    chem, a = small_surrogate(seed=4, hidden=32, n_layers=3)
    X = torch.from_numpy(rng.normal(size=(2048, a.n_in)).astype(np.float32)).cuda()
    Tt = torch.from_numpy(rng.normal(size=(2048, a.n_out)).astype(np.float32)).cuda()
    train(a, X, Tt, 40, batch=256, lr=1e-3, total=40, seed=2, log_every=10000)
    _, b = small_surrogate(seed=4, hidden=32, n_layers=3)
    train(b, X, Tt, 20, batch=256, lr=1e-3, total=40, seed=2, log_every=10000)
    path = str(tmp_path / "ck.bin")
    b.save(path)
    c = Surrogate.load(b.chem, path)
    train(c, X, Tt, 20, batch=256, lr=1e-3, total=40, seed=2, start=c.sampler_pos, log_every=10000)
    sa, ka = a.get_state()
    sc, kc = c.get_state()
    assert ka == kc == 40
    np.testing.assert_array_equal(sa, sc)


def _cells(chem, n, seed):
    from flint_gb300 import mechgen
    T, p, Y, dt = mechgen.c3_states(n, chem.mech, seed=seed)
    return [torch.from_numpy(a).cuda() for a in (T, p, Y, dt)]


def test_rejected_cells_equal_integrator():
    """A gate nothing passes sends every cell to the FP64 integrator."""
    chem, sur = small_surrogate(seed=2)
    T, p, Y, dt = _cells(chem, 200, 41)
    T2, Y2 = T.clone(), Y.clone()
    st_i, ns_i = chem.reactor_advance(T2, p, Y2, dt)
    st, ns, (acc, rej) = sur.advance(T, p, Y, dt, gate={"max_dT_resid": -1.0})
    torch.cuda.synchronize()
    assert acc == 0 and rej == 200
    assert (st.cpu().numpy() == 6).all()          # FLINT_CELL_SURROGATE_REJECTED, re-solved
    assert np.array_equal(ns.cpu().numpy(), ns_i.cpu().numpy())
    np.testing.assert_array_equal(T.cpu().numpy(), T2.cpu().numpy())
    np.testing.assert_array_equal(Y.cpu().numpy(), Y2.cpu().numpy())


def test_accepted_cells_conserve_elements_and_enthalpy():
    """With an open gate every in-domain cell takes the network step, made exactly
    conservative: elements by projection, enthalpy by the Newton temperature."""
    from oracle.oracle import Oracle
    chem, sur = small_surrogate(seed=3, dy_scale=1e-4)
    T, p, Y, dt = _cells(chem, 256, 43)
    T0, Y0 = T.cpu().numpy(), Y.cpu().numpy()
    open_gate = {"max_dT_resid": 1e30, "max_elem_resid": 1e30, "min_Y": -1e30, "T_lo": 0.0, "T_hi": 1e9,
                 "log10p_lo": -1e9, "log10p_hi": 1e9, "log10dt_lo": -1e9, "log10dt_hi": 1e9}
    sur.gate.update(open_gate)
    st, ns, (acc, rej) = sur.advance(T, p, Y, dt)
    torch.cuda.synchronize()
    stn, nsn = st.cpu().numpy(), ns.cpu().numpy()
    ok = (stn == 0) & (nsn == 0)
    assert ok.sum() == acc and acc > 0
    assert (Y.cpu().numpy()[ok] >= 0.0).all()
    T1, Y1 = T.cpu().numpy(), Y.cpu().numpy()
    E = chem.mech.element_matrix()
    W = np.array([s.mw for s in chem.mech.species])
    el0 = (Y0 / W) @ E.T
    el1 = (Y1 / W) @ E.T
    np.testing.assert_allclose(el1[ok], el0[ok], rtol=0, atol=1e-12 * np.abs(el0).max())
    assert np.abs(Y1[ok].sum(1) - Y0[ok].sum(1)).max() < 1e-12
    orc = Oracle(chem.mech)
    P = p.cpu().numpy()
    for i in np.flatnonzero(ok)[:40]:
        _, _, _, h0 = orc.wdot_batch(T0[i:i + 1], P[i:i + 1], Y0[i:i + 1])
        _, _, _, h1 = orc.wdot_batch(T1[i:i + 1], P[i:i + 1], Y1[i:i + 1])
        assert abs(h1[0] - h0[0]) <= 1e-8 * max(abs(h0[0]), 1e5)


def test_advance_captured_in_cuda_graph():
    """Without counts the advance never waits on the host: after a first (sizing)
    call it is captured in a CUDA graph, and a replay reproduces the synchronous
    call cell by cell (accepted and re-solved cells alike)."""
    chem, sur = small_surrogate(seed=5, dy_scale=1e-4)
    # open gate except the domain: cells above 1250 K go to the integrator
    sur.gate.update({"max_dT_resid": 1e30, "max_elem_resid": 1e30, "min_Y": -1e30, "T_lo": 0.0, "T_hi": 1250.0,
                     "log10p_lo": -1e9, "log10p_hi": 1e9, "log10dt_lo": -1e9, "log10dt_hi": 1e9})
    T, p, Y, dt = _cells(chem, 1000, 47)
    T0, Y0 = T.clone(), Y.clone()
    st_ref, ns_ref, (acc, rej) = sur.advance(T, p, Y, dt)
    torch.cuda.synchronize()
    assert acc > 0 and rej > 0
    Tg, Yg = T0.clone(), Y0.clone()
    st = torch.empty_like(st_ref); ns = torch.empty_like(ns_ref)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):                      # warm call on the capture stream
        sur.advance(Tg, p, Yg, dt, status=st, nsteps=ns, wait=False)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="relaxed"):
        sur.advance(Tg, p, Yg, dt, status=st, nsteps=ns, wait=False)
    Tg.copy_(T0); Yg.copy_(Y0)
    g.replay()
    torch.cuda.synchronize()
    assert sur.counts() == (acc, rej)
    np.testing.assert_array_equal(Tg.cpu().numpy(), T.cpu().numpy())
    np.testing.assert_array_equal(Yg.cpu().numpy(), Y.cpu().numpy())
    np.testing.assert_array_equal(st.cpu().numpy(), st_ref.cpu().numpy())
    np.testing.assert_array_equal(ns.cpu().numpy(), ns_ref.cpu().numpy())
