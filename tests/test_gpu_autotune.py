"""The per-mechanism tuning: every choice computes the same numbers, and the
persistent cache applies a stored choice without timing.

* the source-term kernels at 64, 128 and 256 threads per block give wdot and
  the Jacobian bit for bit alike (the block size only regroups warps);
* the reactor gives the same end states, statuses and step counts under every
  layout it can run (shared or global Newton matrices, 8 or 4 warps per block,
  one or two blocks per SM);
* flint_gb300.autotune.tune times, stores a JSON entry keyed by mechanism and
  GPU, and a second call (a fresh handle) applies it from the file;
* a tuning that does not fit is refused and changes nothing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _cuda(*a):
    return [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in a]


@pytest.mark.parametrize("cfg", ["c2", "c5"])
def test_block_sizes_compute_the_same_bits(cfg):
    from flint_gb300 import mechgen
    from flint_gb300.api import Chemistry
    chem = Chemistry.from_config(cfg)
    T, p, Y = _cuda(*mechgen.c2_states(1500, chem.mech, seed=41))
    ref_w, _, _ = chem.wdot(T, p, Y)
    _, ref_J = chem.wdot_jac(T, p, Y, wdot=torch.empty_like(Y))
    ref_w, ref_J = ref_w.clone(), ref_J.clone()
    for bt in (64, 128, 256):
        chem.set_tuning(0, bt, bt)
        assert chem.tuning()["wdot_threads"] == bt
        w, _, _ = chem.wdot(T, p, Y)
        _, J = chem.wdot_jac(T, p, Y, wdot=torch.empty_like(Y))
        torch.cuda.synchronize()
        assert torch.equal(w, ref_w) and torch.equal(J, ref_J), bt


def test_reactor_layouts_compute_the_same_bits():
    from flint_gb300 import mechgen
    from flint_gb300.api import Chemistry
    chem = Chemistry.from_config("c2")
    T0, p, Y0, dt = mechgen.c3_states(300, chem.mech, seed=43)
    pd, dtd = _cuda(p, dt)
    Ta, Ya = _cuda(T0, Y0)
    chem.reactor_autotune(Ta, pd, Ya, dtd)
    layouts = chem.reactor_autotune_times()
    assert set(layouts) >= {1, 2, 3, 4}, layouts   # shared; global 8 / 4 warps; two blocks per SM
    out = {}
    for lay in sorted(layouts):
        chem.set_tuning(lay, 0, 0)
        T, Y = _cuda(T0, Y0)
        st, ns = chem.reactor_advance(T, pd, Y, dtd)
        torch.cuda.synchronize()
        out[lay] = (T.cpu().numpy(), Y.cpu().numpy(), st.cpu().numpy(), ns.cpu().numpy())
    first = out[min(out)]
    for lay, o in out.items():
        for a, b in zip(o, first):
            assert np.array_equal(a, b), lay


def test_tune_caches_and_reapplies(tmp_path):
    from flint_gb300 import autotune, mechgen
    from flint_gb300.api import Chemistry
    from oracle.oracle import Oracle
    cache = str(tmp_path / "tuning.json")
    chem = Chemistry.from_config("c2")
    T, p, Y = _cuda(*mechgen.c2_states(4096, chem.mech, seed=45))
    T3, p3, Y3, dt3 = _cuda(*mechgen.c3_states(512, chem.mech, seed=46))
    e = autotune.tune(chem, T3, p3, Y3, dt3, path=cache)
    assert not e["cached"] and e["reactor_layout"] in (1, 2, 3, 4)
    assert e["wdot_threads"] in (64, 128, 256) and e["jac_threads"] in (64, 128, 256)
    assert e["wdot_kernel"] in ("data-driven", "generated") and e["jac_kernel"] in ("data-driven", "generated")
    # the chosen wdot kernel meets the source-term bar against the oracle
    w, _, _ = chem.wdot(T, p, Y)
    torch.cuda.synchronize()
    w_o, ws_o, _, _ = Oracle(chem.mech).wdot_batch(T.cpu().numpy(), p.cpu().numpy(), Y.cpu().numpy())
    assert np.max(np.abs(w.cpu().numpy().ravel() - w_o) / (ws_o + 1e-300)) < 1e-12
    # a fresh handle takes the stored entry without timing
    chem2 = Chemistry.from_config("c2")
    e2 = autotune.tune(chem2, T3, p3, Y3, dt3, path=cache)
    assert e2["cached"]
    t2 = chem2.tuning()
    assert (t2["reactor_layout"], t2["wdot_threads"], t2["jac_threads"]) == \
        (e["reactor_layout"], e["wdot_threads"], e["jac_threads"])


def test_bad_tuning_is_refused():
    from flint_gb300.api import Chemistry
    chem = Chemistry.from_config("c5")            # 54 species: no shared-memory reactor layout
    before = chem.tuning()
    with pytest.raises(RuntimeError):
        chem.set_tuning(1, 0, 0)
    with pytest.raises(RuntimeError):
        chem.set_tuning(0, 96, 0)
    assert chem.tuning() == before
