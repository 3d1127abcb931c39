"""The allocation-free reactor entry point (flint_reactor_advance_noalloc).

Callers such as CFD solvers that give their whole device memory to their own
pool at start-up cannot let the library call cudaMalloc; this entry point runs
the same reactor kernel on a static device scratch array instead.  The test
works on a handle that has never run flint_reactor_advance (so no handle-owned
scratch exists that a fallback could use): it makes the n = 0 warm-up call,
then two real calls in a row (the second one reuses the scratch the first one
left behind), checks that the device's free memory is unchanged across the
second call, and only then runs flint_reactor_advance on a separate handle and
compares both results with it at the reactor tests' tolerance.  It lives in
its own file, collected last, and needs no state from other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_noalloc_reactor_matches_allocating_entry_point_twice():
    from flint_gb300 import mechgen, native
    from flint_gb300.api import Chemistry

    L = native.lib()
    chem_n = Chemistry.from_config("c2")      # used only through the allocation-free entry
    T0, p, Y0, dt = mechgen.c3_states(600, chem_n.mech, seed=314)
    n = T0.size
    opts = native.reactor_opts()

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    # every device buffer of the two calls exists before the first of them
    T0d, Y0d, pn, dtn = dev(T0), dev(Y0), dev(p), dev(dt)
    Tn, Yn = torch.empty_like(T0d), torch.empty_like(Y0d)
    st = torch.empty(n, dtype=torch.int32, device="cuda")
    nst = torch.empty(n, dtype=torch.int32, device="cuda")
    vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    # warm-up: no cells, NULL arrays; loads the module and sets up the device
    rc = L.flint_reactor_advance_noalloc(chem_n.h, 0, None, None, None, None, C.byref(opts), None, None, None)
    assert rc == 0, L.flint_last_error()
    torch.cuda.synchronize()

    results = []
    free = []
    for call in range(2):
        Tn.copy_(T0d)
        Yn.copy_(Y0d)
        st.fill_(-7)
        nst.zero_()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        rc = L.flint_reactor_advance_noalloc(chem_n.h, n, vp(Tn), vp(pn), vp(Yn), vp(dtn), C.byref(opts),
                                             vp(st), vp(nst), None)
        assert rc == 0, L.flint_last_error()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        results.append((Tn.cpu().numpy(), Yn.cpu().numpy(), st.cpu().numpy(), nst.cpu().numpy()))
    # the second call allocates nothing on the device
    assert free[3] == free[2], f"free device memory changed by {free[2] - free[3]} bytes across the second call"

    # allocating entry point on a separate handle (the comparison)
    chem_a = Chemistry.from_config("c2")
    Tr, Yr = T0d.clone(), Y0d.clone()
    st_r, ns_r = chem_a.reactor_advance(Tr, pn, Yr, dtn)
    torch.cuda.synchronize()
    Tr, Yr, st_r, ns_r = Tr.cpu().numpy(), Yr.cpu().numpy(), st_r.cpu().numpy(), ns_r.cpu().numpy()
    assert (st_r == 0).all()

    for Tc, Yc, sc, nc in results:
        np.testing.assert_array_equal(sc, st_r)
        # same kernel, same per-cell arithmetic: agreement far inside the
        # reactor tests' 1e-6 bound
        np.testing.assert_allclose(Tc, Tr, rtol=1e-12, atol=0)
        np.testing.assert_allclose(Yc, Yr, rtol=1e-12, atol=1e-300)
        assert (nc == ns_r).all()
