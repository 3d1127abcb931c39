"""The allocation-free reactor entry point (flint_reactor_advance_noalloc).

Callers such as CFD solvers that give their whole device memory to their own
pool at start-up cannot let the library call cudaMalloc; this entry point runs
the same reactor kernel on a static device scratch array instead.  The test
calls it through the C-ABI twice in a row (the second call reuses the scratch
the first one left behind) and checks both results against
flint_reactor_advance with the reactor tests' tolerance.  It lives in its own
file, collected last, and needs no state from other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_noalloc_reactor_matches_allocating_entry_point_twice():
    from flint_gb300 import mechgen, native
    from flint_gb300.api import Chemistry

    chem = Chemistry.from_config("c2")
    L = native.lib()
    T0, p, Y0, dt = mechgen.c3_states(600, chem.mech, seed=314)
    opts = native.reactor_opts()

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    # allocating entry point (reference for this test)
    Tr, Yr, pr, dtr = dev(T0), dev(Y0), dev(p), dev(dt)
    st_r, ns_r = chem.reactor_advance(Tr, pr, Yr, dtr)
    torch.cuda.synchronize()
    Tr, Yr, st_r = Tr.cpu().numpy(), Yr.cpu().numpy(), st_r.cpu().numpy()
    assert (st_r == 0).all()

    for call in range(2):
        Tn, Yn, pn, dtn = dev(T0), dev(Y0), dev(p), dev(dt)
        st = torch.full((T0.size,), -7, dtype=torch.int32, device="cuda")
        nst = torch.zeros(T0.size, dtype=torch.int32, device="cuda")
        vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        rc = L.flint_reactor_advance_noalloc(chem.h, T0.size, vp(Tn), vp(pn), vp(Yn), vp(dtn), C.byref(opts),
                                             vp(st), vp(nst), None)
        assert rc == 0, L.flint_last_error()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(st.cpu().numpy(), st_r)
        # same kernel, same per-cell arithmetic: agreement far inside the
        # reactor tests' 1e-6 bound
        np.testing.assert_allclose(Tn.cpu().numpy(), Tr, rtol=1e-12, atol=0)
        np.testing.assert_allclose(Yn.cpu().numpy(), Yr, rtol=1e-12, atol=1e-300)
        assert (nst.cpu().numpy() == ns_r.cpu().numpy()).all()
