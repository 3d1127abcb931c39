"""The GPU kernels against the reference's generated Fortran mechanism routines.

For each of the ten routines in src/lib/Lib_ChemMech/ that utils/YTF.py wrote
(tests/golden/fortran_forms.json), the data-driven warp kernel and the
generated per-mechanism kernel run the mechanism in the routine's form
(Mechanism.ytf_form()), and their wdot must equal the routine's arithmetic
(tests/fortran_forms.py, with the oracle's rate constants) to 1e-12 of the sum
of the absolute terms.  The Troyes routine is also run on the reference's own
Troyes tables against the library's tabulated general loop.
"""
import os

import numpy as np
import pytest

import fortran_forms as FF

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
FORMS = FF.load_forms()


@pytest.mark.parametrize("name", sorted(FORMS))
def test_kernels_compute_the_routine(name):
    from flint_gb300 import mechgen
    from flint_gb300.api import Chemistry
    from flint_gb300.mech import Mechanism
    from oracle.oracle import Oracle
    form = FORMS[name]
    m = Mechanism.load(os.path.join(FF.GOLD, form["mechanism"])).ytf_form()
    T, p, Y = mechgen.c2_states(777, m, seed=73)
    T = np.clip(T, 800.0, 2800.0)
    W = np.array([s.mw for s in m.species])
    rho = p / (m.r_eos * T * (Y / W).sum(1))
    w_ref, sc = FF.omegadot(form, W, rho[:, None] * Y, FF.analytic_rates(Oracle(m), m, T))
    chem = Chemistry(m)
    Tt, pt, Yt = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (T, p, Y))
    for generated in (False, True):
        chem.use_generated(generated)
        w, _, _ = chem.wdot(Tt, pt, Yt)
        torch.cuda.synchronize()
        err = np.abs(w.cpu().numpy() - w_ref) / (sc + 1e-300)
        assert err.max() < 1e-12, (name, generated, err.max())


def test_troyes_routine_on_its_tables_gpu():
    from flint_gb300 import tables
    from test_szl import troyes_tables
    t = troyes_tables()
    form = FORMS["troyes"]
    rng = np.random.default_rng(6)
    n = 4099
    T = rng.uniform(300.0, 2990.0, n)
    Y = rng.dirichlet(np.full(t["ns"], 0.4), n)
    roi = rng.uniform(0.05, 20.0, n)[:, None] * Y
    Ti = T.astype(np.int64)
    Td = T - Ti

    def lerp(tab, j):
        a, b = tab[j, Ti - t["ti1"]], tab[j, Ti + 1 - t["ti1"]]
        return a + (b - a) * Td

    rates = [{"kf": lerp(t["kf_tab"], fr["table_index"] - 1), "kb": lerp(t["kb_tab"], fr["table_index"] - 1)}
             for fr in form["reactions"]]
    w_ref, sc = FF.omegadot(form, t["wm"], roi, rates)
    gpu = tables.Tables(t)
    w = gpu.chemistry_source(torch.from_numpy(roi).cuda(), torch.from_numpy(T).cuda())
    torch.cuda.synchronize()
    assert np.max(np.abs(w.cpu().numpy() - w_ref) / (sc + 1e-300)) < 1e-13
