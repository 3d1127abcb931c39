"""Species thermo on the GPU (flint_species_thermo_batch: cp, h, s, g per
species in mass units, the quantities of cpi / H0i / S0i,
Lib_ThermoTransport.f90:40-97, :233-248) against the oracle's polynomials, on a
NASA-7 mechanism (31 species) and a NASA-9 one (WD), over 300-3000 K."""
import os

import numpy as np
import pytest

from flint_gb300 import mechgen
from flint_gb300.api import Chemistry
from flint_gb300.mech import Mechanism
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", ["c2", "wd"])
def test_species_thermo_vs_oracle(name):
    mech = mechgen.load("c2") if name == "c2" else Mechanism.load(os.path.join(GOLD, f"mech_{name}.json"))
    rng = np.random.default_rng(12)
    T = np.concatenate([rng.uniform(300.0, 3000.0, 997), [300.0, 1000.0, 3000.0]])
    chem = Chemistry(mech)
    cp, h, s, g = (x.cpu().numpy() for x in chem.species_thermo(torch.from_numpy(T).cuda()))
    orc = Oracle(mech)
    W = np.array([sp.mw for sp in mech.species])
    R = mech.r_thermo
    cp_o = np.zeros_like(cp); h_o = np.zeros_like(h); s_o = np.zeros_like(s)
    for i, t in enumerate(T):
        cpR, hRT, sR, _ = orc.species_thermo(t)
        cp_o[i], h_o[i], s_o[i] = cpR * R / W, hRT * R * t / W, sR * R / W
    g_o = h_o - T[:, None] * s_o
    assert cp.shape == (len(T), mech.ns)
    assert np.max(np.abs(cp - cp_o) / cp_o) < 1e-13
    assert np.max(np.abs(h - h_o) / (np.abs(h_o) + cp_o * T[:, None])) < 1e-13
    assert np.max(np.abs(s - s_o) / (np.abs(s_o) + cp_o)) < 1e-13
    assert np.max(np.abs(g - g_o) / (np.abs(h_o) + T[:, None] * (np.abs(s_o) + cp_o))) < 1e-13


def test_species_thermo_null_outputs_and_empty():
    chem = Chemistry(mechgen.load("c1"))
    L = chem.L
    T = torch.full((5,), 1200.0, dtype=torch.float64, device="cuda")
    assert L.flint_species_thermo_batch(chem.h, 5, T.data_ptr(), None, None, None, None, None) == 0
    assert L.flint_species_thermo_batch(chem.h, 0, None, None, None, None, None, None) == 0
    out = torch.empty((5, chem.ns), dtype=torch.float64, device="cuda")
    assert L.flint_species_thermo_batch(chem.h, 5, None, out.data_ptr(), None, None, None, None) == 1
