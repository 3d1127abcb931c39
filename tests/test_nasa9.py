"""NASA-9 thermo (the WD and Cross mechanisms of the reference's tests): the
YAML reader, the oracle's evaluation against an independent NumPy form of the
polynomials, and NASA-7 data entered in their exact NASA-9 form."""
import copy
import os

import numpy as np

from flint_gb300 import mechgen
from flint_gb300.mech import Mechanism
from oracle.oracle import Oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def np_nasa9(sp, T):
    r = [x for x in sp.nasa9 if T <= x[1]]
    a = (r[0] if r else sp.nasa9[-1])[2:]
    if len(sp.nasa9) > 1 and T > sp.nasa9[0][1]:
        a = [x for x in sp.nasa9 if x[0] < T <= x[1]][0][2:]
    cp = a[0] / T ** 2 + a[1] / T + a[2] + a[3] * T + a[4] * T ** 2 + a[5] * T ** 3 + a[6] * T ** 4
    h = (-a[0] / T ** 2 + a[1] * np.log(T) / T + a[2] + a[3] * T / 2 + a[4] * T ** 2 / 3 + a[5] * T ** 3 / 4
         + a[6] * T ** 4 / 5 + a[7] / T)
    s = (-a[0] / T ** 2 / 2 - a[1] / T + a[2] * np.log(T) + a[3] * T + a[4] * T ** 2 / 2 + a[5] * T ** 3 / 3
         + a[6] * T ** 4 / 4 + a[8])
    return cp, h, s


def test_wd_and_cross_parse_as_nasa9():
    for name, ns, nr in (("wd", 5, 3), ("cross", 19, 33)):
        m = Mechanism.load(os.path.join(GOLD, f"mech_{name}.json"))
        assert m.ns == ns and m.nr == nr and all(sp.nasa9 for sp in m.species)
        assert m.to_arrays()["nasa9"].shape == (ns, 32)


def test_oracle_nasa9_vs_numpy():
    m = Mechanism.load(os.path.join(GOLD, "mech_cross.json"))
    orc = Oracle(m)
    for T in (250.0, 999.5, 1000.0, 1000.5, 2345.6, 5900.0):
        cp, h, s, _ = orc.species_thermo(T)
        for k, sp in enumerate(m.species):
            c, hh, ss = np_nasa9(sp, T)
            assert abs(cp[k] - c) <= 1e-13 * abs(c)
            assert abs(h[k] - hh) <= 1e-12 * max(abs(hh), 1.0)
            assert abs(s[k] - ss) <= 1e-13 * abs(ss)


def test_nasa7_in_nasa9_form_is_the_same_thermo():
    m7 = mechgen.load("c2")
    m9 = copy.deepcopy(m7)
    for sp in m9.species:
        lo, hi = list(sp.low), list(sp.high)
        sp.nasa9 = [[sp.tlow, sp.tmid, 0.0, 0.0] + lo[:5] + lo[5:7], [sp.tmid, sp.thigh, 0.0, 0.0] + hi[:5] + hi[5:7]]
    o7, o9 = Oracle(m7), Oracle(m9)
    for T in (400.0, 1000.0, 1700.0, 2900.0):
        for a, b in zip(o7.species_thermo(T), o9.species_thermo(T)):
            np.testing.assert_allclose(b, a, rtol=5e-15, atol=1e-300)
    T, p, Y = mechgen.c2_states(50, m7, seed=2)
    w7, ws7, cp7, h7 = o7.wdot_batch(T, p, Y)
    w9, _, cp9, h9 = o9.wdot_batch(T, p, Y)
    assert np.max(np.abs(w9 - w7) / (ws7 + 1e-300)) < 1e-13
    np.testing.assert_allclose(cp9, cp7, rtol=1e-14)
