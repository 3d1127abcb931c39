"""The surrogate's training-set generators (host logic): the workloads' own
state distributions and the long-step subset used to add training cells where
the networks' errors concentrate."""
import numpy as np

from flint_gb300 import mechgen
from flint_gb300.surrogate import training_states


def test_reactor_states_are_the_fuel_air_distribution():
    mech = mechgen.load("c2")
    a = mechgen.c3_states(2000, mech, seed=5)
    b = mechgen.fuel_air_states(2000, mech, 5)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    c = training_states("c2")(2000, mech, 5)
    for x, y in zip(a, c):
        assert np.array_equal(x, y)


def test_long_step_subset():
    for cfg, (tlo, thi, plo, phi, dlo) in {"c2": (900.0, 1600.0, 1.0, 20.0, -6.0),
                                           "c5": (900.0, 2000.0, 1.0, 40.0, -7.0)}.items():
        mech = mechgen.load(cfg)
        T, p, Y, dt = training_states(cfg, hard=True)(4000, mech, 9)
        ld = np.log10(dt)
        assert ld.min() >= -4.5 - 1e-12 and ld.max() <= -4.0 + 1e-12
        assert T.min() >= tlo and T.max() <= thi
        patm = p / mechgen.P_ATM
        assert patm.min() >= plo - 1e-9 and patm.max() <= phi + 1e-9
        np.testing.assert_allclose(Y.sum(1), 1.0, rtol=0, atol=1e-14)
        # the plain distribution spans the whole dt range
        _, _, _, dt0 = training_states(cfg)(4000, mech, 9)
        assert np.log10(dt0).min() < dlo + 0.1 and np.log10(dt0).max() > -4.1
