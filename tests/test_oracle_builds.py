"""The oracle's two builds compute the same bits.

The portable build checks every parity test; the build tuned for the host CPU
(-mcpu=native / -march=native) is the timed CPU baseline and, in the
benchmark, also judges the GPU's end states on its sample.  Both keep
-ffp-contract=off and no fast-math, so the compiler may neither contract nor
reassociate: the two must agree bit for bit.
"""
import numpy as np

from flint_gb300 import mechgen
from flint_gb300.native import reactor_opts
from oracle.oracle import Oracle


def test_native_build_is_bit_identical():
    mech = mechgen.load("c2")
    T, p, Y = mechgen.c2_states(64, mech)
    a, b = Oracle(mech), Oracle(mech, native=True)
    for x, y in zip(a.wdot_jac_batch(T, p, Y), b.wdot_jac_batch(T, p, Y)):
        assert np.array_equal(x, y)
    T, p, Y, dt = mechgen.c3_states(16, mech, seed=77)
    for x, y in zip(a.reactor_advance(T, p, Y, dt, reactor_opts()), b.reactor_advance(T, p, Y, dt, reactor_opts())):
        assert np.array_equal(x, y)
