"""The mechanism IR blob (flint_ir_parse / flint_mech_create_from_ir): the
Python writer (Mechanism.to_ir) against the library's host-side parser, array
for array, on every in-tree mechanism and the synthetic sets, and the parser's
error returns.  Host only: no GPU."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from flint_gb300 import mechgen, native
from flint_gb300.mech import Mechanism

GOLD = os.path.join(os.path.dirname(__file__), "golden")
MECHS = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLD, "mech_*.json")))


def _parse(blob):
    L = native.lib()
    h = C.c_void_p()
    rc = L.flint_ir_parse(blob, len(blob), C.byref(h))
    return rc, h


def _desc_arrays(h, ns, nr, nasa9):
    L = native.lib()
    d = native.MechDesc()
    assert L.flint_ir_desc(h, C.byref(d)) == 0
    assert (d.ns, d.nr) == (ns, nr)
    shapes = {"mw": (ns,), "nasa7": (ns, 17), "rtype": (nr,), "reversible": (nr,), "arrh": (nr, 3),
              "arrh0": (nr, 3), "troe": (nr, 4), "rsp": (nr, 3), "rnu": (nr, 3), "rord": (nr, 3),
              "psp": (nr, 3), "pnu": (nr, 3), "eff": (nr, ns)}
    out = {}
    for k, shp in shapes.items():
        p = getattr(d, k)
        out[k] = np.ctypeslib.as_array(p, shape=shp).copy() if p and all(shp) else np.zeros(shp)
    out["consts"] = np.array([d.r_eos, d.r_thermo, d.p_ref])
    if nasa9:
        assert d.nasa9
        out["nasa9"] = np.ctypeslib.as_array(d.nasa9, shape=(ns, 32)).copy()
    else:
        assert not d.nasa9
    return out


def _check_roundtrip(m):
    blob = m.to_ir()
    a = m.to_arrays()
    n9 = "nasa9" in a
    assert len(blob) == native.lib().flint_ir_bytes(m.ns, m.nr, int(n9))
    rc, h = _parse(blob)
    assert rc == 0, native.lib().flint_last_error()
    try:
        got = _desc_arrays(h, m.ns, m.nr, n9)
    finally:
        native.lib().flint_ir_free(h)
    for k, v in got.items():
        np.testing.assert_array_equal(v, np.asarray(a[k]).reshape(v.shape), err_msg=k)


@pytest.mark.parametrize("name", MECHS)
def test_roundtrip_intree(name):
    _check_roundtrip(Mechanism.load(os.path.join(GOLD, name)))


@pytest.mark.parametrize("cfg", ["c1", "c2", "c5"])
def test_roundtrip_synthetic(cfg):
    _check_roundtrip(mechgen.load(cfg))


def test_nasa9_section_present():
    assert any("nasa9" in Mechanism.load(os.path.join(GOLD, n)).to_arrays() for n in MECHS), \
        "no in-tree mechanism exercises the NASA-9 section"


@pytest.fixture(scope="module")
def blob():
    return mechgen.load("c1").to_ir()


@pytest.mark.parametrize("case,match", [
    ("short", "48-byte header"), ("magic", "magic"), ("version", "version"), ("counts", "out of range"),
    ("flags", "flags"), ("truncated", "bytes"), ("extra", "bytes")])
def test_parse_errors(blob, case, match):
    b = bytearray(blob)
    if case == "short":
        b = b[:20]
    elif case == "magic":
        b[0:4] = b"FLIX"
    elif case == "version":
        b[4:8] = np.array([2], "<u4").tobytes()
    elif case == "counts":
        b[8:12] = np.array([0], "<i4").tobytes()
    elif case == "flags":
        b[16:20] = np.array([2], "<u4").tobytes()
    elif case == "truncated":
        b = b[:-8]
    elif case == "extra":
        b = b + b"\0" * 8
    rc, h = _parse(bytes(b))
    assert rc == 1 and not h.value
    assert match in native.lib().flint_last_error().decode()


def test_ir_bytes_rejects_bad_sizes():
    L = native.lib()
    assert L.flint_ir_bytes(0, 3, 0) == -1 and L.flint_ir_bytes(4, -1, 0) == -1
    assert L.flint_ir_bytes(6, 2, 1) - L.flint_ir_bytes(6, 2, 0) == 6 * 32 * 8


def test_create_from_ir_null_arguments(blob):
    L = native.lib()
    assert L.flint_mech_create_from_ir(blob, len(blob), None) == 1
    h = C.c_void_p()
    assert L.flint_mech_create_from_ir(None, 0, C.byref(h)) == 1
