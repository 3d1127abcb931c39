"""ctypes view of the C-ABI in include/flint_gpu.h.

The library is built in-tree (flint_gb300/_lib/libflint_gb300.so) by
``flint_gb300.build``.  Loading fails loudly when it is missing: there is no
CPU fallback behind these entry points.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libflint_gb300.so")

FLINT_OK = 0
CELL_MAJOR, SPECIES_MAJOR = 0, 1
CELL_STATUS = {0: "OK", 1: "T_OUT_OF_RANGE", 2: "NAN_INPUT", 3: "MAX_STEPS",
               4: "NEWTON_FAIL", 5: "ERRTEST_FAIL", 6: "SURROGATE_REJECTED"}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class MechDesc(C.Structure):
    """flint_mech_desc."""
    _fields_ = [("ns", C.c_int), ("nr", C.c_int),
                ("mw", _dp), ("nasa7", _dp), ("rtype", _ip), ("reversible", _ip),
                ("arrh", _dp), ("arrh0", _dp), ("troe", _dp),
                ("rsp", _ip), ("rnu", _dp), ("rord", _dp),
                ("psp", _ip), ("pnu", _dp), ("eff", _dp),
                ("r_eos", C.c_double), ("r_thermo", C.c_double), ("p_ref", C.c_double), ("nasa9", _dp)]


class TableDesc(C.Structure):
    """flint_table_desc: FLINT's tabulated module arrays (Fortran layout)."""
    _fields_ = [("ns", C.c_int), ("nr_arrh", C.c_int), ("nr_troe", C.c_int), ("nr_lind", C.c_int),
                ("tmin", C.c_int), ("tmax", C.c_int), ("ti1", C.c_int), ("ti2", C.c_int),
                ("wm", _dp), ("cp_tab", _dp), ("h_tab", _dp), ("kf_tab", _dp), ("kb_tab", _dp),
                ("kinf_troe", _dp), ("k0_troe", _dp), ("kc_troe", _dp), ("fcent_troe", _dp),
                ("kinf_lind", _dp), ("k0_lind", _dp), ("kc_lind", _dp),
                ("ni1_arrh", _dp), ("ni2_arrh", _dp), ("eps_arrh", _dp),
                ("ni1_troe", _dp), ("ni2_troe", _dp), ("eps_troe", _dp),
                ("ni1_lind", _dp), ("ni2_lind", _dp), ("eps_lind", _dp),
                ("runiv", C.c_double), ("mi_tab", _dp), ("k_tab", _dp)]


class ReactorOpts(C.Structure):
    """flint_reactor_opts."""
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("max_steps", C.c_int),
                ("max_order", C.c_int), ("constant_volume", C.c_int), ("reserved", C.c_int),
                ("tmin", C.c_double), ("tmax", C.c_double)]


class Tuning(C.Structure):
    """flint_tuning."""
    _fields_ = [("reactor_layout", C.c_int), ("wdot_threads", C.c_int), ("jac_threads", C.c_int),
                ("reserved", C.c_int)]


def reactor_opts(rtol=1e-8, atol=1e-14, max_steps=20000, max_order=5, tmin=200.0, tmax=6000.0,
                 constant_volume=False):
    return ReactorOpts(rtol, atol, max_steps, max_order, 1 if constant_volume else 0, 0, tmin, tmax)


def ptr(a):
    """ctypes pointer to a contiguous numpy array (or None)."""
    if a is None:
        return None
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_ip)
    raise TypeError(a.dtype)


def mech_desc(mech):
    """Build a MechDesc from a Mechanism; returns (desc, keepalive)."""
    a = mech.to_arrays()
    keep = {k: np.ascontiguousarray(v) for k, v in a.items()}
    d = MechDesc()
    d.ns, d.nr = mech.ns, mech.nr
    for name in ("mw", "nasa7", "rtype", "reversible", "arrh", "arrh0", "troe",
                 "rsp", "rnu", "rord", "psp", "pnu", "eff"):
        setattr(d, name, ptr(keep[name]))
    d.r_eos, d.r_thermo, d.p_ref = (float(x) for x in keep["consts"])
    d.nasa9 = ptr(keep["nasa9"]) if "nasa9" in keep else None
    return d, keep


_lib = None


def lib():
    """Load libflint_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"flint_gb300 native library missing: {LIB_PATH}; "
                           "run flint_gb300.build.build_all() first")
    L = C.CDLL(LIB_PATH)
    vp, i64 = C.c_void_p, C.c_int64
    L.flint_last_error.restype = C.c_char_p
    L.flint_version.restype = C.c_char_p
    L.flint_kernel_launch_count.restype = C.c_int64
    L.flint_mech_create.argtypes = [C.POINTER(MechDesc), C.POINTER(vp)]
    L.flint_mech_destroy.argtypes = [vp]
    L.flint_mech_sizes.argtypes = [vp, _ip, _ip]
    L.flint_thermo_batch.argtypes = [vp, i64, C.c_int, vp, vp, vp, vp, vp]
    L.flint_species_thermo_batch.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp]
    L.flint_wdot_batch.argtypes = [vp, i64, C.c_int, vp, vp, vp, vp, vp, vp, vp]
    L.flint_chemistry_source_batch.argtypes = [vp, i64, vp, vp, vp, vp]
    L.flint_wdot_jac_batch.argtypes = [vp, i64, C.c_int, vp, vp, vp, vp, vp, vp]
    L.flint_rhs_constp_batch.argtypes = [vp, i64, vp, vp, vp, vp, vp]
    L.flint_rhs_constv_batch.argtypes = [vp, i64, vp, vp, vp, vp, vp]
    L.flint_wdot_jac_constv_batch.argtypes = [vp, i64, C.c_int, vp, vp, vp, vp, vp, vp]
    L.flint_reactor_advance.argtypes = [vp, i64, vp, vp, vp, vp, C.POINTER(ReactorOpts), vp, vp, vp]
    L.flint_reactor_autotune.argtypes = [vp, i64, vp, vp, vp, vp, C.POINTER(ReactorOpts), C.POINTER(C.c_int), vp]
    L.flint_reactor_default_opts.argtypes = [C.POINTER(ReactorOpts)]
    L.flint_reactor_advance_noalloc.argtypes = [vp, i64, vp, vp, vp, vp, C.POINTER(ReactorOpts), vp, vp, vp]
    L.flint_reactor_stats.argtypes = [vp, C.POINTER(C.c_int64)]
    L.flint_reactor_autotune_times.argtypes = [vp, _ip, C.POINTER(C.c_float), C.c_int, _ip]
    L.flint_tuning_get.argtypes = [vp, C.POINTER(Tuning)]
    L.flint_tuning_set.argtypes = [vp, C.POINTER(Tuning)]
    L.flint_wdot_autotune.argtypes = [vp, i64, vp, vp, vp, C.POINTER(Tuning), vp]
    L.flint_probe_fp64_peak.argtypes = [C.POINTER(C.c_double)]
    L.flint_selftest_exp.argtypes = [vp, i64, vp, vp, vp]
    L.flint_selftest_log.argtypes = [vp, i64, vp, vp, vp]
    L.flint_mech_create_tables.argtypes = [C.POINTER(TableDesc), C.POINTER(vp)]
    L.flint_tables_read.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp)]
    L.flint_tables_desc.argtypes = [vp, C.POINTER(TableDesc)]
    L.flint_tables_species_name.argtypes = [vp, C.c_int]
    L.flint_tables_species_name.restype = C.c_char_p
    L.flint_tables_free.argtypes = [vp]
    L.flint_mech_create_from_files.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp)]
    L.flint_ir_parse.argtypes = [C.c_char_p, i64, C.POINTER(vp)]
    L.flint_ir_desc.argtypes = [vp, C.POINTER(MechDesc)]
    L.flint_ir_free.argtypes = [vp]
    L.flint_ir_bytes.argtypes = [C.c_int, C.c_int, C.c_int]
    L.flint_ir_bytes.restype = i64
    L.flint_mech_create_from_ir.argtypes = [C.c_char_p, i64, C.POINTER(vp)]
    L.flint_rhs_native_batch.argtypes = [vp, i64, vp, vp, vp]
    L.flint_cons2prim_batch.argtypes = [vp, i64, C.c_int, vp, vp, vp, vp, vp]
    L.flint_transport_batch.argtypes = [vp, i64, vp, vp, vp, vp, vp]
    L.flint_wdot_batch_host.argtypes = [vp, i64, C.c_int, vp, vp, vp, vp, vp, vp]
    L.flint_wdot_jac_batch_host.argtypes = [vp, i64, C.c_int, vp, vp, vp, vp, vp]
    L.flint_reactor_advance_host.argtypes = [vp, i64, vp, vp, vp, vp, C.POINTER(ReactorOpts), vp, vp]
    _lib = L
    return L


def check(rc, what=""):
    if rc != FLINT_OK:
        msg = lib().flint_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed (status {rc}): {msg}")
