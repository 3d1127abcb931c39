"""CPU-side checks of the C-ABI library: it loads and exports every entry point
declared in include/flint_gpu.h (no compute call: there is no GPU here)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(REPO, "include", "flint_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(flint_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("flint_mech_create", "flint_wdot_batch", "flint_wdot_jac_batch", "flint_reactor_advance",
              "flint_chemistry_source_batch", "flint_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from flint_gb300 import native
    if not os.path.exists(native.LIB_PATH):
        from flint_gb300 import build
        build.build_all()
    lib = ctypes.CDLL(native.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_fortran_interface_binds_declared_symbols():
    f90 = open(os.path.join(REPO, "include", "flint_gpu.f90")).read()
    bound = set(re.findall(r"bind\(C,\s*name='(flint_[a-z0-9_]+)'\)", f90))
    assert bound, "no bind(C) interfaces"
    assert bound <= set(declared_symbols())
    # the entry points a CFD caller's time loop needs, including the one for
    # solvers whose memory pool forbids library allocations
    for s in ("flint_reactor_advance", "flint_reactor_advance_noalloc", "flint_chemistry_source_batch",
              "flint_wdot_batch", "flint_mech_destroy"):
        assert s in bound, s


def test_error_reporting_without_gpu():
    """Argument checks run on the host and report through flint_last_error."""
    from flint_gb300 import native
    L = native.lib()
    rc = L.flint_mech_create(None, None)
    assert rc == 1
    assert b"NULL" in L.flint_last_error()


def _c_struct_fields(name):
    txt = open(os.path.join(REPO, "include", "flint_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    body = re.search(r"typedef struct \{([^}]*)\}\s*" + name + r";", txt, flags=re.S).group(1)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        kind = "ptr" if "*" in decl else ("double" if "double" in decl else "int")
        first, *rest = decl.split(",")
        names.append((re.findall(r"[A-Za-z_]\w*", first)[-1], kind))
        names += [(r.strip(), kind) for r in rest]
    return names


def _f90_type_fields(name):
    f90 = open(os.path.join(REPO, "include", "flint_gpu.f90")).read()
    body = re.search(r"type, bind\(C\) :: " + name + r"\n(.*?)end type " + name, f90, flags=re.S).group(1)
    names = []
    for ln in body.splitlines():
        ln = ln.split("!")[0]
        if "::" in ln:
            decl, vars_ = ln.split("::")
            kind = "ptr" if "c_ptr" in decl else ("double" if "c_double" in decl else "int")
            names += [(re.sub(r"=.*", "", v).strip(), kind) for v in vars_.split(",")]
    return [n for n in names if n[0]]


def test_fortran_mirrors_match_c_structs():
    """The bind(C) derived types list the C structs' fields in the same order
    and with the same kinds (int, double, pointer): no Fortran compiler exists
    here to check the layout."""
    for name in ("flint_mech_desc", "flint_table_desc", "flint_reactor_opts"):
        assert _f90_type_fields(name) == _c_struct_fields(name), name
