"""ctypes wrapper of the FP64 CPU oracle (oracle/flint_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the flint_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from flint_gb300.native import MechDesc, ReactorOpts, TableDesc, mech_desc, ptr

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_build", "liboracle.so")
SO_NATIVE = os.path.join(HERE, "_build", "liboracle_native.so")

_libs = {}


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def native_flags():
    """The CPU-tuning flag of the timed baseline build (-mcpu=native / -march=native)."""
    r = subprocess.run(["make", "-s", "-C", HERE, "native-flags"], capture_output=True, text=True)
    return r.stdout.strip()


def lib(native=False):
    """The portable oracle (the checker), or with native=True the same source
    built for the host CPU (the timed CPU baseline)."""
    if native not in _libs:
        # FLINT_ORACLE_SO: another build of the same source (the sanitizer test's)
        so = SO_NATIVE if native else os.environ.get("FLINT_ORACLE_SO", SO)
        if so in (SO, SO_NATIVE) and (not os.path.exists(so) or
                                      os.path.getmtime(so) < os.path.getmtime(os.path.join(HERE, "flint_oracle.c"))):
            build()
        L = C.CDLL(so)
        dp, vp, i64 = C.POINTER(C.c_double), C.c_void_p, C.c_int64
        md = C.POINTER(MechDesc)
        L.orc_species_thermo.argtypes = [md, C.c_double, vp, vp, vp, vp]
        L.orc_rate_constants.argtypes = [md, C.c_double, vp, vp, vp, vp]
        L.orc_wdot_cell.argtypes = [md, C.c_double, C.c_double, vp, vp, vp, vp, vp]
        L.orc_rhs_constp_cell.argtypes = [md, C.c_double, C.c_double, vp, vp]
        L.orc_jac_cell.argtypes = [md, C.c_double, C.c_double, vp, vp, vp, vp]
        L.orc_rhs_constv_cell.argtypes = [md, C.c_double, C.c_double, vp, vp]
        L.orc_jac_constv_cell.argtypes = [md, C.c_double, C.c_double, vp, vp, vp, vp]
        L.orc_jac_constv_batch.argtypes = [md, i64, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_wdot_batch.argtypes = [md, i64, C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_wdot_jac_batch.argtypes = [md, i64, C.c_int, vp, vp, vp, vp, vp, vp, C.c_int]
        L.orc_reactor_advance.argtypes = [md, i64, vp, vp, vp, vp, C.POINTER(ReactorOpts), vp, vp, C.c_int]
        L.orc_max_threads.restype = C.c_int
        td = C.POINTER(TableDesc)
        L.orc_general_batch.argtypes = [td, i64, vp, vp, vp, C.c_int]
        L.orc_rhs_native_batch.argtypes = [td, i64, vp, vp, C.c_int]
        L.orc_cons2prim_batch.argtypes = [td, i64, C.c_int, vp, vp, vp, vp, C.c_int]
        L.orc_transport_batch.argtypes = [td, i64, vp, vp, vp, vp, C.c_int]
        _libs[native] = L
    return _libs[native]


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """Oracle bound to one mechanism."""

    def __init__(self, mech, native=False):
        self.mech = mech
        self.desc, self._keep = mech_desc(mech)
        self.ns, self.nr = mech.ns, mech.nr
        self.L = lib(native)

    def species_thermo(self, T):
        ns = self.ns
        out = [np.zeros(ns) for _ in range(4)]
        self.L.orc_species_thermo(C.byref(self.desc), float(T), *[_vp(o) for o in out])
        return out  # cpR, hRT, sR, dcpR

    def rate_constants(self, T):
        nr = self.nr
        out = [np.zeros(nr) for _ in range(4)]
        self.L.orc_rate_constants(C.byref(self.desc), float(T), *[_vp(o) for o in out])
        return out  # kf, Kc, k0, fcent

    def rhs(self, T, p, Y):
        f = np.zeros(self.ns + 1)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        self.L.orc_rhs_constp_cell(C.byref(self.desc), float(T), float(p), _vp(Y), _vp(f))
        return f

    def jac(self, T, p, Y):
        n = self.ns + 1
        f = np.zeros(n); J = np.zeros(n * n); Js = np.zeros(n * n)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        self.L.orc_jac_cell(C.byref(self.desc), float(T), float(p), _vp(Y), _vp(f), _vp(J), _vp(Js))
        return f, J.reshape(n, n).T.copy(), Js.reshape(n, n).T.copy()  # J[row, col]

    def rhs_constv(self, T, rho, Y):
        """Constant-volume RHS (dY/dt, dT/dt) of one cell at density rho."""
        f = np.zeros(self.ns + 1)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        self.L.orc_rhs_constv_cell(C.byref(self.desc), float(T), float(rho), _vp(Y), _vp(f))
        return f

    def jac_constv(self, T, rho, Y):
        n = self.ns + 1
        f = np.zeros(n); J = np.zeros(n * n); Js = np.zeros(n * n)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        self.L.orc_jac_constv_cell(C.byref(self.desc), float(T), float(rho), _vp(Y), _vp(f), _vp(J), _vp(Js))
        return f, J.reshape(n, n).T.copy(), Js.reshape(n, n).T.copy()  # J[row, col]

    def jac_constv_batch(self, T, rho, Y, nthreads=0):
        """(f (n, ns+1), J, Js) at constant volume; J, Js flat, per cell column-major."""
        T = np.ascontiguousarray(T, dtype=np.float64); rho = np.ascontiguousarray(rho, dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        n, nv = T.shape[0], self.ns + 1
        f = np.zeros(n * nv); J = np.zeros(n * nv * nv); Js = np.zeros(n * nv * nv)
        self.L.orc_jac_constv_batch(C.byref(self.desc), n, _vp(T), _vp(rho), _vp(Y), _vp(f), _vp(J), _vp(Js),
                                    nthreads)
        return f.reshape(n, nv), J, Js

    def wdot_batch(self, T, p, Y, layout=0, nthreads=0):
        T = np.ascontiguousarray(T, dtype=np.float64); p = np.ascontiguousarray(p, dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        n = T.shape[0]
        w = np.zeros(n * self.ns); ws = np.zeros(n * self.ns); cp = np.zeros(n); h = np.zeros(n)
        self.L.orc_wdot_batch(C.byref(self.desc), n, layout, _vp(T), _vp(p), _vp(Y), _vp(w), _vp(ws),
                              _vp(cp), _vp(h), nthreads)
        return w, ws, cp, h

    def wdot_jac_batch(self, T, p, Y, layout=0, nthreads=0, scale=True):
        T = np.ascontiguousarray(T, dtype=np.float64); p = np.ascontiguousarray(p, dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        n = T.shape[0]
        nn = (self.ns + 1) ** 2
        w = np.zeros(n * self.ns); J = np.zeros(n * nn); Js = np.zeros(n * nn) if scale else None
        self.L.orc_wdot_jac_batch(C.byref(self.desc), n, layout, _vp(T), _vp(p), _vp(Y), _vp(w), _vp(J),
                                  _vp(Js), nthreads)
        return w, J, Js

    def reactor_advance(self, T, p, Y, dt, opts, nthreads=0):
        T = np.array(T, dtype=np.float64); p = np.ascontiguousarray(p, dtype=np.float64)
        Y = np.array(Y, dtype=np.float64); dt = np.ascontiguousarray(dt, dtype=np.float64)
        n = T.shape[0]
        st = np.zeros(n, dtype=np.int32); ns_ = np.zeros(n, dtype=np.int32)
        self.L.orc_reactor_advance(C.byref(self.desc), n, _vp(T), _vp(p), _vp(Y), _vp(dt), C.byref(opts),
                                   _vp(st), _vp(ns_), nthreads)
        return T, Y, st, ns_

    @staticmethod
    def max_threads():
        return lib().orc_max_threads()


class TableOracle:
    """Oracle of FLINT's general loop and rhs_native on a table dict."""

    def __init__(self, t, native=False):
        from flint_gb300.tables import table_desc
        self.t = t
        self.desc, self._keep = table_desc(t)
        self.ns = t["ns"]
        self.L = lib(native)

    def general(self, roi, T, nthreads=0):
        roi = np.ascontiguousarray(roi, dtype=np.float64); T = np.ascontiguousarray(T, dtype=np.float64)
        out = np.zeros_like(roi)
        self.L.orc_general_batch(C.byref(self.desc), T.shape[0], _vp(roi), _vp(T), _vp(out), nthreads)
        return out

    def rhs_native(self, Z, nthreads=0):
        Z = np.ascontiguousarray(Z, dtype=np.float64)
        F = np.zeros_like(Z)
        self.L.orc_rhs_native_batch(C.byref(self.desc), Z.shape[0], _vp(Z), _vp(F), nthreads)
        return F

    def transport(self, rhoi, T, nthreads=0):
        """co_k_mi_lam_Wilke over cells: rhoi (n, ns), T (n,) -> (mu, lambda)."""
        rhoi = np.ascontiguousarray(rhoi, dtype=np.float64)
        T = np.ascontiguousarray(T, dtype=np.float64)
        mu, lam = np.zeros_like(T), np.zeros_like(T)
        self.L.orc_transport_batch(C.byref(self.desc), rhoi.shape[0], _vp(rhoi), _vp(T), _vp(mu), _vp(lam), nthreads)
        return mu, lam

    def cons2prim(self, cons, T, nthreads=0):
        """cons (n, ns + ndim + 1) -> (prim (same shape), last Newton T (n,))."""
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        T = np.ascontiguousarray(T, dtype=np.float64)
        prim = np.zeros_like(cons)
        Tout = np.zeros_like(T)
        self.L.orc_cons2prim_batch(C.byref(self.desc), cons.shape[0], cons.shape[1], _vp(cons), _vp(T), _vp(prim),
                                   _vp(Tout), nthreads)
        return prim, Tout
