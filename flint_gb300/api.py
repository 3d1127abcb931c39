"""Host-side mirror of FLINT's chemistry interface over the GB300 C-ABI.

Reference procedure -> this module (paths within the FLINT project):

* ``read_idealgas_thermo`` + ``read_chemistry`` + ``Assign_Mechanism``
  (Load_ThermoTransport.f90:7, Load_Chemistry.f90:7, Lib_Chemistry_wdot.f90:24)
  -> ``Chemistry(mechanism)`` / ``Chemistry.from_config`` (one device handle);
* ``chemistry_source(roi, temp, omegadot)`` (Lib_Chemistry_wdot.f90:6-20)
  -> ``Chemistry.chemistry_source(roi, T)`` over a batch of cells;
* ``f_cp`` / ``H`` (Lib_ThermoTransport.f90:251-271, :40-52) -> ``Chemistry.thermo``;
* ``rhs_native`` (Lib_Chemistry_rhs.f90:15-52) -> ``Chemistry.rhs`` (constant pressure);
* ``setup_odesolver`` / ``run_odesolver`` (test-batchF.f90:81,105)
  -> ``Chemistry.reactor_advance`` (all cells, each over its own dt);
* ``free_chemistry_data`` (Lib_Chemistry_data.f90:168) -> ``Chemistry.close``.

Arguments may be torch CUDA tensors (device path, asynchronous on the current
torch stream) or numpy arrays (host path: the library stages them through its
own device buffers).  Everything runs in the CUDA library; there is no CPU
fallback and a missing library raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .mech import Mechanism

CELL_MAJOR, SPECIES_MAJOR = native.CELL_MAJOR, native.SPECIES_MAJOR


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _dptr(t):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("device path needs CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("tensors must be contiguous")
    return C.c_void_p(t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _hptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Chemistry:
    """One mechanism resident on the GPU (the reference's module globals)."""

    def __init__(self, mech: Mechanism):
        self.mech = mech
        self.L = native.lib()
        desc, keep = native.mech_desc(mech)
        h = C.c_void_p()
        native.check(self.L.flint_mech_create(C.byref(desc), C.byref(h)), "flint_mech_create")
        self.h = h
        self.ns, self.nr = mech.ns, mech.nr
        self._gen, self._use_gen, self._use_gen_jac = None, False, False

    def use_generated(self, on=True, jac=None):
        """Serve wdot (and, with jac, wdot + Jacobian; cell-major device
        tensors) from the mechanism's generated kernels (flint_gb300.ytf_cuda)
        instead of the library's data-driven ones; flint_gb300.autotune makes
        these choices by timing both.  jac=None leaves the Jacobian's choice."""
        if (on or jac) and self._gen is None:
            from .ytf_cuda import GeneratedMechanism
            self._gen = GeneratedMechanism(self.mech)
        self._use_gen = bool(on)
        if jac is not None:
            self._use_gen_jac = bool(jac)

    @classmethod
    def from_ir(cls, blob, mech: Mechanism = None):
        """A handle from an IR blob (flint_mech_create_from_ir).  The kernels
        see only the blob's data; `mech` becomes .mech, which the kinetics,
        thermo and reactor calls do not need but the surrogate's host code does
        (species names and the element matrix are not in the blob)."""
        obj = cls.__new__(cls)
        obj.mech, obj.L = mech, native.lib()
        obj._gen, obj._use_gen, obj._use_gen_jac = None, False, False
        h = C.c_void_p()
        native.check(obj.L.flint_mech_create_from_ir(bytes(blob), len(blob), C.byref(h)), "flint_mech_create_from_ir")
        obj.h = h
        ns, nr = C.c_int(), C.c_int()
        native.check(obj.L.flint_mech_sizes(h, C.byref(ns), C.byref(nr)), "flint_mech_sizes")
        obj.ns, obj.nr = ns.value, nr.value
        return obj

    @classmethod
    def from_config(cls, name):
        from . import mechgen
        return cls(mechgen.load(name))

    def close(self):
        if self.h:
            self.L.flint_mech_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    # -------------------------------------------------------------- kinetics
    def wdot(self, T, p, Y, layout=CELL_MAJOR, wdot=None, cp=None, h=None):
        """Net mass production rates [kg/m^3/s] (+ mixture cp, h) of N cells."""
        n = T.shape[0]
        if _is_torch(T):
            import torch
            if wdot is None:
                wdot = torch.empty_like(Y)
            if self._use_gen and layout == CELL_MAJOR:
                self._gen.wdot(T, p, Y, wdot=wdot, cp=cp, h=h, alloc=False)
                return wdot, cp, h
            native.check(self.L.flint_wdot_batch(self.h, n, layout, _dptr(T), _dptr(p), _dptr(Y), _dptr(wdot),
                                                 _dptr(cp), _dptr(h), _stream()), "flint_wdot_batch")
            return wdot, cp, h
        T, p, Y = (np.ascontiguousarray(a, dtype=np.float64) for a in (T, p, Y))
        w = np.empty_like(Y)
        cpa, ha = np.empty(n), np.empty(n)
        native.check(self.L.flint_wdot_batch_host(self.h, n, layout, _hptr(T), _hptr(p), _hptr(Y), _hptr(w),
                                                  _hptr(cpa), _hptr(ha)), "flint_wdot_batch_host")
        return w, cpa, ha

    def thermo(self, T, Y, layout=CELL_MAJOR, cp=None, h=None):
        """Mixture cp [J/kg/K] and h [J/kg] (device tensors)."""
        native.check(self.L.flint_thermo_batch(self.h, T.shape[0], layout, _dptr(T), _dptr(Y), _dptr(cp),
                                               _dptr(h), _stream()), "flint_thermo_batch")
        return cp, h

    def chemistry_source(self, roi, T, omegadot=None):
        """chemistry_source over N cells: roi (N, ns) kg/m^3 (clamped >= 0 in place)."""
        import torch
        if omegadot is None:
            omegadot = torch.empty_like(roi)
        native.check(self.L.flint_chemistry_source_batch(self.h, T.shape[0], _dptr(roi), _dptr(T),
                                                         _dptr(omegadot), _stream()),
                     "flint_chemistry_source_batch")
        return omegadot

    def wdot_jac(self, T, p, Y, layout=CELL_MAJOR, wdot=None, jac=None):
        """wdot and the constant-pressure reactor Jacobian, jac[cell, col, row]."""
        n, nv = T.shape[0], self.ns + 1
        if _is_torch(T):
            import torch
            if jac is None:
                jac = torch.empty((n, nv, nv), dtype=torch.float64, device=T.device)
            if self._use_gen_jac and layout == CELL_MAJOR:
                self._gen.wdot_jac(T, p, Y, wdot=wdot, jac=jac)
                return wdot, jac
            native.check(self.L.flint_wdot_jac_batch(self.h, n, layout, _dptr(T), _dptr(p), _dptr(Y), _dptr(wdot),
                                                     _dptr(jac), _stream()), "flint_wdot_jac_batch")
            return wdot, jac
        T, p, Y = (np.ascontiguousarray(a, dtype=np.float64) for a in (T, p, Y))
        w = np.empty_like(Y)
        J = np.empty((n, nv, nv))
        native.check(self.L.flint_wdot_jac_batch_host(self.h, n, layout, _hptr(T), _hptr(p), _hptr(Y), _hptr(w),
                                                      _hptr(J)), "flint_wdot_jac_batch_host")
        return w, J

    def species_thermo(self, T):
        """Species cp, h, s (at p_ref) and g = h - T s, mass units, (n, ns) each
        (device tensors)."""
        import torch
        n = T.shape[0]
        out = [torch.empty((n, self.ns), dtype=torch.float64, device=T.device) for _ in range(4)]
        native.check(self.L.flint_species_thermo_batch(self.h, n, _dptr(T), *[_dptr(o) for o in out], _stream()),
                     "flint_species_thermo_batch")
        return tuple(out)

    def wdot_jac_constv(self, T, rho, Y, layout=CELL_MAJOR, wdot=None, jac=None):
        """wdot and the constant-volume reactor Jacobian at density rho (device
        tensors), jac[cell, col, row]."""
        import torch
        n, nv = T.shape[0], self.ns + 1
        if jac is None:
            jac = torch.empty((n, nv, nv), dtype=torch.float64, device=T.device)
        native.check(self.L.flint_wdot_jac_constv_batch(self.h, n, layout, _dptr(T), _dptr(rho), _dptr(Y),
                                                        _dptr(wdot), _dptr(jac), _stream()),
                     "flint_wdot_jac_constv_batch")
        return wdot, jac

    def rhs_constv(self, T, rho, Y, f=None):
        """Constant-volume reactor RHS (dY/dt, dT/dt) at density rho (device tensors), f (n, ns+1)."""
        import torch
        n = T.shape[0]
        if f is None:
            f = torch.empty((n, self.ns + 1), dtype=torch.float64, device=T.device)
        native.check(self.L.flint_rhs_constv_batch(self.h, n, _dptr(T), _dptr(rho), _dptr(Y), _dptr(f), _stream()),
                     "flint_rhs_constv_batch")
        return f

    def rhs(self, T, p, Y, f=None):
        """Constant-pressure RHS (dY/dt, dT/dt), (N, ns+1)."""
        import torch
        if f is None:
            f = torch.empty((T.shape[0], self.ns + 1), dtype=torch.float64, device=T.device)
        native.check(self.L.flint_rhs_constp_batch(self.h, T.shape[0], _dptr(T), _dptr(p), _dptr(Y), _dptr(f),
                                                   _stream()), "flint_rhs_constp_batch")
        return f

    # --------------------------------------------------------------- reactor
    def reactor_autotune(self, T, p, Y, dt, rtol=1e-8, atol=1e-14, max_steps=20000, max_order=5):
        """Time the reactor's layouts on these cells (device tensors, left
        unchanged) and keep the fastest for this handle; returns the layout
        (1 shared memory, 2 global slot / 8 warps per block, 3 global slot / 4 warps,
        4 global slot / two blocks of 8 warps per SM)."""
        opts = native.reactor_opts(rtol, atol, max_steps, max_order)
        lay = C.c_int(0)
        native.check(self.L.flint_reactor_autotune(self.h, T.shape[0], _dptr(T), _dptr(p), _dptr(Y), _dptr(dt),
                                                   C.byref(opts), C.byref(lay), _stream()), "flint_reactor_autotune")
        return lay.value

    def reactor_autotune_times(self):
        """{layout: ms} of the last reactor_autotune on this handle."""
        lays = (C.c_int * 8)()
        ms = (C.c_float * 8)()
        cnt = C.c_int(0)
        native.check(self.L.flint_reactor_autotune_times(self.h, lays, ms, 8, C.byref(cnt)),
                     "flint_reactor_autotune_times")
        return {int(lays[i]): float(ms[i]) for i in range(min(cnt.value, 8))}

    def wdot_autotune(self, T, p, Y):
        """Time the source-term kernels at each block size on these cells (device
        tensors, cell-major) and keep the fastest; returns the handle's tuning."""
        t = native.Tuning()
        native.check(self.L.flint_wdot_autotune(self.h, T.shape[0], _dptr(T), _dptr(p), _dptr(Y), C.byref(t),
                                                _stream()), "flint_wdot_autotune")
        return {f: getattr(t, f) for f, _ in native.Tuning._fields_ if f != "reserved"}

    def tuning(self):
        t = native.Tuning()
        native.check(self.L.flint_tuning_get(self.h, C.byref(t)), "flint_tuning_get")
        return {f: getattr(t, f) for f, _ in native.Tuning._fields_ if f != "reserved"}

    def set_tuning(self, reactor_layout=0, wdot_threads=0, jac_threads=0):
        t = native.Tuning(int(reactor_layout), int(wdot_threads), int(jac_threads), 0)
        native.check(self.L.flint_tuning_set(self.h, C.byref(t)), "flint_tuning_set")

    def reactor_advance(self, T, p, Y, dt, rtol=1e-8, atol=1e-14, max_steps=20000, max_order=5,
                        tmin=200.0, tmax=6000.0, status=None, nsteps=None, constant_volume=False):
        """Advance every cell over its own dt (T, Y updated in place); returns (status, nsteps).
        constant_volume: hold each cell's initial density instead of its pressure."""
        opts = native.reactor_opts(rtol, atol, max_steps, max_order, tmin, tmax, constant_volume)
        n = T.shape[0]
        if _is_torch(T):
            import torch
            if status is None:
                status = torch.empty(n, dtype=torch.int32, device=T.device)
            if nsteps is None:
                nsteps = torch.empty(n, dtype=torch.int32, device=T.device)
            native.check(self.L.flint_reactor_advance(self.h, n, _dptr(T), _dptr(p), _dptr(Y), _dptr(dt),
                                                      C.byref(opts), _dptr(status), _dptr(nsteps), _stream()),
                         "flint_reactor_advance")
            return status, nsteps
        for a in (T, Y):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise ValueError("host arrays T and Y are updated in place: pass contiguous float64 arrays")
        p, dt = (np.ascontiguousarray(a, dtype=np.float64) for a in (p, dt))
        st = np.empty(n, dtype=np.int32)
        nst = np.empty(n, dtype=np.int32)
        native.check(self.L.flint_reactor_advance_host(self.h, n, _hptr(T), _hptr(p), _hptr(Y), _hptr(dt),
                                                       C.byref(opts), _hptr(st), _hptr(nst)),
                     "flint_reactor_advance_host")
        return st, nst


def reactor_stats(chem):
    """Counters of the last reactor launch: rhs, jac, newton, steps, rejected, lu."""
    out = (C.c_int64 * 6)()
    native.check(chem.L.flint_reactor_stats(chem.h, out), "flint_reactor_stats")
    return dict(zip(("rhs", "jac", "newton", "steps", "rejected", "lu"), list(out)))


def kernel_launches():
    """Kernels launched by the library in this process."""
    return native.lib().flint_kernel_launch_count()
