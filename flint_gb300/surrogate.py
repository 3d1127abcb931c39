"""Learned surrogate of the reactor advance: data, training, checkpoints, gate.

The network, its training step (forward, backward, Adam) and the gated
surrogate + fallback advance all run in the CUDA library
(``flint_surrogate_*`` in include/flint_gpu.h); this module drives them:

* ``generate``   runs the FP64 GPU integrator on seeded reactor states and
  returns (state, dt, outcome) samples;
* ``fit_stats``  input / target normalisation from the training samples;
* ``Surrogate``  the device handle (features, targets, train_step, predict,
  advance, state get/set) plus ``save`` / ``load`` of checkpoints holding the
  weights, the Adam moments, the Adam step, the data-sampler position and the
  gate;
* ``train``      Adam with cosine decay on device-resident samples;
* ``calibrate``  gate thresholds from a held-out set judged by the integrator.

Command line: ``python -m flint_gb300.surrogate train --out PATH`` trains the
networks of the benchmark and writes PATH (a checkpoint) next to a JSON
report.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import struct
import time

import numpy as np

from . import native, mechgen
from .api import Chemistry

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)


class SurrogateDesc(C.Structure):
    _fields_ = [("n_layers", C.c_int), ("hidden", C.c_int), ("n_nets", C.c_int), ("bath", C.c_int),
                ("n_elements", C.c_int), ("reserved", C.c_int), ("weights", _fp), ("x_mean", _fp),
                ("x_std", _fp), ("y_mean", _fp), ("y_std", _fp), ("elem", _dp)]


class SurrogateGate(C.Structure):
    _fields_ = [("max_dT_resid", C.c_double), ("max_elem_resid", C.c_double), ("min_Y", C.c_double),
                ("max_ens_dT", C.c_double), ("max_ens_dY", C.c_double), ("T_lo", C.c_double),
                ("T_hi", C.c_double), ("log10p_lo", C.c_double), ("log10p_hi", C.c_double),
                ("log10dt_lo", C.c_double), ("log10dt_hi", C.c_double)]


GATE_KEYS = [f[0] for f in SurrogateGate._fields_]


def _bind(L):
    if getattr(L, "_surrogate_bound", False):
        return
    vp, i64 = C.c_void_p, C.c_int64
    L.flint_surrogate_create.argtypes = [vp, C.POINTER(SurrogateDesc), C.POINTER(vp)]
    L.flint_surrogate_destroy.argtypes = [vp]
    L.flint_surrogate_nparams.argtypes = [vp]
    L.flint_surrogate_nparams.restype = C.c_int64
    L.flint_surrogate_features.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp]
    L.flint_surrogate_targets.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp]
    L.flint_surrogate_train_step.argtypes = [vp, C.c_int, i64, vp, vp, C.c_float, C.POINTER(C.c_double), vp]
    L.flint_surrogate_predict.argtypes = [vp, C.c_int, i64, vp, vp, vp]
    L.flint_surrogate_state.argtypes = [vp, C.c_int, _fp, C.POINTER(C.c_int64), C.c_int]
    L.flint_surrogate_advance.argtypes = [vp, i64, vp, vp, vp, vp, C.POINTER(native.ReactorOpts),
                                          C.POINTER(SurrogateGate), vp, vp, C.POINTER(C.c_int64), vp]
    L.flint_surrogate_counts.argtypes = [vp, C.POINTER(C.c_int64)]
    L.flint_surrogate_evaluate.argtypes = [vp, i64, vp, vp, vp, vp, C.POINTER(SurrogateGate), vp, vp]
    L.flint_surrogate_set_forward.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
    L.flint_surrogate_check.argtypes = [vp, C.POINTER(C.c_int)]
    L._surrogate_bound = True


def layer_dims(ns, hidden=256, n_layers=5):
    return [ns + 2] + [hidden] * (n_layers - 1) + [ns + 1]


def init_weights(dims, seed):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases, per layer W[out][in] then b[out]."""
    rng = np.random.default_rng(seed)
    parts = []
    for i in range(len(dims) - 1):
        bound = 1.0 / math.sqrt(dims[i])
        parts.append(rng.uniform(-bound, bound, dims[i + 1] * dims[i]))
        parts.append(rng.uniform(-bound, bound, dims[i + 1]))
    return np.concatenate(parts).astype(np.float32)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


# ------------------------------------------------------------------ data
def generate(chem, n, seed, states=mechgen.fuel_air_states, **kw):
    """Seeded reactor states advanced by the FP64 GPU integrator (device tensors).

    Returns dict of T0, p, Y0, dt, T1, Y1 (torch, cuda) and the integrator
    statuses; cells that fail are dropped."""
    import torch
    T0, p, Y0, dt = states(n, chem.mech, seed, **kw)
    dev = torch.device("cuda")
    T = torch.from_numpy(T0).to(dev)
    Y = torch.from_numpy(Y0).to(dev)
    P = torch.from_numpy(p).to(dev)
    D = torch.from_numpy(dt).to(dev)
    st, nst = chem.reactor_advance(T, P, Y, D)
    torch.cuda.synchronize()
    ok = (st == 0)
    T0t, Y0t = torch.from_numpy(T0).to(dev), torch.from_numpy(Y0).to(dev)
    return {"T0": T0t[ok].contiguous(), "p": P[ok].contiguous(), "Y0": Y0t[ok].contiguous(),
            "dt": D[ok].contiguous(), "T1": T[ok].contiguous(), "Y1": Y[ok].contiguous(),
            "nsteps": nst[ok].contiguous(), "n_failed": int((~ok).sum().item())}


def fit_stats(d, bath):
    """Normalisation: inputs (log10 Y but bath, T, log10 p, log10 dt) and targets (dY, dT).

    Species targets share a floor of 5 % of the largest species spread so that
    the loss weights mass-fraction errors in absolute terms."""
    Y0 = d["Y0"].cpu().numpy(); Y1 = d["Y1"].cpu().numpy()
    T0 = d["T0"].cpu().numpy(); T1 = d["T1"].cpu().numpy()
    p = d["p"].cpu().numpy(); dt = d["dt"].cpu().numpy()
    ns = Y0.shape[1]
    keep = [k for k in range(ns) if k != bath]
    X = np.hstack([np.log10(np.maximum(Y0[:, keep], 1e-20)), T0[:, None], np.log10(p)[:, None],
                   np.log10(dt)[:, None]])
    xm, xs = X.mean(0), X.std(0)
    xs = np.where(xs > 1e-3, xs, 1.0)
    dY = Y1 - Y0
    dT = T1 - T0
    ym = np.concatenate([dY.mean(0), [dT.mean()]])
    sy = dY.std(0)
    sy = np.maximum(sy, 0.05 * sy.max())
    ys = np.concatenate([sy, [max(dT.std(), 1e-3)]])
    dom = {"T_lo": float(T0.min()), "T_hi": float(T0.max()), "log10p_lo": float(np.log10(p).min()),
           "log10p_hi": float(np.log10(p).max()), "log10dt_lo": float(np.log10(dt).min()),
           "log10dt_hi": float(np.log10(dt).max())}
    return {"x_mean": xm.astype(np.float32), "x_std": xs.astype(np.float32), "y_mean": ym.astype(np.float32),
            "y_std": ys.astype(np.float32), "bath": int(bath), "domain": dom}


DEFAULT_GATE = {"max_dT_resid": 1.0, "max_elem_resid": 1e-4, "min_Y": -1e-4, "max_ens_dT": 1.0, "max_ens_dY": 1e-4,
                "T_lo": 0.0, "T_hi": 1e9, "log10p_lo": -1e9, "log10p_hi": 1e9, "log10dt_lo": -1e9,
                "log10dt_hi": 1e9}


# ---------------------------------------------------------------- handle
class Surrogate:
    """The device surrogate bound to an analytic mechanism handle."""

    def __init__(self, chem: Chemistry, stats, weights=None, n_nets=1, hidden=256, n_layers=5, seed=0):
        self.chem = chem
        self.L = native.lib()
        _bind(self.L)
        self.stats = stats
        self.ns = chem.ns
        self.n_in, self.n_out = chem.ns + 2, chem.ns + 1
        self.dims = layer_dims(chem.ns, hidden, n_layers)
        self.hidden, self.n_layers, self.n_nets = hidden, n_layers, n_nets
        if weights is None:
            weights = np.concatenate([init_weights(self.dims, seed + i) for i in range(n_nets)])
        self._w = np.ascontiguousarray(weights, dtype=np.float32)
        E = chem.mech.element_matrix()
        self._E = np.ascontiguousarray(E, dtype=np.float64)
        self._keep = {k: np.ascontiguousarray(stats[k], dtype=np.float32) for k in ("x_mean", "x_std", "y_mean", "y_std")}
        d = SurrogateDesc(n_layers, hidden, n_nets, int(stats["bath"]), E.shape[0], 0,
                          self._w.ctypes.data_as(_fp), self._keep["x_mean"].ctypes.data_as(_fp),
                          self._keep["x_std"].ctypes.data_as(_fp), self._keep["y_mean"].ctypes.data_as(_fp),
                          self._keep["y_std"].ctypes.data_as(_fp), self._E.ctypes.data_as(_dp))
        h = C.c_void_p()
        native.check(self.L.flint_surrogate_create(chem.h, C.byref(d), C.byref(h)), "flint_surrogate_create")
        self.h = h
        self.P = int(self.L.flint_surrogate_nparams(h))
        self.gate = dict(DEFAULT_GATE, **stats.get("domain", {}))
        self.sampler_pos = 0
        self.rng_state = None

    def close(self):
        if self.h:
            self.L.flint_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    # ---------------------------------------------------------- device ops
    def features(self, T, p, Y, dt):
        import torch
        X = torch.empty((T.shape[0], self.n_in), dtype=torch.float32, device=T.device)
        native.check(self.L.flint_surrogate_features(self.h, T.shape[0], _ptr(T), _ptr(p), _ptr(Y), _ptr(dt),
                                                     _ptr(X), _stream()), "flint_surrogate_features")
        return X

    def targets(self, T0, Y0, T1, Y1):
        import torch
        Yt = torch.empty((T0.shape[0], self.n_out), dtype=torch.float32, device=T0.device)
        native.check(self.L.flint_surrogate_targets(self.h, T0.shape[0], _ptr(T0), _ptr(Y0), _ptr(T1), _ptr(Y1),
                                                    _ptr(Yt), _stream()), "flint_surrogate_targets")
        return Yt

    def train_step(self, X, Yt, lr, net=0, want_loss=False):
        loss = C.c_double(0.0)
        native.check(self.L.flint_surrogate_train_step(self.h, net, X.shape[0], _ptr(X), _ptr(Yt), float(lr),
                                                       C.byref(loss) if want_loss else None, _stream()),
                     "flint_surrogate_train_step")
        return loss.value if want_loss else None

    def predict(self, X, net=0):
        import torch
        Yn = torch.empty((X.shape[0], self.n_out), dtype=torch.float32, device=X.device)
        native.check(self.L.flint_surrogate_predict(self.h, net, X.shape[0], _ptr(X), _ptr(Yn), _stream()),
                     "flint_surrogate_predict")
        return Yn

    def set_forward(self, mode):
        """0: the fused tcgen05 inference kernel where the network fits it (the
        default); 1: one mma.sync GEMM launch per layer.  Returns what runs
        (0 fused, 1 per-layer)."""
        kind = C.c_int(-1)
        native.check(self.L.flint_surrogate_set_forward(self.h, int(mode), C.byref(kind)), "flint_surrogate_set_forward")
        return kind.value

    def check(self):
        """The fused forward's error word (0: every bounded wait completed); waits for the device."""
        e = C.c_int(0)
        native.check(self.L.flint_surrogate_check(self.h, C.byref(e)), "flint_surrogate_check")
        return e.value

    def get_state(self, net=0):
        buf = np.zeros(3 * self.P, dtype=np.float32)
        step = C.c_int64(0)
        native.check(self.L.flint_surrogate_state(self.h, net, buf.ctypes.data_as(_fp), C.byref(step), 1),
                     "flint_surrogate_state")
        return buf, step.value

    def set_state(self, buf, step, net=0):
        buf = np.ascontiguousarray(buf, dtype=np.float32)
        s = C.c_int64(int(step))
        native.check(self.L.flint_surrogate_state(self.h, net, buf.ctypes.data_as(_fp), C.byref(s), 0),
                     "flint_surrogate_state")

    def advance(self, T, p, Y, dt, status=None, nsteps=None, gate=None, rtol=1e-8, atol=1e-14, max_steps=20000,
                wait=True):
        """Gated surrogate + fallback advance in place.  Returns (status, nsteps,
        (accepted, rejected)); with wait=False the call does not wait for the
        stream and the counts are None (the form a CUDA graph captures)."""
        import torch
        g = dict(self.gate, **(gate or {}))
        gs = SurrogateGate(*[float(g[k]) for k in GATE_KEYS])
        opts = native.reactor_opts(rtol, atol, max_steps)
        n = T.shape[0]
        if status is None:
            status = torch.empty(n, dtype=torch.int32, device=T.device)
        if nsteps is None:
            nsteps = torch.empty(n, dtype=torch.int32, device=T.device)
        counts = (C.c_int64 * 2)() if wait else None
        native.check(self.L.flint_surrogate_advance(self.h, n, _ptr(T), _ptr(p), _ptr(Y), _ptr(dt), C.byref(opts),
                                                    C.byref(gs), _ptr(status), _ptr(nsteps), counts, _stream()),
                     "flint_surrogate_advance")
        return status, nsteps, ((counts[0], counts[1]) if wait else None)

    def counts(self):
        """(accepted, rejected) of the last advance, read from the device."""
        c = (C.c_int64 * 2)()
        native.check(self.L.flint_surrogate_counts(self.h, c), "flint_surrogate_counts")
        return c[0], c[1]

    def evaluate(self, T, p, Y, dt):
        """Surrogate result for every cell (T, Y in place) and the gate metrics (n, 6)."""
        import torch
        gs = SurrogateGate(*[float(self.gate[k]) for k in GATE_KEYS])
        M = torch.empty((T.shape[0], 6), dtype=torch.float64, device=T.device)
        native.check(self.L.flint_surrogate_evaluate(self.h, T.shape[0], _ptr(T), _ptr(p), _ptr(Y), _ptr(dt),
                                                     C.byref(gs), _ptr(M), _stream()), "flint_surrogate_evaluate")
        return M

    # ---------------------------------------------------------- checkpoints
    def save(self, path, extra=None, inference_only=False):
        """Checkpoint: JSON header (dims, stats, gate, Adam steps, sampler state) + FP32 blobs
        (weights, Adam first and second moments per network; weights only when inference_only)."""
        nets = [self.get_state(i) for i in range(self.n_nets)]
        if inference_only:
            nets = [(b[:self.P], k) for b, k in nets]
        hdr = {"format": "flint-surrogate-1", "inference_only": bool(inference_only),
               "ns": self.ns, "dims": self.dims, "hidden": self.hidden,
               "n_layers": self.n_layers, "n_nets": self.n_nets, "P": self.P,
               "steps": [s for _, s in nets], "bath": int(self.stats["bath"]),
               "domain": self.stats.get("domain", {}), "gate": self.gate, "sampler_pos": self.sampler_pos,
               "rng_state": self.rng_state, "extra": extra or {}}
        blob = b"".join(self._keep[k].tobytes() for k in ("x_mean", "x_std", "y_mean", "y_std"))
        blob += b"".join(b.tobytes() for b, _ in nets)
        h = json.dumps(hdr).encode()
        with open(path, "wb") as f:
            f.write(struct.pack("<Q", len(h)))
            f.write(h)
            f.write(blob)

    @classmethod
    def load(cls, chem, path, weights_only=False):
        with open(path, "rb") as f:
            (hl,) = struct.unpack("<Q", f.read(8))
            hdr = json.loads(f.read(hl))
            data = np.frombuffer(f.read(), dtype=np.float32)
        ns = hdr["ns"]
        o = 0
        stats = {"bath": hdr["bath"], "domain": hdr["domain"]}
        for k, n in (("x_mean", ns + 2), ("x_std", ns + 2), ("y_mean", ns + 1), ("y_std", ns + 1)):
            stats[k] = data[o:o + n].copy(); o += n
        P = hdr["P"]
        per = P if hdr.get("inference_only") else 3 * P
        states = [data[o + per * i:o + per * (i + 1)].copy() for i in range(hdr["n_nets"])]
        w0 = np.concatenate([s[:P] for s in states])
        s = cls(chem, stats, weights=w0, n_nets=hdr["n_nets"], hidden=hdr["hidden"], n_layers=hdr["n_layers"])
        if not weights_only and not hdr.get("inference_only"):
            for i, st in enumerate(states):
                s.set_state(st, hdr["steps"][i], net=i)
        s.gate = dict(s.gate, **hdr.get("gate", {}))
        s.sampler_pos = hdr.get("sampler_pos", 0)
        s.rng_state = hdr.get("rng_state")
        s.header = hdr
        return s


# ---------------------------------------------------------------- training
def train(sur, X, Yt, steps, batch=4096, lr=1e-3, lr_min=1e-5, net=0, seed=0, log_every=1000, start=0,
          total=None, log=None):
    """Adam with cosine decay over device-resident (X, Yt); returns loss history.

    Mini-batches are drawn by a seeded permutation stream: batch i of the run
    uses generator(seed).permutation epochs, so that resuming at step `start`
    replays exactly the batches of a continuous run."""
    import torch
    n = X.shape[0]
    total = total or steps
    hist = []
    gen = torch.Generator(device=X.device)
    per_epoch = max(1, n // batch)
    epoch = -1
    perm = None
    for it in range(start, start + steps):
        e = it // per_epoch
        if e != epoch:
            gen.manual_seed(seed * 1000003 + e)
            perm = torch.randperm(n, generator=gen, device=X.device)
            epoch = e
        j = it % per_epoch
        idx = perm[j * batch:(j + 1) * batch]
        xb, yb = X.index_select(0, idx).contiguous(), Yt.index_select(0, idx).contiguous()
        a = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * min(it, total) / total))
        want = (it + 1) % log_every == 0
        loss = sur.train_step(xb, yb, a, net=net, want_loss=want)
        if want:
            hist.append((it + 1, loss))
            if log:
                log(f"net {net} step {it + 1} lr {a:.2e} loss {loss:.3e}")
    sur.sampler_pos = start + steps
    return hist


def errors_vs_integrator(Tsur, Ysur, Tref, Yref):
    dT = (Tsur - Tref).abs()
    dY = (Ysur - Yref).abs().amax(dim=1)
    return dT, dY


def search_gate(M, eT, eY, T0, log10dt, gate, n_nets, target_dT=1.0, target_dY=1e-4, margin=0.5):
    """Largest accepted set of validation cells whose every member is within
    margin * (target_dT, target_dY) of the integrator, over gate thresholds on
    the energy residual, the ensemble spreads of dT and dY, and the upper ends
    of the input domain in dt and T0 (the long steps and hot starts where the
    network's errors concentrate).

    For each domain cut and residual threshold the two spread thresholds are
    found exactly: sweeping the dT-spread threshold b over the cells' own
    values, the dY-spread threshold must stay below the smallest dY spread of
    the out-of-tolerance cells with dT spread <= b.  Returns (accepted
    fraction, gate update, max dT, max dY) or None."""
    good = (eT <= margin * target_dT) & (eY <= margin * target_dY)
    bad = ~good
    base = (M[:, 5] > 0) & (M[:, 1] <= gate["max_elem_resid"]) & (M[:, 2] >= gate["min_Y"])
    if not base.any():
        return None
    n = len(eT)
    ens = n_nets > 1
    x = M[:, 3] if ens else np.zeros(n)
    y = M[:, 4] if ens else np.zeros(n)
    dt_cuts = np.unique(np.concatenate([[log10dt.max()], np.quantile(log10dt, [0.95, 0.9, 0.85, 0.8, 0.75, 0.7])]))
    T_cuts = np.unique(np.concatenate([[T0.max()], np.quantile(T0, [0.95, 0.9, 0.85])]))
    rgrid = np.unique(np.concatenate([np.linspace(0.05, 0.9, 10), np.linspace(0.9, 1.0, 21)]))
    bgrid = np.unique(np.concatenate([np.linspace(0.05, 0.9, 12), np.linspace(0.9, 1.0, 29)]))
    best = None
    for dth in dt_cuts:
        for Th in T_cuts:
            dom = base & (log10dt <= dth) & (T0 <= Th)
            if not dom.any():
                continue
            for a in np.quantile(M[dom, 0], rgrid):
                S = dom & (M[:, 0] <= a)
                if not S.any():
                    continue
                cands = np.quantile(x[S], bgrid) if ens else [0.0]
                for bthr in cands:
                    sel = S & (x <= bthr)
                    yb = y[sel & bad]
                    cmax = yb.min() if yb.size else np.inf
                    ok = sel & (y < cmax)
                    cnt = int(ok.sum())
                    if cnt == 0 or (best is not None and cnt <= best[0]):
                        continue
                    c = float(y[ok].max())
                    best = (cnt, {"max_dT_resid": float(a), "max_ens_dT": float(bthr) if ens else 1e30,
                                  "max_ens_dY": c if ens else 1e30, "log10dt_hi": float(dth), "T_hi": float(Th)},
                            float(eT[ok].max()), float(eY[ok].max()))
    if best is None:
        return None
    return (best[0] / n, best[1], best[2], best[3])


def calibrate(sur, d, target_dT=1.0, target_dY=1e-4, margin=0.5):
    """Gate thresholds from held-out samples judged by the integrator.

    The surrogate is applied to every validation cell (``evaluate``) and
    ``search_gate`` picks the thresholds with the largest accepted fraction such
    that every accepted validation cell is within margin * (target_dT,
    target_dY) of the FP64 integrator.  Returns (accept_fraction, gate dict,
    max dT, max dY)."""
    T = d["T0"].clone(); Y = d["Y0"].clone()
    M = sur.evaluate(T, d["p"], Y, d["dt"]).cpu().numpy()
    eT = (T - d["T1"]).abs().cpu().numpy()
    eY = (Y - d["Y1"]).abs().amax(dim=1).cpu().numpy()
    base = (M[:, 5] > 0) & (M[:, 1] <= sur.gate["max_elem_resid"]) & (M[:, 2] >= sur.gate["min_Y"])
    good = (eT <= margin * target_dT) & (eY <= margin * target_dY)
    diag = {"eT_q": [float(x) for x in np.quantile(eT, [0.5, 0.9, 0.99, 0.999, 1.0])],
            "eY_q": [float(x) for x in np.quantile(eY, [0.5, 0.9, 0.99, 0.999, 1.0])],
            "resid_q": [float(x) for x in np.quantile(M[:, 0], [0.5, 0.9, 0.99, 1.0])],
            "ensT_q": [float(x) for x in np.quantile(M[:, 3], [0.5, 0.9, 0.99, 1.0])],
            "ensY_q": [float(x) for x in np.quantile(M[:, 4], [0.5, 0.9, 0.99, 1.0])],
            "elem_q": [float(x) for x in np.quantile(M[:, 1], [0.5, 0.9, 1.0])],
            "minY_q": [float(x) for x in np.quantile(M[:, 2], [0.0, 0.01, 0.5])],
            "base_frac": float(base.mean()), "good_frac": float(good.mean())}
    calibrate.diag = diag
    calibrate.data = {"M": M.astype(np.float32), "eT": eT.astype(np.float32), "eY": eY.astype(np.float32),
                      "T0": d["T0"].cpu().numpy().astype(np.float32), "p": d["p"].cpu().numpy().astype(np.float32),
                      "dt": d["dt"].cpu().numpy().astype(np.float32),
                      "pred_dT": (T - d["T0"]).cpu().numpy().astype(np.float32),
                      "pred_dY": (Y - d["Y0"]).abs().amax(dim=1).cpu().numpy().astype(np.float32),
                      "true_dT": (d["T1"] - d["T0"]).cpu().numpy().astype(np.float32),
                      "worst_species": (Y - d["Y1"]).abs().argmax(dim=1).cpu().numpy().astype(np.int16)}
    return search_gate(M, eT, eY, d["T0"].cpu().numpy(), np.log10(d["dt"].cpu().numpy()), sur.gate, sur.n_nets,
                       target_dT, target_dY, margin)


def training_states(config, hard=False):
    """The state generator of a training set: the workload's own distribution
    (c2: the 31-species reactor states, c5: the 54-species scale-up states), or
    with hard=True the same distribution restricted to the top half-decade of
    dt, where the largest errors of a network trained on the plain
    distribution lie."""
    base = mechgen.c5_states if config == "c5" else mechgen.c3_states
    if not hard:
        return lambda n, mech, seed: base(n, mech, seed)
    return lambda n, mech, seed: base(n, mech, seed, log10dt=(-4.5, -4.0))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "calibrate"],
                    help="train: generate, train, calibrate, save; calibrate: re-derive the gate of a checkpoint")
    ap.add_argument("--checkpoint", help="calibrate: the checkpoint to re-calibrate")
    ap.add_argument("--save-val", action="store_true",
                    help="also write the per-cell validation metrics and errors (<out>_val.npz, tens of MB)")
    ap.add_argument("--out", required=True)
    ap.add_argument("--cells", type=int, default=524288)
    ap.add_argument("--val", type=int, default=65536)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--nets", type=int, default=2)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--margin", type=float, default=0.8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--hard", type=int, default=0,
                    help="extra training cells drawn from the top half-decade of dt only, where the largest "
                         "errors of a network trained on the plain distribution lie (validation stays plain)")
    ap.add_argument("--config", default="c2", choices=["c2", "c5"],
                    help="c2: 31 species, c3 reactor states; c5: 54 species, scale-up states")
    args = ap.parse_args()
    import torch
    chem = Chemistry.from_config(args.config)
    states = training_states(args.config)
    hard_states = training_states(args.config, hard=True)
    if args.cmd == "calibrate":
        sur = Surrogate.load(chem, args.checkpoint)
        v = generate(chem, args.val, seed=6000 + args.seed, states=states)
        best = calibrate(sur, v, margin=args.margin)
        print("calibration diagnostics", json.dumps(getattr(calibrate, "diag", {})))
        if best is not None:
            sur.gate.update(best[1])
        rep = dict(sur.header.get("extra", {}))
        rep["calibration"] = None if best is None else {"accept_frac": best[0], "max_dT": best[2], "max_dY": best[3],
                                                        "val_cells": int(v["T0"].shape[0]), "margin": args.margin}
        rep["gate"] = sur.gate
        rep["diagnostics"] = getattr(calibrate, "diag", {})
        if args.save_val and getattr(calibrate, "data", None) is not None:
            np.savez_compressed(os.path.splitext(args.out)[0] + "_val.npz", **calibrate.data)
        sur.save(args.out, extra=rep, inference_only=bool(sur.header.get("inference_only")))
        print(json.dumps(rep["calibration"]))
        return
    t0 = time.time()
    d = generate(chem, args.cells, seed=5000 + args.seed, states=states)
    if args.hard:
        h = generate(chem, args.hard, seed=7000 + args.seed, states=hard_states)
        d = {k: torch.cat([d[k], h[k]]) if torch.is_tensor(d[k]) else d[k] + h[k] for k in d}
        del h
    v = generate(chem, args.val, seed=6000 + args.seed, states=states)
    tgen = time.time() - t0
    bath = chem.mech.index("N2")
    stats = fit_stats(d, bath)
    sur = Surrogate(chem, stats, n_nets=args.nets, seed=args.seed)
    X = sur.features(d["T0"], d["p"], d["Y0"], d["dt"])
    Yt = sur.targets(d["T0"], d["Y0"], d["T1"], d["Y1"])
    hist = {}
    t1 = time.time()
    for net in range(args.nets):
        hist[net] = train(sur, X, Yt, args.steps, batch=args.batch, net=net, seed=args.seed + net,
                          lr=args.lr, log=print)
    torch.cuda.synchronize()
    ttrain = time.time() - t1
    Xv = sur.features(v["T0"], v["p"], v["Y0"], v["dt"])
    Yv = sur.targets(v["T0"], v["Y0"], v["T1"], v["Y1"])
    val_loss = [float(((sur.predict(Xv, net=i) - Yv) ** 2).mean()) for i in range(args.nets)]
    best = calibrate(sur, v, margin=args.margin)
    print("calibration diagnostics", json.dumps(getattr(calibrate, "diag", {})))
    if best is not None:
        sur.gate.update(best[1])
    rep = {"train_cells": int(d["T0"].shape[0]), "hard_cells": args.hard, "val_cells": int(v["T0"].shape[0]),
           "gen_s": tgen,
           "train_s": ttrain, "steps": args.steps, "batch": args.batch, "val_loss": val_loss,
           "loss_history": {str(k): h for k, h in hist.items()},
           "gate": sur.gate, "diagnostics": getattr(calibrate, "diag", {}),
           "calibration": None if best is None else
           {"accept_frac": best[0], "max_dT": best[2], "max_dY": best[3], "val_cells": int(v["T0"].shape[0]),
            "margin": args.margin}}
    if args.save_val and getattr(calibrate, "data", None) is not None:
        np.savez_compressed(os.path.splitext(args.out)[0] + "_val.npz", **calibrate.data)
    sur.save(args.out, extra=rep)
    sur.save(os.path.splitext(args.out)[0] + "_inference.bin", extra=rep, inference_only=True)
    with open(os.path.splitext(args.out)[0] + ".json", "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps({k: rep[k] for k in ("train_cells", "gen_s", "train_s", "val_loss", "calibration")}))


if __name__ == "__main__":
    main()
