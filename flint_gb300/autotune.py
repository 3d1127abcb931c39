"""Per-mechanism, per-GPU tuning with a persistent cache.

What is tuned (all of it empirically, on a sample of the caller's own cells):

* the reactor's layout (``flint_reactor_autotune``: shared-memory or global
  Newton matrices, 8 or 4 warps per block, one or two blocks per SM);
* the threads per block of the warp-per-cell source-term kernels, for wdot and
  for wdot + Jacobian (``flint_wdot_autotune``: 64, 128 or 256);
* which kernel serves wdot, and which wdot + Jacobian: the data-driven warp
  kernels of the library or the per-mechanism generated ones (``ytf_cuda``,
  every coefficient a literal, thread per cell), when nvcc is there to build
  them.

The choices are stored in a JSON file keyed by the mechanism (a hash of its IR
blob, with ns and nr), the GPU (name, SM count) and the library version, so a
second run on the same mechanism and GPU applies them without timing
(``flint_tuning_set``).  The file is ``$FLINT_TUNING_CACHE`` or
``~/.cache/flint_gb300/tuning.json``.
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import time

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "flint_gb300", "tuning.json")


def cache_path(path=None):
    return path or os.environ.get("FLINT_TUNING_CACHE") or DEFAULT_CACHE


def key(chem):
    """Cache key: mechanism hash, ns, nr, GPU name, SM count, library version."""
    import torch
    from . import native
    blob = chem.mech.to_ir()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    ver = native.lib().flint_version().decode()
    h = hashlib.sha256(bytes(blob)).hexdigest()[:16]
    return f"{h}|ns={chem.ns}|nr={chem.nr}|{props.name}|sms={props.multi_processor_count}|{ver}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply(chem, entry):
    """Put a cached entry into effect on this handle."""
    chem.set_tuning(entry.get("reactor_layout", 0), entry.get("wdot_threads", 0), entry.get("jac_threads", 0))
    chem.use_generated(entry.get("wdot_kernel") == "generated", jac=entry.get("jac_kernel") == "generated")


def _time(fn, reps=3):
    import torch
    fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        fn()
        e1.record(s)
        e1.synchronize()
        t = e0.elapsed_time(e1)
        best = t if best is None else min(best, t)
    return best


def tune(chem, T, p, Y, dt=None, path=None, generated=True, refresh=False):
    """Tune `chem` on a sample of cells (device tensors; dt enables the
    reactor's layout search) or apply the cached choice.  Returns the entry
    (with "cached": True when it came from the file)."""
    import torch
    path = cache_path(path)
    k = key(chem)
    data = _load(path)
    if not refresh and k in data:
        apply(chem, data[k])
        return dict(data[k], cached=True)
    entry = {"when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()), "sample_cells": int(T.shape[0])}
    if dt is not None:
        entry["reactor_layout"] = chem.reactor_autotune(T, p, Y, dt)
        entry["reactor_ms"] = {str(a): b for a, b in chem.reactor_autotune_times().items()}
    t = chem.wdot_autotune(T, p, Y)
    entry["wdot_threads"], entry["jac_threads"] = t["wdot_threads"], t["jac_threads"]
    # data-driven vs generated kernels (wdot with cp, h; wdot + Jacobian)
    w = torch.empty_like(Y)
    cp, h = torch.empty_like(T), torch.empty_like(T)
    J = torch.empty((T.shape[0], chem.ns + 1, chem.ns + 1), dtype=torch.float64, device=T.device)
    chem.use_generated(False, jac=False)
    t_dd = _time(lambda: chem.wdot(T, p, Y, wdot=w, cp=cp, h=h))
    t_ddj = _time(lambda: chem.wdot_jac(T, p, Y, wdot=w, jac=J))
    entry["wdot_ms"] = {"data-driven": t_dd}
    entry["jac_ms"] = {"data-driven": t_ddj}
    entry["wdot_kernel"] = entry["jac_kernel"] = "data-driven"
    if generated and shutil.which(os.environ.get("NVCC", "nvcc")):
        try:
            chem.use_generated(True, jac=True)
            t_gen = _time(lambda: chem.wdot(T, p, Y, wdot=w, cp=cp, h=h))
            t_genj = _time(lambda: chem.wdot_jac(T, p, Y, wdot=w, jac=J))
            entry["wdot_ms"]["generated"] = t_gen
            entry["jac_ms"]["generated"] = t_genj
            if t_gen < t_dd:
                entry["wdot_kernel"] = "generated"
            if t_genj < t_ddj:
                entry["jac_kernel"] = "generated"
        except RuntimeError as ex:   # the generated kernels could not be built: keep the library's
            entry["generated_error"] = str(ex)[:200]
    chem.use_generated(entry["wdot_kernel"] == "generated", jac=entry["jac_kernel"] == "generated")
    data = _load(path)
    data[k] = entry
    _store(path, data)
    return dict(entry, cached=False)
