"""Benchmark: batched stiff 0D constant-pressure reactor advance on one GB300.

Workload (the reactor configuration of the metric): the seeded synthetic
31-species / 160-reaction mechanism (12 third-body, 6 Troe), 262,144 cells with
T0 ~ U(900,1600) K, p ~ U(1,20) atm, phi ~ U(0.5,2) CH4/air, per-cell
dt = 10^U(-6,-4) s, rtol 1e-8, atol 1e-14.  One step = one advance of every
cell over its own dt (one cell-step per cell); the state is reset from the
initial copy at the start of each step.

Metric: cell-steps/s (higher is better).
  value  device-timed (inputs resident in HBM), CUDA events on the launch stream,
         L2 flushed (256 MiB write) between timed steps.
  e2e    the same through the public API with pinned host buffers: per step
         H2D of T, p, Y, dt, the advance, D2H of T, Y and the status word.
  roofline  the reactor kernel against the FP64 pipe: FP64 ops per launch from
         the live work counters x per-event op counts (profiles/), over the
         kernel's event-timed duration; peak = DFMA throughput measured in this
         run by the library's probe kernel.
  cpu_baseline  the FP64 oracle (OpenMP, all host cores) on a bounded sample.

--impl reference times the oracle port of the reference path (FLINT's Fortran
cannot be built: no Fortran compiler exists on these machines) on the same
workload and prints the same JSON line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

from flint_gb300 import dist as fdist  # noqa: E402

CELLS = 262144
METRIC = "cell-steps/s on 1 GB300: surrogate+fallback vs plain FP64 at stated T/Y error"
# FP64 FLOPs per kinetics evaluation (2 x DFMA + DADD + DMUL thread instructions,
# predicated on) of the warp kernels, per state: k_wdot_warp<0> for one RHS and
# k_wdot_warp<1> for one Jacobian, from ncu on the c2-wdot / c2-wdotjac and
# c5-wdot / c5-wdotjac workloads (profiles/fp64_ops_per_state.md).
KINETICS_FLOPS = {"synthetic-31sp-160r": {"rhs": 18800.0, "jac": 40686.0},
                  "synthetic-54sp-320r": {"rhs": 31720.0, "jac": 82537.0}}


# DRAM bytes (read + write) per cell of one k_reactor launch, from ncu
# (profiles/k_reactor_c3_8192cells.md: 2.70 MB for 8,192 cells of the
# 31-species workload); the traffic field scales it by the launch's cells.
REACTOR_DRAM_BYTES_PER_CELL = {"synthetic-31sp-160r": 2.699264e6 / 8192}


def fp64_ops(ev, ns, mech_name="synthetic-31sp-160r"):
    """FP64 FLOPs of a reactor launch from its event counters: kinetics per RHS
    and Jacobian evaluation (measured per state), (2/3) n^3 per LU factorization
    and 2 n^2 per LU solve (n = ns + 1)."""
    k = KINETICS_FLOPS[mech_name]
    n = ns + 1
    return (ev["rhs"] * k["rhs"] + ev["jac"] * k["jac"] + ev["lu"] * (2.0 / 3.0) * n ** 3
            + ev["newton"] * 2.0 * n * n)


def dist_env():
    from flint_gb300.dist import env
    return env()


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0])); smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _oracle_sample_size(orc, T, p, Y, dt, opts, target_s):
    """Cells of a sample that takes about target_s on the host (grown from 256
    on the first cells of the workload); returns (n, seconds, end states)."""
    n = 256
    while True:
        t0 = time.perf_counter()
        out = orc.reactor_advance(T[:n], p[:n], Y[:n], dt[:n], opts)
        el = time.perf_counter() - t0
        if el > 0.7 * target_s or n >= len(T):
            return n, el, out
        n = min(len(T), int(n * min(8.0, max(1.5, target_s / max(el, 1e-3)))))


def cpu_baseline(mech, T, p, Y, dt, target_s=12.0, want_state=False):
    """Oracle reactor (the build tuned for the host CPU) on all host cores over a
    bounded sample; cells/s.  With want_state the oracle's end states of the
    sample come back too (the checker of the GPU results on the same cells; the
    tuned and the portable builds compute the same bits)."""
    from oracle.oracle import Oracle, native_flags
    from flint_gb300.native import reactor_opts
    orc = Oracle(mech, native=True)
    cores = Oracle.max_threads()
    n, el, out = _oracle_sample_size(orc, T, p, Y, dt, reactor_opts(), target_s)
    res = {"value": n / el, "unit": "cell-steps/s", "cores": cores, "kind": "port",
           "sample": f"{n} of the {len(T)} cells (first n), FP64 oracle BDF (gcc -O3 {native_flags()}), {el:.1f} s"}
    if want_state:
        return res, (out[0], out[1], out[2], n)
    return res


def run_reference(args):
    """The reference's CPU implementation of the path (the FP64 oracle port: FLINT's
    Fortran cannot be compiled on these machines) on the default arm's workload:
    the same seeded cells (the 1,048,576-cell C4 set, or the plain path's
    262,144), all host threads.  Every step advances the same bounded sample of
    those cells (its first n, sized once so the whole run takes a few minutes);
    ms_per_step is that sample's measured time, and the per-cell rate scaled to
    the whole workload is reported separately."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from flint_gb300 import mechgen
    from flint_gb300.native import reactor_opts
    from oracle.oracle import Oracle, native_flags
    mech = mechgen.load("c2")
    surrogate = args.path != "plain" and os.path.exists(args.checkpoint)
    n_all = args.cells or (SUR_CELLS if surrogate else CELLS)
    T, p, Y, dt = mechgen.c3_states(n_all, mech, seed=1004 if surrogate else 1003)
    orc = Oracle(mech, native=True)
    opts = reactor_opts()
    per_step = min(args.ref_seconds, max(1.0, 150.0 / max(1, args.warmup + args.steps)))
    n, _, _ = _oracle_sample_size(orc, T, p, Y, dt, opts, per_step)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        orc.reactor_advance(T[:n], p[:n], Y[:n], dt[:n], opts)
        el = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(el)
    t = statistics.mean(times)
    v = n / t
    wl = (f"reactor-c4: surrogate+fallback, 31sp/160r, {n_all} cells, rtol 1e-8 atol 1e-14" if surrogate else
          f"reactor-c3: 31sp/160r constant-p BDF/Newton, {n_all} cells, rtol 1e-8 atol 1e-14")
    sample = (f"the first {n} of the workload's {n_all} cells every step, FP64 oracle BDF "
              f"(gcc -O3 {native_flags()} -fopenmp), {Oracle.max_threads()} threads")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded states, seeded synthetic mechanism)",
            "config": {"workload": wl, "cells": n, "cells_in_workload": n_all,
                       "path": "FP64 BDF oracle (the reference path restated in C; no surrogate)",
                       "note": "each timed step advances the same bounded sample of the workload's cells"},
            "projected_ms_for_all_cells": 1e3 * n_all / v,
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": Oracle.max_threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from flint_gb300 import mechgen
    from flint_gb300.api import Chemistry, reactor_stats, kernel_launches
    from flint_gb300 import native
    c5 = args.workload == "reactor-c5"
    mech = mechgen.load("c5" if c5 else "c2")
    n = args.cells
    if c5:
        T0, p0, Y0, dt0 = mechgen.c5_states(n, mech, seed=1005 + rank)
    else:
        T0, p0, Y0, dt0 = mechgen.c3_states(n, mech, seed=1003 + rank)
    chem = Chemistry(mech)
    Td0 = torch.from_numpy(T0).to(dev)
    Yd0 = torch.from_numpy(Y0).to(dev)
    pd = torch.from_numpy(p0).to(dev)
    dtd = torch.from_numpy(dt0).to(dev)
    Td, Yd = Td0.clone(), Yd0.clone()
    st = torch.empty(n, dtype=torch.int32, device=dev)
    nst = torch.empty(n, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    # the autotuner picks the reactor layout on a sample of these cells (untimed)
    ms = min(n, 16384)
    layout = chem.reactor_autotune(Td0[:ms], pd[:ms], Yd0[:ms], dtd[:ms])

    def direct():
        Td.copy_(Td0)
        Yd.copy_(Yd0)
        chem.reactor_advance(Td, pd, Yd, dtd, status=st, nsteps=nst)

    step = direct
    graph_note = "not used"
    per_replay = 0
    if not args.no_graph:
        # one step (input copy + the persistent reactor launch) captured as a CUDA graph
        try:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                direct()
            torch.cuda.current_stream().wait_stream(side)
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            lc = kernel_launches()
            with torch.cuda.graph(graph, capture_error_mode="relaxed"):
                direct()
            torch.cuda.synchronize()
            per_replay = kernel_launches() - lc
            step = graph.replay
            graph_note = "each step one CUDA graph replay"
        except Exception as ex:   # report it; the timed path is then the direct calls
            graph_note = f"capture failed ({type(ex).__name__}: {ex}); direct calls"
            step = direct

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    times = []
    launches0 = kernel_launches()
    stats = []
    barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        stats.append(reactor_stats(chem))
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    launches = kernel_launches() - launches0
    if step is not direct:
        launches = per_replay * args.steps
    status = st.cpu().numpy()
    steps_per_cell = nst.cpu().numpy()
    t_step = statistics.mean(times)
    t_step = fdist.max_over_ranks(t_step, dev)
    value = n * ws / t_step

    # ---- end to end through the public API with pinned host buffers --------
    Th = torch.from_numpy(T0).pin_memory()
    ph = torch.from_numpy(p0).pin_memory()
    Yh = torch.from_numpy(Y0).pin_memory()
    dth = torch.from_numpy(dt0).pin_memory()
    To = torch.empty_like(Th).pin_memory()
    Yo = torch.empty_like(Yh).pin_memory()
    so = torch.empty(n, dtype=torch.int32).pin_memory()
    Te, pe, Ye, dte = (torch.empty_like(x, device=dev) for x in (Th, ph, Yh, dth))
    h2d = sum(x.numel() * x.element_size() for x in (Th, ph, Yh, dth))
    d2h = sum(x.numel() * x.element_size() for x in (To, Yo, so))
    e2e_times = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Te.copy_(Th, non_blocking=True); pe.copy_(ph, non_blocking=True)
        Ye.copy_(Yh, non_blocking=True); dte.copy_(dth, non_blocking=True)
        chem.reactor_advance(Te, pe, Ye, dte, status=st, nsteps=nst)
        To.copy_(Te, non_blocking=True); Yo.copy_(Ye, non_blocking=True); so.copy_(st, non_blocking=True)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
    e2e_t = statistics.mean(e2e_times)
    e2e_t = fdist.max_over_ranks(e2e_t, dev)
    assert np.array_equal(so.numpy(), status), "e2e run disagrees with the device-timed run"

    # ---- roofline: FP64 pipe ------------------------------------------------
    s = stats[-1]
    ops = fp64_ops(s, chem.ns, chem.mech.name)
    peak = chem_peak_fp64()
    achieved = ops / t_step / 1e12
    roof = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if peak else None,
            "traffic": (REACTOR_DRAM_BYTES_PER_CELL[mech.name] * n if mech.name in REACTOR_DRAM_BYTES_PER_CELL
                        else None),
            "kernel": "k_reactor", "peak_source": "DFMA probe kernel measured in this run (MEASURED_PEAKS.json has no FP64 figure)",
            "ops_per_launch": ops, "events_per_launch": s}
    line = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded states, seeded synthetic mechanism)",
            "config": ({"workload": f"reactor-c5: 54sp/320r constant-p BDF/Newton, {n} cells (sample of the "
                                    "4,194,304-cell scale-up), T0 900-2000 K, p 1-40 atm, phi 0.4-3, dt 1e-7..1e-4 s, "
                                    "rtol 1e-8 atol 1e-14",
                        "cells_per_gpu": n, "mechanism": "synthetic-54sp-320r (20 third-body, 12 Troe)"} if c5 else
                       {"workload": f"reactor-c3: 31sp/160r constant-p BDF/Newton, {n} cells, rtol 1e-8 atol 1e-14",
                        "cells_per_gpu": n, "mechanism": "synthetic-31sp-160r (12 third-body, 6 Troe)"})
                      | {"path": "plain FP64 integrator", "l2": "flushed (256 MiB write) between timed steps",
                         "cuda_graph": graph_note,
                         "reactor_layout": REACTOR_LAYOUTS[layout]
                         + " (autotuned on 16,384 cells)"},
            "e2e": {"value": n * ws / e2e_t, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clk, "roofline": roof,
            "cell_status": {str(k): int(v) for k, v in zip(*np.unique(status, return_counts=True))},
            "internal_steps_per_cell": {"mean": float(steps_per_cell.mean()), "max": int(steps_per_cell.max())},
            "wall_s_timed": wall}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(mech, T0, p0, Y0, dt0)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


REACTOR_LAYOUTS = {0: "by size", 1: "shared memory", 2: "global slot, 8 warps/block",
                   3: "global slot, 4 warps/block", 4: "global slot, 2 blocks of 8 warps/SM (128 registers)"}
SURROGATE_CKPT = os.path.join(REPO, "flint_gb300", "data", "surrogate_c3.bin")
SURROGATE_CKPT_C5 = os.path.join(REPO, "flint_gb300", "data", "surrogate_c5.bin")
SUR_CELLS = 1048576


def run_surrogate(args):
    """Headline: surrogate + fallback advance of 1,048,576 reactor cells vs the
    plain FP64 integrator on the same cells (all of them), which also judges the errors."""
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from flint_gb300 import mechgen
    from flint_gb300.api import Chemistry, reactor_stats, kernel_launches
    from flint_gb300.surrogate import Surrogate
    c5 = args.workload == "reactor-c5"
    chem = Chemistry(mechgen.load("c5" if c5 else "c2"))
    sur = Surrogate.load(chem, args.checkpoint, weights_only=True)
    fwd_kind = sur.set_forward(0)
    n = args.cells or SUR_CELLS
    if c5:
        T0, p0, Y0, dt0 = mechgen.c5_states(n, chem.mech, seed=1005 + rank)
    else:
        T0, p0, Y0, dt0 = mechgen.c3_states(n, chem.mech, seed=1004 + rank)
    Td0, Yd0 = torch.from_numpy(T0).to(dev), torch.from_numpy(Y0).to(dev)
    pd, dtd = torch.from_numpy(p0).to(dev), torch.from_numpy(dt0).to(dev)
    Td, Yd = Td0.clone(), Yd0.clone()
    st = torch.empty(n, dtype=torch.int32, device=dev)
    nst = torch.empty(n, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    counts = {}

    ms = min(n, 16384)
    layout = chem.reactor_autotune(Td0[:ms], pd[:ms], Yd0[:ms], dtd[:ms])

    def direct():
        Td.copy_(Td0)
        Yd.copy_(Yd0)
        _, _, c = sur.advance(Td, pd, Yd, dtd, status=st, nsteps=nst)
        counts["c"] = c

    def async_step():
        Td.copy_(Td0)
        Yd.copy_(Yd0)
        sur.advance(Td, pd, Yd, dtd, status=st, nsteps=nst, wait=False)

    step = direct
    graph_note = "not used"
    if not args.no_graph:
        # one step (input copy + surrogate + fallback) captured as a CUDA graph
        try:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                async_step()
            torch.cuda.current_stream().wait_stream(side)
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            lc = kernel_launches()
            with torch.cuda.graph(graph, capture_error_mode="relaxed"):
                async_step()
            torch.cuda.synchronize()
            per_replay = kernel_launches() - lc
            step = graph.replay
            graph_note = "each step one CUDA graph replay"
        except Exception as ex:   # report it; the timed path is then the direct calls
            graph_note = f"capture failed ({type(ex).__name__}: {ex}); direct calls"
            step = direct

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = kernel_launches()
    times = []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream); step(); e1.record(stream); e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = kernel_launches() - l0
    if step is not direct:
        counts["c"] = sur.counts()
        launches = per_replay * args.steps   # the library kernels captured in one replay
    fb = reactor_stats(chem)
    t_sur = statistics.mean(times)
    t_sur = fdist.max_over_ranks(t_sur, dev)
    acc, rej = counts["c"]
    Ts, Ys, sts, nsts = Td.clone(), Yd.clone(), st.clone(), nst.clone()
    # ---- plain FP64 integrator on a sample of the same cells (timed) + errors
    m = n if args.plain_sample is None else min(args.plain_sample, n)
    Tp, Yp = Td0[:m].clone(), Yd0[:m].clone()
    stp = torch.empty(m, dtype=torch.int32, device=dev); nsp = torch.empty(m, dtype=torch.int32, device=dev)
    flush.zero_()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    chem.reactor_advance(Tp, pd[:m], Yp, dtd[:m], status=stp, nsteps=nsp)
    e1.record(stream); e1.synchronize()
    t_plain = e0.elapsed_time(e1) / 1e3
    plain_stats = reactor_stats(chem)
    plain = m / t_plain
    dT = (Ts[:m] - Tp).abs()
    dY = (Ys[:m] - Yp).abs().amax(dim=1)
    accm = (sts[:m] == 0) & (nsts[:m] == 0)
    # ---- end to end through pinned host buffers, and the dominant kernel alone
    # (--no-e2e skips both: the scale-up run, whose fallback alone takes minutes)
    e2e_line, roof = None, None
    if not args.no_e2e:
        e2e_line, roof = surrogate_e2e_and_roofline(args, chem, sur, dev, stream, flush, T0, p0, Y0, dt0, Td0, Yd0, pd,
                                                    dtd, st, nst, sts, nsts, n, ws, t_sur, plain_stats, t_plain)
    line = {"metric": METRIC, "value": n * ws / t_sur, "unit": "cell-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_sur * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (integrator, gate) + bf16/fp32 (network)",
            "data": "synthetic (seeded states, seeded synthetic mechanism)",
            "config": {"workload": (f"reactor-c5: surrogate+fallback, 54sp/320r, {n} cells, rtol 1e-8 atol 1e-14"
                                    if c5 else
                                    f"reactor-c4: surrogate+fallback, 31sp/160r, {n} cells, rtol 1e-8 atol 1e-14"),
                       "cells_per_gpu": n, "path": "surrogate + FP64 BDF fallback",
                       "network": (f"MLP {'-'.join(str(d) for d in sur.dims)} GELU x{sur.n_nets} (ensemble), "
                                   + ("split-bf16 fused tcgen05 forward (TMEM accumulator), fp32 accumulate"
                                      if fwd_kind == 0 else "split-bf16 mma.sync forward, fp32 accumulate")),
                       "forward_wait_errors": sur.check(),
                       "l2": "flushed (256 MiB write) between timed steps", "cuda_graph": graph_note,
                       "reactor_layout": REACTOR_LAYOUTS[layout]
                       + " (autotuned on 16,384 cells)"},
            "surrogate": {"accepted": int(acc), "rejected": int(rej), "accept_frac": acc / max(acc + rej, 1),
                          "plain_fp64_cell_steps_per_s": plain, "plain_sample_cells": m,
                          "speedup_vs_plain": (n / t_sur) / plain,
                          "max_abs_dT_K": float(dT.max()), "max_abs_dY": float(dY.max()),
                          "max_abs_dT_accepted_K": float(dT[accm].max()) if accm.any() else 0.0,
                          "max_abs_dY_accepted": float(dY[accm].max()) if accm.any() else 0.0,
                          "miss": miss_report(dT, dY, accm, sur),
                          "target": {"dT_K": 1.0, "dY": 1e-4}, "gate": sur.gate},
            "e2e": e2e_line,
            "gpu_launches": launches, "clocks": clk,
            "roofline": roof}
    if rank == 0 and not args.no_cpu_baseline:
        cb, (To, Yo, so_, no) = cpu_baseline(chem.mech, T0, p0, Y0, dt0, want_state=True)
        line["cpu_baseline"] = cb
        # the same cells' end states from the FP64 oracle: the errors the target names
        Tsn, Ysn = Ts[:no].cpu().numpy(), Ys[:no].cpu().numpy()
        acc_o = ((sts[:no] == 0) & (nsts[:no] == 0)).cpu().numpy()
        eTo = np.abs(Tsn - To)
        eYo = np.abs(Ysn - Yo).max(axis=1)
        line["surrogate"]["vs_oracle"] = {
            "cells": int(no), "oracle_failed": int((so_ != 0).sum()),
            "max_abs_dT_K": float(eTo.max()), "max_abs_dY": float(eYo.max()),
            "max_abs_dT_accepted_K": float(eTo[acc_o].max()) if acc_o.any() else 0.0,
            "max_abs_dY_accepted": float(eYo[acc_o].max()) if acc_o.any() else 0.0}
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def surrogate_e2e_and_roofline(args, chem, sur, dev, stream, flush, T0, p0, Y0, dt0, Td0, Yd0, pd, dtd, st, nst,
                               sts, nsts, n, ws, t_sur, plain_stats, t_plain):
    """The surrogate step end to end through pinned host buffers (host copies in
    the timed region), and the fallback reactor timed alone on the rejected
    cells for the roofline.  Returns (e2e, roofline)."""
    import torch
    from flint_gb300 import dist as fdist
    from flint_gb300.api import reactor_stats
    Th = torch.from_numpy(T0).pin_memory(); ph = torch.from_numpy(p0).pin_memory()
    Yh = torch.from_numpy(Y0).pin_memory(); dth = torch.from_numpy(dt0).pin_memory()
    To = torch.empty_like(Th).pin_memory(); Yo = torch.empty_like(Yh).pin_memory()
    so = torch.empty(n, dtype=torch.int32).pin_memory()
    Te, pe, Ye, dte = (torch.empty_like(x, device=dev) for x in (Th, ph, Yh, dth))
    h2d = sum(x.numel() * x.element_size() for x in (Th, ph, Yh, dth))
    d2h = sum(x.numel() * x.element_size() for x in (To, Yo, so))
    e2e = []
    e2e_warm = min(args.warmup, 1)      # the path is already warm from the device-timed loop
    for i in range(e2e_warm + args.steps):
        flush.zero_(); torch.cuda.synchronize()
        t0 = time.perf_counter()
        Te.copy_(Th, non_blocking=True); pe.copy_(ph, non_blocking=True)
        Ye.copy_(Yh, non_blocking=True); dte.copy_(dth, non_blocking=True)
        sur.advance(Te, pe, Ye, dte, status=st, nsteps=nst)
        To.copy_(Te, non_blocking=True); Yo.copy_(Ye, non_blocking=True); so.copy_(st, non_blocking=True)
        torch.cuda.synchronize()
        if i >= e2e_warm:
            e2e.append(time.perf_counter() - t0)
    t_e2e = statistics.mean(e2e)
    t_e2e = fdist.max_over_ranks(t_e2e, dev)
    # ---- the dominant kernel alone: the fallback reactor on the rejected cells
    ridx = torch.nonzero((sts != 0) | (nsts != 0)).squeeze(1)
    Tf, Yf = Td0[ridx].contiguous(), Yd0[ridx].contiguous()
    pf, dtf = pd[ridx].contiguous(), dtd[ridx].contiguous()
    stf = torch.empty(ridx.numel(), dtype=torch.int32, device=dev)
    nsf = torch.empty(ridx.numel(), dtype=torch.int32, device=dev)
    flush.zero_()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    chem.reactor_advance(Tf, pf, Yf, dtf, status=stf, nsteps=nsf)
    e1.record(stream); e1.synchronize()
    t_fb = e0.elapsed_time(e1) / 1e3
    fbk = reactor_stats(chem)
    ops = fp64_ops(fbk, chem.ns, chem.mech.name)
    peak = chem_peak_fp64()
    e2e_line = {"value": n * ws / t_e2e, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    roof = {"bound": "fp64", "kernel": "k_reactor (the fallback: rejected cells, timed alone)",
            "achieved": ops / t_fb / 1e12, "peak": peak, "unit": "TFLOP/s",
            "frac": (ops / t_fb / 1e12) / peak if peak else None,
            "traffic": (REACTOR_DRAM_BYTES_PER_CELL[chem.mech.name] * int(ridx.numel())
                        if chem.mech.name in REACTOR_DRAM_BYTES_PER_CELL else None),
            "traffic_note": "ncu DRAM bytes per cell of a k_reactor launch x cells of this launch",
            "peak_source": "DFMA probe kernel measured in this run (MEASURED_PEAKS.json has no FP64 figure)",
            "kernel_seconds": t_fb, "share_of_step": t_fb / t_sur, "fallback_cells": int(ridx.numel()),
            "events_per_launch": fbk, "ops_per_launch": ops,
            "plain_leg": {"events": plain_stats, "seconds": t_plain}}
    return e2e_line, roof


def miss_report(dT, dY, accm, sur, target_dT=1.0, target_dY=1e-4):
    """Accepted cells of this run (unseen in training and calibration) whose
    error against the FP64 integrator exceeds the target, or the calibration
    margin x target, as fractions of the accepted cells; and the calibration's
    conformal bound: with all n accepted held-out cells inside margin x target,
    an unseen accepted cell (exchangeable with them) lies beyond the largest of
    their errors with probability at most 1/(n + 1)."""
    acc = int(accm.sum())
    cal = (getattr(sur, "header", {}) or {}).get("extra", {}).get("calibration") or {}
    margin = cal.get("margin", 0.5)
    beyond = ((dT > target_dT) | (dY > target_dY)) & accm
    beyond_m = ((dT > margin * target_dT) | (dY > margin * target_dY)) & accm
    n_val_acc = int(round(cal.get("accept_frac", 0.0) * cal.get("val_cells", 0)))
    return {"accepted_cells": acc, "beyond_target": int(beyond.sum()),
            "miss_rate": int(beyond.sum()) / max(acc, 1),
            "calibration_margin": margin, "beyond_margin": int(beyond_m.sum()),
            "miss_rate_margin": int(beyond_m.sum()) / max(acc, 1),
            "calibration_accepted_cells": n_val_acc,
            "conformal_bound_margin": 1.0 / (n_val_acc + 1) if n_val_acc else None}


def run_kernel_workload(args):
    """Source-term workloads: c1-wdot (65,536 states, 2-step CH4/air: wdot, cp, h)
    and c2-wdotjac (1,048,576 states, 31 species: wdot + 32x32 Jacobian); c5-wdot /
    c5-wdotjac the same on the 54-species mechanism (1,048,576 states: the 55x55
    Jacobians of 1 M states are 25 GB)
    Metric states/s, device-timed, L2 flushed between steps."""
    import torch
    from flint_gb300 import mechgen
    from flint_gb300.api import Chemistry, kernel_launches
    dev = torch.device("cuda", 0)
    if args.workload.startswith("c1-"):
        n = args.cells or 65536
        T, p, Y = mechgen.c1_states(n)
        chem = Chemistry.from_config("c1")
    else:
        n = args.cells or 1048576
        chem = Chemistry.from_config("c5" if args.workload.startswith("c5") else "c2")
        T, p, Y = mechgen.c2_states(n, chem.mech)
    Td, pd, Yd = (torch.from_numpy(a).to(dev) for a in (T, p, Y))
    w = torch.empty_like(Yd)
    cp, h = torch.empty_like(Td), torch.empty_like(Td)
    jac = torch.empty((n, chem.ns + 1, chem.ns + 1), dtype=torch.float64, device=dev) \
        if args.workload.endswith("wdotjac") else None
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    gen = None
    tab = None
    if args.workload == "c2-general":
        # FLINT's tabulated path: the general loop on 1-K tables of the same mechanism
        from flint_gb300 import tables
        tab = tables.Tables(tables.generate(chem.mech, 300, 3000))
        Tc = np.clip(T, 300.0, 2990.0)
        W = np.array([sp.mw for sp in chem.mech.species])
        rho = p / (chem.mech.r_eos * Tc * (Y / W).sum(1))
        roi_d = torch.from_numpy(rho[:, None] * Y).to(dev)
        Tc_d = torch.from_numpy(Tc).to(dev)
    if args.generated:
        from flint_gb300.ytf_cuda import GeneratedMechanism
        gen = GeneratedMechanism(chem.mech)
    tuning = None
    if tab is None and gen is None:
        # the source-term kernels' block size, tuned on a sample of these states (untimed)
        ms = min(n, 65536)
        tuning = chem.wdot_autotune(Td[:ms], pd[:ms], Yd[:ms])

    def step():
        if tab is not None:
            tab.chemistry_source(roi_d, Tc_d, omegadot=w)
        elif gen is not None and jac is not None:
            gen.wdot_jac(Td, pd, Yd, wdot=w, jac=jac)
        elif gen is not None:
            gen.wdot(Td, pd, Yd, wdot=w, cp=cp, h=h)
        elif jac is None:
            chem.wdot(Td, pd, Yd, wdot=w, cp=cp, h=h)
        else:
            chem.wdot_jac(Td, pd, Yd, wdot=w, jac=jac)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    l0 = kernel_launches()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream); step(); e1.record(stream); e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = statistics.mean(times)
    parity = None if args.no_parity else parity_sample(chem, T, p, Y, w, jac, tab,
                                                       (roi_d, Tc_d) if tab is not None else None)
    nv = chem.ns + 1
    bytes_per_state = 8 * (2 + 2 * chem.ns) + (8 * nv * nv if jac is not None else 16)
    roof = None
    kf = KINETICS_FLOPS.get(chem.mech.name)
    if kf is not None and tab is None:
        fl = kf["jac" if jac is not None else "rhs"]
        peak = chem_peak_fp64()
        roof = {"bound": "fp64", "kernel": (f"ytf_<mech>_{'jac_' if jac is not None else ''}kernel" if gen else
                                            f"k_wdot_warp<{int(jac is not None)}>"),
                "flops_note": "the data-driven kernel's FP64 operations per state, for both kernels",
                "flops_per_state": fl, "achieved": n * fl / t / 1e12, "peak": peak, "unit": "TFLOP/s",
                "frac": (n * fl / t / 1e12) / peak if peak else None,
                "peak_source": "DFMA probe kernel measured in this run",
                "hbm_gbs_algorithmic": n * bytes_per_state / t / 1e9}
    print(json.dumps({"workload": args.workload,
                      "kernel": "generated (ytf_cuda)" if gen else ("tabulated general loop" if tab else "data-driven"),
                      "metric": "states/s", "value": n / t, "unit": "states/s",
                      "ms_per_step": t * 1e3, "states": n, "steps": args.steps, "warmup": args.warmup,
                      "gpu_launches": kernel_launches() - l0,
                      "hbm_gbs_algorithmic": n * bytes_per_state / t / 1e9,
                      "bytes_per_state": bytes_per_state, "roofline": roof, "parity": parity,
                      "tuning": tuning,
                      "cpu_baseline": None if args.no_cpu_baseline else
                      cpu_baseline_kernels(chem.mech, T, p, Y, jac is not None, tab)}))


PARITY_SAMPLE = 4096
PARITY_BAR = 1e-12


def parity_sample(chem, T, p, Y, w, jac, tab=None, table_in=None, m=PARITY_SAMPLE):
    """The last timed step's outputs against the FP64 oracle on m states spread
    evenly over the whole timed batch: max |GPU - oracle| / (sum of |terms|)
    per entry for wdot (and the Jacobian), the source-term tests' bar; for the
    tabulated general loop, relative to the cell's largest rate."""
    from oracle.oracle import Oracle, TableOracle
    n = T.shape[0]
    idx = np.unique(np.linspace(0, n - 1, min(m, n)).astype(np.int64))
    it = None
    try:
        import torch
        it = torch.from_numpy(idx).to(w.device)
    except ImportError:
        pass
    wg = w.index_select(0, it).cpu().numpy()
    res = {"states": int(idx.size), "of": int(n), "bar": PARITY_BAR, "sampled": "evenly spaced over the batch"}
    if tab is not None:
        roi_d, Tc_d = table_in
        ref = TableOracle(tab.t).general(roi_d.index_select(0, it).cpu().numpy(), Tc_d.index_select(0, it).cpu().numpy())
        sc = np.abs(ref).max(axis=1, keepdims=True)
        res["wdot_max_err"] = float((np.abs(wg - ref) / (sc + 1e-300)).max())
        res["scale"] = "the cell's largest rate"
    else:
        orc = Oracle(chem.mech)
        w_o, ws_o, _, _ = orc.wdot_batch(T[idx], p[idx], Y[idx])
        res["wdot_max_err"] = float((np.abs(wg.ravel() - w_o) / (ws_o + 1e-300)).max())
        res["scale"] = "sum of |terms| per entry"
        if jac is not None:
            _, J_o, Js_o = orc.wdot_jac_batch(T[idx], p[idx], Y[idx])
            Jg = jac.index_select(0, it).cpu().numpy().ravel()
            res["jac_max_err"] = float((np.abs(Jg - J_o) / (Js_o + 1e-300)).max())
    res["pass"] = bool(res["wdot_max_err"] < PARITY_BAR and res.get("jac_max_err", 0.0) < PARITY_BAR)
    return res


def cpu_baseline_kernels(mech, T, p, Y, with_jac, tab=None, target_s=5.0):
    """The oracle's source terms (and Jacobian) on all host cores over a bounded
    sample of the same states; states/s."""
    from oracle.oracle import Oracle, TableOracle
    n = 1024
    while True:
        t0 = time.perf_counter()
        if tab is not None:
            W = np.array([sp.mw for sp in mech.species])
            Tc = np.clip(T[:n], 300.0, 2990.0)
            rho = p[:n] / (mech.r_eos * Tc * (Y[:n] / W).sum(1))
            TableOracle(tab.t).general(rho[:, None] * Y[:n], Tc)
        elif with_jac:
            Oracle(mech).wdot_jac_batch(T[:n], p[:n], Y[:n])
        else:
            Oracle(mech).wdot_batch(T[:n], p[:n], Y[:n])
        el = time.perf_counter() - t0
        if el > 0.5 * target_s or n >= len(T):
            break
        n = min(len(T), int(n * min(8.0, max(1.5, target_s / max(el, 1e-3)))))
    from oracle.oracle import Oracle as _O
    return {"value": n / el, "unit": "states/s", "cores": _O.max_threads(), "kind": "port",
            "sample": f"{n} of the {len(T)} states (first n), FP64 oracle, {el:.2f} s"}


def chem_peak_fp64():
    """FP64 FMA throughput of this GPU [TFLOP/s], measured by the library's probe kernel."""
    import ctypes as C
    from flint_gb300 import native
    L = native.lib()
    out = C.c_double(0.0)
    if L.flint_probe_fp64_peak(C.byref(out)) != 0:
        return None
    return out.value


def run_fp64_math(args):
    """FP64-pipe cost of the CUDA library's math functions on this GPU: time
    per value of torch's elementwise kernels over a 2^27-element FP64 array
    (compute-bound: a copy of the same array takes ~1.5 slots' time), in
    FP64-pipe slots (the time of one DFMA per value at the measured DFMA
    rate).  The kernels' own exp and log are written against these figures."""
    import torch
    dev = torch.device("cuda")
    n = 1 << 27
    x = torch.rand(n, dtype=torch.float64, device=dev) * 2000.0 + 300.0
    y = x * 1e-3
    z = x * 0.5 + 1.0
    out = torch.empty_like(x)

    def timed(f, reps=5):
        f(); torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            f()
        e1.record(); e1.synchronize()
        return e0.elapsed_time(e1) / reps / 1e3

    peak = chem_peak_fp64()                    # TFLOP/s (2 per DFMA)
    slot = 2.0 / (peak * 1e12)                 # seconds per DFMA-value
    fns = {"copy": lambda: out.copy_(x), "mul": lambda: torch.mul(x, x, out=out),
           "log": lambda: torch.log(x, out=out), "log10": lambda: torch.log10(x, out=out),
           "exp": lambda: torch.exp(y, out=out), "reciprocal": lambda: torch.reciprocal(x, out=out),
           "div": lambda: torch.div(x, z, out=out), "sqrt": lambda: torch.sqrt(x, out=out)}
    res = {k: timed(f) for k, f in fns.items()}
    print(json.dumps({"workload": "fp64-math", "values": n, "dfma_peak_tflops": peak,
                      "slots_per_value": {k: v / n / slot for k, v in res.items()},
                      "ms": {k: v * 1e3 for k, v in res.items()}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=None)
    ap.add_argument("--workload", default="reactor",
                    choices=["reactor", "reactor-c5", "c1-wdot", "c1-wdotjac", "c2-wdot", "c2-wdotjac", "c5-wdot",
                             "c5-wdotjac",
                             "c2-general", "fp64-math"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="source-term workloads: skip the oracle check of the timed outputs")
    ap.add_argument("--generated", action="store_true",
                    help="source-term workloads: run the per-mechanism generated kernel (ytf_cuda)")
    ap.add_argument("--ref-seconds", type=float, default=10.0)
    ap.add_argument("--path", default="auto", choices=["auto", "surrogate", "plain"],
                    help="surrogate+fallback (headline, needs the trained checkpoint) or the plain integrator")
    ap.add_argument("--checkpoint", default=SURROGATE_CKPT)
    ap.add_argument("--no-e2e", action="store_true",
                    help="surrogate path: skip the end-to-end timing and the fallback-alone roofline run "
                         "(the 4,194,304-cell scale-up, where each fallback takes minutes)")
    ap.add_argument("--plain-sample", type=int, default=None,
                    help="surrogate path: the plain integrator re-solves (and judges) only the first N cells "
                         "(default: every cell)")
    ap.add_argument("--no-graph", action="store_true", help="surrogate path: direct calls instead of a CUDA graph")
    args = ap.parse_args()
    if args.workload == "reactor-c5":
        if args.path == "surrogate":
            args.checkpoint = args.checkpoint if args.checkpoint != SURROGATE_CKPT else SURROGATE_CKPT_C5
            run_surrogate(args)
            return
        args.cells = args.cells or CELLS
        run_ours(args)
        return
    if args.workload == "fp64-math":
        run_fp64_math(args)
        return
    if args.workload != "reactor":
        run_kernel_workload(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    path = args.path
    if path == "auto":
        path = "surrogate" if os.path.exists(args.checkpoint) else "plain"
    if path == "surrogate":
        run_surrogate(args)
    else:
        args.cells = args.cells or CELLS
        run_ours(args)


if __name__ == "__main__":
    main()
