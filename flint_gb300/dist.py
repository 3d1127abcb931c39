"""Multi-GPU host logic: one process per GPU, cells sharded, no data exchange.

Cells are independent in every procedure of this path (source terms, Jacobian,
reactor advance, surrogate inference), so N GPUs split a batch into N
contiguous ranges and do not communicate inside an advance; the collectives
are the max of the per-rank step times (the job is as slow as its slowest rank)
and the sum of per-rank counts for reporting.  Between advances a caller may
rebalance: rebalance_plan cuts the global cell order by the last advance's
per-cell step counts and redistribute moves the cells' state to their new
ranks.  The process group is whatever torch.distributed was initialised with
(NCCL on GPUs, gloo in the CPU tests).
"""
from __future__ import annotations

import os


def env():
    """(world_size, rank, local_rank) from the torchrun environment (1, 0, 0 without it)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def cell_range(n, rank, world):
    """Contiguous, balanced [start, stop) of n cells for `rank` of `world`
    (the first n % world ranks take one cell more)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def _initialized():
    import torch.distributed as dist
    return dist.is_available() and dist.is_initialized()


def max_over_ranks(x, device=None):
    """Max of a float over all ranks (the step time of the whole job)."""
    if not _initialized():
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, device=None):
    """Sum of a number over all ranks (cells processed, accepted counts ...)."""
    if not _initialized():
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier():
    if _initialized():
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------ rebalancing
# The reactor's cost per cell is very uneven (an igniting cell takes hundreds
# of BDF steps, a cell at equilibrium a handful), so equal cell counts give
# unequal work per rank.  The step counts that flint_reactor_advance returns
# per cell are the cost history: between two advances the ranks gather them,
# cut the global cell order into contiguous ranges of near-equal cost, and move
# the cells' state to their new ranks.  This is the path's one data exchange,
# and it runs only when the caller asks for it.
def weighted_ranges(cost, world):
    """Contiguous [start, stop) ranges, one per rank, of len(cost) cells whose
    cost sums are as even as a contiguous cut allows: boundary k is placed at
    the prefix sum nearest to k/world of the total.  Deterministic, so every
    rank computes the same plan; with zero total cost the cells split evenly."""
    if world < 1:
        raise ValueError("world must be >= 1")
    import numpy as np
    cost = np.asarray(cost, dtype=np.float64)
    if np.any(cost < 0.0) or np.any(np.isnan(cost)):
        raise ValueError("costs must be non-negative")
    c = np.cumsum(cost)
    n = int(c.size)
    if n == 0 or not c[-1] > 0.0:
        return [cell_range(n, r, world) for r in range(world)]
    tot = float(c[-1])
    cuts = [0]
    for k in range(1, world):
        t = tot * k / world
        i = int(np.searchsorted(c, t, side="left"))   # c[i] >= t: cells 0..i reach the target
        b = i + 1 if i == 0 or abs(c[i] - t) <= abs(c[i - 1] - t) else i
        cuts.append(min(max(b, cuts[-1]), n))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def _gather_lengths_and_costs(cost_local, device=None):
    import numpy as np
    import torch
    import torch.distributed as dist
    world = dist.get_world_size()
    cost_local = np.asarray(cost_local, dtype=np.float64)
    n = torch.tensor([cost_local.size], dtype=torch.int64, device=device)
    ns = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(ns, n)
    lens = [int(x.item()) for x in ns]
    m = max(lens + [1])
    buf = torch.zeros(m, dtype=torch.float64, device=device)
    buf[:cost_local.size] = torch.from_numpy(cost_local).to(buf.device)
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    cost = np.concatenate([p[:l].cpu().numpy() for p, l in zip(parts, lens)])
    return lens, cost


def rebalance_plan(cost_local, device=None):
    """(old_ranges, new_ranges) in the global cell order (rank 0's cells first):
    every rank passes the costs of the cells it holds (e.g. the last advance's
    steps per cell + 1) and gets the same plan.  Without an initialised process
    group the plan is the identity on this process's cells."""
    if not _initialized():
        n = len(cost_local)
        return [(0, n)], [(0, n)]
    import torch.distributed as dist
    lens, cost = _gather_lengths_and_costs(cost_local, device)
    old, start = [], 0
    for l in lens:
        old.append((start, start + l))
        start += l
    return old, weighted_ranges(cost, dist.get_world_size())


def redistribute(x, old_ranges, new_ranges):
    """Move this rank's cells (leading dimension of the tensor x, its range in
    old_ranges) to the ranks new_ranges assigns them to; returns this rank's
    cells under the new plan.  Point-to-point sends of the overlapping slices
    (each pair of ranks exchanges at most one slice each way); the local
    overlap is copied.  Works on CPU tensors with gloo and on device tensors
    with NCCL."""
    import torch
    if not _initialized():
        return x
    import torch.distributed as dist
    rank = dist.get_rank()
    (a0, a1), (b0, b1) = old_ranges[rank], new_ranges[rank]
    if x.shape[0] != a1 - a0:
        raise ValueError("x does not hold this rank's old range")
    out = torch.empty((b1 - b0,) + tuple(x.shape[1:]), dtype=x.dtype, device=x.device)
    reqs = []
    for q, ((qa0, qa1), (qb0, qb1)) in enumerate(zip(old_ranges, new_ranges)):
        s0, s1 = max(a0, qb0), min(a1, qb1)          # my old cells that q now owns
        r0, r1 = max(qa0, b0), min(qa1, b1)          # q's old cells that I now own
        if q == rank:
            if s1 > s0:
                out[s0 - b0:s1 - b0] = x[s0 - a0:s1 - a0]
            continue
        if s1 > s0:
            reqs.append(dist.isend(x[s0 - a0:s1 - a0].contiguous(), dst=q))
        if r1 > r0:
            buf = torch.empty((r1 - r0,) + tuple(x.shape[1:]), dtype=x.dtype, device=x.device)
            reqs.append((dist.irecv(buf, src=q), buf, r0 - b0))
    for rq in reqs:
        if isinstance(rq, tuple):
            rq[0].wait()
            out[rq[2]:rq[2] + rq[1].shape[0]] = rq[1]
        else:
            rq.wait()
    return out
