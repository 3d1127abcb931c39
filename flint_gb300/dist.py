"""Multi-GPU host logic: one process per GPU, cells sharded, no data exchange.

Cells are independent in every procedure of this path (source terms, Jacobian,
reactor advance, surrogate inference), so N GPUs split a batch into N
contiguous ranges and never communicate on the data path; the only collective
is the max of the per-rank step times (the job is as slow as its slowest rank)
and the sum of per-rank counts for reporting.  The process group is whatever
torch.distributed was initialised with (NCCL on GPUs, gloo in the CPU tests).
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
