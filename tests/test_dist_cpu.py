"""The N > 1 host logic on CPU: two gloo ranks (spawned processes) shard cells
without overlap, report the job's step time as the max over ranks and the
cells processed as the sum; the per-rank work is the oracle's source terms on
each rank's own range, and the union equals the single-process result."""
import os
import socket

import numpy as np
import pytest

from flint_gb300.dist import cell_range

torch = pytest.importorskip("torch")


def test_cell_range_partitions():
    for n in (0, 1, 7, 100, 1001):
        for world in (1, 2, 3, 8):
            got = [cell_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        cell_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from flint_gb300 import dist as fd, mechgen
    from oracle.oracle import Oracle
    mech = mechgen.load("c2")
    T, p, Y = mechgen.c2_states(101, mech, seed=5)
    a, b = fd.cell_range(len(T), rank, world)
    w, _, _, _ = Oracle(mech).wdot_batch(T[a:b], p[a:b], Y[a:b], nthreads=1)
    t_local = 1.0 + rank            # stand-in step times: the job takes the slowest
    t_job = fd.max_over_ranks(t_local)
    cells = fd.sum_over_ranks(b - a)
    fd.barrier()
    np.save(os.path.join(out_dir, f"w{rank}.npy"), w)
    np.save(os.path.join(out_dir, f"r{rank}.npy"), np.array([a, b, t_job, cells]))
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    from flint_gb300 import mechgen
    from oracle.oracle import Oracle
    mech = mechgen.load("c2")
    T, p, Y = mechgen.c2_states(101, mech, seed=5)
    w_all, _, _, _ = Oracle(mech).wdot_batch(T, p, Y, nthreads=1)
    parts = [np.load(tmp_path / f"w{r}.npy") for r in range(world)]
    np.testing.assert_array_equal(np.concatenate(parts), w_all)
    for r in range(world):
        a, b, t_job, cells = np.load(tmp_path / f"r{r}.npy")
        assert t_job == world and cells == len(T)
