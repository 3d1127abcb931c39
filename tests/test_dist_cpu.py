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


def test_weighted_ranges_balance():
    """Contiguous cuts at the prefix sums nearest k/world of the total: every
    range's cost is within one cell's cost of the even share."""
    from flint_gb300.dist import weighted_ranges
    rng = np.random.default_rng(3)
    for n in (1, 5, 100, 1000):
        for world in (1, 2, 3, 7):
            # step counts: most cells cheap, a few igniting cells expensive
            cost = rng.integers(3, 12, n).astype(float)
            cost[rng.random(n) < 0.05] = rng.integers(200, 600)
            got = weighted_ranges(cost, world)
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] and a[0] <= a[1] for a, b in zip(got, got[1:]))
            share = cost.sum() / world
            for a, b in got:
                assert cost[a:b].sum() <= share + cost.max() + 1e-9
    assert weighted_ranges([0.0, 0.0, 0.0, 0.0], 2) == [(0, 2), (2, 4)]
    assert weighted_ranges([], 3) == [(0, 0)] * 3
    with pytest.raises(ValueError):
        weighted_ranges([1.0, -1.0], 2)


def _rebalance_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from flint_gb300 import dist as fd
    lens = [50, 10, 40]                      # uneven holdings before the rebalance
    start = sum(lens[:rank])
    rng = np.random.default_rng(11)
    cost = rng.integers(3, 12, 100).astype(float)
    cost[20:30] = 400.0                      # rank 0 holds the expensive cells
    T = torch.arange(100, dtype=torch.float64)[start:start + lens[rank]]
    Y = torch.arange(300, dtype=torch.float64).reshape(100, 3)[start:start + lens[rank]]
    old, new = fd.rebalance_plan(cost[start:start + lens[rank]])
    T2 = fd.redistribute(T, old, new)
    Y2 = fd.redistribute(Y, old, new)
    np.save(os.path.join(out_dir, f"plan{rank}.npy"), np.array([old, new]))
    np.save(os.path.join(out_dir, f"T{rank}.npy"), T2.numpy())
    np.save(os.path.join(out_dir, f"Y{rank}.npy"), Y2.numpy())
    dist.destroy_process_group()


def test_rebalance_three_gloo_ranks(tmp_path):
    """Three ranks with uneven cells and uneven step counts: every rank computes
    the same plan, the cost per rank evens out, and the moved state is the
    global state cut by the new ranges."""
    import torch.multiprocessing as mp
    from flint_gb300.dist import weighted_ranges
    world = 3
    mp.start_processes(_rebalance_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn")
    plans = [np.load(tmp_path / f"plan{r}.npy") for r in range(world)]
    assert all(np.array_equal(p, plans[0]) for p in plans)
    old, new = plans[0]
    assert [tuple(x) for x in old] == [(0, 50), (50, 60), (60, 100)]
    rng = np.random.default_rng(11)
    cost = rng.integers(3, 12, 100).astype(float)
    cost[20:30] = 400.0
    assert [tuple(x) for x in new] == weighted_ranges(cost, world)
    before = max(cost[a:b].sum() for a, b in old)
    after = max(cost[a:b].sum() for a, b in new)
    assert after < 0.75 * before
    Tg = np.arange(100, dtype=np.float64)
    Yg = np.arange(300, dtype=np.float64).reshape(100, 3)
    for r, (a, b) in enumerate(new):
        np.testing.assert_array_equal(np.load(tmp_path / f"T{r}.npy"), Tg[a:b])
        np.testing.assert_array_equal(np.load(tmp_path / f"Y{r}.npy"), Yg[a:b])


def _rebalance_empty_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from flint_gb300 import dist as fd
    lens = [0, 30]                           # rank 0 starts with no cells
    start = sum(lens[:rank])
    cost = np.ones(30)
    cost[0] = 1000.0                         # one cell outweighs the rest together
    x = torch.arange(60, dtype=torch.float64).reshape(30, 2)[start:start + lens[rank]]
    old, new = fd.rebalance_plan(cost[start:start + lens[rank]])
    y = fd.redistribute(x, old, new)
    np.save(os.path.join(out_dir, f"plan{rank}.npy"), np.array([old, new]))
    np.save(os.path.join(out_dir, f"x{rank}.npy"), y.numpy())
    dist.destroy_process_group()


def test_rebalance_with_an_empty_rank(tmp_path):
    """A rank that holds no cells takes part in the plan and the exchange; the
    one expensive cell ends up alone on a rank."""
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rebalance_empty_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn")
    old, new = np.load(tmp_path / "plan0.npy")
    assert np.array_equal(old, np.load(tmp_path / "plan1.npy")[0])
    assert [tuple(r) for r in old] == [(0, 0), (0, 30)] and [tuple(r) for r in new] == [(0, 1), (1, 30)]
    xg = np.arange(60, dtype=np.float64).reshape(30, 2)
    for r, (a, b) in enumerate(new):
        np.testing.assert_array_equal(np.load(tmp_path / f"x{r}.npy"), xg[a:b])
