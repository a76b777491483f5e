"""Sharding across ranks, run as two gloo processes on the CPU with the CPU
oracle standing in for the device integration (which needs a GPU).  By
pixels: each rank integrates its contiguous pixel block and the blocks are
gathered; the result equals the single-process integration bit for bit.  By
particles (bench.py's ranks): each rank integrates its own batches onto the
whole screen with no exchange, and the summed traces equal the single-process
integration to rounding."""
import os
import socket

import numpy as np
import pytest

from teufel_gb300 import sharding


def test_shards_partition_the_pixels():
    for n in (0, 1, 7, 441, 40000):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = sharding.shard(n, r, world)
                assert 0 <= lo <= hi <= n
                seen.extend(range(lo, hi))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        sharding.shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, result_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import lw
    from teufel_gb300 import harness as H
    w = H.config1()
    sel = np.arange(0, w.n_pix, 3)
    pos, t0 = w.pix_pos[sel], w.pix_t0[sel]
    lo, hi = sharding.shard(len(sel), rank, world)
    local, rc = lw.integrate_screen(w.traj, pos[lo:hi], t0[lo:hi], w.dt, w.nots, nthreads=1)
    assert rc == 0
    full = sharding.gather_traces(local, len(sel), rank, world, dist)
    if rank == 0:
        np.save(result_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_one(tmp_path):
    import multiprocessing as mp
    from oracle import lw
    from teufel_gb300 import harness as H
    world, port = 2, _free_port()
    path = str(tmp_path / "gathered.npy")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, path)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    gathered = np.load(path)
    w = H.config1()
    sel = np.arange(0, w.n_pix, 3)
    single, rc = lw.integrate_screen(w.traj, w.pix_pos[sel], w.pix_t0[sel], w.dt, w.nots)
    assert rc == 0
    assert np.array_equal(gathered, single)


def test_rank_batches_are_disjoint():
    """Ranks sharing the 1e5-particle bunch by batches (as bench.py's ranks
    do) get disjoint particles while the batches fit in the bunch."""
    n_particles, batch, n_batches = 100000, 1024, 8
    for world in (1, 2, 4, 8):
        seen = set()
        for r in range(world):
            for first in sharding.rank_batches(r, world, n_batches, batch, n_particles):
                idx = set(range(first, first + batch))
                assert not idx & seen
                seen |= idx
        assert len(seen) == world * n_batches * batch
    with pytest.raises(ValueError):
        sharding.rank_batches(2, 2, 1, 1, 10)


def _batch_rank_main(rank, world, port, result_path):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import lw
    from teufel_gb300 import harness as H
    w = H.config2(count=4)
    sel = np.arange(0, w.n_pix, 97)
    parts = [f for f in sharding.rank_batches(rank, world, 1, 2, 4)]
    local = np.zeros((len(sel), w.nots, 6))
    for first in parts:
        sub = w.traj.subset(list(range(first, first + 2)))
        tr, rc = lw.integrate_screen(sub, w.pix_pos[sel], w.pix_t0[sel], w.dt, w.nots,
                                     nthreads=1)
        assert rc == 0
        local += tr
    t = torch.from_numpy(local)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(result_path, t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_with_own_batches_add_up_to_the_bunch(tmp_path):
    """Two ranks integrate their own particle batches onto the whole screen
    with no exchange; summing their traces (the reference's MPI_Reduce)
    gives the single-process integration of all particles, to rounding."""
    import multiprocessing as mp
    from oracle import lw
    from teufel_gb300 import harness as H
    world, port = 2, _free_port()
    path = str(tmp_path / "summed.npy")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_batch_rank_main, args=(r, world, port, path))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    summed = np.load(path)
    w = H.config2(count=4)
    sel = np.arange(0, w.n_pix, 97)
    single, rc = lw.integrate_screen(w.traj, w.pix_pos[sel], w.pix_t0[sel], w.dt, w.nots)
    assert rc == 0 and np.abs(single).max() > 0
    assert np.abs(summed - single).max() <= 1e-12 * np.abs(single).max()
