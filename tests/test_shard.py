"""Multi-GPU sharding logic on the CPU: the lane partition, and a
world-size-2 gloo run in which each rank integrates its range of Kepler
orbits (with the oracle, on the host) and rank 0 gathers a result identical
to the unsharded run."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from hyk import shard


def test_partition_even_and_weighted():
    assert shard.partition(10, 3) == [(0, 3), (3, 6), (6, 10)]
    assert shard.partition(0, 2) == [(0, 0), (0, 0)]
    w = np.array([10.0] + [1.0] * 10)
    parts = shard.partition(11, 2, w)
    assert parts[0][0] == 0 and parts[-1][1] == 11 and parts[0][1] == parts[1][0]
    assert parts[0] == (0, 1)  # the heavy lane alone balances the rest
    rng = np.random.default_rng(0)
    w = rng.exponential(size=1000)
    parts = shard.partition(1000, 4, w)
    sums = [w[a:b].sum() for a, b in parts]
    assert max(sums) - min(sums) <= 2 * w.max()
    with pytest.raises(ValueError):
        shard.partition(5, 0)
    with pytest.raises(ValueError):
        shard.partition(3, 2, [1.0, -1.0, 1.0])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import pyoracle
        from hyk import workloads as W

        st = W.kepler_ics(48, seed=9)
        weights = np.linspace(1.0, 3.0, 48)
        lo, hi = shard.local_range(48, weights)
        o = pyoracle.Oracle(W.kepler_sys(), st[:, lo:hi], order=19, mode=1)
        o.propagate_until(3.0)
        full = shard.gather_lanes(o.state, 48, weights)
        if rank == 0:
            np.save(out_path, full)
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_gather_equals_unsharded(tmp_path, oracle):
    from hyk import workloads as W

    out = str(tmp_path / "full.npy")
    mp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    st = W.kepler_ics(48, seed=9)
    o = oracle.Oracle(W.kepler_sys(), st, order=19, mode=1)
    o.propagate_until(3.0)
    assert np.array_equal(got, o.state)
