"""Instances shard over GPUs with no exchange (the C4 split): every instance on exactly one rank,
loads balanced by cost, and the ranks' timings combine into one rate (slowest rank).  The
multi-rank path runs as two `gloo` processes on the CPU."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from genesis_tissue_simulation_gb300 import batch as BT


def test_shards_cover_every_instance_once():
    w = BT.make_c4(count=24, steps=2)
    costs = BT.instance_costs(w)
    for world in (1, 2, 3, 8):
        shards = BT.shard_instances(costs, world)
        assert len(shards) == world
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(24))
        assert all(s == sorted(s) for s in shards)
        loads = [sum(costs[i] for i in s) for s in shards]
        # longest processing time: the heaviest rank exceeds the mean by at most one instance
        assert max(loads) <= sum(costs) / world + max(costs)
    assert BT.shard_instances(costs, 1) == [list(range(24))]
    with pytest.raises(ValueError):
        BT.shard_instances(costs, 0)


def test_subset_keeps_instances():
    w = BT.make_c4(count=6, steps=2)
    sub = w.subset([4, 1])
    assert [g.positions.shape for g in sub.grids] == [w.grids[4].positions.shape, w.grids[1].positions.shape]
    assert np.array_equal(sub.compliance, w.compliance[[4, 1]])
    assert sub.capsules_at(1) == [w.capsule_paths[4][1], w.capsule_paths[1][1]]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"], os.environ["MASTER_PORT"] = "127.0.0.1", str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = BT.make_c4(count=10, steps=2)
        shards = BT.shard_instances(BT.instance_costs(w), world)
        mine = w.subset(shards[rank])
        # each rank "times" its share (seconds proportional to its cost); the slowest counts
        seconds = torch.tensor([1e-6 * sum(BT.instance_costs(mine))], dtype=torch.float64)
        count = torch.tensor([len(mine.grids)], dtype=torch.float64)
        dist.all_reduce(seconds, op=dist.ReduceOp.MAX)
        dist.all_reduce(count)
        out[rank] = (float(seconds), float(count), shards[rank])
    finally:
        dist.destroy_process_group()


def test_two_ranks_split_and_combine():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    (s0, c0, a), (s1, c1, b) = out[0], out[1]
    assert s0 == s1 and c0 == c1 == 10
    assert sorted(a + b) == list(range(10)) and not set(a) & set(b)
    w = BT.make_c4(count=10, steps=2)
    costs = BT.instance_costs(w)
    assert s0 == pytest.approx(1e-6 * max(sum(costs[i] for i in a), sum(costs[i] for i in b)))


def test_tool_array_matches_ctypes_records():
    """The vectorised XpbdToolState fill gives the bytes of the per-capsule ctypes records."""
    import ctypes as ct
    from genesis_tissue_simulation_gb300.native_backend import Grasper
    w = BT.make_c4(count=12, steps=3)
    for step in (0, 2, 9):
        caps = w.capsules_at(step)
        records = (Grasper * len(caps))(*(BT.capsule_tool(c) for c in caps))
        arr = BT.tool_array(w.capsule_array_at(step))
        assert arr.shape == (12, 23) and ct.sizeof(Grasper) == 92
        assert bytes(records) == arr.tobytes()
