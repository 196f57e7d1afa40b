"""Instances shard over GPUs with no exchange (the C4 split): every instance on exactly one rank,
loads balanced by cost, each rank steps only its own instances, rank 0 gathers the positions (the
only data exchange), and the ranks' timings combine into one rate (slowest rank).  The multi-rank
path runs as two `gloo` processes on the CPU, each stepping its instances through the FP32 oracle."""
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


def _solo_frames(w, i, lib, steps, threads=None):
    """Instance i of a batch workload stepped alone through the FP32 oracle (the CPU stand-in for one
    GPU's share: each instance evolves exactly as it does alone, which the GPU batch tests assert)."""
    from genesis_tissue_simulation_gb300.native_backend import GraspParams, PlainTissue
    from genesis_tissue_simulation_gb300 import workloads as W
    s = PlainTissue(w.grids[i], dt=1 / 60, substeps=w.substeps, ks=1e6, strain_damping_s=w.strain_damping_s,
                    grasp_params=GraspParams(**dict(W.DEFAULT_GRASP, ccd_velocity=0.0)), dll_path=lib)
    try:
        if threads:
            assert s.dll.ORC_SetThreads(threads) == 0
        mu, kappa = s.tet_stiffness()
        scale = w.stiffness_scale()[i]
        s.set_tet_stiffness(mu * scale, kappa * scale)
        s.set_gravity(0.0, -981.0, 0.0)
        s.set_capsule(w.capsule_paths[i][0])
        for k in range(steps):
            s.set_capsule(w.capsule_paths[i][k + 1])
            s.step()
        return s.positions()
    finally:
        s.close()


SHARD_STEPS = 3


def _shard_workload():
    return BT.make_c4(count=8, seed=5, steps=SHARD_STEPS, size_range=((3, 6), (2, 4), (3, 6)))


def _rank(rank, world, port, lib, out):
    os.environ["MASTER_ADDR"], os.environ["MASTER_PORT"] = "127.0.0.1", str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = _shard_workload()
        shards = BT.shard_instances(BT.instance_costs(w), world)
        # each rank steps its own instances only, with no exchange during the frames
        mine = [_solo_frames(w, i, lib, SHARD_STEPS, threads=1) for i in shards[rank]]
        gathered = BT.gather_instance_positions(shards, mine, rank, world)
        seconds = torch.tensor([1e-6 * sum(BT.instance_costs(w.subset(shards[rank])))], dtype=torch.float64)
        count = torch.tensor([len(shards[rank])], dtype=torch.float64)
        dist.all_reduce(seconds, op=dist.ReduceOp.MAX)
        dist.all_reduce(count)
        out[rank] = (float(seconds), float(count), shards[rank], None if gathered is None else [g.tolist() for g in gathered])
    finally:
        dist.destroy_process_group()


def test_two_ranks_step_shards_and_gather(oracle_libs):
    """Two gloo ranks each step their cost-balanced shard of a batch; rank 0 gathers every
    instance's positions, which equal an unsharded run bit for bit."""
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_rank, args=(2, port, str(oracle_libs[0]), out), nprocs=2, join=True, start_method="spawn")
    (s0, c0, a, gathered), (s1, c1, b, none) = out[0], out[1]
    w = _shard_workload()
    assert s0 == s1 and c0 == c1 == len(w.grids)
    assert sorted(a + b) == list(range(len(w.grids))) and not set(a) & set(b) and a and b
    assert none is None and len(gathered) == len(w.grids)
    for i in range(len(w.grids)):
        alone = _solo_frames(w, i, oracle_libs[0], SHARD_STEPS)
        assert np.array_equal(np.asarray(gathered[i], dtype=np.float32), alone), i
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
