"""Batched instances (GBT_Batch* C ABI) against solo runs of the CPU oracle, instance by instance.

A batch packs each instance's own topology into one table, so every instance must evolve exactly as
it does alone: the test compares each instance's nodes after every frame with a solo FP32 oracle
session driven with the same commands, in each launch shape (lockstep grid, one CTA per instance at
256 and 512 threads, thread-block clusters of 2, 4 and 8 CTAs with the positions in distributed shared
memory) and with the frames replayed from a CUDA graph.
"""
import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import batch as BT
from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.native_backend import GraspParams, PlainTissue

pytestmark = pytest.mark.gpu
STEPS = 6
GRASP = dict(W.DEFAULT_GRASP, ccd_velocity=0.0)


@pytest.fixture(scope="module")
def small_batch():
    return BT.make_c4(count=7, seed=11, steps=STEPS, size_range=((4, 9), (3, 6), (4, 9)))


def solo(workload, i, lib):
    g = workload.grids[i]
    s = PlainTissue(g, dt=1 / 60, substeps=workload.substeps, ks=1e6, grasp_params=GraspParams(**GRASP), dll_path=lib)
    try:
        mu, kappa = s.tet_stiffness()
        scale = workload.stiffness_scale()[i]
        s.set_tet_stiffness(mu * scale, kappa * scale)
        s.set_gravity(0.0, -981.0, 0.0)
        s.set_capsule(workload.capsule_paths[i][0])
        frames = []
        for k in range(STEPS):
            s.set_capsule(workload.capsule_paths[i][k + 1])
            s.step()
            frames.append(s.positions())
        return frames
    finally:
        s.close()


def batched(workload, lib, mode, threads, use_graph):
    with BT.TissueBatch(workload.grids, dt=1 / 60, substeps=workload.substeps, ks=1e6,
                        stiffness_scale=workload.stiffness_scale(), grasp_params=GraspParams(**GRASP), dll_path=lib) as b:
        b.set_launch(mode, threads)
        b.set_gravity(0.0, -981.0, 0.0)
        b.set_capsules(workload.capsules_at(0))
        frames = []
        for k in range(STEPS):
            if use_graph:
                b.step_many([workload.capsules_at(k + 1)], use_graph=True)
            else:
                b.set_capsules(workload.capsules_at(k + 1))
                b.step()
            allp = b.positions()
            frames.append([b.instance_positions(allp, i).copy() for i in range(len(workload.grids))])
        info = b.info()
    return frames, info


@pytest.mark.parametrize("mode,threads,use_graph", [(0, 256, False), (0, 256, True), (1, 256, True), (1, 512, False),
                                                    (2, 2, False), (2, 4, True), (2, 8, False)])
def test_batched_instances_match_solo_oracle(gpu_lib, oracle_libs, small_batch, mode, threads, use_graph):
    frames, info = batched(small_batch, gpu_lib, mode, threads, use_graph)
    assert info["instances"] == len(small_batch.grids) and info["mode"] == mode and info["threads"] == threads
    for i in range(len(small_batch.grids)):
        ref = solo(small_batch, i, oracle_libs[0])
        moved = float(np.abs(ref[-1] - small_batch.grids[i].positions).max())
        assert moved > 0.0
        for k in range(STEPS):
            assert np.array_equal(frames[k][i], ref[k]), (i, k, float(np.abs(frames[k][i] - ref[k]).max()))


def test_autotune_keeps_state(gpu_lib, small_batch):
    with BT.TissueBatch(small_batch.grids, dt=1 / 60, substeps=small_batch.substeps, ks=1e6,
                        stiffness_scale=small_batch.stiffness_scale(), grasp_params=GraspParams(**GRASP), dll_path=gpu_lib) as b:
        b.set_gravity(0.0, -981.0, 0.0)
        b.set_capsules(small_batch.capsules_at(0))
        before = b.positions()
        choice = b.autotune(trial_steps=2)
        assert (choice["mode"] in (0, 1) and choice["threads"] in (256, 512)) or (choice["mode"] == 2 and choice["threads"] in (2, 4, 8))
        assert len(choice["ms_per_frame"]) == 6 and all(ms > 0 or ms == -1 for ms in choice["ms_per_frame"])
        assert all(ms > 0 for ms in choice["ms_per_frame"][:3])
        assert np.array_equal(b.positions(), before)
        # the search: lockstep on both element-table forms, every per-instance shape with three packings
        trials = choice["trials"]
        assert len(trials) == 2 + 2 * 3 + 3 * 3
        assert {(t["mode"], t["threads"], t["packing"]) for t in trials if t["mode"] > 0} == \
            {(m, th, pk) for m, ths in ((1, (256, 512)), (2, (2, 4, 8))) for th in ths for pk in range(3)}
        usable = [t for t in trials if t["ms_per_frame"] > 0]
        fastest = min(usable, key=lambda t: t["ms_per_frame"])
        assert (choice["mode"], choice["threads"], choice["element_tables"]) == (fastest["mode"], fastest["threads"], fastest["element_tables"])
        assert choice["mode"] == 0 or choice["packing"] == fastest["packing"]


@pytest.mark.parametrize("mode,threads,packing", [(1, 256, 1), (1, 512, 2), (2, 4, 1), (2, 2, 2)])
def test_packings_match_lockstep(gpu_lib, small_batch, mode, threads, packing):
    """Every instance packing advances every instance exactly as the lockstep grid does."""
    runs = []
    for m, th, pk in ((0, 256, 0), (mode, threads, packing)):
        with BT.TissueBatch(small_batch.grids, dt=1 / 60, substeps=small_batch.substeps, ks=1e6,
                            stiffness_scale=small_batch.stiffness_scale(), grasp_params=GraspParams(**GRASP), dll_path=gpu_lib) as b:
            b.set_packing(pk)
            b.set_launch(m, th)
            assert b.packing() == pk
            b.set_gravity(0.0, -981.0, 0.0)
            b.set_capsules(small_batch.capsules_at(0))
            for k in range(STEPS):
                b.step_many([small_batch.capsules_at(k + 1)], use_graph=k % 2 == 0)
            runs.append(b.positions())
    assert np.array_equal(runs[0], runs[1])


def test_graph_follows_grasp_param_changes(gpu_lib, small_batch):
    """GBT_BatchSetGraspParams between graph replays: the graph is recaptured with the new contact
    parameters, so the graph path stays bit-identical to plain launches."""
    stiffer = GraspParams(**dict(GRASP, contact_compliance=1.0e-9, ccd_omega=0.6, ccd_displacement=0.02))
    runs = []
    for use_graph in (False, True):
        with BT.TissueBatch(small_batch.grids, dt=1 / 60, substeps=small_batch.substeps, ks=1e6,
                            stiffness_scale=small_batch.stiffness_scale(), grasp_params=GraspParams(**GRASP), dll_path=gpu_lib) as b:
            b.set_launch(0, 256)
            b.set_gravity(0.0, -981.0, 0.0)
            b.set_capsules(small_batch.capsules_at(0))
            frames = []
            for k in range(STEPS):
                if k == STEPS // 2:
                    b.set_grasp_params(stiffer)
                b.step_many([small_batch.capsules_at(k + 1)], use_graph=use_graph)
                frames.append(b.positions())
            runs.append(frames)
    plain, graph = runs
    for k in range(STEPS):
        assert np.array_equal(plain[k], graph[k]), (k, float(np.abs(plain[k] - graph[k]).max()))
    assert not np.array_equal(plain[-1], _run_without_change(gpu_lib, small_batch)), "the parameter change had no effect"


def _run_without_change(lib, workload):
    with BT.TissueBatch(workload.grids, dt=1 / 60, substeps=workload.substeps, ks=1e6,
                        stiffness_scale=workload.stiffness_scale(), grasp_params=GraspParams(**GRASP), dll_path=lib) as b:
        b.set_launch(0, 256)
        b.set_gravity(0.0, -981.0, 0.0)
        b.set_capsules(workload.capsules_at(0))
        for k in range(STEPS):
            b.step_many([workload.capsules_at(k + 1)], use_graph=True)
        return b.positions()


def test_c4_batch_instances_match_solo_oracle(gpu_lib, oracle_libs):
    """The C4 table itself (256 uneven instances): the autotuned shape replaying a CUDA graph, and
    four instances spread over the size range (smallest, two middle, largest) each bit-identical to a
    solo FP32 oracle session over 5 frames."""
    steps = 5
    c4 = BT.make_c4(steps=steps)
    with BT.TissueBatch(c4.grids, dt=1 / 60, substeps=c4.substeps, ks=1e6, stiffness_scale=c4.stiffness_scale(),
                        grasp_params=GraspParams(**GRASP), strain_damping_s=0.0, dll_path=gpu_lib) as b:
        b.set_gravity(0.0, -981.0, 0.0)
        b.set_capsules(c4.capsules_at(0))
        choice = b.autotune(trial_steps=2)
        frames = []
        for k in range(steps):
            b.step_many([c4.capsules_at(k + 1)], use_graph=True)
            frames.append(b.positions())
        per_instance = {}
        order = np.argsort([len(g.positions) for g in c4.grids])
        chosen = [int(order[0]), int(order[len(order) // 3]), int(order[2 * len(order) // 3]), int(order[-1])]
        for i in chosen:
            per_instance[i] = [b.instance_positions(f, i).copy() for f in frames]
    assert choice["mode"] in (0, 1, 2)
    for i in chosen:
        g = c4.grids[i]
        s = PlainTissue(g, dt=1 / 60, substeps=c4.substeps, ks=1e6, strain_damping_s=0.0, grasp_params=GraspParams(**GRASP),
                        dll_path=oracle_libs[0])
        try:
            mu, kappa = s.tet_stiffness()
            scale = c4.stiffness_scale()[i]
            s.set_tet_stiffness(mu * scale, kappa * scale)
            s.set_gravity(0.0, -981.0, 0.0)
            s.set_capsule(c4.capsule_paths[i][0])
            for k in range(steps):
                s.set_capsule(c4.capsule_paths[i][k + 1])
                s.step()
                assert np.array_equal(per_instance[i][k], s.positions()), (i, k)
        finally:
            s.close()


@pytest.mark.parametrize("mode,threads", [(0, 256), (1, 512), (2, 4)])
def test_implicit_and_explicit_element_tables_agree(gpu_lib, small_batch, mode, threads):
    """The implicit lattice codes (4 B per tet and edge, nodes from the instance strides and Kuhn
    type) and the explicit element tables give the same frames bit for bit, graph replay included."""
    runs = []
    for implicit in (True, False):
        with BT.TissueBatch(small_batch.grids, dt=1 / 60, substeps=small_batch.substeps, ks=1e6,
                            stiffness_scale=small_batch.stiffness_scale(), grasp_params=GraspParams(**GRASP), dll_path=gpu_lib) as b:
            assert b.element_tables() == "implicit"      # the default for a qualifying batch
            b.set_element_tables(implicit)
            assert b.element_tables() == ("implicit" if implicit else "explicit")
            b.set_launch(mode, threads)
            b.set_gravity(0.0, -981.0, 0.0)
            b.set_capsules(small_batch.capsules_at(0))
            frames = []
            for k in range(STEPS):
                b.step_many([small_batch.capsules_at(k + 1)], use_graph=k % 2 == 0)
                frames.append(b.positions())
            runs.append(frames)
    for k in range(STEPS):
        assert np.array_equal(runs[0][k], runs[1][k]), k


def test_per_tet_stiffness_keeps_explicit_tables(gpu_lib):
    """A batch with per-tet stiffness that varies inside a Kuhn type does not qualify for the codes."""
    wl = BT.make_c4(count=3, seed=2, steps=2, size_range=((3, 5), (2, 4), (3, 5)))
    stiff = []
    for g in wl.grids:
        with PlainTissue(g, dt=1 / 60, substeps=4, ks=1e6, dll_path=gpu_lib) as s:
            mu, kappa = s.tet_stiffness()
        mu = mu * np.linspace(0.5, 1.5, len(mu), dtype=np.float32)
        stiff.append((mu, kappa))
    with BT.TissueBatch(wl.grids, dt=1 / 60, substeps=4, ks=1e6, tet_stiffness=stiff, dll_path=gpu_lib) as b:
        assert b.element_tables() == "explicit"
        with pytest.raises(RuntimeError):
            b.set_element_tables(True)
