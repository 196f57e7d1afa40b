"""CUDA path against the CPU oracle, through the LCS_* C ABI on both sides.

The CUDA kernels evaluate every projection in the oracle's operation order without multiply-add
contraction, so the FP32 trajectories agree bit for bit; the parity tolerance (1e-4 of the
bounding-box diagonal after 100 steps) is asserted as well, and the FP64 oracle error is reported.
"""
import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.native_backend import XPBD_ERR_BAD_DT, LCS_ERR_DEVICE_TIMEOUT, severed_edges

pytestmark = pytest.mark.gpu

SMALL = (4.78, 2.38, 3.98)     # 24 x 12 x 20 cells: the C2/C3 scenarios at a size the oracle runs in seconds


def trajectory(workload, lib, steps, every, launch_mode=None, topology=False):
    session = workload.open(lib)
    try:
        if launch_mode is not None:
            session.check("LCS_SetLaunchMode", launch_mode) if "LCS_SetLaunchMode" in session.functions else None
        frames = []

        def observe(k, s):
            if (k + 1) % every == 0:
                rec = {"pos": s.positions(), "vel": s.velocities()}
                if topology:
                    rec.update(nbr=s.neighbors(), rev=s.topology_revision(), mask=s.voxel_cut_mask(),
                               frac=s.cut_edge_fractions(), bends=s.bend_alive(), dbg=s.cut_debug()[15:17].copy())
                frames.append(rec)
        workload.run(session, steps=steps, observe=observe)
        return frames
    finally:
        session.close()


def _bind_launch_mode(lib):
    import ctypes
    from genesis_tissue_simulation_gb300 import native_backend as nb
    dll = ctypes.CDLL(str(lib))
    return dll


def test_c1_plain_step_matches_oracle(gpu_lib, oracle_libs):
    w = W.make("c1")
    gpu = trajectory(w, gpu_lib, 100, 10)
    cpu = trajectory(w, oracle_libs[0], 100, 10)
    f64 = trajectory(w, oracle_libs[1], 100, 100)
    active = w.grid.active != 0
    tol = 1e-4 * W.bbox_diagonal(w.grid)
    for k, (a, b) in enumerate(zip(gpu, cpu)):
        err = float(np.abs(a["pos"] - b["pos"])[active].max())
        assert err <= tol, f"step {10 * (k + 1)}: |gpu - oracle| = {err} > {tol}"
        assert np.array_equal(a["pos"], b["pos"]), f"step {10 * (k + 1)}: not bit-identical (max {err})"
    fp64_err = float(np.abs(gpu[-1]["pos"] - f64[-1]["pos"])[active].max())
    print(f"C1 100 steps: |gpu - oracle fp32| = 0, |gpu - oracle fp64| = {fp64_err:.3e} cm "
          f"({fp64_err / W.bbox_diagonal(w.grid):.3e} of the diagonal)")
    assert fp64_err <= tol, f"C1 100 steps: |gpu - FP64 oracle| = {fp64_err} > {tol}"


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_launch_modes_agree(gpu_lib, oracle_libs, mode):
    import ctypes
    w = W.make("c1", steps=20)
    dll = ctypes.CDLL(str(gpu_lib))
    dll.LCS_SetLaunchMode(mode)
    try:
        gpu = trajectory(w, gpu_lib, 20, 20)
    finally:
        dll.LCS_SetLaunchMode(0)
    cpu = trajectory(w, oracle_libs[0], 20, 20)
    assert np.array_equal(gpu[-1]["pos"], cpu[-1]["pos"])


def test_c2_capsule_small_matches_oracle(gpu_lib, oracle_libs):
    w = W.make("c2", steps=40, scale=SMALL)
    gpu = trajectory(w, gpu_lib, 40, 10)
    cpu = trajectory(w, oracle_libs[0], 40, 10)
    for a, b in zip(gpu, cpu):
        assert np.array_equal(a["pos"], b["pos"]), float(np.abs(a["pos"] - b["pos"]).max())
        assert np.array_equal(a["vel"], b["vel"]), float(np.abs(a["vel"] - b["vel"]).max())


def test_c3_cut_small_topology_bit_exact(gpu_lib, oracle_libs):
    w = W.make("c3", steps=40, scale=SMALL)
    gpu = trajectory(w, gpu_lib, 40, 10, topology=True)
    cpu = trajectory(w, oracle_libs[0], 40, 10, topology=True)
    assert cpu[-1]["rev"] > 0, "the blade never crossed the tissue"
    for a, b in zip(gpu, cpu):
        assert a["rev"] == b["rev"]
        # the revision counts links severed, each once (V/cut.cu:719-746)
        assert a["rev"] == severed_edges(w.grid.neighbors, a["nbr"])
        for key in ("nbr", "mask", "frac", "bends", "dbg", "pos", "vel"):
            assert np.array_equal(a[key], b[key]), key


def test_c2_full_size_runs_deterministically(gpu_lib):
    w = W.make("c2", steps=10)
    runs = [trajectory(w, gpu_lib, 10, 10)[-1]["pos"] for _ in range(2)]
    assert np.isfinite(runs[0]).all()
    assert np.array_equal(runs[0], runs[1])


def test_bad_dt_and_barrier_timeout_status(gpu_lib):
    import ctypes
    w = W.make("c1", steps=2)
    session = w.open(gpu_lib)
    try:
        assert session.functions["LCS_Step"](0.0) == XPBD_ERR_BAD_DT
        dll = session.dll
        dll.LCS_SetLaunchMode(1)
        dll.LCS_SetBarrierTest.argtypes = (ctypes.c_int, ctypes.c_float)
        assert dll.LCS_SetBarrierTest(1, ctypes.c_float(0.05)) == 0
        assert session.functions["LCS_Step"](1 / 60) == LCS_ERR_DEVICE_TIMEOUT
        assert dll.LCS_SetBarrierTest(0, ctypes.c_float(2.0)) == 0
        assert session.functions["LCS_Step"](1 / 60) == 0    # the context is still usable
        assert np.isfinite(session.positions()).all()
    finally:
        session.dll.LCS_SetLaunchMode(0)
        session.dll.LCS_SetBarrierTest(0, ctypes.c_float(2.0))
        session.close()


@pytest.mark.parametrize("mode", [3, 0])
def test_c2_small_cluster_and_automatic_shapes(gpu_lib, oracle_libs, mode):
    """The 24 x 12 x 20 capsule block on one thread-block cluster (positions in distributed shared
    memory), and in automatic mode, which times one CTA, the whole GPU and the cluster on its 2nd to
    4th frames: bit-identical to the oracle either way."""
    import ctypes
    w = W.make("c2", steps=12, scale=SMALL)
    dll = ctypes.CDLL(str(gpu_lib))
    dll.LCS_SetLaunchMode(mode)
    try:
        gpu = trajectory(w, gpu_lib, 12, 4)
    finally:
        dll.LCS_SetLaunchMode(0)
    cpu = trajectory(w, oracle_libs[0], 12, 4)
    for a, b in zip(gpu, cpu):
        assert np.array_equal(a["pos"], b["pos"])
        assert np.array_equal(a["vel"], b["vel"])



def test_c2_full_size_matches_oracle(gpu_lib, oracle_libs):
    """The C2 workload at its own size (64 x 32 x 48 cells, 589,824 tets, 20 substeps): bit-identical
    positions and velocities to the FP32 oracle after 10 and 20 frames."""
    w = W.make("c2", steps=20)
    gpu = trajectory(w, gpu_lib, 20, 10)
    cpu = trajectory(w, oracle_libs[0], 20, 10)
    for a, b in zip(gpu, cpu):
        assert np.array_equal(a["pos"], b["pos"]), float(np.abs(a["pos"] - b["pos"]).max())
        assert np.array_equal(a["vel"], b["vel"]), float(np.abs(a["vel"] - b["vel"]).max())


def test_c3_full_size_topology_bit_exact(gpu_lib, oracle_libs):
    """The C3 blade workload at its own size over 60 frames: neighbour table, topology revision,
    voxel cut mask, edge fractions, bend liveness and positions identical to the FP32 oracle."""
    w = W.make("c3", steps=60)
    gpu = trajectory(w, gpu_lib, 60, 20, topology=True)
    cpu = trajectory(w, oracle_libs[0], 60, 20, topology=True)
    assert cpu[-1]["rev"] > 0, "the blade never crossed the tissue"
    for a, b in zip(gpu, cpu):
        assert a["rev"] == b["rev"] == severed_edges(w.grid.neighbors, a["nbr"])
        for key in ("nbr", "mask", "frac", "bends", "dbg", "pos", "vel"):
            assert np.array_equal(a[key], b[key]), key


def test_frame_barrier_count_and_floor(gpu_lib):
    """The whole-GPU frame reports the grid barriers it ran (one per phase: at least the edge and tet
    colours of every substep) and the barrier floor is measured on the same grid; a frame in another
    launch shape reports none."""
    import ctypes
    w = W.make("c1", steps=2)
    dll = ctypes.CDLL(str(gpu_lib))
    try:
        dll.LCS_SetLaunchMode(1)
        with w.open(gpu_lib) as s:
            assert s.frame_barriers() is None      # no frame yet
            s.step()
            colours = s.functions["LCS_EdgeColorCount"]() + s.functions["LCS_TetColorCount"]()
            substeps = int(w.params["substeps"])
            barriers = s.frame_barriers()
            assert substeps * colours <= barriers <= substeps * (colours + 6) + 4, (barriers, substeps, colours)
            us = s.grid_barrier_floor(2000)
            assert 0.0 < us < 50.0, us
        dll.LCS_SetLaunchMode(2)
        with w.open(gpu_lib) as s:
            s.step()
            assert s.frame_barriers() is None
    finally:
        dll.LCS_SetLaunchMode(0)
