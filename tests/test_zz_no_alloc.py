"""LCS_StepNoAlloc, the step for hosts that cannot let the library allocate GPU memory.

Engines that manage every device allocation through their own pool or budget, and real-time loops
where an allocation (which may synchronise the device) would stall a frame, call LCS_StepNoAlloc:
it uses a fixed scratch array inside the library instead of any allocation.  These tests check,
through the C ABI, that two calls in a row give the same tissue as two calls of LCS_Step (the
tolerance of the other parity tests, 1e-4 of the bounding-box diagonal, and in fact bit for bit:
positions, velocities, neighbour table, topology revision, particle frames and the rebuilt surface)
in each launch shape, and that a mesh larger than the array's limit is refused.  This file is
collected last.
"""
import ctypes

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W

pytestmark = pytest.mark.gpu
LCS_ERR_SCRATCH_LIMIT = -4003
SMALL = (4.78, 2.38, 3.98)


def two_steps(workload, lib, entry, mode):
    session = workload.open(lib)
    try:
        session.dll.LCS_SetLaunchMode(mode)
        step = getattr(session.dll, entry)
        step.argtypes, step.restype = (ctypes.c_float,), ctypes.c_int
        frames = []
        for k in range(2):
            detect = workload.command(session, k)
            assert step(session.dt) == 0, entry
            if detect:
                session.check("LCS_DetectCut")
            session.check("LCS_Finalize")
            surface = session.surface()
            frames.append(dict(pos=session.positions(), vel=session.velocities(), nbr=session.neighbors(),
                               rev=session.topology_revision(), rot=session.particle_frames(),
                               tri=surface["tri"], spos=surface["pos"]))
        return frames
    finally:
        session.dll.LCS_SetLaunchMode(0)
        session.close()


# launch mode 0 picks one CTA for these meshes (their nodes stage in shared memory), 1 the
# whole-GPU cooperative kernel, whose barrier counter and status words live in the scratch array,
# 2 one CTA explicitly
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("name,scale", [("c1", None), ("c2", SMALL), ("c3", SMALL)])
def test_no_alloc_step_matches_step(gpu_lib, name, scale, mode):
    w = W.make(name, steps=2, scale=scale)
    tol = 1e-4 * W.bbox_diagonal(w.grid)
    ref = two_steps(w, gpu_lib, "LCS_Step", mode)
    out = two_steps(w, gpu_lib, "LCS_StepNoAlloc", mode)
    for a, b in zip(ref, out):
        assert float(np.abs(a["pos"] - b["pos"]).max()) <= tol
        for key in ("pos", "vel", "nbr", "rot", "tri", "spos"):
            assert np.array_equal(a[key], b[key]), key
        assert a["rev"] == b["rev"]


def test_no_alloc_step_refuses_meshes_beyond_its_limit(gpu_lib):
    w = W.make("c2", steps=1)          # 589,824 tets > 524,288
    session = w.open(gpu_lib)
    try:
        step = session.dll.LCS_StepNoAlloc
        step.argtypes, step.restype = (ctypes.c_float,), ctypes.c_int
        before = session.positions()
        assert step(session.dt) == LCS_ERR_SCRATCH_LIMIT
        assert np.array_equal(session.positions(), before)
    finally:
        session.close()
