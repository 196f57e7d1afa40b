"""Debug-build gather checks (libgbtissue_debug.so, compiled with GBT_DEBUG_BOUNDS), the stand-in
for a memory checker: every element gather index -- edge ends, bend nodes, tet nodes and the
neighbour-table slots of the liveness refresh -- is checked against the nodes the kernel serves
(the instance's own nodes in the one-CTA-per-instance batch kernels).  The GPU tests run the plain
step in every launch shape, the capsule, blade, tissue-guard and friction workloads, the batch in
every launch shape and the differentiable rollout on the debug library and require zero violations,
and the debug library's results to equal the release library's bit for bit."""
import ctypes

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import batch as BT
from genesis_tissue_simulation_gb300 import build as native_build
from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.native_backend import GraspParams

SMALL = (4.78, 2.38, 3.98)


def test_release_build_reports_unsupported():
    dll = ctypes.CDLL(str(native_build.build()))
    out = (ctypes.c_uint * 3)()
    assert dll.GBT_DebugBoundsRead(out) == -4001
    assert dll.GBT_BatchDebugBoundsRead(out) == -4001


@pytest.fixture(scope="module")
def debug_lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    return native_build.build(debug=True)


def _read(dll, name="GBT_DebugBoundsRead"):
    out = (ctypes.c_uint * 3)()
    assert getattr(dll, name)(out) == 0
    return list(out)


def _run(workload, lib, steps, mode=0):
    s = workload.open(lib)
    try:
        s.dll.LCS_SetLaunchMode(mode)
        workload.run(s, steps=steps)
        rec = _read(s.dll) if "debug" in str(lib) else None
        return s.positions(), rec
    finally:
        s.dll.LCS_SetLaunchMode(0)
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale,steps,mode", [("c1", None, 6, 0), ("c1", None, 6, 1), ("c1", None, 6, 2), ("c1", None, 6, 3),
                                                   ("c2", SMALL, 8, 0), ("c3", SMALL, 12, 1), ("c3", SMALL, 12, 2)])
def test_plain_workloads_have_no_out_of_range_gathers(gpu_lib, debug_lib, name, scale, steps, mode):
    w = W.make(name, steps=steps, scale=scale)
    pos, rec = _run(w, debug_lib, steps, mode)
    assert rec[0] == 0, f"{rec[0]} out-of-range gathers, first index {rec[1]} at site {rec[2]}"
    ref, _ = _run(w, gpu_lib, steps, mode)
    assert np.array_equal(pos, ref), "the checks changed the arithmetic"


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_guard_and_friction_have_no_out_of_range_gathers(debug_lib, mode):
    from test_guard import guarded_run
    from test_friction_contact import friction_run
    records = []
    guarded_run(debug_lib, steps=4, launch_mode=mode, on_close=lambda s: records.append(_read(s.dll)))
    friction_run(debug_lib, steps=4, closing=True, launch_mode=mode, on_close=lambda s: records.append(_read(s.dll)))
    assert len(records) == 2 and all(r[0] == 0 for r in records), records


@pytest.mark.gpu
@pytest.mark.parametrize("mode,threads", [(0, 256), (1, 256), (1, 512), (2, 2), (2, 8)])
def test_batch_has_no_out_of_range_gathers(debug_lib, mode, threads):
    wl = BT.make_c4(count=7, seed=11, steps=4, size_range=((4, 9), (3, 6), (4, 9)))
    grasp = GraspParams(**dict(W.DEFAULT_GRASP, ccd_velocity=0.0))
    with BT.TissueBatch(wl.grids, dt=1 / 60, substeps=wl.substeps, ks=1e6, stiffness_scale=wl.stiffness_scale(),
                        grasp_params=grasp, dll_path=debug_lib) as b:
        b.set_launch(mode, threads)
        b.set_gravity(0.0, -981.0, 0.0)
        b.set_capsules(wl.capsules_at(0))
        for k in range(4):
            b.step_many([wl.capsules_at(k + 1)], use_graph=k % 2 == 1)
        rec = _read(b.dll, "GBT_BatchDebugBoundsRead")
        assert np.isfinite(b.positions()).all()
    assert rec[0] == 0, f"{rec[0]} out-of-range gathers, first index {rec[1]} at site {rec[2]}"


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_differentiable_rollout_has_no_out_of_range_gathers(debug_lib, mode):
    import torch
    from diff_cases import Case
    from test_gpu_adjoint import gpu_tissue
    case = Case()
    with gpu_tissue(case, debug_lib, mode) as t:
        theta = torch.tensor(case.theta(t.session.tet_count), device="cuda")
        path = torch.tensor(case.path, device="cuda")
        x = t.forward(theta, path)
        grads = t.backward(torch.ones_like(x))
        assert torch.isfinite(grads["theta"]).all()
        rec = _read(t.session.dll)
    assert rec[0] == 0, f"{rec[0]} out-of-range gathers, first index {rec[1]} at site {rec[2]}"
