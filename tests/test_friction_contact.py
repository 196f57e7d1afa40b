"""Contact model 1 without a reconstructed surface (LCS_SetContactModel(1, ...); the reference's
k_FindToolContacts + k_SolveFrictionContacts, V/contact/friction_contact.cuh:3-169): the shaft
capsule and both jaw boxes of the instrument against every lattice node, swept over each substep,
with unilateral normal and Coulomb friction projection.

Two instrument motions cover both time-of-impact paths: a pure translation of the jaws (the exact
piecewise-quadratic box path) and a closing jaw that turns the boxes (conservative advancement).
CPU tests check the oracle (FP32 against FP64, the contact acts); GPU tests check the CUDA frame
against the FP32 oracle bit for bit."""
import ctypes

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import Grasper, GraspParams, PlainTissue, V3

GRASP = dict(W.DEFAULT_GRASP, ccd_velocity=0.0)


def grasper(top, k, steps, closing):
    """Shaft capsule above the block and a jaw pair whose lower box is pressed into the top face."""
    f = (k + 1) / steps
    y = top + 0.45 - 0.55 * f
    gap = (0.5 - 0.4 * f) if closing else 0.3
    return Grasper(V3(-0.4, y + 0.9, 0.1), V3(0.4, y + 1.6, 0.1), 0.25, V3(-0.6, y, 0.0), V3(1.0, 0.0, 0.15), V3(0.0, y, 0.0),
                   V3(0.0, 1.0, 0.0), 0.35, 1.2, gap, 0.0)


def surfaceless_grid():
    """The C1 lattice with no surface edges: the reconstructed surface has no triangles, so the
    reference's contact model 1 takes its node-contact branch (k_FindToolContacts +
    k_SolveFrictionContacts, xpbd_solver.cu:3655-3665), the branch this library implements; with a
    surface it contacts the triangle soup instead (the unified solver's surface contact)."""
    g = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    return g.__class__(**{**vars(g), "surface_edges": np.zeros((0, 8), dtype=np.int32)})


def friction_run(lib, steps=10, closing=False, launch_mode=None, enabled=1, reference=False, on_close=None):
    g = surfaceless_grid()
    s = PlainTissue(g, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, strain_damping_s=0.0, grasp_params=GraspParams(**GRASP),
                    dll_path=lib, reference=reference)
    try:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(launch_mode)
        s.set_gravity(0.0, -981.0, 0.0)
        s.check("LCS_SetContactModel", enabled, ctypes.c_float(0.6), ctypes.c_float(0.4), ctypes.c_float(0.1), ctypes.c_float(0.01))
        top = float(g.positions[g.active != 0, 1].max())
        s.check("LCS_SetGraspTool", ctypes.byref(grasper(top, -1, steps, closing)))
        frames = []
        for k in range(steps):
            s.check("LCS_SetGraspTool", ctypes.byref(grasper(top, k, steps, closing)))
            s.step()
            frames.append(s.positions())
        if on_close is not None:
            on_close(s)
        return g, frames
    finally:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(0)
        s.close()


@pytest.mark.parametrize("closing", [False, True])
def test_friction_contact_oracle_acts_and_fp32_tracks_fp64(oracle_libs, closing):
    g, f32 = friction_run(oracle_libs[0], closing=closing)
    _, f64 = friction_run(oracle_libs[1], closing=closing)
    _, free = friction_run(oracle_libs[0], closing=closing, enabled=0)   # contact model 0: the jaw slab only
    active = g.active != 0
    assert np.isfinite(f32[-1]).all()
    assert float(np.abs(f32[-1] - f64[-1])[active].max()) < 1e-3
    assert float(np.abs(f32[-1] - free[-1])[active].max()) > 1e-2        # the jaw boxes push the top face


def test_anchor_assist_is_refused(oracle_libs):
    g = build_grid(0.2, size=(1.18, 0.58, 1.18), density=1000.0)
    with PlainTissue(g, dt=1 / 60, substeps=4, ks=1e6, dll_path=oracle_libs[0]) as s:
        assert s.functions["LCS_SetContactModel"](2, 0.6, 0.4, 0.1, 0.01) == -4001


@pytest.mark.gpu
@pytest.mark.parametrize("closing,mode", [(False, 2), (True, 1), (True, 2)])
def test_friction_contact_matches_oracle(gpu_lib, oracle_libs, closing, mode):
    _, gpu = friction_run(gpu_lib, closing=closing, launch_mode=mode)
    _, cpu = friction_run(oracle_libs[0], closing=closing)
    for k, (a, b) in enumerate(zip(gpu, cpu)):
        assert np.array_equal(a, b), (k, float(np.abs(a - b).max()))
