"""The oracle's operation-order rewrites against the reference's own order (CPU).

liboracle_f32.so evaluates the tet projection in the CUDA library's order (frame-constant
reciprocals of the damping scales, one reciprocal of the 2x2 pivot, own J^(-2/3), log and arccos
routines); liboracle_f32w.so (ORACLE_AS_WRITTEN) evaluates it as the reference writes it
(xpbd_solver.cu:553, 773-816: its divisions, powf, logf, acosf).  Every arithmetic rewrite of the
CUDA path is therefore checked against the as-written order, not only against a co-edited oracle:
on the C1 block (16 x 8 x 16 cells, no strain damping) both stay within 1e-4 of the bounding-box
diagonal of each other and of the FP64 build over 100 free-running steps, and with bending and the
tissue guard armed over 20."""
import ctypes

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import PlainTissue, pointer
from conftest import ROOT

WRITTEN = ROOT / "oracle" / "_build" / "liboracle_f32w.so"


def rollout(lib, steps, record, kb=0.0, guard=False):
    g = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    out = {}
    with PlainTissue(g, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, poisson=0.25, strain_damping_s=0.0, kb=kb,
                     dll_path=lib) as s:
        s.set_gravity(0.0, -981.0, 0.0)
        if guard:
            s.check("LCS_SetTissueGuard", ctypes.c_float(0.5), 1, len(g.positions), pointer(g.inside), 1)
        for k in range(steps):
            s.step()
            if k + 1 in record:
                out[k + 1] = s.positions()
    return g, out


@pytest.mark.parametrize("kb,guard,steps", [(0.0, False, 100), (0.1, False, 20), (0.0, True, 20)])
def test_library_order_tracks_the_reference_order(oracle_libs, kb, guard, steps):
    record = (1, 2, 5, 10, 20, 50, 100)
    g, f32 = rollout(oracle_libs[0], steps, record, kb, guard)
    _, f32w = rollout(WRITTEN, steps, record, kb, guard)
    _, f64 = rollout(oracle_libs[1], steps, record, kb, guard)
    active = g.active != 0
    diag = W.bbox_diagonal(g)
    for k in f32:
        a = float(np.abs(f32[k] - f32w[k])[active].max()) / diag
        b = float(np.abs(f32w[k] - f64[k])[active].max()) / diag
        assert a <= 1e-4 and b <= 1e-4, (k, a, b)
    assert not np.array_equal(f32[steps], f32w[steps]), "the two orders should round differently"


def test_damped_step_rounding_floor(oracle_libs):
    """Why the strain-damped block's replayed steps have a wider bound than 1e-4: replayed from FP64
    states (each step started from the FP64 oracle's state), FP32 in the reference's own operation
    order (the as-written oracle) lands farther than 1e-4 of the diagonal from the FP64 step at some
    step of the 100, and FP32 in either order stays within the 5e-4 the GPU replay uses.  With 0.04 s
    of Kelvin-Voigt damping one step amplifies rounding near the deviatoric constraint's singularity
    (C_D = sqrt(q) at q -> 0)."""
    import replay_harness as RH
    from test_replay_parity import DAMPED_STEP_TOL, TOL, scenario

    sc = scenario("c1_damped")
    libs = {"library": oracle_libs[0], "written": WRITTEN}
    exact = sc.open(oracle_libs[1])
    sessions = {k: sc.open(v) for k, v in libs.items()}
    try:
        states, replayed = RH.replay(exact, sessions, sc.steps, sc.cmd)
    finally:
        for s in [exact, *sessions.values()]:
            s.close()
    active = sc.grid.active != 0
    diag = W.bbox_diagonal(sc.grid)
    worst = {k: max(RH.diff(replayed[k][i], states[i], active, diag)["pos"] for i in range(sc.steps)) for k in libs}
    assert worst["written"] > TOL, worst
    assert max(worst.values()) <= DAMPED_STEP_TOL, worst
