"""Pin the CPU oracle against the reference's own CUDA solver (oracle/_ref, built from the
reference's sources by oracle/build_ref.sh), through the same LCS_* harness.

Only configurations the reference ABI expresses are used: uniform (E, nu) material, lattice-edge
stiffness, capsule contact model 0 and the geometric blade.  The reference contracts multiply-adds
and uses the CUDA power function, so its FP32 trajectory differs from the oracle's in the last bits;
positions are compared within the benchmark spec's tolerance (1e-4 of the bounding-box diagonal) on
horizons where those rounding differences have not grown, and cut topology bit-exactly.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import Capsule, PlainTissue, GraspParams

pytestmark = pytest.mark.gpu
from conftest import results_dir

OUT = results_dir()
SMALL = (4.78, 2.38, 3.98)


def run(lib, grid, steps, reference, ks=1e6, substeps=10, capsule=None, blades=None, record=(1, 2, 5, 10, 20), guard=None):
    s = PlainTissue(grid, dt=1 / 60, substeps=substeps, ks=ks, young_pa=6000.0, poisson=0.25, strain_damping_s=0.04,
                    dll_path=lib, reference=reference,
                    grasp_params=GraspParams(**dict(W.DEFAULT_GRASP, ccd_velocity=0.0)) if capsule else None)
    out = {}
    try:
        s.set_gravity(0.0, -981.0, 0.0)
        if guard:   # the reference adapter's guard: minimum relative volume, passes; strength 80, bulk damping 0.01 s
            import ctypes
            from genesis_tissue_simulation_gb300.native_backend import pointer
            s.check("LCS_SetTissueGuard", ctypes.c_float(guard[0]), guard[1], len(grid.positions), pointer(grid.inside), 1)
            s.check("LCS_SetTissueMaterial", ctypes.c_float(80.0), ctypes.c_float(0.01))
        if capsule:
            s.set_capsule(capsule[0])
        for k in range(steps):
            if capsule:
                s.set_capsule(capsule[1][k])
            detect = False
            if blades:
                s.set_blade(blades[k])
                detect = True
            s.step(detect_cut=detect)
            if k + 1 in record:
                out[k + 1] = dict(pos=s.positions(), nbr=s.neighbors(), rev=s.topology_revision(),
                                  frac=s.cut_edge_fractions())
        out["colors"] = (s.functions["LCS_EdgeColorCount"](), s.functions["LCS_TetColorCount"](), s.functions["LCS_TetCount"]())
        ids = np.empty((out["colors"][2], 4), dtype=np.int32)
        s.check("LCS_GetTetIds", ids.ctypes.data_as(__import__("ctypes").c_void_p))
        out["ids"] = ids
    finally:
        s.close()
    return out


def report(name, grid, ref, orc):
    active = grid.active != 0
    diag = W.bbox_diagonal(grid)
    rows = {k: float(np.abs(ref[k]["pos"] - orc[k]["pos"])[active].max()) / diag for k in ref if isinstance(k, int)}
    OUT.mkdir(exist_ok=True)
    with open(OUT / "reference_parity.jsonl", "a") as f:
        f.write(json.dumps({"case": name, "err_over_diag": rows}) + "\n")
    print(name, rows)
    return rows


def test_tet_mesh_and_colouring_match_reference(reference_lib, oracle_libs):
    grid = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    ref = run(reference_lib, grid, 1, True, record=(1,))
    orc = run(oracle_libs[0], grid, 1, False, record=(1,))
    assert ref["colors"] == orc["colors"]
    np.testing.assert_array_equal(ref["ids"], orc["ids"])


@pytest.mark.parametrize("ks", [1e6, 0.0])
def test_plain_step_matches_reference(reference_lib, oracle_libs, ks):
    grid = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    ref = run(reference_lib, grid, 20, True, ks=ks)
    orc = run(oracle_libs[0], grid, 20, False, ks=ks)
    rows = report(f"c1_grid_ks{ks:g}", grid, ref, orc)
    assert rows[1] <= 1e-4


def test_capsule_contact_matches_reference(reference_lib, oracle_libs):
    w = W.make("c2", steps=10, scale=SMALL)
    cap = (w.initial_capsule, w.capsule_path)
    ref = run(reference_lib, w.grid, 10, True, substeps=20, capsule=cap, record=(1, 2, 5, 10))
    orc = run(oracle_libs[0], w.grid, 10, False, substeps=20, capsule=cap, record=(1, 2, 5, 10))
    rows = report("c2_small_capsule", w.grid, ref, orc)
    assert rows[1] <= 1e-4


def test_blade_cut_topology_matches_reference(reference_lib, oracle_libs):
    w = W.make("c3", steps=10, scale=SMALL)
    ref = run(reference_lib, w.grid, 10, True, substeps=20, blades=w.blade_path, record=(1, 2, 5, 10))
    orc = run(oracle_libs[0], w.grid, 10, False, substeps=20, blades=w.blade_path, record=(1, 2, 5, 10))
    report("c3_small_blade", w.grid, ref, orc)
    with open(OUT / "reference_parity.jsonl", "a") as f:
        f.write(json.dumps({"case": "c3_small_blade_topology", "rev": {k: [ref[k]["rev"], orc[k]["rev"]] for k in (1, 2, 5, 10)},
                            "nbr_diff": {k: int((ref[k]["nbr"] != orc[k]["nbr"]).sum()) for k in (1, 2, 5, 10)}}) + "\n")
    assert ref[1]["rev"] == orc[1]["rev"]
    np.testing.assert_array_equal(ref[1]["nbr"], orc[1]["nbr"])


def test_tall_block_sag_matches_reference(reference_lib, oracle_libs):
    """The plain branch's single Gauss-Seidel pass per substep lets a 16-cell column sag far below its
    elastic equilibrium; the oracle must show the same sag as the reference."""
    grid = build_grid(0.2, size=(3.18, 3.18, 3.18), density=1000.0)
    ref = run(reference_lib, grid, 10, True, ks=0.0, record=(10,))
    orc = run(oracle_libs[0], grid, 10, False, ks=0.0, record=(10,))
    active = grid.active != 0
    sag = [float((r[10]["pos"] - grid.positions)[active, 1].mean()) for r in (ref, orc)]
    with open(OUT / "reference_parity.jsonl", "a") as f:
        f.write(json.dumps({"case": "tall_block_sag", "reference": sag[0], "oracle": sag[1]}) + "\n")
    assert abs(sag[0] - sag[1]) <= 0.05 * abs(sag[0]) + 1e-3


@pytest.mark.parametrize("minimum,passes", [(0.15, 1), (0.9, 1)])
def test_guarded_step_matches_reference(reference_lib, oracle_libs, minimum, passes):
    """The tissue guard chain (guarded tet form, tensile passes, feasibility chain) against the
    reference's own: a capsule pressed into the C1 block; at minimum 0.9 the repair and the vertex
    line search run in most substeps."""
    grid = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    top = float(grid.positions[grid.active != 0, 1].max())
    caps = [Capsule((-1.0, top + 0.25 - 0.6 * k / 10, 0.0), (1.0, top + 0.25 - 0.6 * k / 10, 0.2), 0.25) for k in range(11)]
    cap = (caps[0], caps[1:])
    ref = run(reference_lib, grid, 10, True, capsule=cap, record=(1, 2, 5, 10), guard=(minimum, passes))
    orc = run(oracle_libs[0], grid, 10, False, capsule=cap, record=(1, 2, 5, 10), guard=(minimum, passes))
    rows = report(f"c1_guard_min{minimum:g}_passes{passes}", grid, ref, orc)
    assert rows[1] <= 1e-4


@pytest.mark.parametrize("closing", [False, True])
def test_friction_contact_matches_reference(reference_lib, oracle_libs, closing):
    """Contact model 1 without a surface (shaft capsule + jaw boxes, swept contact, Coulomb
    friction) against the reference's own kernels."""
    from test_friction_contact import friction_run
    grid, ref = friction_run(reference_lib, closing=closing, reference=True)
    _, orc = friction_run(oracle_libs[0], closing=closing)
    active = grid.active != 0
    diag = W.bbox_diagonal(grid)
    rows = {k + 1: float(np.abs(ref[k] - orc[k])[active].max()) / diag for k in (0, 1, 4, 9)}
    with open(OUT / "reference_parity.jsonl", "a") as f:
        f.write(json.dumps({"case": f"c1_friction_contact_closing{int(closing)}", "err_over_diag": rows}) + "\n")
    assert rows[1] <= 1e-4
