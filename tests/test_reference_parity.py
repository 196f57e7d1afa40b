"""Structural pins of the CPU oracle against the reference's own CUDA solver (oracle/_ref, built from
the reference's sources by oracle/build_ref.sh), through the same LCS_* harness: the Kuhn tet mesh
in storage order and both colourings, and the sag of a tall block (the plain branch's signature).
Step-by-step dynamics and cut topology against the reference are the replay tests
(test_replay_parity.py), which start every compared step from the reference's own state.
"""
import json

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import PlainTissue, GraspParams

pytestmark = pytest.mark.gpu
from conftest import results_dir

OUT = results_dir()


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


def test_tet_mesh_and_colouring_match_reference(reference_lib, oracle_libs):
    grid = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    ref = run(reference_lib, grid, 1, True, record=(1,))
    orc = run(oracle_libs[0], grid, 1, False, record=(1,))
    assert ref["colors"] == orc["colors"]
    np.testing.assert_array_equal(ref["ids"], orc["ids"])


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
