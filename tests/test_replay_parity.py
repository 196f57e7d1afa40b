"""Replay-mode parity against the reference's own CUDA build (oracle/_ref, compiled from the
reference's sources by oracle/build_ref.sh), at every step of each scenario.

The reference build free-runs a scenario; the CUDA library, the FP32 oracle (the library's operation
order) and the as-written FP32 oracle (the reference's divisions, library power and logarithm) each
step from the reference's state of every step under the same commands (tests/replay_harness.py).
The FP64 oracle is replayed from the same states too, and each step's distance of the FP32 results
from it is recorded.  Asserted at every replayed step: positions within the parity tolerance, 1e-4
of the bounding-box diagonal, of the reference's next state (5e-4 for the strain-damped block, whose
steps amplify FP32 rounding past 1e-4 in the reference's own operation order, see DAMPED_STEP_TOL);
the integer topology (neighbour table, bend liveness, active flags, voxel cut mask, cut
edges, topology revision) identical; the CUDA library bit-identical
to the FP32 oracle in positions, velocities and topology.  Free-running differences over the whole
horizon (against the reference build and the FP64 oracle) are recorded, and asserted within the
tolerance where the scenario is not chaotic in FP32 (strain damping 0).

Only what the reference ABI expresses is used: uniform (E, nu) material, lattice-edge stiffness,
capsule contact model 0 (with and without its approach-speed gate), contact model 1 without a
surface, the tissue guard, bending, perpendicular edge damping, the geometric blade and the tear law.
"""
from __future__ import annotations

import ctypes
import json
from dataclasses import dataclass, field

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import Capsule, GraspParams, PlainTissue, severed_edges
from conftest import ROOT, results_dir
import replay_harness as RH

pytestmark = pytest.mark.gpu

C1 = (3.18, 1.58, 3.18)        # 16 x 8 x 16 cells
SMALL = (4.78, 2.38, 3.98)     # 24 x 12 x 20 cells
ORACLE_WRITTEN = ROOT / "oracle" / "_build" / "liboracle_f32w.so"
TOL = 1e-4
# The strain-damped block's per-step bound.  With 0.04 s of Kelvin-Voigt damping a single step
# amplifies FP32 rounding near the deviatoric constraint's singularity so far that FP32 evaluations
# in the reference's own operation order land up to 3.5e-4 of the diagonal from the FP64 step
# (tests/test_oracle_as_written.py::test_damped_step_rounding_floor); 1e-4 lies below that floor.
DAMPED_STEP_TOL = 5e-4


@dataclass
class Scenario:
    name: str
    grid: object
    steps: int
    kwargs: dict
    setup: object = None        # setup(session) after construction (gravity is always set)
    command: object = None      # command(session, k) -> rod-phase cut after the step
    free_tolerance: bool = False   # assert the free-running difference too
    step_tol: float = TOL          # bound of every replayed step
    extra: dict = field(default_factory=dict)

    def open(self, lib, reference=False):
        s = PlainTissue(self.grid, dll_path=lib, reference=reference, **self.kwargs)
        try:
            s.set_gravity(0.0, -981.0, 0.0)
            if self.setup:
                self.setup(s)
        except Exception:
            s.close()
            raise
        return s

    def cmd(self, s, k):
        return bool(self.command(s, k)) if self.command else False


def _base(substeps=10, ks=1e6, damping=0.0, **kw):
    return dict(dt=1 / 60, substeps=substeps, ks=ks, young_pa=6000.0, poisson=0.25, strain_damping_s=damping, **kw)


def _capsule_scenario(name, grid_scale, steps, gate):
    w = W.make("c2", steps=steps, scale=grid_scale)
    grasp = GraspParams(**dict(W.DEFAULT_GRASP, ccd_velocity=gate))
    return Scenario(name, w.grid, steps, _base(substeps=20, grasp_params=grasp),
                    setup=lambda s: s.set_capsule(w.initial_capsule),
                    command=lambda s, k: s.set_capsule(w.capsule_path[k]))


def _blade_scenario(name, grid_scale, steps, tear=0.0):
    w = W.make("c3", steps=steps, scale=grid_scale)
    return Scenario(name, w.grid, steps, _base(substeps=20, tear_ratio=tear),
                    command=lambda s, k: (s.set_blade(w.blade_path[k]), True)[1])


def _guard_scenario(minimum):
    grid = build_grid(0.2, size=C1, density=1000.0)
    top = float(grid.positions[grid.active != 0, 1].max())
    caps = [Capsule((-1.0, top + 0.25 - 0.6 * k / 10, 0.0), (1.0, top + 0.25 - 0.6 * k / 10, 0.2), 0.25) for k in range(11)]

    def setup(s):
        from genesis_tissue_simulation_gb300.native_backend import pointer
        s.check("LCS_SetTissueGuard", ctypes.c_float(minimum), 1, len(grid.positions), pointer(grid.inside), 1)
        s.check("LCS_SetTissueMaterial", ctypes.c_float(80.0), ctypes.c_float(0.01))
        s.set_capsule(caps[0])
    return Scenario(f"c1_guard_min{minimum:g}", grid, 10,
                    _base(damping=0.04, grasp_params=GraspParams(**dict(W.DEFAULT_GRASP, ccd_velocity=0.0))),
                    setup=setup, command=lambda s, k: s.set_capsule(caps[k + 1]))


def _friction_scenario(closing):
    from test_friction_contact import GRASP, grasper, surfaceless_grid
    grid = surfaceless_grid()     # the reference's node-contact branch of contact model 1
    top = float(grid.positions[grid.active != 0, 1].max())
    steps = 10

    def setup(s):
        s.check("LCS_SetContactModel", 1, ctypes.c_float(0.6), ctypes.c_float(0.4), ctypes.c_float(0.1), ctypes.c_float(0.01))
        s.check("LCS_SetGraspTool", ctypes.byref(grasper(top, -1, steps, closing)))
    return Scenario(f"c1_friction_closing{int(closing)}", grid, steps, _base(grasp_params=GraspParams(**GRASP)), setup=setup,
                    command=lambda s, k: s.check("LCS_SetGraspTool", ctypes.byref(grasper(top, k, steps, closing))))


def scenario(name):
    c1 = build_grid(0.2, size=C1, density=1000.0)
    table = {
        # the C1 workload (16 x 8 x 16 cells, 10 substeps): strain damping 0 is not chaotic in FP32
        "c1": lambda: Scenario("c1", c1, 100, _base(), free_tolerance=True),
        # the reference adapter's 0.04 s strain damping: FP32 and FP64 of one algorithm part within
        # 10 frames on this block, so only the replayed steps are held to the tolerance
        "c1_damped": lambda: Scenario("c1_damped", c1, 100, _base(damping=0.04), step_tol=DAMPED_STEP_TOL),
        "c1_ks0": lambda: Scenario("c1_ks0", c1, 20, _base(ks=0.0), free_tolerance=True),
        "c1_bending": lambda: Scenario("c1_bending", c1, 20, _base(kb=0.1, cb=1e-5), free_tolerance=True),
        "c1_perp_damping": lambda: Scenario("c1_perp_damping", c1, 20, _base(cs=1e-3), free_tolerance=True),
        "c2_small": lambda: _capsule_scenario("c2_small", SMALL, 40, 0.0),
        "c2_small_gate": lambda: _capsule_scenario("c2_small_gate", SMALL, 40, 0.5),
        "c3_small": lambda: _blade_scenario("c3_small", SMALL, 40),
        "c3_small_tear": lambda: _blade_scenario("c3_small_tear", SMALL, 20, tear=1.008),
        # lattices at the edges of the layout: a 2 x 9 x 2 column bending under gravity, the capsule on
        # an 8 x 5 x 6 block, the blade through a 10 x 3 x 9 sheet
        "c1_column": lambda: Scenario("c1_column", build_grid(0.2, size=(0.2, 1.8, 0.2), density=1000.0), 20, _base()),
        "c2_odd": lambda: _capsule_scenario("c2_odd", (1.5, 0.9, 1.1), 20, 0.0),
        "c3_sheet": lambda: _blade_scenario("c3_sheet", (2.0, 0.4, 1.6), 20),
        "c2_full": lambda: _capsule_scenario("c2_full", None, 20, 0.0),
        "c3_full": lambda: _blade_scenario("c3_full", None, 30),
        "c1_guard_min0.15": lambda: _guard_scenario(0.15),
        "c1_guard_min0.9": lambda: _guard_scenario(0.9),
        "c1_friction_closing0": lambda: _friction_scenario(False),
        "c1_friction_closing1": lambda: _friction_scenario(True),
    }
    return table[name]()


def run_scenario(sc, reference_lib, gpu_lib, oracle_libs):
    grid = sc.grid
    active = grid.active != 0
    diag = W.bbox_diagonal(grid)
    libs = {"gpu": gpu_lib, "oracle": oracle_libs[0], "written": ORACLE_WRITTEN}
    replayers = dict(libs, fp64=oracle_libs[1])   # the FP64 oracle: exact-arithmetic stand-in for each step
    sessions = {}
    try:
        ref = sc.open(reference_lib, reference=True)
        sessions["reference"] = ref
        for name, lib in replayers.items():
            sessions[name] = sc.open(lib)
        ref_states, replayed = RH.replay(ref, {k: sessions[k] for k in replayers}, sc.steps, sc.cmd)
    finally:
        for s in sessions.values():
            s.close()
    # free runs: the CUDA library and the FP64 oracle over the whole horizon
    last = {sc.steps}
    free = {}
    for name, lib in (("gpu", gpu_lib), ("fp64", oracle_libs[1])):
        with sc.open(lib) as s:
            free[name] = RH.free_run(s, sc.steps, sc.cmd, record=last)[sc.steps]
    rows = []
    for k in range(sc.steps):
        row = {"step": k + 1}
        for name in libs:
            row[name] = RH.diff(replayed[name][k], ref_states[k], active, diag)
        row["gpu_vs_oracle"] = RH.diff(replayed["gpu"][k], replayed["oracle"][k], active, diag)
        # recorded: how far the reference's own FP32 step and the as-written oracle's (the same
        # operation order on the CPU) land from the FP64 evaluation of the same step
        exact = replayed["fp64"][k]["pos"]
        row["floor"] = max(float(np.abs(exact - ref_states[k]["pos"])[active].max()),
                           float(np.abs(exact - replayed["written"][k]["pos"])[active].max())) / diag
        rows.append(row)
    summary = {
        "case": sc.name, "steps": sc.steps, "nodes": int(active.sum()),
        "replay_max_err_over_diag": {name: max(r[name]["pos"] for r in rows) for name in libs},
        "replay_err_over_diag_by_step": {name: [r[name]["pos"] for r in rows] for name in libs},
        "fp32_floor_by_step": [r["floor"] for r in rows],
        "free_run_err_over_diag": {
            "gpu_vs_reference": float(np.abs(free["gpu"]["pos"] - ref_states[-1]["pos"])[active].max()) / diag,
            "gpu_vs_fp64_oracle": float(np.abs(free["gpu"]["pos"] - free["fp64"]["pos"])[active].max()) / diag,
            "reference_vs_fp64_oracle": float(np.abs(ref_states[-1]["pos"] - free["fp64"]["pos"])[active].max()) / diag,
        },
        "revision": [int(ref_states[-1]["rev"]), int(free["gpu"]["rev"])],
        "tears": [int(ref_states[-1]["tears"]), int(free["gpu"]["tears"])],
    }
    with open(results_dir() / "replay_parity.jsonl", "a") as f:
        f.write(json.dumps(summary) + "\n")
    return rows, ref_states, replayed, free, summary


CASES = ["c1", "c1_damped", "c1_ks0", "c1_bending", "c1_perp_damping", "c2_small", "c2_small_gate", "c3_small",
         "c3_small_tear", "c1_guard_min0.15", "c1_guard_min0.9", "c1_friction_closing0", "c1_friction_closing1",
         "c1_column", "c2_odd", "c3_sheet", "c2_full", "c3_full"]


@pytest.mark.parametrize("case", CASES)
def test_replay_matches_reference(reference_lib, gpu_lib, oracle_libs, case):
    sc = scenario(case)
    rows, ref_states, replayed, free, summary = run_scenario(sc, reference_lib, gpu_lib, oracle_libs)
    for r in rows:
        k = r["step"]
        tol = sc.step_tol
        for name in ("gpu", "oracle", "written"):
            d = r[name]
            assert d["pos"] <= tol, f"{case} step {k}: |{name} - reference| = {d['pos']:.3e} of the diagonal (bound {tol:.1e})"
            for key in ("nbr", "bends", "active", "rev", "mask", "frac_cut"):
                assert d[key], f"{case} step {k}: {name} {key} differs from the reference"
        g = r["gpu_vs_oracle"]
        assert g["pos"] == 0.0 and g["vel"] == 0.0, f"{case} step {k}: gpu differs from the FP32 oracle"
        assert all(g[key] for key in ("nbr", "bends", "active", "rev", "mask", "frac_cut"))
    for k in range(sc.steps):
        gpu = replayed["gpu"][k]
        assert np.array_equal(gpu["own_mask"], gpu["mask"]), "mask rebuilt from fractions differs from the library's"
        assert np.array_equal(replayed["gpu"][k]["frac"], replayed["oracle"][k]["frac"])
    if sc.free_tolerance:
        err = summary["free_run_err_over_diag"]["gpu_vs_reference"]
        assert err <= TOL, f"{case}: free-running |gpu - reference| after {sc.steps} steps = {err:.3e} of the diagonal"
    if case == "c3_small_tear":
        assert ref_states[-1]["tears"] > 0 and replayed["gpu"][-1]["tears"] > 0, "the tear law severed nothing"
    if case.startswith("c3"):
        assert ref_states[-1]["rev"] > 0, "the blade never crossed the tissue"
        assert ref_states[-1]["rev"] == severed_edges(sc.grid.neighbors, ref_states[-1]["nbr"])
