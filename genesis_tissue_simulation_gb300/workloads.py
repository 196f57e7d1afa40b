"""Named synthetic workloads of the tissue step (parameter files in ``params/``).

Each workload fixes a lattice (``build_grid``), the XPBD parameters, per-tet material, gravity and
an optional scripted instrument: a capsule pressed into the top surface (contact model 0) or a
planar blade swept along a polyline (geometric cut).  All randomness comes from
``numpy.random.default_rng(seed)``.  Native units: cm, y up, gravity -981 cm/s^2 on y.

Material: the reference bakes mu*V and kappa*V from (E, nu) per tet (xpbd_solver.cu:1632-1731);
``per_tet_compliance`` draws a compliance c_t per tet (storage order, log-uniform, in 1/Pa) and
gives the tet Young's modulus 1/c_t, i.e. both rows of the bake scaled by 1/(c_t E);
``young_deviatoric_uniform_volume`` keeps the (E, nu) deviatoric bake and gives every tet the
hydrostatic compliance ``volume_compliance``.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .grid import METERS_PER_UNIT, TissueGrid, build_grid
from .native_backend import Capsule, GraspParams, PlainTissue, blade_sweep

PARAMS_DIR = Path(__file__).resolve().parent / "params"
WORKLOADS = {"c1": "c1_plain.json", "c2": "c2_capsule.json", "c3": "c3_cutting.json", "c5": "c5_identification.json"}

# Contact defaults of the reference (g_gp, xpbd_solver.cu:284-287); the capsule workload changes
# only the approach-speed gate.
DEFAULT_GRASP = dict(capture=0.5, release=0.3, closed_gap=0.02, core_fraction=0.55, friction=0.3,
                     contact_compliance=1.0e-7, skin=0.02, ccd_velocity=0.5, ccd_displacement=0.045,
                     ccd_omega=0.25, grasp_omega=0.25, core_compliance=1.0e-7, break_force=150.0,
                     grasp_displacement=0.045, exempt_rings=1)


def load_params(name: str) -> dict:
    path = PARAMS_DIR / WORKLOADS.get(name, name)
    return json.loads(path.read_text())


def grid_for(params: dict, scale=None) -> TissueGrid:
    g = params["grid"]
    size = g["size"] if scale is None else scale
    return build_grid(g["spacing"], size=tuple(size), density=g["density_kg_m3"])


def material_moduli(young_pa, poisson):
    """Native-unit shear and bulk moduli in float32, as the reference bakes them."""
    e = np.float32(young_pa * METERS_PER_UNIT)
    nu = np.float32(poisson)
    mu = e / (np.float32(2) * (np.float32(1) + nu))
    kappa = e / (np.float32(3) * (np.float32(1) - np.float32(2) * nu))
    return np.float32(mu), np.float32(kappa)


def tet_stiffness(params: dict, baked_mu_v: np.ndarray, baked_kappa_v: np.ndarray):
    """Per-tet (mu*V, kappa*V) of a workload, storage order."""
    m = params["tet_material"]
    if m["mode"] == "young_deviatoric_uniform_volume":
        kappa_v = np.full(len(baked_mu_v), 1.0 / m["volume_compliance"], dtype=np.float32)
        return baked_mu_v.astype(np.float32), kappa_v
    if m["mode"] == "per_tet_compliance":
        scale = young_scale(per_tet_compliance(len(baked_mu_v), m["low"], m["high"], m["seed"]), scale_modulus(m))
        return (baked_mu_v * scale).astype(np.float32), (baked_kappa_v * scale).astype(np.float32)
    raise ValueError(f"unknown material mode {m['mode']}")


def scale_modulus(material: dict) -> float:
    """The modulus M of the compliance map scale = 1 / (c M).  Without a ``compliance_reference``,
    c is the tet's Young's compliance (1/Pa) and M the bake's Young's modulus; with one, c is
    relative to it (c = compliance_reference leaves the bake unscaled) and M = 1 / reference."""
    ref = material.get("compliance_reference")
    return float(material["young_pa"]) if ref is None else 1.0 / float(ref)


def young_scale(compliance, young_pa):
    """Stiffness multiplier of tets whose Young's modulus is 1/compliance (Pa), relative to the bake."""
    return (np.float32(1) / (compliance * np.float32(young_pa))).astype(np.float32)


def per_tet_compliance(count, low, high, seed):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(low), np.log(high), count)).astype(np.float32)


@dataclass
class Workload:
    """A ready-to-step scenario: grid, parameters and the per-step command schedule."""
    name: str
    params: dict
    grid: TissueGrid
    steps: int
    capsule_path: list = field(default_factory=list)   # Capsule per step (after the initial one)
    blade_path: list = field(default_factory=list)     # CutTool per step
    initial_capsule: Capsule | None = None

    def open(self, dll_path=None) -> PlainTissue:
        p = self.params
        grasp = None
        if p.get("instrument"):
            g = dict(DEFAULT_GRASP)
            g["ccd_velocity"] = p["instrument"]["ccd_velocity"]
            grasp = GraspParams(**g)
        m = p["tet_material"]
        tear = (p.get("blade") or {}).get("tear_ratio", 0.0)
        session = PlainTissue(self.grid, dt=p["dt"], substeps=p["substeps"], ks=1.0 / p["edge_compliance"],
                              young_pa=m["young_pa"], poisson=m["poisson"], strain_damping_s=p["strain_damping_s"],
                              tear_ratio=tear, grasp_params=grasp, dll_path=dll_path)
        try:
            baked_mu, baked_kappa = session.tet_stiffness()
            session.set_tet_stiffness(*tet_stiffness(p, baked_mu, baked_kappa))
            session.set_gravity(*p["gravity"])
            if self.initial_capsule is not None:
                session.set_capsule(self.initial_capsule)
        except Exception:
            session.close()
            raise
        return session

    def command(self, session: PlainTissue, step: int):
        """Send step ``step``'s instrument/blade pose; returns True when the rod-phase cut follows the step."""
        if self.capsule_path:
            session.set_capsule(self.capsule_path[step])
        if self.blade_path:
            session.set_blade(self.blade_path[step])
            return True
        return False

    def run(self, session: PlainTissue, steps=None, start=0, observe=None):
        for k in range(start, start + (self.steps if steps is None else steps)):
            detect = self.command(session, k)
            session.step(detect_cut=detect)
            if observe is not None:
                observe(k, session)


def _top(grid: TissueGrid) -> float:
    return float(grid.positions[grid.active != 0, 1].max())


def _half_extent(grid: TissueGrid):
    p = grid.positions[grid.active != 0]
    return (p.max(axis=0) - p.min(axis=0)) / 2, (p.max(axis=0) + p.min(axis=0)) / 2


def capsule_schedule(params: dict, grid: TissueGrid, steps: int):
    """Capsule of radius r and length L, axis horizontal at a seeded angle, centre at a seeded point of
    the top face; it starts ``clearance`` above the surface and descends linearly to ``press_depth``
    below it over ``steps`` steps."""
    ins = params["instrument"]
    rng = np.random.default_rng(ins["seed"])
    half, mid = _half_extent(grid)
    cx = mid[0] + rng.uniform(-0.4 * half[0], 0.4 * half[0])
    cz = mid[2] + rng.uniform(-0.4 * half[2], 0.4 * half[2])
    angle = rng.uniform(0.0, np.pi)
    axis = np.array((np.cos(angle), 0.0, np.sin(angle)))
    r, length = ins["radius"], ins["length"]
    top = _top(grid)
    y0, y1 = top + r + ins["clearance"], top + r - ins["press_depth"]

    def pose(y):
        c = np.array((cx, y, cz))
        return Capsule(tuple(c - axis * length / 2), tuple(c + axis * length / 2), r)

    return pose(y0), [pose(y0 + (y1 - y0) * (k + 1) / steps) for k in range(steps)]


def blade_schedule(params: dict, grid: TissueGrid, steps: int):
    """Blade edge: a vertical segment of length ``width`` whose lower end sits ``depth`` below the top
    surface, carried along a seeded polyline of ``segments`` segments across the top face at uniform
    arc-length speed; step k sweeps it from its pose at k-1 to its pose at k."""
    b = params["blade"]
    rng = np.random.default_rng(b["seed"])
    half, mid = _half_extent(grid)
    xs = mid[0] + np.linspace(-0.8 * half[0], 0.8 * half[0], b["segments"] + 1)
    zs = mid[2] + np.clip(np.cumsum(rng.uniform(-0.35, 0.35, b["segments"] + 1)) * half[2] * 0.3,
                          -0.7 * half[2], 0.7 * half[2])
    points = np.stack((xs, zs), axis=1)
    seg = np.linalg.norm(np.diff(points, axis=0), axis=1)
    arc = np.concatenate(([0.0], np.cumsum(seg)))
    top = _top(grid)
    lower, upper = top - b["depth"], top - b["depth"] + b["width"]

    def at(s):
        x = np.interp(s, arc, points[:, 0])
        z = np.interp(s, arc, points[:, 1])
        return (x, upper, z), (x, lower, z)

    poses = [at(arc[-1] * k / steps) for k in range(steps + 1)]
    tools = []
    for k in range(steps):
        (sp, ep), (s, e) = poses[k], poses[k + 1]
        tools.append(blade_sweep(sp, ep, s, e))
    return tools


def make(name: str, steps=None, scale=None) -> Workload:
    params = load_params(name)
    grid = grid_for(params, scale)
    n = params["steps"] if steps is None else steps
    w = Workload(params["name"], params, grid, n)
    if params.get("instrument"):
        w.initial_capsule, w.capsule_path = capsule_schedule(params, grid, max(n, params["steps"]))
    if params.get("blade"):
        w.blade_path = blade_schedule(params, grid, max(n, params["steps"]))
    return w


def bbox_diagonal(grid: TissueGrid) -> float:
    p = grid.positions[grid.active != 0]
    return float(np.linalg.norm(p.max(axis=0) - p.min(axis=0)))


def constraint_projections(grid_or_session, substeps: int, steps: int, live_edges: int, live_tets: int, contacts=0) -> int:
    """Projections per run: (live edge + live tet + contact) projections summed over substeps."""
    return int((live_edges + live_tets + contacts) * substeps * steps)
