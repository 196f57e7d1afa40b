"""Small differentiable-rollout cases shared by the adjoint tests: a lattice, a capsule path that
presses into its top, log-compliances, and the oracle's ORC_Diff* bindings."""
from __future__ import annotations

import ctypes as ct
import importlib.util
from pathlib import Path

import numpy as np

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import GraspParams, PlainTissue

ROOT = Path(__file__).resolve().parents[1]
F, I, D, P = ct.c_float, ct.c_int32, ct.c_double, ct.c_void_p
YOUNG = 6000.0
GRASP = dict(W.DEFAULT_GRASP, ccd_velocity=0.0)


def torch_rollout_module():
    spec = importlib.util.spec_from_file_location("torch_rollout", ROOT / "oracle" / "torch_rollout.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def bind_oracle(dll):
    for name, args, res in (("ORC_DiffBegin", (D, I, I), I), ("ORC_DiffForward", (F, I, P, P, D, P), I),
                            ("ORC_DiffBackward", (P,) * 6, I), ("ORC_DiffEnd", (), None), ("ORC_TopologySizes", (P,), I),
                            ("ORC_ExportTopology", (P,) * 13, I), ("ORC_Parameters", (P,), I)):
        fn = getattr(dll, name)
        fn.argtypes, fn.restype = args, res
    return dll


def ptr(a):
    return None if a is None else a.ctypes.data_as(P)


class Case:
    """A small lattice with a capsule pressed into its top over ``frames`` frames."""

    def __init__(self, size=(1.38, 0.78, 1.18), frames=4, substeps=4, every=3, seed=3, press=0.35, dt=1 / 60):
        self.grid = build_grid(0.2, size=size, density=1000.0)
        self.frames, self.substeps, self.every, self.dt = frames, substeps, every, dt
        params = {"instrument": {"radius": 0.25, "length": 0.9, "press_depth": press, "clearance": 0.02, "seed": seed}}
        first, rest = W.capsule_schedule(params, self.grid, frames)
        caps = [first] + rest[:frames]
        self.path = np.array([list(c.a) + list(c.b) for c in caps], dtype=np.float32)
        self.radius = 0.25
        rng = np.random.default_rng(seed)
        self.n = len(self.grid.positions)
        self.rng = rng

    def session(self, lib):
        s = PlainTissue(self.grid, dt=self.dt, substeps=self.substeps, ks=1e6, young_pa=YOUNG, poisson=0.25, strain_damping_s=0.04,
                        grasp_params=GraspParams(**GRASP), dll_path=lib)
        s.set_gravity(0.0, -981.0, 0.0)
        return s

    def theta(self, tets, seed=7):
        rng = np.random.default_rng(seed)
        return rng.uniform(np.log(1e-7), np.log(1e-5), tets).astype(np.float32)


class C5Oracle:
    """The C5 identification workload on an oracle build (FP32 or FP64): target, loss gradient."""

    def __init__(self, lib, frames=None):
        from genesis_tissue_simulation_gb300 import diff as D
        self.c5 = c5 = D.make_c5(frames=frames)
        p, m = c5.params, c5.params["tet_material"]
        self.session = PlainTissue(c5.grid, dt=p["dt"], substeps=p["substeps"], ks=1 / p["edge_compliance"], young_pa=m["young_pa"],
                                   poisson=m["poisson"], strain_damping_s=p["strain_damping_s"], grasp_params=GraspParams(**GRASP), dll_path=lib)
        self.session.set_gravity(*p["gravity"])
        self.dll = bind_oracle(self.session.dll)
        self.n, self.T, self.dt = len(c5.grid.positions), self.session.tet_count, p["dt"]
        assert self.dll.ORC_DiffBegin(W.scale_modulus(m), p["checkpoint_every"], c5.frames) == 0
        self.target = self.positions(c5.theta_hidden, c5.path)

    def positions(self, theta, path):
        out = np.zeros((self.n, 3))
        rc = self.dll.ORC_DiffForward(self.dt, self.c5.frames, ptr(np.ascontiguousarray(theta, np.float64)),
                                      ptr(np.ascontiguousarray(path, np.float64)), self.c5.radius, ptr(out))
        assert rc == 0, rc
        return out

    def loss(self, theta, path):
        x, top = self.positions(theta, path), self.c5.top
        return float(((x[top] - self.target[top]) ** 2).mean())

    def loss_gradient(self, x):
        top = self.c5.top
        g = np.zeros((self.n, 3))
        g[top] = 2.0 * (x[top] - self.target[top]) / (3 * len(top))
        return g

    def gradient(self, theta, path):
        x = self.positions(theta, path)
        gt, gp = np.zeros(self.T), np.zeros((self.c5.frames + 1, 6))
        assert self.dll.ORC_DiffBackward(ptr(self.loss_gradient(x)), ptr(gt), ptr(gp), None, None, None) == 0
        return gt, gp

    def close(self):
        self.dll.ORC_DiffEnd()
        self.session.close()


def oracle_rollout(dll, case: Case, theta, path, every=None, frames=None):
    """(final positions [N, 3], hand adjoint function) of an oracle session already begun."""
    frames = case.frames if frames is None else frames
    th = np.ascontiguousarray(theta, dtype=np.float64)
    pa = None if path is None else np.ascontiguousarray(path, dtype=np.float64)
    out = np.zeros((case.n, 3))
    rc = dll.ORC_DiffForward(case.dt, frames, ptr(th), ptr(pa), case.radius, ptr(out))
    assert rc == 0, rc
    return out


def oracle_adjoint(dll, case: Case, grad_pos, tets, frames=None, rest=False, origin=False):
    frames = case.frames if frames is None else frames
    g = np.ascontiguousarray(grad_pos, dtype=np.float64)
    gt = np.zeros(tets)
    gp = np.zeros((frames + 1, 6))
    gl = np.zeros((case.n, 6)) if rest else None
    gb = np.zeros((tets, 9)) if rest else None
    go = np.zeros((2, case.n, 3)) if origin else None
    rc = dll.ORC_DiffBackward(ptr(g), ptr(gt), ptr(gp), ptr(gl), ptr(gb), ptr(go))
    assert rc == 0, rc
    return {"theta": gt, "path": gp, "rest_length": gl, "rest_inverse": gb, "origin": go}
