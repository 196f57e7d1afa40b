"""Differentiable tissue rollouts: the GBT_Diff* C ABI behind a ``torch.autograd.Function``.

A rollout advances F frames of the plain XPBD step (predict, lattice edges, unguarded Neo-Hookean
tets, capsule contact, velocity) from a fixed origin, with per-tet log-compliances ``theta`` (tet
storage order, as ``LCS_SetTetStiffness``) and a capsule path of F + 1 commands (end points a, b),
and returns the final node positions.  The backward is the library's hand-written adjoint of the
substep: node states are checkpointed every k substeps in the forward; the backward recomputes
each segment with a tape and sweeps it in reverse (tet colours last to first, then edge colours,
then predict), on the GPU, in one launch.

The reference solver is not differentiable; the forward is the plain path of its XPBD step
(V/xpbd/xpbd_solver.cu:3460-3721 plain branch, "V/" = endoscopic_tissue/native/vendor/cuda/) with
the material expressed as a per-tet compliance scale of the baked Neo-Hookean stiffness.

The C5 identification workload (:func:`make_c5`): 32 x 16(up) x 32 cells, a hidden seeded
log-compliance field produces the target top-surface positions; the loss is their MSE.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np
import torch

from . import workloads as W
from .grid import TissueGrid
from .native_backend import GraspParams, PlainTissue

F, I, P = ct.c_float, ct.c_int32, ct.c_void_p

SIGNATURES = (
    ("GBT_DiffBegin", (F, I, I), I), ("GBT_DiffForward", (F, I, P, P, F, P), I),
    ("GBT_DiffBackward", (P, P, P, P, P, P), I), ("GBT_DiffInfo", (P,), I), ("GBT_DiffEnd", (), None),
    ("LCS_SetLaunchMode", (I,), I),
)


def _ptr(t: torch.Tensor | None):
    return None if t is None else ct.c_void_p(t.data_ptr())


class DifferentiableTissue:
    """A differentiable rollout on one tissue grid (one LCS session; one instance per process).

    ``launch_mode``: 0 automatic, 1 whole-GPU cooperative grid, 2 one CTA.  ``max_frames`` sizes the
    checkpoint buffers; ``checkpoint_every`` is k in substeps.  A log-compliance theta scales the
    (E, nu) bake of each tet by 1 / (exp(theta) M), M = ``scale_modulus`` (default: ``young_pa``, so
    exp(theta) is the tet's Young's compliance in 1/Pa).
    """

    def __init__(self, grid: TissueGrid, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, poisson=0.25, strain_damping_s=0.04,
                 gravity=(0.0, -981.0, 0.0), grasp_params: GraspParams | None = None, capsule_radius=0.25, checkpoint_every=5,
                 max_frames=50, launch_mode=0, dll_path=None, scale_modulus=None):
        if not torch.cuda.is_available():
            raise RuntimeError("the differentiable rollout runs on a CUDA device; no CUDA device is visible")
        self.grid, self.dt, self.substeps, self.radius = grid, float(dt), int(substeps), float(capsule_radius)
        self.young_pa, self.max_frames, self.every = float(young_pa), int(max_frames), int(checkpoint_every)
        self.session = PlainTissue(grid, dt=dt, substeps=substeps, ks=ks, young_pa=young_pa, poisson=poisson,
                                   strain_damping_s=strain_damping_s, grasp_params=grasp_params, dll_path=dll_path)
        try:
            self.f = {}
            for name, args, result in SIGNATURES:
                fn = self.session.dll[name]
                fn.argtypes, fn.restype = args, result
                self.f[name] = fn
            self.session.set_gravity(*gravity)
            self._check("LCS_SetLaunchMode", int(launch_mode))
            self.scale_modulus = float(scale_modulus if scale_modulus is not None else young_pa)
            self._check("GBT_DiffBegin", self.scale_modulus, self.every, self.max_frames)
        except Exception:
            self.session.close()
            raise
        self.n_nodes = len(grid.positions)
        self.tet_count = self.session.tet_count
        self.device = torch.device("cuda", torch.cuda.current_device())
        self._generation = 0
        self._frames = 0

    def _check(self, name, *args):
        rc = self.f[name](*args)
        if rc != 0:
            raise RuntimeError(f"{name} failed with native status {rc}")

    def info(self):
        out = np.zeros(4, dtype=np.int32)
        self._check("GBT_DiffInfo", out.ctypes.data_as(P))
        return {"grid_launch": bool(out[0]), "ctas": int(out[1]), "checkpoint_every": int(out[2]), "max_frames": int(out[3])}

    # -- raw calls (no autograd) ----------------------------------------------------------------
    def forward(self, log_compliance: torch.Tensor, capsule_path: torch.Tensor | None, frames: int | None = None) -> torch.Tensor:
        """Final node positions [N, 3] of a rollout; ``frames`` defaults to len(capsule_path) - 1."""
        theta = log_compliance.detach().to(self.device, torch.float32).contiguous()
        if theta.numel() != self.tet_count:
            raise ValueError(f"log_compliance has {theta.numel()} entries, the mesh has {self.tet_count} tets")
        path = None
        if capsule_path is not None:
            path = capsule_path.detach().to(self.device, torch.float32).contiguous()
            if path.dim() != 2 or path.shape[1] != 6:
                raise ValueError("capsule_path must be [frames + 1, 6]")
            frames = path.shape[0] - 1
        if frames is None or frames < 1:
            raise ValueError("a rollout needs at least one frame")
        out = torch.empty((self.n_nodes, 3), dtype=torch.float32, device=self.device)
        torch.cuda.current_stream(self.device).synchronize()
        self._check("GBT_DiffForward", self.dt, int(frames), _ptr(theta), _ptr(path), self.radius, _ptr(out))
        self._generation += 1
        self._frames = int(frames)
        return out

    def backward(self, grad_positions: torch.Tensor, rest_shape=False, origin=False) -> dict:
        """Adjoints of the last forward: ``theta`` [T], ``path`` [F + 1, 6]; with ``rest_shape`` also
        ``rest_length`` [N, 6] (per directed lattice slot) and ``rest_inverse`` [T, 3, 3]; with
        ``origin`` the origin state's ``origin_position`` and ``origin_velocity`` [N, 3]."""
        g = grad_positions.detach().to(self.device, torch.float32).contiguous()
        dev = dict(dtype=torch.float32, device=self.device)
        out = {"theta": torch.empty(self.tet_count, **dev), "path": torch.empty((self._frames + 1, 6), **dev)}
        rest_len = torch.empty((self.n_nodes, 6), **dev) if rest_shape else None
        rest_inv = torch.empty((self.tet_count, 3, 3), **dev) if rest_shape else None
        org = torch.empty((2, self.n_nodes, 3), **dev) if origin else None
        torch.cuda.current_stream(self.device).synchronize()
        self._check("GBT_DiffBackward", _ptr(g), _ptr(out["theta"]), _ptr(out["path"]), _ptr(rest_len), _ptr(rest_inv), _ptr(org))
        if rest_shape:
            out["rest_length"], out["rest_inverse"] = rest_len, rest_inv
        if origin:
            out["origin_position"], out["origin_velocity"] = org[0], org[1]
        return out

    # -- autograd -------------------------------------------------------------------------------
    def rollout(self, log_compliance: torch.Tensor, capsule_path: torch.Tensor | None = None, frames: int | None = None) -> torch.Tensor:
        """Final node positions, differentiable with respect to ``log_compliance`` and ``capsule_path``.
        One rollout at a time: its backward must run before the next rollout's forward."""
        path = capsule_path if capsule_path is not None else torch.empty(0, device=self.device)
        return _Rollout.apply(log_compliance, path, self, frames)

    def close(self):
        if getattr(self, "session", None) is not None and not self.session.closed:
            self.f["GBT_DiffEnd"]()
            self.session.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, log_compliance, capsule_path, tissue: DifferentiableTissue, frames):
        has_path = capsule_path.numel() > 0
        out = tissue.forward(log_compliance, capsule_path if has_path else None, frames)
        ctx.tissue, ctx.generation, ctx.has_path = tissue, tissue._generation, has_path
        ctx.theta_dtype, ctx.path_dtype = log_compliance.dtype, capsule_path.dtype
        return out

    @staticmethod
    def backward(ctx, grad_positions):
        tissue = ctx.tissue
        if tissue._generation != ctx.generation:
            raise RuntimeError("another rollout ran after this one; its checkpoints are gone (backward one rollout at a time)")
        g = tissue.backward(grad_positions)
        g_theta = g["theta"].to(ctx.theta_dtype) if ctx.needs_input_grad[0] else None
        g_path = g["path"].to(ctx.path_dtype) if (ctx.needs_input_grad[1] and ctx.has_path) else None
        return g_theta, g_path, None, None


def rest_position_gradient(grid: TissueGrid, tet_ids: np.ndarray, rest_length: np.ndarray, rest_inverse: np.ndarray) -> np.ndarray:
    """Chain the rest-shape adjoints to the rest node positions X [N, 3] (lumped masses and baked
    stiffnesses held fixed): each tet's rest inverse is Dm^-1 with Dm = [X1 - X0, X2 - X0, X3 - X0]
    (d Dm^-1 = -Dm^-1 dDm Dm^-1), each lattice edge's rest length is |X_nbr - X_p|."""
    X = grid.positions.astype(np.float64)
    g = np.zeros_like(X)
    ids = np.asarray(tet_ids, dtype=np.int64)
    Dm = np.stack([X[ids[:, k]] - X[ids[:, 0]] for k in (1, 2, 3)], axis=2)      # columns
    B = np.linalg.inv(Dm)
    gB = np.asarray(rest_inverse, dtype=np.float64).reshape(-1, 3, 3)
    gDm = -np.einsum("tji,tjk,tlk->til", B, gB, B)                                # -B^T gB B^T
    for k in (1, 2, 3):
        np.add.at(g, ids[:, k], gDm[:, :, k - 1])
        np.add.at(g, ids[:, 0], -gDm[:, :, k - 1])
    gl = np.asarray(rest_length, dtype=np.float64).reshape(-1, 6)
    p, s = np.nonzero(gl)
    q = grid.neighbors[p, s]
    ok = q >= 0
    p, s, q = p[ok], s[ok], q[ok]
    d = X[q] - X[p]
    u = d / np.linalg.norm(d, axis=1, keepdims=True)
    np.add.at(g, q, u * gl[p, s, None])
    np.add.at(g, p, -u * gl[p, s, None])
    return g


# ------------------------------------------------------------------------------------------------
# C5: differentiable identification
# ------------------------------------------------------------------------------------------------
@dataclass
class Identification:
    params: dict
    grid: TissueGrid
    frames: int
    theta_hidden: np.ndarray     # [T] log-compliance producing the target (storage order)
    theta_initial: np.ndarray    # [T] the estimate gradients are taken at
    path: np.ndarray             # [frames + 1, 6] capsule end points per command
    radius: float
    top: np.ndarray              # node ids of the top surface

    def open(self, dll_path=None, launch_mode=0, max_frames=None) -> DifferentiableTissue:
        p = self.params
        m = p["tet_material"]
        grasp = GraspParams(**dict(W.DEFAULT_GRASP, ccd_velocity=p["instrument"]["ccd_velocity"]))
        return DifferentiableTissue(self.grid, dt=p["dt"], substeps=p["substeps"], ks=1.0 / p["edge_compliance"], young_pa=m["young_pa"],
                                    poisson=m["poisson"], strain_damping_s=p["strain_damping_s"], gravity=tuple(p["gravity"]),
                                    grasp_params=grasp, capsule_radius=self.radius, checkpoint_every=p["checkpoint_every"],
                                    max_frames=max_frames or self.frames, launch_mode=launch_mode, dll_path=dll_path,
                                    scale_modulus=W.scale_modulus(m))


def make_c5(frames=None, scale=None) -> Identification:
    params = W.load_params("c5")
    grid = W.grid_for(params, scale)
    n = params["steps"] if frames is None else frames
    initial, path = W.capsule_schedule(params, grid, n)
    caps = [initial] + path[:n]
    arr = np.array([list(c.a) + list(c.b) for c in caps], dtype=np.float32)
    m = params["tet_material"]
    tets = _tet_count(grid)
    hidden = np.log(W.per_tet_compliance(tets, m["low"], m["high"], m["seed"])).astype(np.float32)
    initial_theta = np.full(tets, params["initial_log_compliance"], dtype=np.float32)
    top_y = grid.positions[grid.active != 0, 1].max()
    top = np.nonzero((grid.active != 0) & (np.abs(grid.positions[:, 1] - top_y) < 1e-6))[0]
    return Identification(params, grid, n, hidden, initial_theta, arr, float(params["instrument"]["radius"]), top)


def _tet_count(grid: TissueGrid) -> int:
    """Kuhn tets of the lattice: 6 per cell whose 8 corners are active."""
    a = (grid.active != 0).reshape(grid.dims[2] + 1, grid.dims[1] + 1, grid.dims[0] + 1)
    cell = a[:-1, :-1, :-1] & a[1:, :-1, :-1] & a[:-1, 1:, :-1] & a[1:, 1:, :-1] & a[:-1, :-1, 1:] & a[1:, :-1, 1:] & a[:-1, 1:, 1:] & a[1:, 1:, 1:]
    return int(cell.sum()) * 6


def identification_loss(positions: torch.Tensor, target: torch.Tensor, top: torch.Tensor) -> torch.Tensor:
    """MSE between the top-surface node positions and the target's."""
    return ((positions[top] - target[top]) ** 2).mean()
