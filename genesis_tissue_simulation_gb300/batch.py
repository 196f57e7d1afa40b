"""Batched tissue instances through the GBT_Batch* C ABI (one persistent launch per frame for all).

Each instance is a lattice from :func:`grid.build_grid` with the topology its own plain session
would build, so instance i of a batch evolves exactly as a :class:`native_backend.PlainTissue` of
the same grid and commands.  The C4 workload (``make_c4``) draws 256 instances of uneven size.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np

from .grid import METERS_PER_UNIT, TissueGrid, build_grid
from .native_backend import DEFAULT_DLL, Capsule, Grasper, GraspParams, V3, pointer

F, I, P = ct.c_float, ct.c_int32, ct.c_void_p


class GbtInstanceDesc(ct.Structure):
    _fields_ = [("dims_x", I), ("dims_y", I), ("dims_z", I), ("corner_pos", P), ("mass", P), ("pinned", P), ("active", P),
                ("nbr_idx", P), ("rest_nbr", P), ("bend_pairs", P), ("bend_pair_count", I), ("tet_mu_v", P),
                ("tet_kappa_v", P), ("stiffness_scale", F)]


class GbtBatchParams(ct.Structure):
    _fields_ = [("substeps", I)] + [(n, F) for n in ("ks", "cs", "kb", "cb", "alpha", "young", "poisson", "strain_damping")]


SIGNATURES = (
    ("GBT_BatchInit", (I, P, P), I), ("GBT_BatchSetGravity", (F, F, F), I), ("GBT_BatchSetGraspParams", (P,), None),
    ("GBT_BatchSetTools", (P,), I), ("GBT_BatchStep", (F,), I), ("GBT_BatchStepMany", (F, I, P, I), I),
    ("GBT_BatchGetPositions", (P,), I), ("GBT_BatchNodeRange", (I, P, P), I), ("GBT_BatchInfo", (P,), I),
    ("GBT_BatchSetLaunch", (I, I), I), ("GBT_BatchAutotune", (F, I, P, P, P), I), ("GBT_BatchProfileEnable", (I,), None),
    ("GBT_BatchProfileRead", (P,), I), ("GBT_BatchShutdown", (), None),
    ("GBT_BatchSetElementTables", (I,), I), ("GBT_BatchElementTables", (), I),
    ("GBT_BatchSetPacking", (I,), I), ("GBT_BatchPacking", (), I), ("GBT_BatchAutotuneTable", (I, P, P), I),
)


def capsule_tool(c: Capsule) -> Grasper:
    """XpbdToolState of a contact model 0 capsule; the jaw box is parked far away (zero size)."""
    far = (0.0, 1.0e4, 0.0)
    return Grasper(V3(*c.a), V3(*c.b), c.radius, V3(*far), V3(0, 0, 1), V3(*far), V3(1, 0, 0), 0.0, 0.0, 0.0, 0.0)


def tool_array(capsules) -> np.ndarray:
    """The same XpbdToolState records (23 float32, 92 B each) for capsules given as an array
    [..., 7] = (a xyz, b xyz, radius): one numpy fill instead of one ctypes record per instance."""
    c = np.asarray(capsules, dtype=np.float32)
    if c.shape[-1] != 7:
        raise ValueError("tool_array: capsules must be [..., 7] = (a xyz, b xyz, radius)")
    out = np.zeros(c.shape[:-1] + (23,), dtype=np.float32)
    out[..., :7] = c
    out[..., 8] = out[..., 14] = 1.0e4      # hinge and jaw centre parked at (0, 1e4, 0)
    out[..., 12] = 1.0                      # jaw axis (0, 0, 1)
    out[..., 16] = 1.0                      # jaw normal (1, 0, 0)
    return out


class TissueBatch:
    """Many tissue instances advanced together.  ``tet_stiffness[i]`` = (mu*V, kappa*V) per tet in storage
    order, or None for the (E, nu) bake; ``stiffness_scale[i]`` multiplies an instance's stiffnesses."""

    def __init__(self, grids, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, poisson=0.25, strain_damping_s=0.04,
                 tet_stiffness=None, stiffness_scale=None, grasp_params: GraspParams | None = None, dll_path=None):
        self.grids, self.dt = list(grids), float(dt)
        self.dll = ct.CDLL(str(dll_path or DEFAULT_DLL))
        self.f = {}
        for name, args, res in SIGNATURES:
            fn = self.dll[name]
            fn.argtypes, fn.restype = args, res
            self.f[name] = fn
        self._keep = []
        descs = (GbtInstanceDesc * len(self.grids))()
        for i, g in enumerate(self.grids):
            mu = kappa = None
            if tet_stiffness is not None and tet_stiffness[i] is not None:
                mu = np.ascontiguousarray(tet_stiffness[i][0], dtype=np.float32)
                kappa = np.ascontiguousarray(tet_stiffness[i][1], dtype=np.float32)
                self._keep += [mu, kappa]
            descs[i] = GbtInstanceDesc(*g.dims, pointer(g.positions), pointer(g.mass), pointer(g.pinned), pointer(g.active),
                                       pointer(g.neighbors), pointer(g.rest_neighbors), pointer(g.bends), len(g.positions) * 15,
                                       pointer(mu) if mu is not None else None, pointer(kappa) if kappa is not None else None,
                                       float(stiffness_scale[i]) if stiffness_scale is not None else 0.0)
        params = GbtBatchParams(int(substeps), ks, 0.0, 0.0, 0.0, 0.0, young_pa * METERS_PER_UNIT, poisson, strain_damping_s)
        self.check("GBT_BatchInit", len(self.grids), ct.byref(descs), ct.byref(params))
        self.closed = False
        if grasp_params is not None:
            self.f["GBT_BatchSetGraspParams"](ct.byref(grasp_params))
        self.ranges = []
        for i in range(len(self.grids)):
            base, count = I(), I()
            self.check("GBT_BatchNodeRange", i, ct.byref(base), ct.byref(count))
            self.ranges.append((base.value, count.value))
        self.total_nodes = sum(c for _, c in self.ranges)

    def check(self, name, *args):
        rc = self.f[name](*args)
        if rc != 0:
            raise RuntimeError(f"{name} failed with native status {rc}")

    def info(self):
        out = np.zeros(8, dtype=np.int32)
        self.check("GBT_BatchInfo", pointer(out))
        keys = ("instances", "nodes", "edges", "tets", "edge_colours", "tet_colours", "mode", "threads")
        return dict(zip(keys, (int(v) for v in out)))

    def set_grasp_params(self, grasp_params: GraspParams):
        """Contact parameters of every instance (XpbdGraspParams); a captured CUDA graph is recaptured."""
        self.f["GBT_BatchSetGraspParams"](ct.byref(grasp_params))

    def set_gravity(self, gx, gy, gz):
        self.check("GBT_BatchSetGravity", gx, gy, gz)

    def set_capsules(self, capsules):
        tools = (Grasper * len(self.grids))(*(capsule_tool(c) for c in capsules))
        self.check("GBT_BatchSetTools", ct.byref(tools))

    def step(self):
        self.check("GBT_BatchStep", self.dt)

    def step_many(self, capsules_per_step=None, steps=None, use_graph=True):
        """Advance ``steps`` frames (or ``len(capsules_per_step)``), one capsule per instance per frame:
        lists of Capsule per frame, or an array [frames, instances, 7] (a xyz, b xyz, radius)."""
        if isinstance(capsules_per_step, np.ndarray):
            if capsules_per_step.ndim != 3 or capsules_per_step.shape[1] != len(self.grids):
                raise ValueError("step_many: capsule array must be [frames, instances, 7]")
            tools = np.ascontiguousarray(tool_array(capsules_per_step))
            self.check("GBT_BatchStepMany", self.dt, int(tools.shape[0]), tools.ctypes.data_as(ct.c_void_p), int(use_graph))
        elif capsules_per_step is not None:
            steps = len(capsules_per_step)
            tools = (Grasper * (steps * len(self.grids)))(*(capsule_tool(c) for frame in capsules_per_step for c in frame))
            self.check("GBT_BatchStepMany", self.dt, steps, ct.byref(tools), int(use_graph))
        else:
            self.check("GBT_BatchStepMany", self.dt, int(steps), None, int(use_graph))

    def set_element_tables(self, implicit_codes: bool):
        """Implicit lattice codes (True) or explicit element tables (False) in the frame kernels."""
        self.check("GBT_BatchSetElementTables", int(bool(implicit_codes)))

    def element_tables(self) -> str:
        return "implicit" if self.f["GBT_BatchElementTables"]() else "explicit"

    def set_launch(self, mode, threads=256):
        self.check("GBT_BatchSetLaunch", mode, threads)

    def set_packing(self, packing):
        """Instance packing of the per-instance shapes: 0 LPT on tets, 1 LPT on tets + edges + nodes,
        2 size-ordered serpentine deal."""
        self.check("GBT_BatchSetPacking", int(packing))

    def packing(self) -> int:
        return int(self.f["GBT_BatchPacking"]())

    def autotune(self, trial_steps=3):
        """Time every launch configuration and keep the fastest.  Returns the chosen mode and threads,
        the best ms per frame of each of the six launch shapes, and every trial (mode, threads,
        packing, element tables, ms per frame; -1 where it cannot run this batch)."""
        mode, threads, ms = I(), I(), (F * 6)()
        self.check("GBT_BatchAutotune", self.dt, trial_steps, ct.byref(mode), ct.byref(threads), ms)
        n = int(self.f["GBT_BatchAutotuneTable"](0, None, None))
        shape = np.zeros((max(n, 1), 4), dtype=np.int32)
        times = np.zeros(max(n, 1), dtype=np.float32)
        self.f["GBT_BatchAutotuneTable"](n, pointer(shape), pointer(times))
        trials = [{"mode": int(r[0]), "threads": int(r[1]), "packing": int(r[2]), "element_tables": "implicit" if r[3] else "explicit",
                   "ms_per_frame": float(t)} for r, t in zip(shape[:n], times[:n])]
        return {"mode": mode.value, "threads": threads.value, "packing": self.packing(), "element_tables": self.element_tables(),
                "ms_per_frame": [float(v) for v in ms], "trials": trials}

    def positions(self, out=None):
        """Every instance's node positions [total_nodes, 3]; into `out` when given (float32, C order)."""
        if out is None:
            out = np.empty((self.total_nodes, 3), dtype=np.float32)
        elif out.shape != (self.total_nodes, 3) or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("positions: out must be a C-ordered float32 array of shape (total_nodes, 3)")
        self.check("GBT_BatchGetPositions", pointer(out))
        return out

    def instance_positions(self, all_positions, i):
        base, count = self.ranges[i]
        return all_positions[base:base + count]

    def profile(self, enabled):
        self.f["GBT_BatchProfileEnable"](int(enabled))

    def profile_read(self):
        ms = F()
        self.check("GBT_BatchProfileRead", ct.byref(ms))
        return ms.value

    def close(self):
        if not getattr(self, "closed", True):
            self.f["GBT_BatchShutdown"]()
            self.closed = True

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


@dataclass
class BatchWorkload:
    grids: list
    compliance: np.ndarray            # per instance, 1/Pa (Young's modulus 1/c)
    capsule_paths: list               # per instance: [initial, step 1, ..., step n]
    steps: int
    substeps: int = 10
    strain_damping_s: float = 0.0     # tall instances flatten under Kelvin-Voigt strain damping (see make_c4)

    def stiffness_scale(self, young_pa=6000.0):
        """Per-instance multiplier of the (E, nu) bake: Young's modulus 1/c (Pa) over E, in FP32."""
        return (np.float32(1) / (self.compliance.astype(np.float32) * np.float32(young_pa))).astype(np.float32)

    def capsules_at(self, step):
        return [path[min(step, len(path) - 1)] for path in self.capsule_paths]

    def capsule_array_at(self, step):
        """capsules_at(step) as an array [instances, 7] = (a xyz, b xyz, radius)."""
        if getattr(self, "_capsule_table", None) is None:
            longest = max(len(p) for p in self.capsule_paths)
            self._capsule_table = np.array([[(*p[min(k, len(p) - 1)].a, *p[min(k, len(p) - 1)].b, p[min(k, len(p) - 1)].radius)
                                             for k in range(longest)] for p in self.capsule_paths], dtype=np.float32)
        return self._capsule_table[:, min(step, self._capsule_table.shape[1] - 1)]

    def subset(self, indices):
        """The instances `indices` (in that order) as a workload of their own."""
        idx = [int(i) for i in indices]
        return BatchWorkload([self.grids[i] for i in idx], self.compliance[idx], [self.capsule_paths[i] for i in idx],
                             self.steps, self.substeps, self.strain_damping_s)


def shard_instances(costs, world):
    """Split instances over `world` GPUs with no exchange between them: longest-processing-time
    assignment by cost (e.g. tets + edges per instance), ties to the lowest rank.  Returns one
    ascending index list per rank; every instance lands on exactly one rank."""
    costs = np.asarray(costs, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be at least 1")
    loads = np.zeros(world)
    shards = [[] for _ in range(world)]
    for i in np.argsort(-costs, kind="stable"):
        r = int(np.argmin(loads))
        shards[r].append(int(i))
        loads[r] += costs[i]
    return [sorted(s) for s in shards]


def gather_instance_positions(shards, local, rank, world, dst=0):
    """The only exchange of a sharded batch: rank `dst` receives every rank's instance positions.
    `shards` is shard_instances' split, `local` this rank's positions of its own instances (list, in
    its shard's order).  Returns the positions of all instances in instance order on `dst`, None on
    the other ranks.  Uses torch.distributed (gloo or NCCL; with NCCL the current CUDA device must
    be set)."""
    import torch.distributed as dist
    if world == 1:
        return list(local)
    if len(local) != len(shards[rank]):
        raise ValueError("gather_instance_positions: one array per instance of this rank's shard")
    parts = [None] * world if rank == dst else None
    dist.gather_object([np.ascontiguousarray(p) for p in local], parts, dst=dst)
    if rank != dst:
        return None
    out = [None] * sum(len(s) for s in shards)
    for r, shard in enumerate(shards):
        for j, i in enumerate(shard):
            out[i] = parts[r][j]
    return out


def instance_costs(workload):
    """Per-instance cost for sharding: lattice edges plus tets, from the grids alone."""
    costs = []
    for g in workload.grids:
        cells = int(np.prod(g.dims))
        costs.append(float(len(g.edges)) + 6.0 * cells)
    return costs


def make_c4(count=256, seed=4, steps=100, substeps=10, low=1e-7, high=1e-5, size_range=((8, 32), (4, 16), (8, 32))):
    """256 instances with cells x, y(up), z drawn uniformly from [8,32] x [4,16] x [8,32], one log-uniform
    compliance per instance, and a capsule per instance pressed into its top face over ``steps`` steps.

    Strain damping is 0: with the 0.04 s default, each substep's elastic correction is divided by
    1 + 0.04/h = 25, and one Gauss-Seidel pass per substep then lets columns taller than about eight
    cells flatten under gravity."""
    rng = np.random.default_rng(seed)
    grids, paths = [], []
    for _ in range(count):
        cells = [int(rng.integers(lo, hi + 1)) for lo, hi in size_range]
        size = tuple(np.float64(c) * 0.2 - 0.02 for c in cells)
        g = build_grid(0.2, size=size, density=1000.0)
        grids.append(g)
        p = g.positions[g.active != 0]
        lo, hi = p.min(axis=0), p.max(axis=0)
        mid, half = (lo + hi) / 2, (hi - lo) / 2
        angle = rng.uniform(0.0, np.pi)
        axis = np.array((np.cos(angle), 0.0, np.sin(angle)))
        length = 0.6 * float(min(half[0], half[2])) * 2
        r = 0.25
        cx = mid[0] + rng.uniform(-0.2, 0.2) * half[0]
        cz = mid[2] + rng.uniform(-0.2, 0.2) * half[2]
        y0, y1 = hi[1] + r + 0.05, hi[1] + r - 0.25 * (hi[1] - lo[1])

        def pose(y, cx=cx, cz=cz, axis=axis, length=length, r=r):
            c = np.array((cx, y, cz))
            return Capsule(tuple(c - axis * length / 2), tuple(c + axis * length / 2), r)

        paths.append([pose(y0)] + [pose(y0 + (y1 - y0) * (k + 1) / steps) for k in range(steps)])
    compliance = np.exp(rng.uniform(np.log(low), np.log(high), count))
    return BatchWorkload(grids, compliance, paths, steps, substeps)
