"""ctypes adapter for the LCS_* C ABI of the tissue solver.

Mirrors the reference adapter ``endoscopic_tissue/native_backend.py`` (structs 22-81, ``Settings`` 84-123,
``Command`` 126-137, ``NativeTissue`` 212-483): the same struct layouts, the same signature table style
and the same error behaviour (a non-zero native status raises ``RuntimeError(name + status)``,
native_backend.py:284-287).  The default library is this package's CUDA build
``csrc/_build/libgbtissue.so``; passing ``dll_path`` drives any library exporting the same ABI.

Two session classes sit on top of the ABI:

* :class:`NativeTissue` keeps the reference class's constructor and call sequence unchanged.  Its
  initialisation arms the reference's unified contact/grasp solver, which this library does not
  provide, so against this library it stops with the native status of the first unsupported call.
* :class:`PlainTissue` drives the plain XPBD branch through the same entry points: lattice upload,
  physics, cut, gravity, step, optional capsule instrument and geometric blade, observation.
"""
from __future__ import annotations

import ctypes as ct
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .grid import METERS_PER_UNIT, TissueGrid

F = ct.c_float
I = ct.c_int32
P = ct.c_void_p
V3 = F * 3

PACKAGE_DIR = Path(__file__).resolve().parent
DEFAULT_DLL = PACKAGE_DIR / "csrc" / "_build" / "libgbtissue.so"

# Status codes (xpbd_solver.h:25-33 band, plus this library's "not available in this build").
XPBD_ERR_NOT_READY = -1000
XPBD_ERR_NO_FRAME = -1001
XPBD_ERR_BAD_DT = -1002
XPBD_ERR_COLOR_OVERFLOW = -1003
XPBD_ERR_BAD_ARG = -1004
XPBD_ERR_IRREGULAR_REST = -1005
LCS_ERR_UNSUPPORTED = -4001
LCS_ERR_DEVICE_TIMEOUT = -4002


class ReconDesc(ct.Structure):
    _fields_ = [(name, I) for name in (
        "voxels", "nodes", "intersections", "surface_edges", "tri_capacity", "nx", "ny", "nz")]
    _fields_ += [("spacing", F), ("qef_iterations", I)]


class PhysicsDesc(ct.Structure):
    _fields_ = [("nodes", I), ("bends", I)]
    _fields_ += [(name, F) for name in ("ks", "cs", "kb", "cb", "h_init", "h_max")]
    _fields_ += [("substeps", I)]
    _fields_ += [(name, F) for name in ("alpha", "young", "poisson", "strain_damping")]


class CutDesc(ct.Structure):
    _fields_ = [(name, I) for name in (
        "voxels", "nodes", "edges", "intersections", "tri_capacity", "nx", "ny", "nz")]
    _fields_ += [("spacing", F), ("origin", V3), ("point_capacity", I), ("interpolation", F), ("tear_ratio", F)]


class CutTool(ct.Structure):
    _fields_ = [(name, V3) for name in ("t1a", "t1b", "t1c", "t2a", "t2b", "t2c", "normal")]
    _fields_ += [("thickness", F), ("valid", I), ("low", V3), ("high", V3)]


class Grasper(ct.Structure):
    _fields_ = [("shaft_a", V3), ("shaft_b", V3), ("radius", F)]
    _fields_ += [(name, V3) for name in ("hinge", "axis", "mid", "normal")]
    _fields_ += [(name, F) for name in ("half_width", "length", "gap", "closure")]


class GraspParams(ct.Structure):
    _fields_ = [(name, F) for name in (
        "capture", "release", "closed_gap", "core_fraction", "friction", "contact_compliance",
        "skin", "ccd_velocity", "ccd_displacement", "ccd_omega", "grasp_omega",
        "core_compliance", "break_force", "grasp_displacement")]
    _fields_ += [("exempt_rings", I)]


class Blade(ct.Structure):
    _fields_ = [("a", V3), ("b", V3)]
    _fields_ += [(name, F) for name in ("radius", "start_force", "cut_force", "stiffness", "mass", "friction")]
    _fields_ += [("enabled", I)]


class ScissorsBack(ct.Structure):
    _fields_ = [(name, V3) for name in ("center", "half_size", "axis_x", "axis_y")]


class ScissorsControl(ct.Structure):
    _fields_ = [(name, V3) for name in ("hinge", "axis", "normal", "left_a", "left_b", "right_a", "right_b")]
    _fields_ += [(name, F) for name in ("length", "gap", "max_gap", "jaw_speed", "start_force", "cut_force",
                                      "stiffness", "mass", "friction", "jaw_mass", "jaw_stiffness")]
    _fields_ += [(name, I) for name in ("enabled", "cutting", "guided")]
    _fields_ += [("left_back", ScissorsBack), ("right_back", ScissorsBack), ("back_contact", I), ("squeeze", F)]


class ScissorsResult(ct.Structure):
    _fields_ = [(name, V3) for name in ("hinge", "axis", "normal", "left_a", "left_b", "right_a", "right_b")]
    _fields_ += [(name, F) for name in ("gap", "radius", "pressure", "mass", "jaw_mass")]
    _fields_ += [("force", V3), ("phase", I), ("contacts", I)]


@dataclass(frozen=True)
class Settings:
    """Session settings; field names and defaults of native_backend.py:84-123."""
    dt: float = 1 / 30
    substeps: int = 3
    young_pa: float = 6000
    poisson: float = 0.25
    strain_damping_s: float = 0.04
    density_kg_m3: float = 1050
    jaw_length: float = 1.99
    jaw_width: float = 0.52
    jaw_open_gap: float = 1.0
    jaw_axis: tuple = (0.0, -0.8, 0.6)
    jaw_normal: tuple = (1.0, 0.0, 0.0)
    blade_length: float = 1.6
    blade_radius: float = 0.04
    blade_axis: tuple = (2 ** -.5, 0.0, 2 ** -.5)
    start_force_n: float = 0.2
    cut_force_n: float = 0.12
    blade_drive_stiffness: float = 1200
    blade_mass_kg: float = 0.02
    blade_friction: float = 0.15
    blade_preload_n: float = 1.0
    contact_refine_passes: int = 8
    has_knife_body: bool = True
    instrument_model: str = "davinci"
    cutting_tool: str = "knife"
    scissors_jaw_stiffness: float = 150
    scissors_squeeze_cm: float = .2
    contact_model: int = 2


@dataclass(frozen=True)
class Command:
    """Per-step instrument command; fields of native_backend.py:126-137."""
    hinge: tuple = (-1.4, 3.384, -2.288)
    closure: float = 0.0
    blade_center: tuple = (0.2, 2.2, -0.6)
    blade_enabled: bool = True
    scissors_closure: float = 0.0
    scissors_cutting: bool = False
    scissors_pitch_deg: float = 19.9
    scissors_roll_deg: float = 0.0
    scissors_yaw_deg: float = 0.0


@dataclass
class Observation:
    """Per-step readback (native_backend.py:182-196); fields this library has no data for stay empty."""
    nodes: np.ndarray
    neighbors: np.ndarray
    grip_flags: np.ndarray
    hinge: np.ndarray
    jaw_gap: float
    grip_points: int
    grip_error_m: float
    blade: np.ndarray
    reaction_n: np.ndarray
    scissors: object = None
    jaw_load_n: tuple = (0.0, 0.0)


def pointer(array):
    assert array.flags.c_contiguous
    return array.ctypes.data_as(P)


# Entry points of the plain path: (name, argtypes, restype).  The reference's own table is
# native_backend.py:230-256; the last block lists this library's diagnostics and extensions.
CORE_SIGNATURES = (
    ("LCS_Init", (P,) * 7, I), ("LCS_InitPhysics", (P,) * 8, I),
    ("LCS_InitCut", (P,) * 5, I), ("LCS_SetTool", (P,), None),
    ("LCS_PhysicsAbiVersion", (), I), ("LCS_GraspToolAbiVersion", (), I), ("LCS_ContactModelVersion", (), I),
    ("LCS_SetGraspParams", (P,), None), ("LCS_SetGraspTool", (P,), I),
    ("LCS_SetPressureCutMode", (I,), None), ("LCS_SetContactModel", (I, F, F, F, F), I),
    ("LCS_SetTissueGuard", (F, I, I, P, I), I), ("LCS_SetTissueMaterial", (F, F), I),
    ("LCS_SetGravity", (F, F, F), I), ("LCS_Step", (F,), I), ("LCS_Finalize", (), I), ("LCS_DetectCut", (), I),
    ("LCS_GetCornerPos", (P,), I), ("LCS_GetNbrIdx", (P,), I), ("LCS_GetTopologyRevision", (P,), I),
    ("LCS_GetCutEdgeFractions", (P,), I), ("LCS_GetCutDebug", (P, P), I),
    ("LCS_ProfileEnable", (I,), None), ("LCS_ProfileRead", (I, P), I), ("LCS_Shutdown", (), None),
    ("LCS_GetSurfaceCounts", (P, P), I), ("LCS_GetSurface", (P, P, P), I), ("LCS_GetSurfaceAux", (P,), I),
)
EXTENSION_SIGNATURES = (
    ("LCS_SetTetStiffness", (I, P, P), I), ("LCS_GetTetStiffness", (P, P), I), ("LCS_TetCount", (), I), ("LCS_TetColorCount", (), I),
    ("LCS_EdgeColorCount", (), I), ("LCS_EdgeCount", (), I), ("LCS_GetTetIds", (P,), I),
    ("LCS_GetTetColors", (P,), I), ("LCS_GetEdgeColors", (P,), I), ("LCS_GetVelocities", (P,), I),
    ("LCS_GetBendPairs", (P,), I), ("LCS_GetVoxelCutMask", (P,), I), ("GBT_GetParticleRot", (P,), I),
    ("GBT_GetSurfaceTriangles", (P,), I), ("GBT_CutTopologyBuild", (P,), I), ("GBT_GetCutTopology", (P, P, P, P), I),
)
UNIFIED_SIGNATURES = (
    ("LCS_PressureBladeAbiVersion", (), I), ("LCS_SetPressureBlade", (P,), I),
    ("LCS_ScissorsAbiVersion", (), I), ("LCS_ScissorsResultAbiVersion", (), I),
    ("LCS_SetScissors", (P,), I), ("LCS_GetScissors", (P,), I),
    ("LCS_SetJawGeometry", (P,), I), ("LCS_SetKnifeGeometry", (I, P), I), ("LCS_KnifeBodyDepth", (P,), I),
    ("LCS_RefineContactSurface", (I,), I), ("LCS_SurfaceDepth", (P,), I),
    ("LCS_SetGraspPatch", (F, F, F), I), ("LCS_SetToolDynamics", (F, F, F, F), I),
    ("LCS_SetJawDynamics", (F, F, F, F), I), ("LCS_SetInstrumentControl", (I,), I),
    ("LCS_GetGraspCoreFlags", (I, P), I), ("LCS_GetSolvedTool", (P, P, P), I), ("LCS_GetSolvedJaw", (P,), I),
    ("LCS_GetPressureBlade", (P,), I), ("LCS_GetContactReaction", (P, P), I), ("LCS_GetJawLoad", (P,), I),
    ("LCS_GetMaterialQuality", (P,), I), ("LCS_GetScissorsLoads", (P,), I), ("LCS_SetScissorsWrist", (F, F, F), I),
)


# The reference plugin exports its solver module's own diagnostics under their module names
# (xpbd_solver.h:170-208); a reference build is driven through these aliases.
REFERENCE_ALIASES = {
    "LCS_TetCount": "xpbd_tet_count", "LCS_TetColorCount": "xpbd_tet_color_count",
    "LCS_EdgeColorCount": "xpbd_color_count", "LCS_EdgeCount": "xpbd_get_edge_count",
    "LCS_GetTetIds": "xpbd_readback_tet_ids", "LCS_GetVelocities": "xpbd_get_velocities",
}


def load_library(dll_path=None, extensions=True):
    """Open an LCS_* library and bind its signature table.  Raises if the library or a symbol is missing.

    ``extensions``: True binds this library's diagnostics and extensions as well; ``"reference"`` binds
    only those a reference plugin build provides, through :data:`REFERENCE_ALIASES`.
    """
    path = Path(dll_path) if dll_path else DEFAULT_DLL
    if not path.exists():
        raise FileNotFoundError(f"tissue solver library not built: {path} (run __graft_entry__.build())")
    dll = ct.CDLL(str(path.resolve()))
    functions = {}
    for name, args, result in CORE_SIGNATURES:
        function = dll[name]
        function.argtypes, function.restype = args, result
        functions[name] = function
    for name, args, result in EXTENSION_SIGNATURES:
        symbol = name if extensions is True else REFERENCE_ALIASES.get(name) if extensions == "reference" else None
        if symbol is None:
            continue
        function = dll[symbol]
        function.argtypes, function.restype = args, result
        functions[name] = function
    return dll, functions


class _Session:
    """Shared call/check plumbing; one process-global native session per library (native_backend.py:212-218)."""
    open_libraries: set = set()

    def _open(self, dll_path, extensions):
        self.dll_path = Path(dll_path) if dll_path else DEFAULT_DLL
        key = str(self.dll_path.resolve())
        if key in _Session.open_libraries:
            raise RuntimeError("CUDA solver is single-session; use separate processes for separate environments")
        self.dll, self.functions = load_library(self.dll_path, extensions)
        for name, structure in (("LCS_PhysicsAbiVersion", PhysicsDesc), ("LCS_GraspToolAbiVersion", Grasper)):
            actual = self.functions[name]()
            if actual != ct.sizeof(structure):
                raise RuntimeError(f"{name}: DLL size {actual}, Python size {ct.sizeof(structure)}")
        if self.functions["LCS_ContactModelVersion"]() != 28:
            raise RuntimeError("This adapter requires the snapshotted contact model version 28")
        self._key = key
        _Session.open_libraries.add(key)
        self.closed = False

    def check(self, name, *args):
        result = self.functions[name](*args)
        if result != 0:
            raise RuntimeError(f"{name} failed with native status {result}")

    def close(self):
        if not getattr(self, "closed", True):
            self.functions["LCS_Shutdown"]()
            self.closed = True
            _Session.open_libraries.discard(self._key)

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc, traceback):
        self.close()

    # -- shared initialisation of the lattice, physics and cut buffers (native_backend.py:289-307) --
    def _upload(self, grid: TissueGrid, physics: PhysicsDesc, tear_ratio=0.0):
        g = grid
        n, v = len(g.positions), len(g.corners)
        self.tri_capacity = 6 * len(g.surface_edges) + 1024 + 2 * len(g.edges)
        rd = ReconDesc(v, n, len(g.intersections), len(g.surface_edges), self.tri_capacity, *g.dims, g.spacing, 8)
        self.check("LCS_Init", ct.byref(rd), pointer(g.positions), pointer(g.corners), pointer(g.offsets),
                   pointer(g.counts), pointer(g.intersections), pointer(g.surface_edges))
        external = np.zeros_like(g.positions)
        self.check("LCS_InitPhysics", ct.byref(physics), pointer(g.mass), pointer(g.pinned), pointer(g.active),
                   pointer(external), pointer(g.neighbors), pointer(g.rest_neighbors), pointer(g.bends))
        cd = CutDesc(v, n, len(g.edges), len(g.intersections), self.tri_capacity, *g.dims, g.spacing,
                     V3(*g.origin), 4 * len(g.edges), 0, tear_ratio)
        self.check("LCS_InitCut", ct.byref(cd), pointer(g.connectivity), pointer(g.edges), pointer(g.occupied),
                   pointer(g.inside))


class NativeTissue(_Session):
    """The reference session class with its unchanged call sequence (native_backend.py:212-339).

    Its initialisation enables the unified contact/grasp solver (contact model 2, tissue guard,
    grasp patch, tool dynamics, pressure blade).  This library implements the plain XPBD branch
    only; it exports the unified entry points with the reference's record sizes, so the whole
    signature table binds, and constructing a ``NativeTissue`` against it raises ``RuntimeError``
    at the first unified call (``LCS_SetGraspPatch failed with native status -4001``).  Use
    :class:`PlainTissue`.
    """

    def __init__(self, grid: TissueGrid, settings=Settings(), dll_path=None, initial_command=Command()):
        self.grid, self.settings = grid, settings
        self.initial_command = initial_command
        if settings.cutting_tool not in ("knife", "scissors"):
            raise ValueError(f"Unknown cutting tool: {settings.cutting_tool}")
        self.closed = True
        self._open(dll_path, extensions=False)
        try:
            for name, args, result in UNIFIED_SIGNATURES:
                try:
                    function = self.dll[name]
                except AttributeError as missing:
                    raise RuntimeError(f"{name} is not exported: the unified solver is not part of this library") from missing
                function.argtypes, function.restype = args, result
                self.functions[name] = function
            self.initialize()
        except (RuntimeError, ValueError, OSError):
            self.close()
            raise

    def initialize(self):
        g, s = self.grid, self.settings
        n = len(g.positions)
        pd = PhysicsDesc(n, n * 15, 0, 0, 0, 0, 0.0001, 0.0015, s.substeps, 0, s.young_pa * METERS_PER_UNIT,
                         s.poisson, s.strain_damping_s)
        self._upload(g, pd)
        self.check("LCS_SetTissueGuard", 0.15, 1, n, pointer(g.inside), 1)
        self.check("LCS_SetTissueMaterial", 80, 0.01)
        self.check("LCS_SetGraspPatch", 0.35, 1 / 100000, 0.005)
        self.check("LCS_SetToolDynamics", 0.02, 1200, 10, g.spacing * 0.25)
        self.check("LCS_SetContactModel", s.contact_model, 0.6, 0.4, 0.1, 0.01)


@dataclass(frozen=True)
class Capsule:
    """Capsule instrument: the shaft segment ``a``-``b`` and its radius, in native cm."""
    a: tuple
    b: tuple
    radius: float


class PlainTissue(_Session):
    """Plain XPBD branch session: lattice + physics + cut through the LCS_* ABI.

    ``ks`` is the lattice-edge stiffness (edge compliance = 1/ks), ``tet_mu_v``/``tet_kappa_v`` are
    optional per-tet material stiffnesses in tet storage order (``LCS_SetTetStiffness``).  An
    instrument is armed with :meth:`set_capsule`; a blade with :meth:`set_blade`.
    """

    def __init__(self, grid: TissueGrid, dt=1 / 60, substeps=10, ks=0.0, young_pa=6000.0, poisson=0.25,
                 strain_damping_s=0.04, cs=0.0, kb=0.0, cb=0.0, alpha=0.0, tet_mu_v=None, tet_kappa_v=None,
                 tear_ratio=0.0, grasp_params: GraspParams | None = None, dll_path=None, reference=False):
        self.grid, self.dt, self.closed = grid, float(dt), True
        self.reference = reference
        self._open(dll_path, extensions="reference" if reference else True)
        try:
            n = len(grid.positions)
            pd = PhysicsDesc(n, n * 15, ks, cs, kb, cb, 0.0001, 0.0015, int(substeps), alpha,
                             young_pa * METERS_PER_UNIT, poisson, strain_damping_s)
            self._upload(grid, pd, tear_ratio)
            self.check("LCS_SetContactModel", 0, 0.6, 0.4, 0.1, 0.01)
            self.functions["LCS_SetPressureCutMode"](0)
            if grasp_params is not None:
                self.functions["LCS_SetGraspParams"](ct.byref(grasp_params))
            if tet_mu_v is not None or tet_kappa_v is not None:
                self.set_tet_stiffness(tet_mu_v, tet_kappa_v)
            self.gravity = (0.0, 0.0, 0.0)
        except (RuntimeError, ValueError, OSError):
            self.close()
            raise

    # -- configuration --------------------------------------------------------------------------
    @property
    def tet_count(self):
        return int(self.functions["LCS_TetCount"]())

    def tet_ids(self):
        out = np.empty((self.tet_count, 4), dtype=np.int32)
        self.check("LCS_GetTetIds", pointer(out))
        return out

    def tet_colors(self):
        out = np.empty(self.tet_count, dtype=np.int32)
        self.check("LCS_GetTetColors", pointer(out))
        return out

    def cut_topology(self):
        """The cut topology of the live mesh (GBT_CutTopologyBuild, GBT_GetCutTopology; this library's
        own product, the reference keeps a static colouring and one vertex per lattice node): the live
        tets in emission order as vertex quadruples over the lattice nodes and their duplicates
        (``tet_nodes`` [L, 4]), each tet's storage index (``tet_source``), its colour in the greedy
        re-colouring (``tet_colour``), the lattice node of every duplicated vertex (``dup_parent``,
        vertex N + j duplicates node dup_parent[j]), the colour count and, from the CUDA library, the
        relaxation sweeps its colouring took."""
        counts = np.zeros(4, dtype=np.int32)
        self.check("GBT_CutTopologyBuild", pointer(counts))
        live, dups = int(counts[0]), int(counts[1])
        nodes = np.empty((live, 4), dtype=np.int32)
        source = np.empty(live, dtype=np.int32)
        colour = np.empty(live, dtype=np.int32)
        parent = np.empty(max(dups, 1), dtype=np.int32)
        self.check("GBT_GetCutTopology", pointer(nodes), pointer(source), pointer(colour), pointer(parent))
        return dict(tet_nodes=nodes, tet_source=source, tet_colour=colour, dup_parent=parent[:dups],
                    colours=int(counts[2]), sweeps=int(counts[3]))

    def frame_barriers(self):
        """Grid barriers the last frame executed on the whole-GPU grid (GBT_FrameBarriers; CUDA
        library only), or None when that frame ran in another launch shape."""
        f = self.dll.GBT_FrameBarriers
        f.argtypes, f.restype = (ct.c_void_p,), ct.c_int
        out = ct.c_uint(0)
        rc = f(ct.byref(out))
        if rc == XPBD_ERR_NOT_READY:
            return None
        if rc != 0:
            raise RuntimeError(f"GBT_FrameBarriers failed with native status {rc}")
        return int(out.value)

    def grid_barrier_floor(self, barriers=20000):
        """Microseconds per grid barrier with no work between barriers, on the whole-GPU frame grid
        (GBT_GridBarrierFloor; CUDA library only)."""
        f = self.dll.GBT_GridBarrierFloor
        f.argtypes, f.restype = (ct.c_int, ct.c_void_p), ct.c_int
        out = ct.c_float(0.0)
        rc = f(int(barriers), ct.byref(out))
        if rc != 0:
            raise RuntimeError(f"GBT_GridBarrierFloor failed with native status {rc}")
        return float(out.value)

    def edge_colors(self):
        out = np.empty((len(self.grid.positions), 6), dtype=np.int32)
        self.check("LCS_GetEdgeColors", pointer(out))
        return out

    def tet_stiffness(self):
        mu = np.empty(self.tet_count, dtype=np.float32)
        kappa = np.empty(self.tet_count, dtype=np.float32)
        self.check("LCS_GetTetStiffness", pointer(mu), pointer(kappa))
        return mu, kappa

    def set_tet_stiffness(self, mu_v, kappa_v):
        mu_v = np.ascontiguousarray(mu_v, dtype=np.float32)
        kappa_v = np.ascontiguousarray(kappa_v, dtype=np.float32)
        self.check("LCS_SetTetStiffness", len(mu_v), pointer(mu_v), pointer(kappa_v))

    def set_gravity(self, gx, gy, gz):
        self.gravity = (gx, gy, gz)
        self.check("LCS_SetGravity", gx, gy, gz)

    def set_capsule(self, capsule: Capsule):
        """Arm the shaft capsule of the contact model 0 path; the jaw slab is parked far away."""
        far = (0.0, 1.0e4, 0.0)
        tool = Grasper(V3(*capsule.a), V3(*capsule.b), capsule.radius, V3(*far), V3(0, 0, 1), V3(*far),
                       V3(1, 0, 0), 0.0, 0.0, 0.0, 0.0)
        self.check("LCS_SetGraspTool", ct.byref(tool))

    def set_blade(self, tool: CutTool):
        self.functions["LCS_SetTool"](ct.byref(tool))

    # -- stepping -------------------------------------------------------------------------------
    def step(self, detect_cut=False):
        if self.closed:
            raise RuntimeError("Native session is closed")
        self.check("LCS_Step", self.dt)
        if detect_cut:
            self.check("LCS_DetectCut")
        self.check("LCS_Finalize")

    # -- readback -------------------------------------------------------------------------------
    def positions(self):
        out = np.empty((len(self.grid.positions), 3), dtype=np.float32)
        self.check("LCS_GetCornerPos", pointer(out))
        return out

    def velocities(self):
        out = np.empty((len(self.grid.positions), 3), dtype=np.float32)
        self.check("LCS_GetVelocities", pointer(out))
        return out

    def neighbors(self):
        out = np.empty((len(self.grid.positions), 6), dtype=np.int32)
        self.check("LCS_GetNbrIdx", pointer(out))
        return out

    def particle_frames(self):
        """Current particle frames, (nodes, 3, 3) float32: R with column k the world direction of the
        node's lattice axis k (physics_particle_rot, V/physics.cu:414)."""
        n = len(self.grid.positions)
        if not self.reference:
            out = np.empty((n, 3, 3), dtype=np.float32)
            self.check("GBT_GetParticleRot", pointer(out))
            return out
        # a reference build keeps them in device memory behind its physics module's accessor
        accessor = getattr(self.dll, "_Z20physics_particle_rotv")
        accessor.restype = ct.c_void_p
        return _device_floats(accessor(), 9 * n).reshape(n, 3, 3)

    def surface(self):
        """The reconstructed surface (LCS_GetSurface*): a triangle soup ``pos``, ``nrm`` (3T, 3) and
        ``aux`` (3T, 4), plus ``tri`` (3T,) — the voxel id of each soup vertex (its feature point)."""
        count, indices = ct.c_int32(0), ct.c_int32(0)
        self.check("LCS_GetSurfaceCounts", ct.byref(count), ct.byref(indices))
        n = count.value
        pos, nrm = np.empty((n, 3), dtype=np.float32), np.empty((n, 3), dtype=np.float32)
        idx, aux = np.empty(n, dtype=np.int32), np.empty((n, 4), dtype=np.float32)
        if n:
            self.check("LCS_GetSurface", pointer(pos), pointer(nrm), pointer(idx))
            self.check("LCS_GetSurfaceAux", pointer(aux))
        if not self.reference:
            tri = np.empty(n, dtype=np.int32)
            if n:
                self.check("GBT_GetSurfaceTriangles", pointer(tri))
        else:   # a reference build keeps the tagged voxel ids in device memory (recon_tri)
            accessor = getattr(self.dll, "_Z9recon_triv")
            accessor.restype = ct.c_void_p
            tri = _device_floats(accessor(), n).view(np.int32) if n else np.empty(0, dtype=np.int32)
        return dict(pos=pos, nrm=nrm, aux=aux, tri=tri)

    def bend_alive(self):
        out = np.empty(len(self.grid.positions) * 15 * 8, dtype=np.int32)
        self.check("LCS_GetBendPairs", pointer(out))
        return out.reshape(-1, 8)[:, 4].copy()

    def voxel_cut_mask(self):
        out = np.empty(len(self.grid.corners), dtype=np.uint32)
        self.check("LCS_GetVoxelCutMask", pointer(out))
        return out

    def cut_edge_fractions(self):
        out = np.empty((len(self.grid.positions), 6), dtype=np.float32)
        self.check("LCS_GetCutEdgeFractions", pointer(out))
        return out

    def topology_revision(self):
        r = ct.c_uint()
        self.check("LCS_GetTopologyRevision", ct.byref(r))
        return r.value

    def cut_debug(self):
        out = np.zeros(18, dtype=np.uint32)
        alpha = F()
        self.check("LCS_GetCutDebug", pointer(out), ct.byref(alpha))
        return out

    def observe(self):
        nodes = self.positions()
        if not np.isfinite(nodes).all():
            raise RuntimeError("Non-finite native state; simulation stopped")
        return Observation(nodes, self.neighbors(), np.zeros(len(nodes), np.int32), np.zeros(3), 0.0, 0, 0.0,
                           np.zeros(10, np.float32), np.zeros(3, np.float32))


def _device_floats(address, count):
    """Copy `count` float32 values at a CUDA device address (current device) to a host array."""
    import torch

    class _View:
        __cuda_array_interface__ = {"shape": (count,), "typestr": "<f4", "data": (int(address), False), "version": 2}

    torch.cuda.synchronize()
    return torch.as_tensor(_View(), device="cuda").cpu().numpy()


def severed_edges(baseline, current):
    """Lattice links cut since `baseline` (scenario.py:392-394): both are neighbour tables [N, 6]
    (slot 2a: -axis a, 2a+1: +axis a); each undirected link is counted once, on its +axis slot."""
    before, after = np.asarray(baseline)[:, 1::2], np.asarray(current)[:, 1::2]
    return int(np.count_nonzero((before >= 0) & (after < 0)))


def blade_sweep(prev_start, prev_end, start, end, thickness=0.02):
    """Swept blade quad as the two triangles T1=(Sprev,Eprev,E), T2=(Sprev,E,S) of a ``CutTool`` (V/cut.h:29-38).

    The ribbon tick cuts against the current segment S=t2c, E=t1c.
    """
    sp, ep, s, e = (np.asarray(v, dtype=np.float64) for v in (prev_start, prev_end, start, end))
    normal = np.cross(ep - sp, e - sp)
    length = np.linalg.norm(normal)
    valid = int(length > 1e-10)
    normal = normal / length if valid else np.array((0.0, 1.0, 0.0))
    points = np.stack((sp, ep, s, e))
    tool = CutTool(V3(*sp), V3(*ep), V3(*e), V3(*sp), V3(*e), V3(*s), V3(*normal), thickness, valid,
                   V3(*points.min(axis=0)), V3(*points.max(axis=0)))
    return tool


def library_path_from_env(default=None):
    """Library path chosen by ``GBTISSUE_LIBRARY`` (used by the parity harness), else ``default``."""
    value = os.environ.get("GBTISSUE_LIBRARY")
    return Path(value) if value else default
