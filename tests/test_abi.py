"""C ABI contracts checked without a GPU: struct layouts of the reference ABI
(endoscopic_tissue/test_core.py:64-67), and that every library exports every entry point
include/gbtissue.h declares (the CUDA library is loaded, never called, here)."""
import ctypes
import re
from pathlib import Path

import pytest

from genesis_tissue_simulation_gb300 import build as native_build
from genesis_tissue_simulation_gb300.native_backend import (Blade, CutDesc, CutTool, Grasper, GraspParams, PhysicsDesc,
                                                            ReconDesc, ScissorsControl, ScissorsResult)

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "gbtissue.h"


# entry points of the reference's unified solver: exported by the CUDA library (defined status), not by the oracle
UNIFIED = ("LCS_SetPressureBlade", "LCS_SetScissors", "LCS_GetScissors", "LCS_SetJawGeometry", "LCS_SetKnifeGeometry",
           "LCS_KnifeBodyDepth", "LCS_RefineContactSurface", "LCS_SurfaceDepth", "LCS_SetGraspPatch",
           "LCS_SetToolDynamics", "LCS_SetJawDynamics", "LCS_SetInstrumentControl", "LCS_GetGraspCoreFlags",
           "LCS_GetSolvedTool", "LCS_GetSolvedJaw", "LCS_GetPressureBlade", "LCS_GetContactReaction",
           "LCS_GetJawLoad", "LCS_GetMaterialQuality", "LCS_GetScissorsLoads", "LCS_SetScissorsWrist")
UNIFIED_SIZES = ("LCS_PressureBladeAbiVersion", "LCS_ScissorsAbiVersion", "LCS_ScissorsResultAbiVersion")


def declared_symbols(prefixes=("LCS_",)):
    names = re.findall(r"LCS_API\s+[\w\s\*]+?\b((?:LCS|GBT)_\w+)\s*\(", HEADER.read_text())
    return sorted(n for n in set(names) if n.startswith(prefixes))


def test_abi_layout():
    for structure, expected in ((ReconDesc, 40), (PhysicsDesc, 52), (CutDesc, 60), (Grasper, 92), (GraspParams, 60),
                                (Blade, 52), (CutTool, 116), (ScissorsControl, 244), (ScissorsResult, 124)):
        assert ctypes.sizeof(structure) == expected, structure.__name__


def test_header_declares_plain_path():
    names = declared_symbols()
    for required in ("LCS_Init", "LCS_InitPhysics", "LCS_InitCut", "LCS_SetGravity", "LCS_Step", "LCS_Finalize",
                     "LCS_GetCornerPos", "LCS_GetNbrIdx", "LCS_GetTopologyRevision", "LCS_GetCutEdgeFractions",
                     "LCS_SetTool", "LCS_DetectCut", "LCS_SetPressureCutMode", "LCS_PhysicsAbiVersion",
                     "LCS_GraspToolAbiVersion", "LCS_SetGraspTool", "LCS_SetGraspParams", "LCS_SetContactModel",
                     "LCS_ContactModelVersion", "LCS_SetTissueGuard", "LCS_SetTissueMaterial", "LCS_ProfileEnable",
                     "LCS_ProfileRead", "LCS_Shutdown"):
        assert required in names


def test_cuda_library_exports_declared_symbols():
    lib = native_build.build()
    dll = ctypes.CDLL(str(lib))
    names = declared_symbols(("LCS_", "GBT_"))
    assert any(n.startswith("GBT_Diff") for n in names) and any(n.startswith("GBT_Batch") for n in names)
    missing = [n for n in names if not hasattr(dll, n)]
    assert not missing, missing


def test_oracle_exports_declared_symbols(oracle_libs):
    for path in oracle_libs:
        dll = ctypes.CDLL(str(path))
        skip = ("LCS_SetLaunchMode", "LCS_SetBarrierTest", "LCS_StepNoAlloc") + UNIFIED + UNIFIED_SIZES
        missing = [n for n in declared_symbols() if n not in skip and not hasattr(dll, n)]
        assert not missing, (path.name, missing)


def test_oracle_abi_versions(oracle_libs):
    dll = ctypes.CDLL(str(oracle_libs[0]))
    assert dll.LCS_PhysicsAbiVersion() == 52
    assert dll.LCS_GraspToolAbiVersion() == 92
    assert dll.LCS_ContactModelVersion() == 28


def _adapter_table():
    import json
    data = json.loads((ROOT / "tests" / "golden" / "adapter_signatures.json").read_text())
    return data["signatures"] + data["scissors_signatures"]


def test_reference_adapter_table_binds():
    """Every entry point the reference adapter binds (native_backend.py:229-263, the scissors pair
    included; tests/golden/make_adapter_signatures.py) exists in libgbtissue.so with the adapter's
    argtypes/restype, the record-size checks the adapter makes pass, and every entry point of the
    unified solver answers LCS_ERR_UNSUPPORTED.  Only host-side calls are made (no session)."""
    lib = native_build.build()
    dll = ctypes.CDLL(str(lib))
    kinds = {"P": ctypes.c_void_p, "I": ctypes.c_int32, "F": ctypes.c_float, None: None}
    bound = {}
    for name, args, res in _adapter_table():
        fn = dll[name]
        fn.argtypes, fn.restype = tuple(kinds[a] for a in args), kinds[res]
        bound[name] = (fn, args)
    for name, structure in (("LCS_PhysicsAbiVersion", PhysicsDesc), ("LCS_GraspToolAbiVersion", Grasper),
                            ("LCS_PressureBladeAbiVersion", Blade), ("LCS_ScissorsAbiVersion", ScissorsControl),
                            ("LCS_ScissorsResultAbiVersion", ScissorsResult)):
        assert bound[name][0]() == ctypes.sizeof(structure), name
    assert bound["LCS_ContactModelVersion"][0]() == 28
    buf = (ctypes.c_float * 4096)()
    dummy = {"P": ctypes.cast(buf, ctypes.c_void_p), "I": 1, "F": 0.5}
    for name in UNIFIED:
        fn, args = bound[name]
        assert fn(*(dummy[a] for a in args)) == -4001, name
    assert len(bound) == 49
