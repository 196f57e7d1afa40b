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
        missing = [n for n in declared_symbols() if n not in ("LCS_SetLaunchMode", "LCS_SetBarrierTest", "LCS_StepNoAlloc") and not hasattr(dll, n)]
        assert not missing, (path.name, missing)


def test_oracle_abi_versions(oracle_libs):
    dll = ctypes.CDLL(str(oracle_libs[0]))
    assert dll.LCS_PhysicsAbiVersion() == 52
    assert dll.LCS_GraspToolAbiVersion() == 92
    assert dll.LCS_ContactModelVersion() == 28
