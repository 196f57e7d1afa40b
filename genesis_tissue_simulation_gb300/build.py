"""In-tree build of the CUDA library (libgbtissue.so) for sm_103a.

Two translation units are compiled in parallel with nvcc and linked into
``csrc/_build/libgbtissue.so``.  Flags that matter for results:

* ``-fmad=false``: no implicit multiply-add contraction; the projections contract explicitly
  (``fmaf``) exactly where the FP32 CPU restatement calls ``std::fma``, so every projection rounds as
  it does;
* ``-Xcompiler -ffp-contract=off``: the host-side coefficient arithmetic (h, compliances, rest
  shapes) rounds identically on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
CSRC = PACKAGE_DIR / "csrc"
BUILD = CSRC / "_build"
INCLUDE = PACKAGE_DIR.parent / "include"
LIBRARY = BUILD / "libgbtissue.so"
# the same sources with every element gather index checked (GBT_DEBUG_BOUNDS): tests only
DEBUG_BUILD = CSRC / "_build_debug"
DEBUG_LIBRARY = DEBUG_BUILD / "libgbtissue_debug.so"
SOURCES = ("frame_kernels.cu", "lcs_api.cu", "mesh_build.cu", "batch_api.cu", "adjoint_kernels.cu", "adjoint_api.cu",
           "surface_kernels.cu", "cut_topology.cu")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path():
    for candidate in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError("nvcc not found")


def common_flags():
    return [ARCH, "-O3", "-std=c++17", "-lineinfo", "-fmad=false", f"-I{INCLUDE}",
            "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden"]


def _compile(source: str, debug: bool = False) -> Path:
    obj = (DEBUG_BUILD if debug else BUILD) / (Path(source).stem + ".o")
    cmd = [nvcc_path(), *common_flags(), *(["-DGBT_DEBUG_BOUNDS"] if debug else []), "-c", str(CSRC / source), "-o", str(obj)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"nvcc failed for {source}:\n{result.stderr}")
    return obj


def _stale(library: Path = LIBRARY) -> bool:
    if not library.exists():
        return True
    built = library.stat().st_mtime
    inputs = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > built for p in inputs)


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> Path:
    """Compile libgbtissue.so (debug: libgbtissue_debug.so, gather indices checked) unless it is newer
    than every source; returns its path."""
    library, folder = (DEBUG_LIBRARY, DEBUG_BUILD) if debug else (LIBRARY, BUILD)
    if not force and not _stale(library):
        return library
    folder.mkdir(parents=True, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        objects = list(pool.map(lambda src: _compile(src, debug), SOURCES))
    tmp = library.with_suffix(".so.tmp")
    cmd = [nvcc_path(), ARCH, "-shared", "-o", str(tmp), *map(str, objects)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"link failed:\n{result.stderr}")
    os.replace(tmp, library)
    if verbose:
        print(f"built {library}", file=sys.stderr)
    return library


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
