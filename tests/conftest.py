"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; everything else runs on the CPU."""
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

ORACLE_F32 = ROOT / "oracle" / "_build" / "liboracle_f32.so"
ORACLE_F64 = ROOT / "oracle" / "_build" / "liboracle_f64.so"
REFERENCE_LIB = ROOT / "oracle" / "_ref" / "libLiverCudaSim.so"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle_libs():
    """The FP32 and FP64 builds of the CPU oracle (built on demand with make)."""
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    return ORACLE_F32, ORACLE_F64


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree; requires a GPU."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from genesis_tissue_simulation_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def reference_lib():
    """The reference's own CUDA plugin built by oracle/build_ref.sh from staged sources, if present."""
    if not REFERENCE_LIB.exists():
        staged = ROOT / "oracle" / "_ref" / "src" / "cuda"
        if not staged.exists():
            pytest.skip("reference sources not staged (oracle/build_ref.sh stage)")
        subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh"), "build"], check=True)
    return REFERENCE_LIB


def results_dir():
    """Where GPU tests append the figures they measure (JSON lines): $GBT_RESULTS_DIR, else
    test_results/ at the repository root (git-ignored)."""
    import os
    path = Path(os.environ.get("GBT_RESULTS_DIR", ROOT / "test_results"))
    path.mkdir(parents=True, exist_ok=True)
    return path
