"""Settings a session shutdown restores.

The reference keeps its tissue material (tensile strength, bulk damping) in module statics that
xpbd_shutdown puts back to 80 and 0.003125 s (xpbd_solver.cu:3829), and physics_init shuts a live
physics session down first (physics.cu:218).  So a session that never calls LCS_SetTissueMaterial
runs with the defaults whatever an earlier session in the same process set.  Checked on the oracle
(CPU) and on the CUDA library (GPU): a guarded C1 run after a session that changed the material
equals, bit for bit, a run that sets the defaults explicitly."""
import ctypes

import numpy as np
import pytest

from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import PlainTissue, pointer

STEPS = 3


def guarded(lib, material=None, steps=STEPS):
    g = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    with PlainTissue(g, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, strain_damping_s=0.0, dll_path=lib) as s:
        s.set_gravity(0.0, -981.0, 0.0)
        s.check("LCS_SetTissueGuard", ctypes.c_float(0.5), 1, len(g.positions), pointer(g.inside), 1)
        if material is not None:
            s.check("LCS_SetTissueMaterial", ctypes.c_float(material[0]), ctypes.c_float(material[1]))
        for _ in range(steps):
            s.step()
        return s.positions()


def check_reset(lib):
    changed = guarded(lib, material=(40.0, 0.02), steps=1)
    after = guarded(lib)
    explicit = guarded(lib, material=(80.0, 0.003125))
    assert np.array_equal(after, explicit)
    assert not np.array_equal(guarded(lib, material=(40.0, 0.02)), explicit), "the material should matter"
    return changed


def test_oracle_shutdown_restores_tissue_material(oracle_libs):
    check_reset(oracle_libs[0])


@pytest.mark.gpu
def test_cuda_library_shutdown_restores_tissue_material(gpu_lib):
    check_reset(gpu_lib)
