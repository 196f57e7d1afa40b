"""The tissue guard chain (LCS_SetTissueGuard with passes > 0; xpbd_solver.cu:588-741 and the guarded
form of k_solve_tet, 749-829): guarded Neo-Hookean projection (log J with a floor, bulk damping,
trust region), tensile fibre passes, and the feasibility chain after contact (minimum-volume
repair, conservative inversion test, eight-colour vertex line search).

CPU tests check the oracle (its own logarithm, FP32 against FP64, the chain actually running); the
GPU tests check the CUDA frame against the FP32 oracle bit for bit in both launch shapes."""
import ctypes

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import Capsule, GraspParams, PlainTissue, pointer

GRASP = dict(W.DEFAULT_GRASP, ccd_velocity=0.0)


def guarded_run(lib, steps=12, minimum=0.9, passes=1, launch_mode=None, press=0.6, on_close=None):
    """C1 lattice, guard armed as the reference adapter arms it (strength 80, bulk damping 0.01 s),
    a capsule pressed ``press`` cm into the top.  Returns positions after every step and the
    oracle's feasibility counters (None for the CUDA library)."""
    g = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    s = PlainTissue(g, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, strain_damping_s=0.0, grasp_params=GraspParams(**GRASP),
                    dll_path=lib)
    try:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(launch_mode)
        s.set_gravity(0.0, -981.0, 0.0)
        s.check("LCS_SetTissueGuard", ctypes.c_float(minimum), passes, len(g.positions), pointer(g.inside), 1)
        s.check("LCS_SetTissueMaterial", ctypes.c_float(80.0), ctypes.c_float(0.01))
        top = float(g.positions[g.active != 0, 1].max())
        frames = []
        for k in range(steps):
            y = top + 0.25 - press * (k + 1) / steps
            s.set_capsule(Capsule((-1.0, y, 0.0), (1.0, y, 0.2), 0.25))
            s.step()
            frames.append(s.positions())
        stats = None
        if hasattr(s.dll, "ORC_GuardStats"):
            stats = np.zeros(3, dtype=np.int64)
            s.dll.ORC_GuardStats(stats.ctypes.data_as(ctypes.c_void_p))
        if on_close is not None:
            on_close(s)
        return g, frames, stats
    finally:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(0)
        s.close()


def test_pow_minus_two_thirds_accuracy(oracle_libs):
    """J^(-2/3) of the Neo-Hookean deviatoric term (own Newton routine, identical on host and device)
    against float64 pow: within 2.5 ulp on [0.05, 1e6]."""
    dll = ctypes.CDLL(str(oracle_libs[0]))
    dll.ORC_PowMinusTwoThirds.argtypes, dll.ORC_PowMinusTwoThirds.restype = (ctypes.c_double,), ctypes.c_double
    xs = np.float32(np.concatenate([np.geomspace(0.05, 1e6, 8000), np.linspace(0.9, 1.1, 2001), [1.0, 0.05, 8.0, 27.0]]))
    got = np.array([dll.ORC_PowMinusTwoThirds(float(x)) for x in xs], dtype=np.float32).astype(np.float64)
    ref = xs.astype(np.float64) ** (-2.0 / 3.0)
    err = np.abs(got - ref) / np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert err.max() <= 2.5, (float(err.max()), float(xs[err.argmax()]))


def test_acos_bend_accuracy(oracle_libs):
    """The FP32 arccos of the bending angle (own routine, identical on host and device; coefficients
    derived by oracle/fit_acos.py) against float64 arccos: within 1.1 ulp on [-1, 1], and equal bit for
    bit to the same operation sequence evaluated in numpy float32."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("fit_acos", str(oracle_libs[0].parents[1] / "fit_acos.py"))
    fit = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fit)
    dll = ctypes.CDLL(str(oracle_libs[0]))
    dll.ORC_AcosBend.argtypes, dll.ORC_AcosBend.restype = (ctypes.c_double,), ctypes.c_double
    rng = np.random.default_rng(1)
    xs = np.float32(np.concatenate([np.linspace(-1, 1, 6001), rng.uniform(-1, 1, 4000), 1 - rng.uniform(0, 1e-4, 500),
                                    0.5 + rng.uniform(-1e-4, 1e-4, 500), [-1.0, -0.5, 0.0, 0.5, 1.0]]))
    got = np.array([dll.ORC_AcosBend(float(x)) for x in xs], dtype=np.float32)
    ref = np.arccos(xs.astype(np.float64))
    err = np.abs(got.astype(np.float64) - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    assert float(err.max()) <= 1.1, (float(err.max()), float(xs[err.argmax()]))
    coef = np.float32([0.1666666, 0.075005025, 0.044517495, 0.03180234, 0.014460857, 0.03748363])
    assert np.array_equal(fit.acos_bend(xs, coef), got)
    assert np.array_equal(fit.fit(), coef), "the routine's coefficients are the fit's"


def test_log_positive_accuracy(oracle_libs):
    """The FP32 logarithm of the guarded bulk strain (own routine, identical on host and device)
    against numpy's: within 2 ulp on [0.05, 1e4]."""
    dll = ctypes.CDLL(str(oracle_libs[0]))
    dll.ORC_LogPositive.argtypes, dll.ORC_LogPositive.restype = (ctypes.c_double,), ctypes.c_double
    xs = np.float32(np.concatenate([np.geomspace(0.05, 1e4, 4000), np.linspace(0.9, 1.1, 2001), [1.0, 2.0, 0.5, 1.41421356]]))
    got = np.array([dll.ORC_LogPositive(float(x)) for x in xs], dtype=np.float32)
    ref = np.log(xs.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    err = np.abs(got.astype(np.float64) - ref) / np.maximum(ulp, np.spacing(np.float32(1e-7)))
    assert float(err.max()) <= 2.0, float(err.max())
    assert got[np.where(xs == 1.0)[0][0]] == 0.0


def test_guarded_oracle_fp32_tracks_fp64_and_runs_the_chain(oracle_libs):
    g, f32, stats32 = guarded_run(oracle_libs[0])
    _, f64, stats64 = guarded_run(oracle_libs[1])
    active = g.active != 0
    assert np.isfinite(f32[-1]).all()
    assert float(np.abs(f32[-1] - f64[-1])[active].max()) < 1e-3
    # every stage ran: candidates below the minimum, repairs that did not suffice, vertex line searches
    assert stats32[0] > 0 and stats32[1] > 0 and stats32[2] > 0, stats32
    assert stats64[0] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("minimum,passes,mode", [(0.9, 1, 2), (0.9, 2, 1), (0.15, 1, 1)])
def test_guarded_step_matches_oracle(gpu_lib, oracle_libs, minimum, passes, mode):
    g, gpu, _ = guarded_run(gpu_lib, minimum=minimum, passes=passes, launch_mode=mode)
    _, cpu, stats = guarded_run(oracle_libs[0], minimum=minimum, passes=passes)
    if minimum > 0.5:
        assert stats[2] > 0                     # the feasibility line search ran in this case
    for k, (a, b) in enumerate(zip(gpu, cpu)):
        assert np.array_equal(a, b), (k, float(np.abs(a - b).max()))
