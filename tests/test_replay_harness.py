"""CPU checks of the replay harness (tests/replay_harness.py) and of GBT_SetState on the oracle: a
state captured and loaded back is the identity, a step from a loaded state equals the step the
session would have taken, the voxel mask rebuilt from the edge fractions equals the oracle's own,
and the FP32 oracles replayed against the FP64 oracle stay within the parity tolerance with
identical topology."""
import ctypes

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.native_backend import PlainTissue
from conftest import ROOT
import replay_harness as RH

SMALL = (2.38, 1.58, 1.98)   # 12 x 8 x 10 cells


def blade_session(lib, steps):
    w = W.make("c3", steps=steps, scale=SMALL)
    s = PlainTissue(w.grid, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, strain_damping_s=0.0, dll_path=lib)
    s.set_gravity(0.0, -981.0, 0.0)
    return w, s


def command(w):
    return lambda s, k: (s.set_blade(w.blade_path[k]), True)[1]


def test_set_state_round_trip_and_continuation(oracle_libs):
    w, a = blade_session(oracle_libs[0], 40)
    _, b = blade_session(ROOT / "oracle" / "_build" / "liboracle_f32w.so", 40)   # a second library, same state layout
    try:
        cmd = command(w)
        for k in range(30):
            cmd(a, k)
            a.step(detect_cut=True)
        st = RH.capture(a)
        assert st["rev"] > 0, "the blade severed nothing"
        assert np.array_equal(st["mask"], st["own_mask"]), "mask rebuilt from the fractions differs from the oracle's"
        RH.load(a, st)
        again = RH.capture(a)
        for key in ("pos", "vel", "nbr", "bends", "active", "rot", "frac", "mask"):
            assert np.array_equal(st[key], again[key]), key
        assert again["rev"] == st["rev"]
        for k in range(30):     # the second session continues from the loaded state with the same commands
            cmd(b, k)
        RH.load(b, st)
        for k in range(30, 36):
            cmd(a, k); a.step(detect_cut=True)
            cmd(b, k); b.step(detect_cut=True)
        x, y = RH.capture(a), RH.capture(b)
        for key in ("nbr", "bends", "active", "mask"):
            assert np.array_equal(x[key], y[key]), key
        assert x["rev"] == y["rev"]
        assert float(np.abs(x["pos"] - y["pos"]).max()) < 1e-4 * W.bbox_diagonal(w.grid)
    finally:
        a.close()
        b.close()


def test_set_state_rejects_bad_tables(oracle_libs):
    w, s = blade_session(oracle_libs[0], 2)
    try:
        st = RH.capture(s)
        f = s.dll.GBT_SetState
        f.argtypes = (ctypes.c_void_p,) * 8 + (ctypes.c_int, ctypes.c_uint)
        nbr = st["nbr"].copy()
        nbr[0, 1] = 5            # not node 0's +x neighbour
        assert f(None, None, nbr.ctypes.data_as(ctypes.c_void_p), None, None, None, None, None, 0, 0) == -1004
        bends = st["bends"].copy()
        bends[0, 1] += 1         # only the alive flag may change
        assert f(None, None, None, bends.ctypes.data_as(ctypes.c_void_p), None, None, None, None, 0, 0) == -1004
        pos = st["pos"].copy()
        pos[3, 1] = np.nan
        assert f(pos.ctypes.data_as(ctypes.c_void_p), None, None, None, None, None, None, None, 0, 0) == -1004
        assert np.array_equal(RH.capture(s)["nbr"], st["nbr"])
    finally:
        s.close()


def test_fp32_oracles_replayed_against_fp64(oracle_libs):
    """The harness end to end on the CPU: FP64 oracle as the free-running solver, both FP32 oracles
    replayed from its states; every step within 1e-4 of the diagonal, topology identical."""
    steps = 30
    w, ref = blade_session(oracle_libs[1], steps)
    _, f32 = blade_session(oracle_libs[0], steps)
    _, f32w = blade_session(ROOT / "oracle" / "_build" / "liboracle_f32w.so", steps)
    try:
        ref_states, out = RH.replay(ref, {"f32": f32, "f32w": f32w}, steps, command(w))
    finally:
        for s in (ref, f32, f32w):
            s.close()
    active = w.grid.active != 0
    diag = W.bbox_diagonal(w.grid)
    assert ref_states[-1]["rev"] > 0
    for name, states in out.items():
        for k, st in enumerate(states):
            d = RH.diff(st, ref_states[k], active, diag)
            assert d["pos"] < 1e-5, (name, k, d["pos"])
            assert all(d[key] for key in ("nbr", "bends", "active", "rev", "mask", "frac_cut")), (name, k, d)
