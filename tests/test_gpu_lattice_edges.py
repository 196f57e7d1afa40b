"""CUDA path against the CPU oracle on lattices at the edges of the layout (`edge_lattices.py`):
the smallest block (2 x 2 x 2 cells), a rod along x, a column, a two-cell-thick sheet, an odd-sized
capsule block, a thin sheet the blade cuts through and a small cube the blade misses.  Each runs in
every launch shape (whole GPU, one CTA, one thread-block cluster) and must match the FP32 oracle bit
for bit: positions, velocities and, for the blade, the neighbour table and topology revision.

Few colours, colour ranges shorter than a warp, nodes of a colour spread over one or two CTAs and
edges that end on the lattice margin are what these shapes exercise that the C1-C3 sizes do not.
"""
import ctypes

import numpy as np
import pytest

from edge_lattices import CASES, STEPS, run
from genesis_tissue_simulation_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle_runs(oracle_libs):
    return {case: run(W.make(case[0], steps=STEPS, scale=case[1]), oracle_libs[0], case[0] == "c3") for case in CASES}


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{'x'.join(str(v) for v in c[1])}")
def test_edge_lattices_match_oracle(gpu_lib, oracle_runs, case, mode):
    w = W.make(case[0], steps=STEPS, scale=case[1])
    dll = ctypes.CDLL(str(gpu_lib))
    dll.LCS_SetLaunchMode(mode)
    try:
        gpu = run(w, gpu_lib, case[0] == "c3")
    finally:
        dll.LCS_SetLaunchMode(0)
    cpu = oracle_runs[case]
    assert np.isfinite(gpu["pos"]).all()
    for key in cpu:
        if key == "rev":
            assert gpu[key] == cpu[key]
        else:
            assert np.array_equal(gpu[key], cpu[key]), (key, float(np.abs(gpu[key].astype(np.float64) - cpu[key]).max()))
