"""The edge lattices of the GPU parity test, on the FP32 oracle: each builds, steps to finite
positions and exercises what it is there for (the blade severs links in the thin sheet and none in
the small cube; the column bends under gravity)."""
import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W

from edge_lattices import CASES, STEPS, run


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{'x'.join(str(v) for v in c[1])}")
def test_edge_lattices_on_the_oracle(oracle_libs, case):
    w = W.make(case[0], steps=STEPS, scale=case[1])
    out = run(w, oracle_libs[0], case[0] == "c3")
    active = w.grid.active != 0
    assert active.sum() > 0 and np.isfinite(out["pos"]).all()
    moved = float(np.abs(out["pos"] - w.grid.positions)[active].max())
    assert moved > 0
    if case == ("c3", (2.0, 0.4, 1.6)):
        assert out["rev"] > 0
    if case == ("c3", (0.6, 0.6, 0.6)):
        assert out["rev"] == 0
    if case == ("c1", (0.2, 1.8, 0.2)):
        assert moved > 0.1
