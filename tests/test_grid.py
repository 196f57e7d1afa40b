"""The lattice producer against the reference's own output (golden hashes) and the reference's
CPU grid contracts (endoscopic_tissue/test_core.py:64-113, 198-208)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from genesis_tissue_simulation_gb300.grid import EDGE_CORNERS, Tab, build_grid, connectivity_table, to_genesis

GOLDEN = Path(__file__).resolve().parent / "golden"
HASHES = json.loads((GOLDEN / "grid_hashes.json").read_text())


def _kwargs(case):
    kw = dict(case)
    if "tab" in kw:
        low, high, attached = kw["tab"]
        kw["tab"] = Tab(tuple(low), tuple(high), attached)
    if "size" in kw:
        kw["size"] = tuple(kw["size"])
    return kw


@pytest.mark.parametrize("name", sorted(HASHES["cases"]))
def test_grid_matches_reference_hashes(name):
    grid = build_grid(**_kwargs(HASHES["cases"][name]))
    want = HASHES["grids"][name]
    assert list(grid.dims) == want["dims"]
    for field, ref in want.items():
        if not isinstance(ref, dict):
            continue
        a = np.ascontiguousarray(getattr(grid, field))
        assert a.dtype.str == ref["dtype"] and list(a.shape) == ref["shape"], field
        assert hashlib.sha256(a.tobytes()).hexdigest() == ref["sha256"], field


def test_grid_matches_reference_arrays_small():
    ref = np.load(GOLDEN / "grid_small.npz")
    grid = build_grid(0.6)
    for field in ref.files:
        np.testing.assert_array_equal(getattr(grid, field), ref[field], err_msg=field)


def test_connectivity_exhaustive():
    table = connectivity_table()
    for mask in range(4096):
        visited, groups = set(), []
        for start in range(8):
            if start in visited:
                continue
            group, pending = set(), [start]
            while pending:
                node = pending.pop()
                if node in group:
                    continue
                group.add(node)
                for bit, (a, b) in enumerate(EDGE_CORNERS):
                    if not mask & (1 << bit):
                        if node == a:
                            pending.append(int(b))
                        elif node == b:
                            pending.append(int(a))
            groups.append(group)
            visited |= group
        assert table[mask, 0] == len(groups)
        for label, group in enumerate(groups):
            assert all(table[mask, n + 1] == label for n in group)


def test_grid_boundary_and_reciprocal_neighbors():
    grid = build_grid(0.6)
    assert grid.intersections.dtype.itemsize == 40 and grid.bends.dtype.itemsize == 32
    assert grid.counts.sum() == len(grid.intersections)
    assert np.any(grid.pinned)
    supported = np.all(grid.active[grid.corners] != 0, axis=1)
    np.testing.assert_allclose(grid.mass.sum(), np.count_nonzero(supported) * (grid.spacing * .01) ** 3 * 1000, rtol=1e-6)
    assert np.all(grid.mass[grid.active == 0] == 0)
    for slot in range(6):
        nodes = np.flatnonzero(grid.neighbors[:, slot] >= 0)
        other = grid.neighbors[nodes, slot]
        np.testing.assert_array_equal(grid.neighbors[other, slot ^ 1], nodes)
        assert np.all(grid.active[nodes] & grid.active[other])
    assert np.all((grid.intersections["t"] >= 0) & (grid.intersections["t"] <= 1))
    distances = (np.abs(grid.intersections["position"]) - (3.0, 0.7, 2.0)).max(axis=1)
    np.testing.assert_allclose(distances, 0, atol=1e-6)


def test_rest_neighbors_and_envelope_mass():
    grid = build_grid(.2, vertical_spacing=.05)
    for slot in range(6):
        ids = np.flatnonzero(grid.neighbors[:, slot] >= 0)
        delta = grid.positions[grid.neighbors[ids, slot]] - grid.positions[ids]
        np.testing.assert_allclose(grid.rest_neighbors[ids, slot], delta, atol=3e-7)
    active = grid.positions[grid.active != 0]
    volume = np.prod((active.max(axis=0) - active.min(axis=0)) * .01)
    np.testing.assert_allclose(grid.mass.sum(), volume * 1000, rtol=2e-6)


def test_workload_lattice_sizes():
    c1 = build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)
    assert len(c1.positions) == 5733 and int(c1.active.sum()) == 2601 and int(c1.pinned.sum()) == 289
    np.testing.assert_allclose(c1.mass.sum(), 0.016384, rtol=1e-5)


def test_units_and_orientation():
    axes = to_genesis(np.eye(3))
    np.testing.assert_allclose(np.linalg.norm(axes, axis=1), 0.01)
    assert np.linalg.det(axes) > 0


def test_invalid_spacing_rejected():
    with pytest.raises(ValueError):
        build_grid(0.05)
    with pytest.raises(ValueError):
        build_grid(0.2, vertical_spacing=0.3)


def test_severed_edges_counts_each_link_once():
    """Known answer of the reference's undirected cut count (test_core.py:233-236): one link between
    nodes 0 and 1, seen from both ends, cut once."""
    from genesis_tissue_simulation_gb300.native_backend import severed_edges
    baseline = np.full((2, 6), -1, dtype=np.int32)
    baseline[0, 1], baseline[1, 0] = 1, 0
    assert severed_edges(baseline, np.full_like(baseline, -1)) == 1
    assert severed_edges(baseline, baseline) == 0
    g = build_grid(0.5, size=(2.0, 1.0, 1.5))
    cut = g.neighbors.copy()
    live = np.argwhere(cut[:, 1::2] >= 0)
    i, a = live[len(live) // 2]
    j = cut[i, 2 * a + 1]
    cut[i, 2 * a + 1] = cut[j, 2 * a] = -1
    assert severed_edges(g.neighbors, cut) == 1

