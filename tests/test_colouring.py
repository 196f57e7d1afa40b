"""The Gauss-Seidel colourings the oracle builds (xpbd_solver.cu:1204-1279 edges, 1600-1848 tets):
members of a colour share no node, and every element of colour k meets an element of each colour
below k (first-fit greedy, so colour membership matches the reference's order-dependent colouring).
The CUDA library builds the same colourings: the GPU test compares them entry for entry."""
import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W

SMALL = (4.78, 2.38, 3.98)


def _sessions(lib):
    for name, scale in (("c1", None), ("c2", SMALL)):
        w = W.make(name, steps=1, scale=scale)
        s = w.open(lib)
        try:
            yield name, w, s.tet_ids(), s.tet_colors(), s.edge_colors()
        finally:
            s.close()


def _edges(grid, edge_colors):
    """(node a, node b, colour) of every coloured lattice edge, keyed by its +axis slot."""
    slot = np.argwhere(edge_colors >= 0)
    a, s = slot[:, 0], slot[:, 1]
    return a, grid.neighbors[a, s], edge_colors[a, s]


def _greedy_and_disjoint(members, colours, n_nodes):
    """members [M, k] node ids, colours [M]: node-disjoint colour classes, first-fit lower colours."""
    flat = members.ravel()
    rep_colour = np.repeat(colours, members.shape[1])
    for c in np.unique(colours):
        nodes = flat[rep_colour == c]
        assert len(np.unique(nodes)) == len(nodes), f"colour {c} repeats a node"
    seen = np.zeros(n_nodes, dtype=np.int64)        # per node: OR of 1 << colour over its elements
    np.bitwise_or.at(seen, flat, np.left_shift(np.int64(1), rep_colour.astype(np.int64)))
    around = np.bitwise_or.reduce(seen[members], axis=1)
    below = np.left_shift(np.int64(1), colours.astype(np.int64)) - 1
    assert np.all((around & below) == below), "an element skips a lower colour it could have taken"


def test_oracle_colourings(oracle_libs):
    for name, w, ids, tcol, ecol in _sessions(oracle_libs[0]):
        n = len(w.grid.positions)
        assert tcol.min() == 0 and ecol.max() >= 0
        _greedy_and_disjoint(ids, tcol, n)
        a, b, c = _edges(w.grid, ecol)
        assert np.all(b >= 0)
        _greedy_and_disjoint(np.stack([a, b], axis=1), c, n)
        assert int(c.max()) + 1 == 6, (name, int(c.max()) + 1)
        if name == "c1":
            assert int(tcol.max()) + 1 == 31


@pytest.mark.gpu
def test_cuda_colourings_equal_oracle(gpu_lib, oracle_libs):
    for (name, _, ids_g, tcol_g, ecol_g), (_, _, ids_c, tcol_c, ecol_c) in zip(_sessions(gpu_lib), _sessions(oracle_libs[0])):
        assert np.array_equal(ids_g, ids_c), name
        assert np.array_equal(tcol_g, tcol_c), name
        assert np.array_equal(ecol_g, ecol_c), name
