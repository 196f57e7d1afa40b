"""Tissue lattice producer: the host-side input of the XPBD tissue step.

This module rebuilds the reference's lattice producer (``endoscopic_tissue/grid.py:176-281``,
``build_grid`` / ``TissueGrid``) so that a caller of the reference can swap imports and get
byte-identical arrays in the same ABI dtypes.  Units are native: 1 unit = 1 cm, y points up
(``endoscopic_tissue/grid.py:3``).

Array conventions (all C-contiguous, the dtypes are part of the C ABI):

* node id ``i = x + nx*(y + ny*z)`` with ``nx = dims[0]+1``; ``positions`` float32 ``[N,3]``;
* ``neighbors`` int32 ``[N,6]``: slot ``2a`` is the ``-a`` neighbour, ``2a+1`` the ``+a`` one, ``-1`` none;
* ``rest_neighbors`` float32 ``[N,6,3]``: rest offset to each live neighbour;
* ``bends`` 32-byte records ``(i, j, k, theta, alive, pad[3])``, 15 per node (all slot pairs);
* ``mass`` float32 ``[N]``: a quarter of each Kuhn tetrahedron's mass lumped on its corners;
* ``edges`` int32 ``[E,4]``: ``(axis, x, y, z)`` of every lattice edge whose four incident voxels
  lie inside the grid (the cut detector's edge list, ``GridEdgeGpu2``).

The construction is written independently: voxel, edge and slot tables are derived with
explicit integer arithmetic, and the floating-point steps are ordered to reproduce the
reference's numpy promotion rules exactly (they are pinned by golden hashes in ``tests/``).
"""
from __future__ import annotations

import functools
from dataclasses import dataclass

import numpy as np

# Local corner c of a voxel sits at the offset below (the reference's Fig 2.4 numbering,
# endoscopic_tissue/grid.py:11-13); the 12 voxel edges join the corner pairs in EDGE_CORNERS
# (grid.py:14-16).  Both tables are part of the cut-connectivity format (Conn4096).
CORNER_OFFSETS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                           [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=np.int32)
EDGE_CORNERS = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [4, 5], [5, 6],
                         [6, 7], [7, 4], [0, 4], [1, 5], [2, 6], [3, 7]], dtype=np.int32)

# Record layouts shared with the C ABI (IsectGpu 40 B, BendPairGpu 32 B).
ISECT_DTYPE = np.dtype([("position", "<f4", 3), ("normal", "<f4", 3), ("a", "<i4"), ("b", "<i4"),
                        ("t", "<f4"), ("inside_a", "<i4")])
BEND_DTYPE = np.dtype([("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("theta", "<f4"),
                       ("alive", "<i4"), ("padding", "<i4", 3)])

METERS_PER_UNIT = 0.01
# Native (x, y, z) -> Genesis (x, -z, y), a proper rotation (grid.py:24-25).
TO_GENESIS = np.array([[1, 0, 0], [0, 0, -1], [0, 1, 0]], dtype=np.float32)
BLOCK_SIZE = (6.0, 1.4, 4.0)

# Kuhn split of a cell along its main diagonal; corners in "binary" numbering (bit a = +axis a).
KUHN_TETS = np.array([[0, 1, 3, 7], [0, 3, 2, 7], [0, 2, 6, 7],
                      [0, 6, 4, 7], [0, 4, 5, 7], [0, 5, 1, 7]], dtype=np.int64)


@dataclass(frozen=True)
class Tab:
    """Box of tissue grown from one positive face of the block, in cm (grid.py:28-37).

    ``low``/``high`` are its outer corners; its ``low`` face along ``attached`` lies on the block's
    positive face of that axis.  Faces within 1e-6 cm of a block face are snapped onto it.
    """
    low: tuple
    high: tuple
    attached: int


@dataclass
class TissueGrid:
    """Output of :func:`build_grid`; field names and meanings follow grid.py:40-61."""
    spacing: float
    cell_size: np.ndarray
    dims: tuple
    origin: np.ndarray
    positions: np.ndarray
    inside: np.ndarray
    active: np.ndarray
    pinned: np.ndarray
    mass: np.ndarray
    neighbors: np.ndarray
    rest_neighbors: np.ndarray
    bends: np.ndarray
    corners: np.ndarray
    occupied: np.ndarray
    intersections: np.ndarray
    offsets: np.ndarray
    counts: np.ndarray
    surface_edges: np.ndarray
    edges: np.ndarray
    connectivity: np.ndarray


def lattice_coordinates(extent):
    """Integer (x, y, z) of every site of a box of ``extent`` sites, x varying fastest."""
    nx, ny, nz = (int(v) for v in extent)
    idx = np.arange(nx * ny * nz, dtype=np.int64)
    return np.stack((idx % nx, (idx // nx) % ny, idx // (nx * ny)), axis=1).astype(np.int32)


# The reference exposes the same helper under this name (grid.py:64-66).
coordinates = lattice_coordinates


def connectivity_table():
    """Component labels of the 8 voxel corners for each of the 2^12 edge-cut masks (a fresh copy)."""
    return _connectivity_table().copy()


@functools.lru_cache(maxsize=1)
def _connectivity_table():
    """Component labels of the 8 voxel corners for each of the 2^12 edge-cut masks (grid.py:69-82).

    Row ``m`` holds ``(count, label_0 .. label_7)``: bit ``b`` of ``m`` set means voxel edge ``b``
    (EDGE_CORNERS order) is cut.  Labels number the connected components in order of their
    lowest corner.  Computed with a union-find per mask.
    """
    table = np.zeros((4096, 9), dtype=np.int32)
    for mask in range(4096):
        parent = list(range(8))

        def root(c):
            while parent[c] != c:
                c = parent[c]
            return c

        for bit in range(12):
            if mask >> bit & 1:
                continue
            a, b = (int(v) for v in EDGE_CORNERS[bit])
            ra, rb = root(a), root(b)
            if ra != rb:
                parent[max(ra, rb)] = min(ra, rb)
        label_of_root, labels = {}, []
        for c in range(8):
            r = root(c)
            if r not in label_of_root:
                label_of_root[r] = len(label_of_root)
            labels.append(label_of_root[r])
        table[mask, 0] = len(label_of_root)
        table[mask, 1:] = labels
    return table


def union_exit(points, axis, direction, lows, highs):
    """Coordinate at which axis-parallel rays leave a union of open boxes (grid.py:85-105).

    Ray ``r`` starts at ``points[r]`` and runs along ``axis[r]`` with sign ``direction[r]``.  A box
    holds the ray when the ray's cross-section lies strictly inside it; overlapping held boxes
    chain into one interval, and the ray leaves at the far end of the chain that contains it.
    Written as a fixed-point iteration over the boxes in the ray's own forward coordinate.
    """
    points = np.asarray(points)
    n, nb = len(points), len(lows)
    rows = np.arange(n)
    strict = (lows[None, :, :] < points[:, None, :]) & (points[:, None, :] < highs[None, :, :])
    strict[rows, :, axis] = True
    holds = strict.all(axis=2)                              # [n, boxes]
    forward = direction[:, None] > 0
    near = np.where(forward, lows[:, axis].T, -highs[:, axis].T)   # entry, forward coordinate
    far = np.where(forward, highs[:, axis].T, -lows[:, axis].T)    # exit, forward coordinate
    start = direction * points[rows, axis]
    reach = np.full(n, -np.inf, dtype=np.result_type(far, start))
    frontier = start
    # Each round extends every ray through the held boxes that contain its current frontier;
    # nb rounds suffice because every round must add a new box to a chain.
    for _ in range(nb):
        inside = holds & (near < frontier[:, None]) & (frontier[:, None] < far)
        step = np.where(inside, far, -np.inf).max(axis=1)
        reach = np.maximum(reach, step)
        frontier = reach
    assert np.isfinite(reach).all(), "an interior point lies outside every box"
    return direction * reach


@dataclass(frozen=True)
class BoxUnion:
    """Tissue as a union of axis-aligned boxes: the block (centred at the origin) and an optional tab.

    The tissue bed is the block's bottom face; ``half`` holds the block's half extents (grid.py:111-151).
    """
    lows: np.ndarray
    highs: np.ndarray
    half: np.ndarray

    @property
    def low(self):
        return self.lows.min(axis=0)

    @property
    def high(self):
        return self.highs.max(axis=0)

    def inside(self, positions):
        within = (self.lows[None] < positions[:, None, :]) & (positions[:, None, :] < self.highs[None])
        return within.all(axis=2).any(axis=1)

    def boundary(self, positions, a, b, inside):
        """Crossing fraction from ``a`` to ``b`` and outward normal of each surface-crossing lattice edge.

        The lattice is axis aligned, so an edge leaves the union through a face normal to its own
        axis; the exit coordinate comes from :func:`union_exit`.
        """
        axis = np.abs(positions[b] - positions[a]).argmax(axis=1)
        a_in = inside[a] != 0
        interior = np.where(a_in, a, b)
        exterior = np.where(a_in, b, a)
        rows = np.arange(len(a))
        direction = np.sign(positions[exterior, axis] - positions[interior, axis])
        exit_coord = union_exit(positions[interior], axis, direction, self.lows, self.highs)
        t = (exit_coord - positions[a, axis]) / (positions[b, axis] - positions[a, axis])
        normals = np.zeros((len(a), 3), dtype=np.float32)
        normals[rows, axis] = direction
        return t, normals

    def bed(self, positions):
        return positions[:, 1] <= -self.half[1]


def implicit_boundary(distance, positions, a, b):
    """Zero crossing of a signed distance along lattice edges, by 40 bisections (grid.py:154-173).

    ``distance`` maps ``(n,3)`` points to signed distances (negative inside).  Returns the fraction
    from ``a`` to ``b`` and the unit central-difference gradient (step 1e-4) at the crossing.
    """
    pa = positions[a].astype(np.float64)
    pb = positions[b].astype(np.float64)
    lo = np.zeros(len(a))
    hi = np.ones(len(a))
    sign_a = np.sign(distance(pa))
    for _ in range(40):
        mid = (lo + hi) / 2
        same = np.sign(distance(pa + (pb - pa) * mid[:, None])) == sign_a
        lo = np.where(same, mid, lo)
        hi = np.where(same, hi, mid)
    t = (lo + hi) / 2
    hit = pa + (pb - pa) * t[:, None]
    grad = np.stack([distance(hit + 1e-4 * e) - distance(hit - 1e-4 * e) for e in np.eye(3)], axis=1)
    return t, (grad / np.linalg.norm(grad, axis=1, keepdims=True)).astype(np.float32)


def _block_shape(size, cell_size, tab):
    half = np.asarray(size, dtype=np.float32) / 2
    lows, highs = [-half], [half]
    if tab is not None:
        low = np.asarray(tab.low, dtype=np.float32).copy()
        high = np.asarray(tab.high, dtype=np.float32).copy()
        ok = (np.isfinite(np.stack((low, high))).all() and tab.attached in (0, 1, 2)
              and bool(np.all(high - low >= 2 * cell_size - 1e-6))
              and abs(low[tab.attached] - half[tab.attached]) < 1e-6)
        if not ok:
            raise ValueError("tab must span two cells per axis and grow from a positive face of the block")
        # Snap faces flush with a block face onto it, then let the tab reach one cell into the block
        # so nodes on the shared face belong to a box interior (grid.py:198-205).
        for bound in (low, high):
            for face in (-half, half):
                flush = np.abs(bound - face) < 1e-6
                bound[flush] = face[flush]
        low[tab.attached] = half[tab.attached] - cell_size[tab.attached]
        lows.append(low)
        highs.append(high)
    return BoxUnion(np.array(lows), np.array(highs), half)


def build_grid(spacing=0.6, size=BLOCK_SIZE, density=1000.0, vertical_spacing=None, tab=None, shape=None):
    """Build the tissue lattice of a block (optionally with a tab) or of an implicit ``shape``.

    Same signature, validation and outputs as the reference producer (grid.py:176-281).  A ``shape``
    supplies ``low``, ``high``, ``inside(positions)``, ``boundary(positions, a, b, inside)`` and
    ``bed(positions)``.
    """
    if not np.isfinite(spacing) or not 0.1 <= spacing <= 0.7:
        raise ValueError("spacing must be 0.1..0.7 native units (1..7 mm)")
    cell = np.full(3, spacing, dtype=np.float32)
    if vertical_spacing is not None:
        if not np.isfinite(vertical_spacing) or not 0.01 <= vertical_spacing <= spacing:
            raise ValueError("vertical spacing must be 0.01..spacing native units")
        cell[1] = vertical_spacing
    if shape is None:
        shape = _block_shape(size, cell, tab)

    low, high = shape.low, shape.high
    # Two empty cells of margin on every side: the lattice covers the tissue's bounding box.
    dims = tuple(int(v) + 4 for v in np.ceil((high - low) / cell).astype(int))
    origin = (low + high) / 2 - np.array(dims, dtype=np.float32) * cell / 2
    nodes_per_axis = np.array(dims, dtype=np.int64) + 1
    nx, ny, _ = (int(v) for v in nodes_per_axis)
    node_xyz = lattice_coordinates(nodes_per_axis)
    stride = np.array([1, nx, nx * ny], dtype=np.int64)
    # int32 * float32 promotes to float64 in numpy; the sum is rounded to float32 once.
    positions = np.ascontiguousarray(origin.astype(np.float64) + node_xyz * cell.astype(np.float64),
                                     dtype=np.float32)
    n_nodes = len(positions)
    inside = shape.inside(positions).astype(np.int32)

    voxel_xyz = lattice_coordinates(dims).astype(np.int64)
    voxel_base = voxel_xyz @ stride
    corner_step = CORNER_OFFSETS.astype(np.int64) @ stride
    corners = (voxel_base[:, None] + corner_step[None, :]).astype(np.int32)
    occupied = (inside[corners] != 0).any(axis=1).astype(np.int32)
    active = np.zeros(n_nodes, dtype=np.int32)
    active[corners[occupied != 0].ravel()] = 1
    pinned = (shape.bed(positions) & (active != 0)).astype(np.int32)

    # Surface crossings of every voxel edge, listed voxel by voxel in EDGE_CORNERS order.
    end_a = corners[:, EDGE_CORNERS[:, 0]]
    end_b = corners[:, EDGE_CORNERS[:, 1]]
    crossing = inside[end_a] != inside[end_b]
    counts = crossing.sum(axis=1, dtype=np.int32)
    offsets = (np.cumsum(counts, dtype=np.int32) - counts).astype(np.int32)
    cross_a, cross_b = end_a[crossing], end_b[crossing]
    frac, normals = shape.boundary(positions, cross_a, cross_b, inside)
    hit = positions[cross_a] + (positions[cross_b] - positions[cross_a]) * frac[:, None]
    intersections = np.zeros(len(hit), dtype=ISECT_DTYPE)
    intersections["position"] = hit
    intersections["normal"] = normals
    intersections["a"] = cross_a
    intersections["b"] = cross_b
    intersections["t"] = frac
    intersections["inside_a"] = inside[cross_a]

    neighbors = np.full((n_nodes, 6), -1, dtype=np.int32)
    rest = np.zeros((n_nodes, 6, 3), dtype=np.float32)
    edge_lists, surface_lists = [], []
    for axis in range(3):
        has_next = node_xyz[:, axis] < dims[axis]
        lower = np.flatnonzero(has_next)
        upper = lower + stride[axis]
        linked = (active[lower] != 0) & (active[upper] != 0)
        lo_ids, hi_ids = lower[linked], upper[linked]
        neighbors[lo_ids, 2 * axis + 1] = hi_ids
        neighbors[hi_ids, 2 * axis] = lo_ids
        rest[lo_ids, 2 * axis + 1, axis] = cell[axis]
        rest[hi_ids, 2 * axis, axis] = -cell[axis]
        # The edge list keeps edges whose four incident voxels exist (complete dual-contouring quad).
        interior = has_next.copy()
        for other in range(3):
            if other != axis:
                interior &= (node_xyz[:, other] > 0) & (node_xyz[:, other] < dims[other])
        base = np.flatnonzero(interior)
        records = np.empty((len(base), 4), dtype=np.int32)
        records[:, 0] = axis
        records[:, 1:] = node_xyz[base]
        edge_lists.append(records)
        flips = inside[base] != inside[base + stride[axis]]
        surface = np.zeros((int(flips.sum()), 8), dtype=np.int32)
        surface[:, :4] = records[flips]
        surface[:, 4] = inside[base[flips]]
        surface_lists.append(surface)

    # Bend elements: every pair (s0 < s1) of the 6 neighbour slots of every node.
    slot_pairs = np.array([(s0, s1) for s0 in range(6) for s1 in range(s0 + 1, 6)], dtype=np.int64)
    bends = np.zeros((n_nodes, 15), dtype=BEND_DTYPE)
    bends["i"] = np.arange(n_nodes, dtype=np.int32)[:, None]
    bends["j"] = neighbors[:, slot_pairs[:, 0]]
    bends["k"] = neighbors[:, slot_pairs[:, 1]]
    bends["alive"] = ((bends["j"] >= 0) & (bends["k"] >= 0)).astype(np.int32)
    straight = (slot_pairs[:, 0] // 2) == (slot_pairs[:, 1] // 2)
    bends["theta"] = np.where(straight, np.pi, np.pi / 2)

    # Lumped mass: each Kuhn tetrahedron of a cell with 8 active corners puts a quarter of its mass
    # (cell volume / 6) on each of its corners, i.e. density * cell volume / 24 per corner use.
    binary = corners[:, [0, 1, 3, 2, 4, 5, 7, 6]]
    full_cells = (active[binary] != 0).all(axis=1)
    tet_nodes = binary[full_cells][:, KUHN_TETS].reshape(-1)
    uses = np.bincount(tet_nodes, minlength=n_nodes)
    cell_volume_m3 = np.prod(cell * METERS_PER_UNIT)
    mass = (uses * density * cell_volume_m3 / 24).astype(np.float32)
    assert np.all(mass[active != 0] > 0)

    return TissueGrid(spacing, cell, dims, origin, positions, inside, active, pinned, mass,
                      neighbors, rest, bends, corners, occupied, intersections, offsets, counts,
                      np.concatenate(surface_lists), np.concatenate(edge_lists), connectivity_table())


def to_genesis(points):
    """Native cm, y up -> Genesis metres, z up (grid.py:284-285)."""
    return points @ TO_GENESIS.T * METERS_PER_UNIT
