"""Dual-contouring surface of the deformed lattice (recon_build_static, V/dc_recon.cu:507-541):
rebuilt at LCS_Init and in every LCS_Finalize, read back with LCS_GetSurfaceCounts / LCS_GetSurface
/ LCS_GetSurfaceAux.

CPU tests check the oracle's restatement on properties the construction guarantees: the rest skin
of a block is a closed, consistently oriented triangle surface with outward normals whose enclosed
volume is the block's; feature points lie in their voxels; once the rest surface exists an intact
voxel's point is its rest point carried trilinearly by the deformed corners.  GPU tests check the
CUDA surface against the FP32 oracle bit for bit (rest, sagging, capsule contact, a blade that
severs surface crossings) and pin the oracle against the reference's own build (same triangles by
voxel ids, positions within tolerance; the reference appends triangles in arrival order, so the
comparison is by voxel-id triple)."""
import json

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import PlainTissue

SMALL = (4.78, 2.38, 3.98)
SIZE = (3.18, 1.58, 3.18)


def c1_grid():
    return build_grid(0.2, size=SIZE, density=1000.0)


def open_session(lib, grid, reference=False):
    return PlainTissue(grid, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, strain_damping_s=0.0, dll_path=lib,
                       reference=reference)


def triangles(surface):
    return surface["tri"].reshape(-1, 3)


def voxel_coords(grid, v):
    dx, dy, _ = grid.dims
    return np.stack([v % dx, (v // dx) % dy, v // (dx * dy)], axis=-1)


def test_rest_surface_closed_oriented_outward(oracle_libs):
    g = c1_grid()
    with open_session(oracle_libs[0], g) as s:
        surf = s.surface()
    tri = triangles(surf)
    assert len(tri) > 100
    # every directed edge once, its reverse once: a closed, consistently oriented surface
    directed = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
    keys = directed[:, 0].astype(np.int64) * (1 << 32) + directed[:, 1]
    rev = directed[:, 1].astype(np.int64) * (1 << 32) + directed[:, 0]
    assert len(np.unique(keys)) == len(keys)
    assert np.array_equal(np.sort(keys), np.sort(rev))
    # outward: the divergence theorem gives the enclosed volume with a positive sign
    p = surf["pos"].reshape(-1, 3, 3).astype(np.float64)
    volume = np.einsum("ij,ij->i", p[:, 0], np.cross(p[:, 1], p[:, 2])).sum() / 6
    block = float(np.prod(SIZE))
    assert 0.9 * block < volume < 1.1 * block, (volume, block)
    # every feature point inside its voxel's rest box
    lo = g.positions[g.corners[surf["tri"], 0]]
    hi = g.positions[g.corners[surf["tri"], 6]]
    assert np.all(surf["pos"] > lo) and np.all(surf["pos"] < hi)
    # unit normals, pointing along the face normals around them
    n = surf["nrm"]
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-5)
    face = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    assert (np.einsum("ij,ij->i", n.reshape(-1, 3, 3)[:, 0].astype(np.float64), face) > 0).mean() > 0.99
    # the rest anchors of the first build are unset (the rest snapshot is taken after it)
    assert not surf["aux"].any()


def test_intact_surface_follows_the_lattice(oracle_libs):
    """After deformation an intact voxel's feature point is its rest point carried trilinearly by the
    voxel's deformed corners (k_AdvectIntactSurface)."""
    g = c1_grid()
    with open_session(oracle_libs[1], g) as s:
        rest = s.surface()
        s.set_gravity(0.0, -981.0, 0.0)
        for _ in range(6):
            s.step()
        now = s.surface()
        pos = np.empty((len(g.positions), 3), dtype=np.float64)
        import ctypes
        assert s.dll.ORC_GetCornerPos64(pos.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.array_equal(triangles(rest), triangles(now))
    v = now["tri"]
    corners = g.corners[v].astype(np.int64)
    a, b = g.positions[corners[:, 0]].astype(np.float64), g.positions[corners[:, 6]].astype(np.float64)
    r = now["aux"][:, :3].astype(np.float64)                 # rest anchor = rest feature point
    assert np.array_equal(r, rest["pos"].astype(np.float64))
    uv = np.clip((r - a) / (b - a), 0, 1)
    off = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    w = np.prod(np.where(off[None], uv[:, None], 1 - uv[:, None]), axis=2)
    want = np.einsum("nk,nkj->nj", w, pos[corners])
    assert np.abs(now["pos"] - want).max() < 1e-6   # the getter returns float32
    assert np.abs(now["pos"] - rest["pos"]).max() > 1e-3


def test_fp32_and_fp64_oracles_agree(oracle_libs):
    g = c1_grid()
    out = []
    for lib in oracle_libs:
        with open_session(lib, g) as s:
            s.set_gravity(0.0, -981.0, 0.0)
            for _ in range(3):
                s.step()
            out.append(s.surface())
    assert np.array_equal(out[0]["tri"], out[1]["tri"])
    assert np.abs(out[0]["pos"] - out[1]["pos"]).max() < 1e-4


def skin_cut_run(lib, steps=10, launch_mode=None):
    """C1 block under gravity; a horizontal blade along z sweeps across x just below the top skin, so
    the rod-phase cut severs the skin-crossing lattice edges: their crossings are rebuilt from the
    inside particle's frame."""
    from genesis_tissue_simulation_gb300.native_backend import blade_sweep
    g = c1_grid()
    y = float(g.intersections["position"][:, 1].max()) - 0.04
    xs = np.linspace(-2.5, 2.5, steps + 1)
    s = open_session(lib, g)
    try:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(launch_mode)
        s.set_gravity(0.0, -981.0, 0.0)
        out = [s.surface()]
        for k in range(steps):
            s.set_blade(blade_sweep((xs[k], y, -2.5), (xs[k], y, 2.5), (xs[k + 1], y, -2.5), (xs[k + 1], y, 2.5)))
            s.step(detect_cut=True)
            out.append(s.surface())
        nbr = s.neighbors()
    finally:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(0)
        s.close()
    a, b = g.intersections["a"], g.intersections["b"]
    d = b - a
    axis = np.where(np.abs(d) == 1, 0, np.where(np.abs(d) == g.dims[0] + 1, 1, 2))
    severed = int((nbr[a, 2 * axis + (d > 0)] < 0).sum())
    return out, severed


def test_skin_cut_severs_crossings(oracle_libs):
    out, severed = skin_cut_run(oracle_libs[0])
    assert severed > 100
    assert all(np.isfinite(o["pos"]).all() and len(o["tri"]) > 0 for o in out)


def rest_cut_run(lib, reference=False, sweeps=6):
    """C1 block at rest: a vertical blade from above the top to mid-height sweeps across x in
    `sweeps` rod-phase detections (LCS_SetTool, LCS_DetectCut, LCS_Finalize; no physics step), so
    positions and particle frames stay at rest and every library sees the same cut.  Returns the
    surface after each sweep and the final neighbour table."""
    from genesis_tissue_simulation_gb300.native_backend import blade_sweep
    g = c1_grid()
    s = PlainTissue(g, dt=1 / 60, substeps=20, ks=1e6, young_pa=6000.0, poisson=0.25, strain_damping_s=0.04,
                    dll_path=lib, reference=reference)
    try:
        xs = np.linspace(-2.3, 2.3, sweeps + 1)
        z, top, low = 0.031, 1.3, 0.05
        out = []
        for k in range(sweeps):
            s.set_blade(blade_sweep((xs[k], top, z), (xs[k], low, z), (xs[k + 1], top, z), (xs[k + 1], low, z)))
            s.check("LCS_DetectCut")
            s.check("LCS_Finalize")
            out.append(s.surface())
        return out, s.neighbors()
    finally:
        s.close()


def directed_edges(tri):
    t = tri.reshape(-1, 3).view(np.uint32).astype(np.uint64)
    d = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    return (d[:, 0] << np.uint64(32)) | d[:, 1], (d[:, 1] << np.uint64(32)) | d[:, 0]


def test_cut_surface_walls(oracle_libs):
    """After a blade has cut the block, the surface has wall triangles made of component feature
    points (tag bits 31 and 30, aux flag 1); it stays consistently oriented (no directed edge twice)
    and closed but for the crack front and rims where fewer than three component points exist
    (1.5 % of the edges here); every component point lies in its voxel."""
    out, nbr = rest_cut_run(oracle_libs[0])
    surf = out[-1]
    tags = surf["tri"].view(np.uint32)
    wall = (tags & 0x40000000) != 0
    assert wall.sum() > 30 and np.array_equal(surf["aux"][:, 3] == 1, wall)
    assert np.all((tags[wall] & 0x80000000) != 0)
    keys, rev = directed_edges(surf["tri"])
    assert len(np.unique(keys)) == len(keys)
    assert np.isin(keys, rev).mean() > 0.97
    assert np.isfinite(surf["pos"]).all() and np.isfinite(surf["nrm"]).all()
    g = c1_grid()
    cut = (tags & 0x80000000) != 0
    vox = (tags[cut] & 0x3FFFFFFF) >> 3
    lo, hi = g.positions[g.corners[vox, 0]], g.positions[g.corners[vox, 6]]
    assert np.all(surf["pos"][cut] >= lo - 1e-5) and np.all(surf["pos"][cut] <= hi + 1e-5)


# ---------------------------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------------------------
@pytest.mark.gpu
def test_gpu_surface_bit_exact_rest_cut(gpu_lib, oracle_libs):
    gpu, nbr_g = rest_cut_run(gpu_lib)
    cpu, nbr_c = rest_cut_run(oracle_libs[0])
    assert np.array_equal(nbr_g, nbr_c)
    for a, b in zip(gpu, cpu):
        assert_same_surface(a, b)


@pytest.mark.gpu
def test_cut_surface_against_reference_build(reference_lib, oracle_libs):
    """The cut feature-point chain, the cut walls and the internal-face cancellation against the
    reference's own build: the same rod-phase cuts of a block at rest give the same neighbour table
    and the same triangles (multisets of vertex tags: voxel ids and component slots, wall marks
    included), positions within 1e-5 of the diagonal (the reference sums cut points with float
    atomics and contracts multiply-adds)."""
    from conftest import results_dir
    ref, nbr_r = rest_cut_run(reference_lib, reference=True)
    orc, nbr_o = rest_cut_run(oracle_libs[0])
    assert np.array_equal(nbr_r, nbr_o)
    diag = W.bbox_diagonal(c1_grid())
    rows = []
    for a, b in zip(ref, orc):
        ta, pa, _ = _by_triangle(a)
        tb, pb, _ = _by_triangle(b)
        assert np.array_equal(ta, tb)
        rows.append({"triangles": int(len(ta)), "walls": int(((a["tri"].view(np.uint32) & 0x40000000) != 0).sum() // 3),
                     "pos_err_over_diag": float(np.abs(pa - pb).max()) / diag})
    with open(results_dir() / "reference_parity.jsonl", "a") as f:
        f.write(json.dumps({"case": "cut surface at rest, c1 grid", "sweeps": rows}) + "\n")
    assert rows[-1]["walls"] > 10
    assert max(r["pos_err_over_diag"] for r in rows) < 1e-5, rows


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2, 3])
def test_gpu_surface_bit_exact_skin_cut(gpu_lib, oracle_libs, mode):
    gpu, severed = skin_cut_run(gpu_lib, launch_mode=mode)
    cpu, _ = skin_cut_run(oracle_libs[0])
    assert severed > 100
    for a, b in zip(gpu, cpu):
        assert_same_surface(a, b)


def surface_run(workload, lib, steps, every, launch_mode=None):
    s = workload.open(lib)
    try:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(launch_mode)
        out = [s.surface()]
        for k in range(steps):
            detect = workload.command(s, k)
            s.step(detect_cut=detect)
            if (k + 1) % every == 0:
                out.append(s.surface())
        return out
    finally:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(0)
        s.close()


def assert_same_surface(a, b):
    for key in ("tri", "pos", "nrm", "aux"):
        assert a[key].shape == b[key].shape, (key, a[key].shape, b[key].shape)
        assert np.array_equal(a[key], b[key]), (key, float(np.abs(a[key].astype(np.float64) - b[key]).max()))


@pytest.mark.gpu
@pytest.mark.parametrize("name,steps,scale,mode", [("c1", 20, None, 2), ("c1", 20, None, 1), ("c2", 20, SMALL, None),
                                                   ("c3", 30, SMALL, None)])
def test_gpu_surface_bit_exact(gpu_lib, oracle_libs, name, steps, scale, mode):
    w = W.make(name, steps=steps, scale=scale)
    gpu = surface_run(w, gpu_lib, steps, 5, launch_mode=mode)
    cpu = surface_run(w, oracle_libs[0], steps, 5)
    for a, b in zip(gpu, cpu):
        assert_same_surface(a, b)


def _by_triangle(surface):
    tri = triangles(surface).view(np.uint32)
    order = np.lexsort(tri.T[::-1])
    return tri[order], surface["pos"].reshape(-1, 3, 3)[order], surface["nrm"].reshape(-1, 3, 3)[order]


@pytest.mark.gpu
def test_oracle_surface_against_reference_build(reference_lib, oracle_libs):
    """The reference build and the oracle from the same C1 grid: the same triangles (voxel-id
    triples, as multisets) at rest and after one sagging frame; vertex positions within 1e-5 of
    the diagonal at rest and 1e-4 after the frame (the reference contracts multiply-adds)."""
    from conftest import results_dir
    g = c1_grid()
    diag = W.bbox_diagonal(g)
    rows = {}
    ref = PlainTissue(g, dt=1 / 60, substeps=20, ks=1e6, young_pa=6000.0, poisson=0.25, strain_damping_s=0.04,
                      dll_path=reference_lib, reference=True)
    try:
        with PlainTissue(g, dt=1 / 60, substeps=20, ks=1e6, young_pa=6000.0, poisson=0.25, strain_damping_s=0.04,
                         dll_path=oracle_libs[0]) as orc:
            for label in ("rest", "frame 1"):
                if label != "rest":
                    for s in (ref, orc):
                        s.set_gravity(0.0, -981.0, 0.0)
                        s.step()
                ta, pa, na = _by_triangle(ref.surface())
                tb, pb, nb = _by_triangle(orc.surface())
                assert np.array_equal(ta, tb), label
                rows[label] = {"triangles": int(len(ta)), "pos_err_over_diag": float(np.abs(pa - pb).max()) / diag,
                               "nrm_err": float(np.abs(na - nb).max())}
    finally:
        ref.close()
    with open(results_dir() / "reference_parity.jsonl", "a") as f:
        f.write(json.dumps({"case": "dual-contouring surface, c1 grid", **rows}) + "\n")
    assert rows["rest"]["pos_err_over_diag"] < 1e-5 and rows["frame 1"]["pos_err_over_diag"] < 1e-4, rows
    assert rows["rest"]["nrm_err"] < 1e-4 and rows["frame 1"]["nrm_err"] < 1e-2, rows
