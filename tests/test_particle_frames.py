"""Particle coordinate frames (k_ComputeParticleRot, V/physics.cu:109-205; physics_compute_rotations,
V/physics.cu:399-411): run at the end of LCS_Step, after a ribbon tick that emitted cut points, and
in LCS_Finalize.

CPU tests check the oracle's restatement on properties the algorithm guarantees (identity at rest,
proper orthonormal frames, convergence to a rigid rotation through the previous-frame blend, the
cross-product recovery of one lost axis, identity where two axes are lost or the node is pinned)
and against an independent float64 numpy restatement.  GPU tests check the CUDA frames against the
FP32 oracle bit for bit (plain frames, a blade that severs the lattice mid-frame, both launch
shapes) and pin the oracle against the reference's own build."""
import ctypes
import json

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import PlainTissue, pointer

SMALL = (4.78, 2.38, 3.98)


def c1_grid():
    return build_grid(0.2, size=(3.18, 1.58, 3.18), density=1000.0)


def free(grid, active=None):
    """The grid with no pinned nodes (pinned nodes keep identity frames, which the neighbours' blend
    would mix into a rigidly rotated field) and, optionally, other active flags."""
    fields = {**vars(grid), "pinned": np.zeros_like(grid.pinned)}
    if active is not None:
        fields["active"] = active
    return grid.__class__(**fields)


def rotation(axis, angle):
    u = np.asarray(axis, dtype=np.float64)
    u = u / np.linalg.norm(u)
    K = np.array([[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def open_session(lib, grid):
    return PlainTissue(grid, dt=1 / 60, substeps=10, ks=1e6, young_pa=6000.0, strain_damping_s=0.0, dll_path=lib)


def place(session, positions):
    """Overwrite the oracle's live corner positions (replay entry point)."""
    p = np.ascontiguousarray(positions, dtype=np.float32)
    assert session.dll.ORC_SetCornerPos(p.ctypes.data_as(ctypes.c_void_p)) == 0


def numpy_frames(pos, nbr, active, pinned, prev):
    """Independent float64 restatement of one frame pass (vectorised over nodes where it can be)."""
    n = len(pos)
    out = np.tile(np.eye(3), (n, 1, 1))
    for c in range(n):
        if pinned[c] or not active[c]:
            continue
        live = [s for s in range(6) if nbr[c, s] >= 0 and active[nbr[c, s]]]
        axes = [None, None, None]
        for k in range(3):
            p, m = nbr[c, 2 * k + 1], nbr[c, 2 * k]
            okp, okm = 2 * k + 1 in live, 2 * k in live
            if okp and okm:
                e = pos[p] - pos[m]
            elif okp:
                e = pos[p] - pos[c]
            elif okm:
                e = pos[c] - pos[m]
            else:
                continue
            if np.linalg.norm(e) < 1e-12:
                continue
            d = e / np.linalg.norm(e)
            if live:
                ps = sum(prev[nbr[c, s]][:, k] for s in live)
                if np.linalg.norm(ps) > 1e-6:
                    b = d + ps / np.linalg.norm(ps)
                    if np.linalg.norm(b) > 0.25:
                        d = b / np.linalg.norm(b)
            axes[k] = d
        missing = [k for k in range(3) if axes[k] is None]
        if len(missing) == 1:
            k = missing[0]
            cx = np.cross(axes[(k + 1) % 3], axes[(k + 2) % 3])
            if np.linalg.norm(cx) > 1e-9:
                axes[k] = cx / np.linalg.norm(cx)
        if any(a is None for a in axes):
            continue
        M = np.stack(axes, axis=1)
        if np.linalg.det(M) <= 1e-4:
            continue
        R = M.copy()
        for _ in range(16):
            R = 0.5 * (R + np.linalg.inv(R).T)
        G = R.T @ R
        if max(np.abs(np.diag(G) - 1).max(), abs(G[0, 1]), abs(G[0, 2]), abs(G[1, 2])) > 1e-3:
            continue
        out[c] = R
    return out


def frames64(session):
    n = len(session.grid.positions)
    out = np.empty((n, 3, 3), dtype=np.float64)
    assert session.dll.ORC_GetParticleRot64(out.ctypes.data_as(ctypes.c_void_p)) == 0
    return out


def test_rest_frames_are_identity(oracle_libs):
    g = c1_grid()
    with open_session(oracle_libs[0], g) as s:
        assert np.array_equal(s.particle_frames(), np.tile(np.eye(3, dtype=np.float32), (len(g.positions), 1, 1)))
        s.check("LCS_Finalize")
        assert np.array_equal(s.particle_frames(), np.tile(np.eye(3, dtype=np.float32), (len(g.positions), 1, 1)))


@pytest.mark.parametrize("which", [0, 1])
def test_rigid_rotation_converges_through_blend(oracle_libs, which):
    """Every pass blends the lattice direction with the neighbours' previous axes, so on a rigidly
    rotated lattice the frames walk from the identity to the rotation, halving the gap per pass
    (down to the float32 rounding of the rotated positions); pinned nodes stay at the identity."""
    base = c1_grid()
    g = free(base)
    Q = rotation((0.3, 1.0, -0.5), 0.9)
    centre = g.positions.mean(axis=0)
    moved = (g.positions - centre) @ Q.T + centre
    live = g.active != 0
    with open_session(oracle_libs[which], g) as s:
        place(s, moved)
        errors = []
        for _ in range(40):
            s.check("LCS_Finalize")
            R = frames64(s)
            errors.append(float(np.abs(R[live] - Q).max()))
        frozen = R[~live]
    tol = 1e-6
    assert errors[0] > 0.1 and errors[-1] < tol, errors[::8]
    assert all(b <= a * 0.75 + tol for a, b in zip(errors[:20], errors[1:21])), errors[:21]
    assert np.array_equal(frozen, np.tile(np.eye(3), (len(frozen), 1, 1)))
    with open_session(oracle_libs[which], base) as s:   # pinned nodes: identity whatever moves
        place(s, moved)
        s.check("LCS_Finalize")
        R = frames64(s)
    pinned = base.pinned != 0
    assert pinned.any() and np.array_equal(R[pinned], np.tile(np.eye(3), (int(pinned.sum()), 1, 1)))


def test_frames_are_proper_rotations(oracle_libs):
    """After a deforming run the frames are orthonormal with determinant +1 (or the identity)."""
    g = c1_grid()
    with open_session(oracle_libs[0], g) as s:
        s.set_gravity(0.0, -981.0, 0.0)
        for _ in range(10):
            s.step()
        R = s.particle_frames().astype(np.float64)
    gram = np.einsum("nji,njk->nik", R, R)
    assert np.abs(gram - np.eye(3)).max() < 1e-5
    assert np.abs(np.linalg.det(R) - 1).max() < 1e-5
    assert np.abs(R - np.eye(3)).max() > 1e-4, "gravity sag should tilt some frames"


def test_oracle_against_numpy_restatement(oracle_libs):
    """One pass of the FP64 oracle against the float64 numpy restatement on a sagged, partly
    deactivated lattice with a rotated previous frame field."""
    g = build_grid(0.4, size=(3.18, 1.58, 3.18), density=1000.0)
    active = g.active.copy()
    live_ids = np.flatnonzero(active)
    rng = np.random.default_rng(3)
    active[rng.choice(live_ids, size=len(live_ids) // 8, replace=False)] = 0
    g2 = g.__class__(**{**vars(g), "active": active})
    with open_session(oracle_libs[1], g2) as s:
        s.set_gravity(0.0, -981.0, 0.0)
        for _ in range(6):
            s.step()
        prev = frames64(s)
        pos = np.empty((len(g.positions), 3), dtype=np.float64)
        assert s.dll.ORC_GetCornerPos64(pos.ctypes.data_as(ctypes.c_void_p)) == 0
        nbr = s.neighbors()
        s.check("LCS_Finalize")
        got = frames64(s)
    want = numpy_frames(pos, nbr, active, g.pinned, prev)
    assert np.abs(got - want).max() < 1e-12


def test_lost_axes(oracle_libs):
    """One lost axis is recovered as the cross product of the other two (the frame still converges
    to the rigid rotation); two lost axes give the identity."""
    g = c1_grid()
    nx, ny, nz = (d + 1 for d in g.dims)
    cid = lambda x, y, z: x + nx * (y + ny * z)
    one = cid(3, 4, 3)            # interior node: drop both x neighbours
    two = cid(9, 4, 9)            # interior node: drop both x and both z neighbours
    active = g.active.copy()
    assert active[one] and active[two]
    for x, y, z in ((2, 4, 3), (4, 4, 3), (8, 4, 9), (10, 4, 9), (9, 4, 8), (9, 4, 10)):
        active[cid(x, y, z)] = 0
    g2 = free(g, active)
    Q = rotation((1.0, 0.2, 0.4), 0.6)
    centre = g.positions.mean(axis=0)
    with open_session(oracle_libs[1], g2) as s:
        place(s, (g.positions - centre) @ Q.T + centre)
        for _ in range(40):
            s.check("LCS_Finalize")
        R = frames64(s)
    assert np.abs(R[one] - Q).max() < 1e-6
    assert np.array_equal(R[two], np.eye(3))


# ---------------------------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------------------------
def frames_run(workload, lib, steps, every, launch_mode=None):
    s = workload.open(lib)
    try:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(launch_mode)
        out = []
        for k in range(steps):
            detect = workload.command(s, k)
            s.step(detect_cut=detect)
            if (k + 1) % every == 0:
                out.append(dict(rot=s.particle_frames(), dbg=s.cut_debug()[15:17].copy()))
        return out
    finally:
        if launch_mode is not None:
            s.dll.LCS_SetLaunchMode(0)
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2, 3])
def test_gpu_frames_bit_exact_c1(gpu_lib, oracle_libs, mode):
    w = W.make("c1", steps=30)
    gpu = frames_run(w, gpu_lib, 30, 10, launch_mode=mode)
    cpu = frames_run(w, oracle_libs[0], 30, 10)
    for a, b in zip(gpu, cpu):
        assert np.array_equal(a["rot"], b["rot"]), float(np.abs(a["rot"] - b["rot"]).max())
    assert np.abs(cpu[-1]["rot"] - np.eye(3)).max() > 1e-4


def ticking_blade(workload):
    """A static blade segment along z just below the second node layer from the top: the first
    frame's sag carries lattice edges across it, so ribbon ticks inside LCS_Step emit cut points."""
    from genesis_tissue_simulation_gb300.native_backend import blade_sweep
    g = workload.grid
    act = g.active != 0
    lo, hi = g.positions[act].min(axis=0), g.positions[act].max(axis=0)
    y = float(hi[1]) - 0.2 - 0.002
    x = 0.5 * float(lo[0] + hi[0]) + 0.013
    start, end = (x, y, float(lo[2]) - 0.2), (x, y, float(hi[2]) + 0.2)
    return blade_sweep(start, end, start, end)


def tick_run(lib, steps=6):
    w = W.make("c3", steps=steps, scale=SMALL)
    s = w.open(lib)
    try:
        s.set_blade(ticking_blade(w))
        out = []
        for _ in range(steps):
            s.check("LCS_Step", s.dt)
            out.append(dict(rot=s.particle_frames(), dbg=s.cut_debug()[15:17].copy(), nbr=s.neighbors()))
        passes = int(s.dll.ORC_FramePasses()) if hasattr(s.dll, "ORC_FramePasses") else None
        return out, passes
    finally:
        s.close()


def test_oracle_tick_runs_mid_frame_pass(oracle_libs):
    """The ticking blade scenario emits cut points inside LCS_Step before the last substep, so the
    oracle runs more than one frame pass per step (the mid-frame pass, V/physics.cu:368-379)."""
    import ctypes as c
    dll = c.CDLL(str(oracle_libs[0]))
    dll.ORC_FramePasses.restype = c.c_longlong
    before = dll.ORC_FramePasses()
    out, _ = tick_run(oracle_libs[0], steps=2)
    assert out[0]["dbg"][1] > 0
    assert dll.ORC_FramePasses() - before > 2


@pytest.mark.gpu
def test_gpu_frames_bit_exact_tick(gpu_lib, oracle_libs):
    """Frames at the end of LCS_Step after ribbon ticks that emitted cut points mid-frame."""
    gpu, _ = tick_run(gpu_lib)
    cpu, _ = tick_run(oracle_libs[0])
    assert cpu[0]["dbg"][1] > 0, "the ticks emitted no cut points"
    for a, b in zip(gpu, cpu):
        assert np.array_equal(a["dbg"], b["dbg"]) and np.array_equal(a["nbr"], b["nbr"])
        assert np.array_equal(a["rot"], b["rot"]), float(np.abs(a["rot"] - b["rot"]).max())


@pytest.mark.gpu
def test_gpu_frames_bit_exact_quad_cut(gpu_lib, oracle_libs):
    """The swept blade of the rod phase severs the lattice (LCS_DetectCut); LCS_Finalize's frames
    follow the post-sever lattice, bit for bit."""
    w = W.make("c3", steps=40, scale=SMALL)
    gpu = frames_run(w, gpu_lib, 40, 5)
    cpu = frames_run(w, oracle_libs[0], 40, 5)
    assert cpu[-1]["dbg"][1] > 0, "the blade emitted no cut points"
    for a, b in zip(gpu, cpu):
        assert np.array_equal(a["dbg"], b["dbg"])
        assert np.array_equal(a["rot"], b["rot"]), float(np.abs(a["rot"] - b["rot"]).max())


def _reference_positions(session):
    """Writable float32 (nodes, 3) torch view of a reference build's corner positions (device)."""
    import torch
    accessor = getattr(session.dll, "_Z16recon_corner_posv")
    accessor.restype = ctypes.c_void_p
    n = len(session.grid.positions)

    class _View:
        __cuda_array_interface__ = {"shape": (n, 3), "typestr": "<f4", "data": (int(accessor()), False), "version": 2}
    return torch.as_tensor(_View(), device="cuda")


def _reference_frame_pass(session):
    import torch
    compute = getattr(session.dll, "_Z25physics_compute_rotationsv")
    compute.restype = ctypes.c_int
    assert compute() == 0
    torch.cuda.synchronize()


def _pair_session(grid, lib, reference):
    """The configuration the reference parity tests drive both libraries with."""
    return PlainTissue(grid, dt=1 / 60, substeps=20, ks=1e6, young_pa=6000.0, poisson=0.25, strain_damping_s=0.04,
                       dll_path=lib, reference=reference)


@pytest.mark.gpu
def test_oracle_frames_against_reference_build(reference_lib, oracle_libs):
    """Pin the oracle's frame pass on the reference's own kernel: both sessions get the same corner
    positions (a rigid rotation plus seeded noise, then others, so every pass blends with frames the
    previous pass produced) and run one frame pass; entries agree within 1e-5 (the reference
    contracts multiply-adds).  A deactivated band exercises one-sided edges and axis recovery."""
    import torch
    from conftest import results_dir
    g = c1_grid()
    active = g.active.copy()
    nx, ny, nz = (d + 1 for d in g.dims)
    for z in range(nz):
        for y in range(ny):
            active[5 + nx * (y + ny * z)] = 0            # a plane of removed nodes: x axis one-sided beside it
    g2 = g.__class__(**{**vars(g), "active": active})
    rng = np.random.default_rng(11)
    centre = g.positions.mean(axis=0)
    ref = _pair_session(g2, reference_lib, True)
    try:
        with _pair_session(g2, oracle_libs[0], False) as orc:
            view = _reference_positions(ref)
            errors = []
            for axis, angle in (((0.3, 1.0, -0.5), 0.5), ((1.0, 0.0, 0.2), 1.4), ((0.0, 0.2, 1.0), -0.8)):
                Q = rotation(axis, angle)
                pos = ((g.positions - centre) @ Q.T + centre + rng.normal(scale=0.02, size=g.positions.shape)).astype(np.float32)
                view.copy_(torch.from_numpy(pos).cuda())
                torch.cuda.synchronize()
                place(orc, pos)
                _reference_frame_pass(ref)
                orc.check("LCS_Finalize")
                a, b = ref.particle_frames(), orc.particle_frames()
                errors.append(float(np.abs(a - b).max()))
                assert np.abs(b - np.eye(3)).max() > 0.1
            assert max(errors) < 1e-5, errors
    finally:
        ref.close()
    with open(results_dir() / "reference_parity.jsonl", "a") as f:
        f.write(json.dumps({"case": "particle frames, same positions", "max_abs_entry": errors}) + "\n")


@pytest.mark.gpu
def test_oracle_frames_after_blade_match_reference(reference_lib, oracle_libs):
    """After a blade has severed the lattice in both (same topology), both get the same positions and
    repeat the frame pass until the previous-frame history no longer matters: the severed lattice's
    frames (one-sided edges, recovered axes, identity where two axes are lost) agree within 1e-5."""
    import torch
    from conftest import results_dir
    w = W.make("c3", steps=10, scale=SMALL)
    sessions = []
    try:
        ref = _pair_session(w.grid, reference_lib, True)
        sessions.append(ref)
        orc = _pair_session(w.grid, oracle_libs[0], False)
        sessions.append(orc)
        for s in (ref, orc):
            s.set_gravity(0.0, -981.0, 0.0)
            for k in range(10):
                s.set_blade(w.blade_path[k])
                s.step(detect_cut=True)
        nbr = ref.neighbors()
        assert (nbr < 0).sum() > (w.grid.neighbors < 0).sum(), "the blade severed nothing"
        assert np.array_equal(nbr, orc.neighbors())
        pos = ref.positions()
        place(orc, pos)
        for _ in range(40):
            _reference_frame_pass(ref)
            orc.check("LCS_Finalize")
        a, b = ref.particle_frames(), orc.particle_frames()
        err = float(np.abs(a - b).max())
        assert err < 1e-5, err
    finally:
        for s in sessions:
            s.close()
    with open(results_dir() / "reference_parity.jsonl", "a") as f:
        f.write(json.dumps({"case": "particle frames after blade", "max_abs_entry": err}) + "\n")
