"""Replay-mode parity harness (test infrastructure).

A free-running comparison of two FP32 XPBD solvers mixes two things: a difference in what one step
computes, and the growth of last-bit rounding differences over many steps (the plain branch's
single Gauss-Seidel pass on a soft block amplifies them).  Replay separates them: the reference's
own build free-runs a scenario and its state after every step is captured; each other solver then
steps from the reference's state after step k-1, under the same commands, and its result is
compared with the reference's state after step k.  A per-step difference at rounding level with a
free-running difference that grows is rounding growth; a per-step difference that jumps is an
operator difference.

The state one frame carries into the next is what the reference keeps between `LCS_Step` calls:
corner positions (recon_corner_pos), velocities (xpbd_get_velocities), the live neighbour table
(physics_nbr_idx), the bend records' alive flags (physics_bend_pairs), the active flags
(physics_active), the cut module's voxel mask, first-cut edge fractions and topology revision, and
the particle frames (physics_particle_rot).  The reference build exposes no accessor for its voxel
mask; it is rebuilt from the edge fractions (MarkAndEmit, V/cut.cu:218-254, writes a lattice edge's
fraction exactly when it first sets the edge's bits in the occupied voxels of its stencil), and the
same rebuild is checked against the CUDA library's own mask.  Everything is loaded through
`GBT_SetState`, which the CUDA library and the oracle both export.
"""
from __future__ import annotations

import ctypes

import numpy as np

from genesis_tissue_simulation_gb300.native_backend import _device_floats, pointer

# Voxels around a lattice edge and the edge's local index in each (ES_VoxelOffset / ES_LocalEdge,
# V/cut.cuh:113-160): edge (axis, base corner) borders voxel base + OFF[axis][s] as its edge EDGE[axis][s].
ES_OFF = np.array([[[0, 0, 0], [0, -1, 0], [0, -1, -1], [0, 0, -1]],
                   [[0, 0, 0], [0, 0, -1], [-1, 0, -1], [-1, 0, 0]],
                   [[0, 0, 0], [-1, 0, 0], [-1, -1, 0], [0, -1, 0]]], dtype=np.int64)
ES_EDGE = np.array([[0, 2, 6, 4], [3, 7, 5, 1], [8, 9, 10, 11]], dtype=np.int64)


def mask_from_fractions(grid, frac):
    """Cumulative voxel cut mask implied by the first-cut fractions: every grid edge whose +axis
    directed slot holds a fraction >= 0 sets its bit in each occupied voxel of its stencil."""
    dx, dy, dz = grid.dims
    edges = np.asarray(grid.edges, dtype=np.int64).reshape(-1, 4)
    axis, base = edges[:, 0], edges[:, 1:4]
    nx, nxy = dx + 1, (dx + 1) * (dy + 1)
    a = base[:, 0] + nx * base[:, 1] + nxy * base[:, 2]
    cut = np.asarray(frac, dtype=np.float32).reshape(-1)[6 * a + 2 * axis + 1] >= 0
    mask = np.zeros(dx * dy * dz, dtype=np.uint32)
    occupied = np.asarray(grid.occupied).reshape(-1) != 0
    for s in range(4):
        v = base + ES_OFF[axis, s]
        inside = (v >= 0).all(axis=1) & (v[:, 0] < dx) & (v[:, 1] < dy) & (v[:, 2] < dz) & cut
        vid = v[inside, 0] + dx * (v[inside, 1] + dy * v[inside, 2])
        keep = occupied[vid]
        np.bitwise_or.at(mask, vid[keep], (np.uint32(1) << ES_EDGE[axis[inside], s][keep].astype(np.uint32)))
    return mask


def _reference_ints(session, symbol, count):
    accessor = getattr(session.dll, symbol)
    accessor.restype = ctypes.c_void_p
    return _device_floats(accessor(), count).view(np.int32).copy()


def capture(session, cut=True):
    """The state a frame of `session` hands to the next (see the module docstring)."""
    g = session.grid
    n = len(g.positions)
    st = dict(pos=session.positions(), vel=session.velocities(), nbr=session.neighbors())
    if session.reference:
        st["bends"] = _reference_ints(session, "_Z18physics_bend_pairsv", 15 * n * 8).reshape(-1, 8)
        st["active"] = _reference_ints(session, "_Z14physics_activev", n)
    else:
        bends = np.empty((15 * n, 8), dtype=np.int32)
        session.check("LCS_GetBendPairs", pointer(bends))
        st["bends"] = bends
        active = np.empty(n, dtype=np.int32)
        assert session.dll.GBT_GetActive(pointer(active)) == 0
        st["active"] = active
    st["rot"] = np.ascontiguousarray(session.particle_frames(), dtype=np.float32)
    if cut:
        st["frac"] = session.cut_edge_fractions()
        st["rev"] = session.topology_revision()
        st["tears"] = int(session.cut_debug()[15])
        st["mask"] = mask_from_fractions(g, st["frac"])
        if not session.reference:
            st["own_mask"] = session.voxel_cut_mask()
    return st


def load(session, st, cut=True):
    """Overwrite `session`'s carried state with `st` (GBT_SetState)."""
    f = session.dll.GBT_SetState
    f.argtypes = (ctypes.c_void_p,) * 8 + (ctypes.c_int, ctypes.c_uint)
    f.restype = ctypes.c_int
    arrays = [np.ascontiguousarray(st[k]) for k in ("pos", "vel", "nbr", "bends", "active")]
    if cut:
        arrays += [np.ascontiguousarray(st["mask"], dtype=np.uint32), np.ascontiguousarray(st["frac"], dtype=np.float32)]
    else:
        arrays += [None, None]
    arrays.append(np.ascontiguousarray(st["rot"], dtype=np.float32))
    ptrs = [a.ctypes.data_as(ctypes.c_void_p) if a is not None else None for a in arrays]
    rc = f(*ptrs, 1 if cut else 0, int(st["rev"]) if cut else 0)
    assert rc == 0, f"GBT_SetState failed with {rc}"


def diff(a, b, active, diag):
    """Per-state differences: max |position| and |velocity| difference over active nodes (positions as
    a fraction of the bounding-box diagonal), and whether the integer topology is identical."""
    out = dict(pos=float(np.abs(a["pos"] - b["pos"])[active].max()) / diag,
               vel=float(np.abs(a["vel"] - b["vel"])[active].max()),
               nbr=bool(np.array_equal(a["nbr"], b["nbr"])),
               bends=bool(np.array_equal(a["bends"][:, 4], b["bends"][:, 4])),
               active=bool(np.array_equal(a["active"], b["active"])))
    if "rev" in a and "rev" in b:
        out.update(rev=a["rev"] == b["rev"], mask=bool(np.array_equal(a["mask"], b["mask"])),
                   frac_cut=bool(np.array_equal(a["frac"] >= 0, b["frac"] >= 0)))
    return out


def replay(reference, others, steps, command, cut=True):
    """Free-run `reference` for `steps` steps, then step every session of `others` (name -> session)
    from the reference's state of each step.  `command(session, k)` sends step k's commands and
    returns whether the rod-phase cut follows the step.  Returns (reference states, {name: [states]})
    where states[k] is the state after step k + 1."""
    ref_states = []
    for k in range(steps):
        detect = command(reference, k)
        reference.step(detect_cut=detect)
        ref_states.append(capture(reference, cut))
    out = {name: [] for name in others}
    for name, s in others.items():
        for k in range(steps):
            detect = command(s, k)
            if k > 0:
                load(s, ref_states[k - 1], cut)
            s.step(detect_cut=detect)
            out[name].append(capture(s, cut))
    return ref_states, out


def free_run(session, steps, command, cut=True, record=()):
    """Step `session` freely; returns {step: state} for the steps in `record` (1-based)."""
    rec = {}
    for k in range(steps):
        detect = command(session, k)
        session.step(detect_cut=detect)
        if k + 1 in record:
            rec[k + 1] = capture(session, cut)
    return rec
