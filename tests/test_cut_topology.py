"""Cut topology of the live mesh (GBT_CutTopologyBuild / GBT_GetCutTopology): live tets, vertex
duplication and greedy re-colouring, a product of this library with no counterpart in the
reference (whose cut severs links and keeps the bind-time colouring).

CPU: the oracle (oracle/cut_topology_oracle.inc) against an independent pure-Python restatement on
small lattices with links severed at random through GBT_SetState (duplications occur there), and
its properties on the C3 blade workload: with nothing cut it returns every tet and the bind-time
colouring; after cuts every colour class is vertex-disjoint and every tet holds the smallest colour
its earlier neighbours leave free.
GPU: the CUDA library's product equals the oracle's bit for bit (tets, vertex ids, duplication map,
colours) on the same topologies, up to the full-size C3 lattice after 30 blade frames.
"""
import ctypes
import json

import numpy as np
import pytest

from genesis_tissue_simulation_gb300 import workloads as W
from genesis_tissue_simulation_gb300.grid import build_grid
from genesis_tissue_simulation_gb300.native_backend import PlainTissue
from conftest import results_dir

SMALL_C3 = (4.78, 2.38, 3.98)     # 24 x 12 x 20 cells
KUHN = [(0, 1, 3, 7), (0, 3, 2, 7), (0, 2, 6, 7), (0, 6, 4, 7), (0, 4, 5, 7), (0, 5, 1, 7)]


def set_topology(session, nbr, active=None):
    f = session.dll.GBT_SetState
    f.argtypes = (ctypes.c_void_p,) * 8 + (ctypes.c_int, ctypes.c_uint)
    f.restype = ctypes.c_int
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    act = None if active is None else np.ascontiguousarray(active, dtype=np.int32)
    rc = f(None, None, nbr.ctypes.data_as(ctypes.c_void_p), None,
           None if act is None else act.ctypes.data_as(ctypes.c_void_p), None, None, None, 0, 0)
    assert rc == 0, rc


def sever_at_random(grid, fraction, seed, box=None):
    """The grid's neighbour table with a random `fraction` of the live links inside `box` (a node
    predicate) cut on both halves."""
    nbr = grid.neighbors.reshape(-1, 6).copy()
    rng = np.random.default_rng(seed)
    for i in range(len(nbr)):
        if box is not None and not box(i):
            continue
        for a in range(3):
            j = nbr[i, 2 * a + 1]
            if j >= 0 and rng.random() < fraction:
                nbr[i, 2 * a + 1] = -1
                nbr[j, 2 * a] = -1
    return nbr.reshape(-1)


def restated(session):
    """The product restated independently: liveness from the neighbour table, groups by a breadth-
    first search over shared faces, first-fit colours with Python sets."""
    g = session.grid
    nbr = session.neighbors().reshape(-1, 6)
    ids = session.tet_ids()
    active = g.active != 0
    dx, dy, _ = g.dims
    nx, nxy = dx + 1, (dx + 1) * (dy + 1)
    N = len(active)

    def off(c):
        return (c & 1) + ((c >> 1) & 1) * nx + ((c >> 2) & 1) * nxy

    typ = [next(t for t, q in enumerate(KUHN) if off(q[1]) == d) for d in ids[:, 1] - ids[:, 0]]
    live = []
    for d in sorted(range(len(ids)), key=lambda d: (int(ids[d, 0]), typ[d])):
        q, n0 = KUHN[typ[d]], int(ids[d, 0])
        ok = all(active[ids[d]])
        for a in range(4):
            for b in range(a + 1, 4):
                diff = q[a] ^ q[b]
                if diff in (1, 2, 4):
                    axis = {1: 0, 2: 1, 4: 2}[diff]
                    low = q[b] if (q[a] >> axis) & 1 else q[a]
                    ok = ok and nbr[n0 + off(low), 2 * axis + 1] >= 0
        if ok:
            live.append(d)
    around = [[] for _ in range(N)]
    for t, d in enumerate(live):
        for v in ids[d]:
            around[v].append(t)
    group = {}
    groups = np.zeros(N, dtype=np.int64)
    for v in range(N):
        members, label = around[v], {}
        for t in members:                      # members in emission order: a new label per first member
            if t in label:
                continue
            label[t] = len(set(label.values()))
            queue = [t]
            while queue:
                a = queue.pop()
                for b in members:
                    if b not in label and len(set(ids[live[a]]) & set(ids[live[b]])) >= 3:
                        label[b] = label[t]
                        queue.append(b)
        groups[v] = len(set(label.values()))
        for t in members:
            group[(t, int(v))] = label[t]
    extra = np.maximum(groups - 1, 0)
    base = np.concatenate([[0], np.cumsum(extra)[:-1]])
    parent = [v for v in range(N) for _ in range(extra[v])]
    nodes = np.array([[v if group[(t, int(v))] == 0 else N + base[v] + group[(t, int(v))] - 1 for v in ids[d]]
                      for t, d in enumerate(live)], dtype=np.int64).reshape(-1, 4)
    colour, used = [], {}
    for t in range(len(live)):
        taken = set().union(*(used.get(int(v), set()) for v in nodes[t]))
        c = 0
        while c in taken:
            c += 1
        colour.append(c)
        for v in nodes[t]:
            used.setdefault(int(v), set()).add(c)
    return dict(tet_nodes=nodes, tet_source=np.array(live), tet_colour=np.array(colour), dup_parent=np.array(parent, dtype=np.int64))


def assert_same(a, b):
    for k in ("tet_nodes", "tet_source", "tet_colour", "dup_parent"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def check_properties(session, ct):
    """Every colour class vertex-disjoint; every tet's colour the smallest its earlier neighbours
    leave free; the duplication map names nodes; vertex ids below N + D."""
    nodes, colour = ct["tet_nodes"], ct["tet_colour"]
    N = len(session.grid.positions)
    assert nodes.max(initial=-1) < N + len(ct["dup_parent"])
    assert np.all(ct["dup_parent"] < N)
    for c in range(ct["colours"]):
        members = nodes[colour == c].ravel()
        assert len(members) == len(np.unique(members)), c
    seen = {}
    for t in range(len(colour)):
        taken = set().union(*(seen.get(int(v), set()) for v in nodes[t]))
        c = 0
        while c in taken:
            c += 1
        assert colour[t] == c, t
        for v in nodes[t]:
            seen.setdefault(int(v), set()).add(int(colour[t]))


def small_grid():
    return build_grid(0.5, size=(3.0, 1.5, 2.5))


def open_small(lib):
    s = PlainTissue(small_grid(), dt=1 / 60, substeps=4, ks=1e6, dll_path=lib)
    s.set_gravity(0.0, -981.0, 0.0)
    return s


@pytest.mark.parametrize("fraction,seed", [(0.0, 0), (0.15, 1), (0.3, 2), (0.6, 3)])
def test_oracle_matches_restatement_on_random_cuts(oracle_libs, fraction, seed):
    with open_small(oracle_libs[0]) as s:
        set_topology(s, sever_at_random(s.grid, fraction, seed))
        ct = s.cut_topology()
        assert_same(ct, restated(s))
        check_properties(s, ct)
        if fraction >= 0.3:
            assert len(ct["dup_parent"]) > 0, "the random cut should split some node's tets"


def test_oracle_on_blade_workload(oracle_libs):
    w = W.make("c3", scale=SMALL_C3)
    with w.open(dll_path=oracle_libs[0]) as s:
        static = s.tet_colors()
        ct = s.cut_topology()
        assert len(ct["tet_source"]) == s.tet_count and len(ct["dup_parent"]) == 0
        assert np.array_equal(ct["tet_source"][np.argsort(ct["tet_source"])], np.arange(s.tet_count))
        assert np.array_equal(ct["tet_colour"], static[ct["tet_source"]]), "uncut: the bind-time colouring"
        w.run(s, steps=40)
        assert s.topology_revision() > 0
        ct = s.cut_topology()
        assert len(ct["tet_source"]) < s.tet_count
        check_properties(s, ct)


# ---- GPU: the CUDA library against the oracle ------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("fraction,seed", [(0.0, 0), (0.3, 2), (0.6, 3)])
def test_cuda_matches_oracle_on_random_cuts(gpu_lib, oracle_libs, fraction, seed):
    out = []
    for lib in (gpu_lib, oracle_libs[0]):
        with open_small(lib) as s:
            set_topology(s, sever_at_random(s.grid, fraction, seed))
            out.append(s.cut_topology())
    assert_same(*out)
    assert out[0]["colours"] == out[1]["colours"]
    if fraction > 0:
        assert len(out[0]["dup_parent"]) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("scale,frames", [(SMALL_C3, 40), (None, 30)])
def test_cuda_matches_oracle_on_blade_workload(gpu_lib, oracle_libs, scale, frames):
    """The CUDA library runs the blade workload; the oracle takes its topology (neighbour table and
    active flags) and builds the product from it."""
    w = W.make("c3", scale=scale) if scale else W.make("c3")
    with w.open(dll_path=gpu_lib) as s:
        before = s.cut_topology()
        assert before["sweeps"] == 1 and len(before["dup_parent"]) == 0
        w.run(s, steps=frames)
        gpu = s.cut_topology()
        again = s.cut_topology()     # nothing severed since: the product stands, no relaxation
        nbr = s.neighbors()
        prior = np.full(s.tet_count, -1)
        prior[before["tet_source"]] = before["tet_colour"]
    assert_same(gpu, again)
    assert gpu["sweeps"] >= 1 and again["sweeps"] == 0
    with w.open(dll_path=oracle_libs[0]) as o:
        set_topology(o, nbr)
        cpu = o.cut_topology()
    assert_same(gpu, cpu)
    assert gpu["colours"] == cpu["colours"]
    changed = int((gpu["tet_colour"] != prior[gpu["tet_source"]]).sum())
    with open(results_dir() / "cut_topology.jsonl", "a") as f:
        f.write(json.dumps(dict(scale=scale, frames=frames, live=len(gpu["tet_source"]), duplicates=len(gpu["dup_parent"]),
                                colours=gpu["colours"], sweeps=gpu["sweeps"], recoloured=changed)) + "\n")


@pytest.mark.gpu
def test_cuda_rebuilt_every_step_matches_oracle(gpu_lib, oracle_libs):
    """Built after every step of the blade workload, each relaxation starting from the previous
    step's colouring: at every fifth step the product equals the oracle's sequential build on the
    same topology, and the last equals a single build of the same topology from the uncut colouring
    (the fixed point does not depend on the start; the sweeps each took are recorded).  A step that
    severs nothing keeps the previous product without a relaxation (0 sweeps)."""
    w = W.make("c3", scale=SMALL_C3, steps=40)
    sweeps = []
    with w.open(dll_path=gpu_lib) as s, w.open(dll_path=oracle_libs[0]) as o:
        s.cut_topology()
        revision = s.topology_revision()
        for k in range(40):
            s.step(detect_cut=w.command(s, k))
            gpu = s.cut_topology()
            sweeps.append(gpu["sweeps"])
            severed = s.topology_revision() != revision
            revision = s.topology_revision()
            assert (gpu["sweeps"] > 0) == severed, (k, gpu["sweeps"], severed)
            if k % 5 == 4:
                set_topology(o, s.neighbors())
                assert_same(gpu, o.cut_topology())
        assert s.topology_revision() > 0
    with w.open(dll_path=gpu_lib) as fresh:     # the same topology from the uncut colouring in one build
        w.run(fresh, steps=40)
        scratch = fresh.cut_topology()
    assert_same(gpu, scratch)
    with open(results_dir() / "cut_topology.jsonl", "a") as f:
        f.write(json.dumps(dict(per_step_sweeps=sweeps, from_uncut_sweeps=scratch["sweeps"])) + "\n")
