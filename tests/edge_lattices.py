"""The edge lattices shared by the GPU parity test and its oracle check (tissue extents in cells,
the builder's active nodes): the smallest block, a rod along x, a column, a two-cell-thick sheet,
an odd-sized capsule block, a thin sheet the blade cuts through and a small cube the blade misses."""
STEPS = 20
CASES = [
    ("c1", (0.2, 0.2, 0.2)),    # 2 x 2 x 2 cells (27 nodes) in a 5 x 5 x 5 lattice
    ("c1", (2.2, 0.2, 0.2)),    # a rod along x, 11 x 2 x 2 cells
    ("c1", (0.2, 1.8, 0.2)),    # a column, 2 x 9 x 2 cells, standing on its bed
    ("c1", (1.6, 0.2, 1.2)),    # a sheet two cells thick, 9 x 2 x 6
    ("c2", (1.5, 0.9, 1.1)),    # the capsule press on an odd-sized block, 8 x 5 x 6
    ("c3", (2.0, 0.4, 1.6)),    # the blade through a thin sheet, 10 x 3 x 9 (it severs links)
    ("c3", (0.6, 0.6, 0.6)),    # the blade path on a 4 x 4 x 4 cube it never reaches
]


def run(workload, lib, topology):
    session = workload.open(lib)
    try:
        workload.run(session, steps=STEPS)
        out = {"pos": session.positions(), "vel": session.velocities()}
        if topology:
            out.update(nbr=session.neighbors(), rev=session.topology_revision())
        return out
    finally:
        session.close()
