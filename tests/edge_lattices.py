"""The edge lattices shared by the GPU parity test and its oracle check: one cell, a rod of cells
along x, a one-cell column, a one-cell-thick sheet, an odd-sized capsule block, a thin sheet the
blade cuts through and a small cube the blade misses."""
STEPS = 20
CASES = [
    ("c1", (0.2, 0.2, 0.2)),    # one cell of tissue in a 5 x 5 x 5 lattice
    ("c1", (2.2, 0.2, 0.2)),    # a rod of cells along x
    ("c1", (0.2, 1.8, 0.2)),    # a one-cell column standing on its bed
    ("c1", (1.6, 0.2, 1.2)),    # a one-cell-thick sheet
    ("c2", (1.5, 0.9, 1.1)),    # the capsule press on an odd-sized block
    ("c3", (2.0, 0.4, 1.6)),    # the blade through a thin sheet (it severs links)
    ("c3", (0.6, 0.6, 0.6)),    # the blade path on a small cube it never reaches
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
