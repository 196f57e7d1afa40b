"""The implicit lattice element codes of batched instances decode to the explicit tables (CPU).

Batched lattices address a tet by (corner-0 node, Kuhn type) and derive its four nodes and its
three link slots with ``kuhnNodes`` / ``kuhnOwners`` (csrc/tissue_device.cuh).  The explicit tables
come from mesh_build.cu: the Kuhn corner lists and, for the link slots, the scan of corner pairs that
differ in one axis bit, each owned by its lower end's +axis slot.  This test compiles the two decode
functions into a host program (nvcc, no GPU needed) and compares every Kuhn type on a few lattice
shapes with a restatement of that scan, so a decode that disagrees with the tables fails here
rather than as a wrong trajectory on the GPU.
"""
import subprocess
import textwrap
from pathlib import Path

import pytest

from genesis_tissue_simulation_gb300 import build

ROOT = Path(__file__).resolve().parents[1]
KUHN = [(0, 1, 3, 7), (0, 3, 2, 7), (0, 2, 6, 7), (0, 6, 4, 7), (0, 4, 5, 7), (0, 5, 1, 7)]
SHAPES = [(5, 4), (9, 63), (65, 33 * 65)]


def corner_offset(c, nx, nxy):
    return (c & 1) + ((c >> 1) & 1) * nx + ((c >> 2) & 1) * nxy


def table_nodes_and_owners(t, n0, nx, nxy):
    """mesh_build.cu's tet: the corner list of Kuhn type t and its axis-edge owners in pair-scan order."""
    q = KUHN[t]
    nodes = [n0 + corner_offset(c, nx, nxy) for c in q]
    owners = []
    for a in range(4):
        for b in range(a + 1, 4):
            diff = q[a] ^ q[b]
            if diff not in (1, 2, 4) or len(owners) == 3:
                continue
            axis = {1: 0, 2: 1, 4: 2}[diff]
            low = q[b] if (q[a] >> axis) & 1 else q[a]
            owners.append(6 * (n0 + corner_offset(low, nx, nxy)) + 2 * axis + 1)
    return nodes, owners


@pytest.fixture(scope="module")
def decode_program(tmp_path_factory):
    folder = tmp_path_factory.mktemp("kuhn")
    src = folder / "kuhn.cu"
    src.write_text(textwrap.dedent("""
        #include <cstdio>
        #include <cstdlib>
        #include "tissue_device.cuh"
        using namespace gbt;
        int main(int argc, char** argv) {
            const int n0 = atoi(argv[1]), nx = atoi(argv[2]), nxy = atoi(argv[3]);
            for (int t = 0; t < 6; t++) {
                int4 d = kuhnNodes(t, n0, nx, nxy);
                int o[3];
                kuhnOwners(t, n0, nx, nxy, o);
                printf("%d %d %d %d %d %d %d\\n", d.x, d.y, d.z, d.w, o[0], o[1], o[2]);
            }
            return 0;
        }
    """))
    exe = folder / "kuhn"
    cmd = [build.nvcc_path(), *build.common_flags(), f"-I{build.CSRC}", str(src), "-o", str(exe)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    assert result.returncode == 0, result.stderr
    return exe


@pytest.mark.parametrize("nx,nxy", SHAPES)
def test_implicit_tet_decode_matches_tables(decode_program, nx, nxy):
    n0 = 3 * nxy + 2 * nx + 1
    out = subprocess.run([str(decode_program), str(n0), str(nx), str(nxy)], capture_output=True, text=True, check=True)
    rows = [list(map(int, line.split())) for line in out.stdout.split("\n") if line.strip()]
    assert len(rows) == 6
    for t, row in enumerate(rows):
        nodes, owners = table_nodes_and_owners(t, n0, nx, nxy)
        assert row[:4] == nodes, (t, row[:4], nodes)
        assert row[4:] == owners, (t, row[4:], owners)
