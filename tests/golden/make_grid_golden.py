"""Generate the grid golden fixtures from the reference's own producer (endoscopic_tissue/grid.py).

Run where the reference tree is mounted:  python tests/golden/make_grid_golden.py <reference_root>
Writes grid_hashes.json (SHA-256, shape and dtype of every TissueGrid array for several build_grid
configurations) and grid_small.npz (all arrays of one small lattice).
"""
import hashlib
import importlib.util
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
if len(sys.argv) != 2:
    sys.exit("usage: make_grid_golden.py <reference_root>")
ROOT = Path(sys.argv[1])
CASES = {
    "c1_16x8x16": dict(spacing=0.2, size=(3.18, 1.58, 3.18), density=1000.0),
    "default_block_0p6": dict(spacing=0.6),
    "block_vertical_0p05": dict(spacing=0.2, vertical_spacing=0.05),
    "tab_x": dict(spacing=0.2, density=1000, vertical_spacing=.05, tab=((3.0, .3, -1.0), (4.2, .7, 1.0), 0)),
    "tab_y": dict(spacing=0.2, density=1000, vertical_spacing=.05, tab=((0.0, .7, 1.4), (2.5, 1.7, 1.8), 1)),
    "c5_32x16x32": dict(spacing=0.2, size=(6.38, 3.18, 6.38), density=1000.0),
    "c2_64x32x48": dict(spacing=0.2, size=(12.78, 6.38, 9.58), density=1000.0),
}


def digest(array):
    a = np.ascontiguousarray(array)
    return {"sha256": hashlib.sha256(a.tobytes()).hexdigest(), "shape": list(a.shape), "dtype": a.dtype.str}


def main():
    spec = importlib.util.spec_from_file_location("reference_grid", ROOT / "endoscopic_tissue" / "grid.py")
    ref = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref)
    out = {}
    for name, kwargs in CASES.items():
        kw = dict(kwargs)
        if "tab" in kw:
            low, high, attached = kw["tab"]
            kw["tab"] = ref.Tab(low, high, attached)
        g = ref.build_grid(**kw)
        entry = {"dims": list(g.dims), "spacing": g.spacing}
        for field in g.__dataclass_fields__:
            value = getattr(g, field)
            if isinstance(value, np.ndarray):
                entry[field] = digest(value)
        out[name] = entry
        if name == "default_block_0p6":
            arrays = {f: getattr(g, f) for f in g.__dataclass_fields__ if isinstance(getattr(g, f), np.ndarray)}
            np.savez_compressed(HERE / "grid_small.npz", **arrays)
    (HERE / "grid_hashes.json").write_text(json.dumps({"cases": {k: {kk: (list(vv) if isinstance(vv, tuple) else vv) for kk, vv in v.items()} for k, v in CASES.items()}, "grids": out}, indent=1))


if __name__ == "__main__":
    main()
