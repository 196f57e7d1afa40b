"""Generate adapter_signatures.json: the ctypes signature table the reference adapter binds
(endoscopic_tissue/native_backend.py:229-263, NativeTissue.__init__), read from its source text with
`ast` (the module itself imports trimesh, which is not installed), so a CPU test can bind exactly that
table against libgbtissue.so.

Run where the reference tree is mounted:
    python tests/golden/make_adapter_signatures.py <reference_root>
"""
import ast
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def table(node):
    """[(name, [argtypes], restype)] from a tuple of ("name", (P,) * 7 | (I, F, ...), I | None) literals."""
    names = {"P": "P", "I": "I", "F": "F"}

    def args(expr):
        if isinstance(expr, ast.BinOp) and isinstance(expr.op, ast.Mult):     # (P,) * 7
            return args(expr.left) * expr.right.value
        if isinstance(expr, ast.Tuple):
            return [names[e.id] for e in expr.elts]
        raise ValueError(ast.dump(expr))

    out = []
    for item in node.elts:
        name, argtuple, res = item.elts
        out.append([name.value, args(argtuple), None if isinstance(res, ast.Constant) else names[res.id]])
    return out


def main(root):
    src = (Path(root) / "endoscopic_tissue" / "native_backend.py").read_text()
    tree = ast.parse(src)
    signatures, scissors = None, None
    for node in ast.walk(tree):
        if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
            if node.targets[0].id == "signatures" and isinstance(node.value, ast.Tuple):
                signatures = table(node.value)
        if isinstance(node, ast.AugAssign) and isinstance(node.target, ast.Name) and node.target.id == "signatures":
            scissors = table(node.value)
    assert signatures and scissors
    out = {"source": "endoscopic_tissue/native_backend.py (NativeTissue.__init__)", "signatures": signatures,
           "scissors_signatures": scissors}
    lines = ['{', f' "source": {json.dumps(out["source"])},']
    for key in ("signatures", "scissors_signatures"):
        rows = [" " * 2 + json.dumps(r) for r in out[key]]
        lines.append(f' "{key}": [\n' + ",\n".join(rows) + "\n ]" + ("," if key == "signatures" else ""))
    lines.append("}")
    (HERE / "adapter_signatures.json").write_text("\n".join(lines) + "\n")
    print(f"{len(signatures)} + {len(scissors)} entry points")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_adapter_signatures.py <reference_root>")
    main(sys.argv[1])
