"""Extract the reference's known-answer vectors into golden.json.

Run in a container where the reference sources are present:

    python tests/golden/make_golden.py /root/reference

The reference package cannot be imported (quimb / primme / tensornetwork are
absent), so its test files and notebook are read as text: every ``np.array``
literal the known-answer tests compare against is parsed with ``ast`` and
evaluated with only ``np`` in scope. The notebook ED spectrum is read from the
printed cell output. Output: ``tests/golden/golden.json`` (committed); nothing
at test time reads the reference.
"""
from __future__ import annotations

import ast
import json
import re
import sys
from pathlib import Path

import numpy as np


def _arrays(path: Path):
    """All np.array(...) literals of a file, in source order, with their line numbers."""
    src = path.read_text()
    tree = ast.parse(src)
    out = []
    for node in ast.walk(tree):
        if (
            isinstance(node, ast.Call)
            and isinstance(node.func, ast.Attribute)
            and node.func.attr == "array"
            and isinstance(node.func.value, ast.Name)
            and node.func.value.id == "np"
            and node.args
            and isinstance(node.args[0], ast.List)
        ):
            expr = ast.get_source_segment(src, node)
            val = eval(expr, {"__builtins__": {}, "np": np})  # noqa: S307 (literal arrays only)
            arr = np.asarray(val)
            if not np.iscomplexobj(arr):
                out.append((node.lineno, arr.astype(float)))
    out.sort(key=lambda t: t[0])
    return out


def main(ref: str):
    ref = Path(ref)
    g = {"source": "tanlin2013/tnpy test files and docs/source/notebooks/tsdrg.ipynb"}

    ops = _arrays(ref / "tests/test_operators.py")
    # TestFullHamiltonian params, in order: RandomHeisenberg(n=2,h=0), (n=3,h=0), XXZ(n=2,0.5), XXZ(n=3,0.5)
    mats = [a for _, a in ops if a.ndim == 2 and a.shape[0] in (4, 8)]
    g["full_hamiltonian"] = [
        {"model": "random_heisenberg", "n": 2, "h": 0.0, "matrix": mats[0].tolist(),
         "ref": "tests/test_operators.py:42-46"},
        {"model": "random_heisenberg", "n": 3, "h": 0.0, "matrix": mats[1].tolist(),
         "ref": "tests/test_operators.py:48-63"},
        {"model": "xxz", "n": 2, "delta": 0.5, "matrix": mats[2].tolist(),
         "ref": "tests/test_operators.py:66-71"},
        {"model": "xxz", "n": 3, "delta": 0.5, "matrix": mats[3].tolist(),
         "ref": "tests/test_operators.py:73-88"},
    ]

    ed = _arrays(ref / "tests/test_exact_diagonalization.py")
    g["ed_n2"] = {
        "model": "random_heisenberg", "n": 2, "h": 0.0,
        "matrix": ed[0][1].tolist(), "evals": ed[1][1].tolist(), "evecs": ed[2][1].tolist(),
        "ref": "tests/test_exact_diagonalization.py:15-42",
    }

    ts = _arrays(ref / "tests/test_tsdrg.py")
    g["tsdrg_block"] = {
        "model": "random_heisenberg", "n": 8, "h": 0.0, "chi": 64,
        "block_hamiltonian": ts[0][1].tolist(), "evecs": ts[1][1].tolist(),
        "ref": "tests/test_tsdrg.py:116-140",
    }

    nb = json.loads((ref / "docs/source/notebooks/tsdrg.ipynb").read_text())
    text = None
    for cell in nb["cells"]:
        if cell.get("cell_type") != "code":
            continue
        src = "".join(cell.get("source", []))
        if "ExactDiagonalization(model.mpo)" in src and "print(ed.evals)" in src:
            text = "".join("".join(o.get("text", [])) for o in cell.get("outputs", []))
            break
    vals = [float(v) for v in re.findall(r"-?\d+\.\d+(?:e[-+]\d+)?", text)]
    g["notebook_ed"] = {
        "model": "random_heisenberg", "n": 6, "h": 3.0, "seed": 2021, "evals": vals,
        "printed_decimals": 8, "ref": "docs/source/notebooks/tsdrg.ipynb:140-152",
    }
    tsdrg_text = None
    for cell in nb["cells"]:
        src = "".join(cell.get("source", []))
        if cell.get("cell_type") == "code" and "TreeTensorNetworkSDRG(model.mpo, chi=4)" in src:
            tsdrg_text = "".join("".join(o.get("text", [])) for o in cell.get("outputs", []))
            break
    merges = re.findall(r"merging TreeNode\((\d+)\) and TreeNode\((\d+)\)", tsdrg_text)
    last = tsdrg_text.split("Obtain ground state energies")[-1]
    g["notebook_tsdrg"] = {
        "model": "random_heisenberg", "n": 6, "h": 3.0, "seed": 2021, "chi": 4,
        "evals": [float(v) for v in re.findall(r"-?\d+\.\d+", last)],
        "merged_pairs_old_ids": [[int(a), int(b)] for a, b in merges],
        "printed_decimals": 8, "ref": "docs/source/notebooks/tsdrg.ipynb:180-200",
    }
    g["fdmrg_vs_ed"] = {"model": "xxz", "n": 10, "delta": 0.5, "bond_dim": 32, "atol": 1e-8,
                        "ref": "tests/test_finite_dmrg.py:9-23"}
    g["tsdrg_vs_ed"] = {"model": "random_heisenberg", "n": 4, "h": 0.1, "chi": 4, "atol": 1e-8,
                        "ref": "tests/test_tsdrg.py:98-147"}

    out = Path(__file__).with_name("golden.json")
    out.write_text(json.dumps(g, indent=1))
    print(f"wrote {out}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the tnpy source tree>")
    main(sys.argv[1])
