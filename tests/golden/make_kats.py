"""Extract the known-answer cases of the reference's own tests into kats.json.

Reads ``src/pytest/test_pair.py``, ``src/pytest/test_bond.py`` (also the
``test_image_harmonic`` parameter list) and ``src/pytest/test_wall.py`` of the
azplugins tree AS TEXT (``ast``; the files import hoomd, which is not needed):
every ``PotentialTestCase(...)`` call becomes one record with its line number.

Usage: python tests/golden/make_kats.py [/path/to/azplugins]
"""

from __future__ import annotations

import ast
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _value(node):
    # dict(k=v, ...) calls are literals too
    if isinstance(node, ast.Call) and getattr(node.func, "id", None) == "dict":
        return {kw.arg: ast.literal_eval(kw.value) for kw in node.keywords}
    return ast.literal_eval(node)


def cases(path, fields):
    tree = ast.parse(open(path).read())
    out = []
    for node in ast.walk(tree):
        if isinstance(node, ast.Call) and getattr(node.func, "id", None) == "PotentialTestCase":
            pot = node.args[0]
            name = pot.attr  # hoomd.azplugins.pair.<Name>
            vals = [_value(a) for a in node.args[1:]]
            rec = {"potential": name, "line": node.lineno}
            rec.update(dict(zip(fields, vals)))
            out.append(rec)
    return out


def image_bond_cases(path):
    """The parametrize list of test_image_harmonic: positions and images of the
    two bonded particles (the test computes the expected values from them)."""
    tree = ast.parse(open(path).read())
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name == "test_image_harmonic":
            for dec in node.decorator_list:
                if isinstance(dec, ast.Call) and ast.unparse(dec.func).endswith("parametrize"):
                    rows = ast.literal_eval(dec.args[1])
                    return [{"position_1": r[0], "position_2": r[1], "image_1": r[2], "image_2": r[3],
                             "line": node.lineno, "source": f"src/pytest/test_bond.py:{dec.lineno}"} for r in rows]
    return []


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AZP_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_kats.py <azplugins source tree> (or set AZP_REFERENCE_ROOT)")
    pair = cases(os.path.join(root, "src", "pytest", "test_pair.py"),
                 ["params", "r_cut", "shift", "distance", "energy", "force"])
    bond = cases(os.path.join(root, "src", "pytest", "test_bond.py"), ["params", "distance", "energy", "force"])
    wall = cases(os.path.join(root, "src", "pytest", "test_wall.py"), ["params", "position", "energy", "force"])
    image_bond = image_bond_cases(os.path.join(root, "src", "pytest", "test_bond.py"))
    for r in pair:
        r["source"] = f"src/pytest/test_pair.py:{r['line']}"
    for r in bond:
        r["source"] = f"src/pytest/test_bond.py:{r['line']}"
    for r in wall:
        r["source"] = f"src/pytest/test_wall.py:{r['line']}"
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump({"pair": pair, "bond": bond, "wall": wall, "image_bond": image_bond}, f, indent=1)
    print(f"{len(pair)} pair, {len(bond)} bond, {len(wall)} wall and {len(image_bond)} image-bond cases")


if __name__ == "__main__":
    main()
