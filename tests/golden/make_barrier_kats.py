"""Extract the known answers of the reference's harmonic-barrier tests into
barrier_kats.json.

Reads ``src/pytest/test_external.py`` of the azplugins tree AS TEXT (``ast``; the
file imports hoomd, which is not needed). For ``test_planar_harmonic_barrier`` and
``test_spherical_harmonic_barrier`` it records the box, positions, type ids and
the ``CustomVariant(z=...)`` of the test, then one stage per ``sim.run(n)``: the
timestep reached, the per-type ``params`` in force, and every expected energy and
force of the assertions that follow (their expressions evaluated with the test's
own constants kA, dB, kB).

Usage: python tests/golden/make_barrier_kats.py [/path/to/azplugins]
"""

from __future__ import annotations

import ast
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = ("test_planar_harmonic_barrier", "test_spherical_harmonic_barrier")


def _eval(node, env):
    return eval(compile(ast.Expression(node), "<kat>", "eval"), {"__builtins__": {}}, dict(env))


def _dict_call(node, env):
    return {kw.arg: float(_eval(kw.value, env)) for kw in node.keywords}


def _walk(stmts, env, case, stage):
    for st in stmts:
        if isinstance(st, ast.If):
            _walk(st.body, env, case, stage)
            continue
        if isinstance(st, ast.Assign) and len(st.targets) == 1:
            t = st.targets[0]
            src = ast.unparse(t)
            if isinstance(t, ast.Name):
                try:
                    env[t.id] = _eval(st.value, env)
                except Exception:
                    pass
            elif src == "snap.configuration.box":
                case["box"] = _eval(st.value, env)
            elif src == "snap.particles.position[:]":
                case["position"] = _eval(st.value, env)
            elif src == "snap.particles.typeid[:]":
                case["typeid"] = _eval(st.value, env)
            elif src == "snap.particles.types":
                case["types"] = _eval(st.value, env)
            elif src.startswith("barrier.params["):
                case["params"][_eval(t.slice, env)] = _dict_call(st.value, env)
            elif src == "barrier.params":
                pass
            if isinstance(st.value, ast.Call) and ast.unparse(st.value.func).endswith("HarmonicBarrier"):
                for kw in st.value.keywords:
                    if kw.arg == "location":
                        case["location"] = ast.unparse(kw.value)
            continue
        if isinstance(st, ast.Expr) and isinstance(st.value, ast.Call):
            call = st.value
            fn = ast.unparse(call.func)
            if fn == "sim.run":
                case["timestep"] += int(_eval(call.args[0], env))
                stage = {"timestep": case["timestep"], "line": st.lineno,
                         "params": json.loads(json.dumps(case["params"])), "energies": {}, "forces": {}}
                case["stages"].append(stage)
            elif fn == "numpy.testing.assert_allclose" and ast.unparse(call.args[0]).startswith("forces["):
                i = int(_eval(call.args[0].slice, env))
                stage["forces"][str(i)] = [float(x) for x in _eval(call.args[1], env)]
            continue
        if isinstance(st, ast.Assert) and isinstance(st.test, ast.Call):
            call = st.test
            if ast.unparse(call.func) == "numpy.isclose" and ast.unparse(call.args[0]).startswith("energies["):
                i = int(_eval(call.args[0].slice, env))
                stage["energies"][str(i)] = float(_eval(call.args[1], env))
    return stage


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AZP_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_barrier_kats.py <azplugins source tree> (or set AZP_REFERENCE_ROOT)")
    path = os.path.join(root, "src", "pytest", "test_external.py")
    tree = ast.parse(open(path).read())
    out = {"source": "src/pytest/test_external.py"}
    z = None
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name == "custom_variant_fixture":
            for sub in ast.walk(node):
                if isinstance(sub, ast.Call) and ast.unparse(sub.func) == "CustomVariant":
                    z = float(_eval(sub.keywords[0].value, {}))
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name in TESTS:
            case = {"line": node.lineno, "params": {}, "stages": [], "timestep": 0}
            _walk(node.body, {}, case, None)
            # CustomVariant (src/pytest/test_external.py:11-27): z up to timestep 1, z - 1 after
            case["variant_z"] = z
            del case["timestep"]
            out["planar" if "planar" in node.name else "spherical"] = case
    with open(os.path.join(HERE, "barrier_kats.json"), "w") as f:
        json.dump(out, f, indent=1)
    print({k: len(v["stages"]) for k, v in out.items() if isinstance(v, dict)})


if __name__ == "__main__":
    main()
