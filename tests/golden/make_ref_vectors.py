"""Golden vectors from the reference's OWN evaluator code.

Imports ``oracle/_ref/azp_ref`` (built by ``oracle/build_ref.sh`` from the
azplugins headers in place) and records, for seeded random parameters and
distances, the reference's (evaluated, force/r, energy), its param_type fields
and asDict round trip, and the flow-field values. The fixture travels to
machines without the reference tree; tests compare the oracle and the GPU to it.

Also records sizeof(param_type) of every evaluator in the reference's double- and
single-precision layouts (``oracle/_ref/ref_sizes_*``), which pins the C ABI's
record strides.

Usage: python tests/golden/make_ref_vectors.py (after oracle/build_ref.sh)
"""

from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))

import azp_ref  # noqa: E402


def pair_cases(rng):
    out = []
    for _ in range(60):
        sigma = rng.uniform(0.6, 1.4)
        d = dict(epsilon=rng.uniform(0.2, 3.0), sigma=sigma, attraction_scale_factor=rng.choice([0.0, 0.5, 1.0, rng.uniform()]))
        rcut = rng.uniform(1.1, 3.5) * sigma
        out.append(("PerturbedLennardJones", d, rcut, rng.uniform(0.8 * sigma, 1.1 * rcut)))
    for _ in range(40):
        delta = rng.uniform(0.0, 1.0)
        kappa = rng.uniform(0.5, 3.0)
        d = dict(epsilon=rng.uniform(0.2, 3.0), kappa=kappa, delta=delta)
        rcut = delta + 5.0 / kappa
        out.append(("ExpandedYukawa", d, rcut, rng.uniform(delta + 0.05, 1.1 * rcut)))
    for _ in range(30):
        rcut = rng.uniform(1.0, 3.0)
        out.append(("Hertz", dict(epsilon=rng.uniform(0.1, 5.0)), rcut, rng.uniform(0.1, 1.1 * rcut)))
    for _ in range(60):
        form = rng.integers(3)
        a1 = 0.0 if form == 0 else rng.uniform(0.5, 3.0)
        a2 = rng.uniform(0.5, 3.0) if form == 2 else 0.0
        if rng.uniform() < 0.5:
            a1, a2 = a2, a1
        d = dict(A=rng.uniform(10.0, 150.0), a_1=a1, a_2=a2, sigma=rng.uniform(0.8, 1.2))
        contact = a1 + a2 if form == 2 else max(a1, a2)
        rcut = contact + rng.uniform(2.0, 5.0)
        out.append(("Colloid", d, rcut, rng.uniform(contact + 0.6, 1.1 * rcut)))
    return out


def bond_cases(rng):
    out = []
    for _ in range(50):
        d = dict(k=rng.uniform(100, 2000), r_0=rng.uniform(1.2, 1.8), b_1=rng.uniform(-1.0, 0.0),
                 b_2=rng.uniform(-0.5, 0.5), U_0=rng.uniform(10, 100), sigma=rng.choice([0.0, 1.0, rng.uniform(0.8, 1.2)]),
                 epsilon=rng.choice([0.0, 1.0, rng.uniform(0.5, 2.0)]), delta=rng.choice([0.0, rng.uniform(0.0, 0.6)]))
        out.append(("Quartic", d, rng.uniform(0.85 + d["delta"], 2.0 + d["delta"])))
    for _ in range(30):
        r0 = rng.uniform(0.5, 1.5)
        d = dict(r_0=r0, r_1=r0 + rng.uniform(0.3, 1.5), U_1=rng.uniform(0.5, 6.0), U_tilt=rng.uniform(-1.0, 1.0))
        out.append(("DoubleWell", d, rng.uniform(0.3, 3.5)))
    return out


def main():
    rng = np.random.Generator(np.random.PCG64(20261203))
    pair = []
    for name, d, rcut, r in pair_cases(rng):
        d = {k: float(v) for k, v in d.items()}
        for shift in (False, True):
            ok, f, e = azp_ref.pair_eval(name, d, r * r, rcut * rcut, shift)
            pair.append(dict(name=name, params=d, rcut=rcut, r=r, shift=shift, ok=bool(ok), force_divr=f, energy=e,
                             raw=list(azp_ref.pair_raw(name, d)), asdict=azp_ref.pair_roundtrip(name, d)))
    bond = []
    for name, d, r in bond_cases(rng):
        d = {k: float(v) for k, v in d.items()}
        ok, f, e = azp_ref.bond_eval(name, d, r * r)
        bond.append(dict(name=name, params=d, r=r, ok=bool(ok), force_divr=f, energy=e,
                         raw=list(azp_ref.bond_raw(name, d)), asdict=azp_ref.bond_roundtrip(name, d)))
    flow = []
    for _ in range(20):
        U = tuple(float(x) for x in rng.uniform(-2, 2, size=3))
        r = tuple(float(x) for x in rng.uniform(-5, 5, size=3))
        flow.append(dict(kind="constant", U=U, r=r, u=list(azp_ref.constant_flow(U, r))))
        mv, sep = float(rng.uniform(0.1, 3.0)), float(rng.uniform(2.0, 20.0))
        out = azp_ref.parabolic_flow(mv, sep, r)
        flow.append(dict(kind="parabolic", mean_velocity=mv, separation=sep, r=r, u=list(out[:3]),
                         get_mean_velocity=out[3], get_separation=out[4]))
    # sizeof(param_type) of every evaluator, double- and single-precision HOOMD
    # builds, printed by oracle/ref_sizes.cpp compiled from the reference headers
    sizes = {}
    for tag in ("double", "single"):
        exe = os.path.join(REPO, "oracle", "_ref", f"ref_sizes_{tag}")
        sizes[tag] = json.loads(subprocess.run([exe], check=True, capture_output=True, text=True).stdout)
    with open(os.path.join(HERE, "ref_vectors.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_ref_vectors.py", "pair": pair, "bond": bond, "flow": flow,
                   "record_bytes": sizes}, f)
    print(f"{len(pair)} pair, {len(bond)} bond, {len(flow)} flow vectors; record sizes {sizes}")


if __name__ == "__main__":
    main()
