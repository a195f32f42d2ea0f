"""ImageHarmonic bond on the CPU: the oracle against the reference test's cases
(src/pytest/test_bond.py:240-309, golden/kats.json "image_bond": box 5, k = 2,
r0 = 1, energy (d - 1)^2 split in halves, force -2 (d - 1) along the unwrapped
bond), the oracle's per-particle loop (the MD loop's form) against its bond-list
loop, energy conservation of the oracle's MD loop with image bonds across the
box faces, and the parameter builders of the C ABI."""

import numpy as np
import pytest

from helpers import image_chains, load_golden

CASES = load_golden("kats.json")["image_bond"]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['image_1']}-{c['image_2']}")
def test_oracle_matches_reference(orc, case):
    L = np.array([5.0, 5.0, 5.0])
    p1, p2 = np.array(case["position_1"], float), np.array(case["position_2"], float)
    i1, i2 = np.array(case["image_1"]), np.array(case["image_2"])
    rec = np.zeros(8)
    rec[:2] = [2.0, 1.0]
    pos = np.array([[*p1, 0.0], [*p2, 0.0]])
    F, U, W = orc.image_bond_forces(pos, np.array([i1, i2], dtype=np.int32), L, [[0, 1]], [0], "ImageHarmonic",
                                    rec[None])
    u1, u2 = p1 + i1 * L, p2 + i2 * L
    d = np.linalg.norm(u2 - u1)
    e = (d - 1) ** 2
    np.testing.assert_allclose(U, [0.5 * e, 0.5 * e], rtol=1e-12)
    fv = -2 * (d - 1) * (-(u2 - u1) / d)
    np.testing.assert_allclose(F, [fv, -fv], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(W[0], W[1])


def test_param_builders(orc):
    from azplugins_gb300 import _lib

    L = _lib.load()
    vals = np.array([25.0, 1.2])
    rec = np.zeros(8)
    assert L.azp_bond_params_from_values(2, vals.ctypes.data, rec.ctypes.data) == 0
    np.testing.assert_array_equal(rec, orc.bond_params("ImageHarmonic", dict(k=25.0, r0=1.2)))
    back = np.zeros(2)
    assert L.azp_bond_params_to_values(2, rec.ctypes.data, back.ctypes.data) == 0
    np.testing.assert_array_equal(back, vals)
    assert L.azp_bond_num_values(2) == 2


def test_front_end():
    import azplugins_gb300 as az

    ih = az.bond.ImageHarmonic()
    ih.params["A-A"] = dict(k=25.0, r0=1.0)
    assert ih.kind == 2
    np.testing.assert_array_equal(ih._table(["A-A"])[0, :2], [25.0, 1.0])
    assert ih.record_to_dict(ih._table(["A-A"])[0]) == dict(k=25.0, r0=1.0)
    with pytest.raises(KeyError):
        ih.params["B-B"] = dict(k=1.0)


def _rec():
    rec = np.zeros((2, 8))
    rec[0, :2] = [30.0, 1.0]
    rec[1, :2] = [5.0, 1.5]
    return rec


def test_per_particle_loop_matches_bond_loop(orc):
    pos, img, un, bonds, btypes, L = image_chains()
    pos4 = np.concatenate([pos, np.zeros((len(pos), 1))], axis=1)
    F, U, W = orc.image_bond_forces(pos4, img, L, bonds, btypes, "ImageHarmonic", _rec())
    F2, U2, W2 = np.zeros_like(F), np.zeros_like(U), np.zeros_like(W)
    orc.image_bond_forces_pp(pos4, img, L, orc.bond_table(len(pos), bonds, btypes), "ImageHarmonic", _rec(), F2, U2,
                             W2)
    scale = np.abs(F).max()
    assert np.abs(F2 - F).max() <= 1e-13 * scale
    assert np.abs(U2 - U).max() <= 1e-13 * np.abs(U).max()
    assert np.abs(W2 - W).max() <= 1e-13 * np.abs(W).max()
    # Newton's third law on the unwrapped bond vectors
    assert np.abs(F2.sum(axis=0)).max() <= 1e-11 * scale


def test_oracle_md_conserves_energy_across_faces(orc):
    """Velocity Verlet (the Langevin step without drag or noise) on chains whose
    bonds cross the box faces: the images the step updates enter the bond
    vectors, so a missed image update would show as an energy jump."""
    pos, img, un, bonds, btypes, L = image_chains(n_chains=60)
    N = len(pos)
    rng = np.random.Generator(np.random.PCG64(3))
    system = dict(pos4=np.concatenate([pos, np.zeros((N, 1))], axis=1),
                  vel4=np.concatenate([rng.normal(0, 1.0, size=(N, 3)), np.ones((N, 1))], axis=1),
                  accel=np.zeros((N, 3)), image=img.copy(), types=np.zeros(N, dtype=np.int32),
                  tags=np.arange(N, dtype=np.uint32), L=L, ntypes=1, bonds=bonds.astype(np.int32), btypes=btypes)
    md = orc.OracleMD(system, bond=dict(name="ImageHarmonic", params=_rec()), method="langevin", gamma=[0.0], kT=0.0,
                      dt=0.001, seed=1, noiseless=True)
    F, U, _ = md.forces()
    md.s["accel"][:] = F
    energies = []
    for _ in range(20):
        md.run(25)
        F, U, _ = md.forces()
        v = md.s["vel4"][:, :3]
        energies.append(U.sum() + 0.5 * (v * v).sum())
    wrapped = np.abs(md.s["image"] - img).sum()
    assert wrapped > 10
    e = np.array(energies)
    assert np.abs(e - e[0]).max() < 1e-3 * abs(e[0])
