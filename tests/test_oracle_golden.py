"""The CPU oracle pinned against the reference: its own known-answer tests
(src/pytest/test_pair.py:22-306, src/pytest/test_bond.py:20-193), vectors of the
reference evaluators compiled in place (tests/golden/ref_vectors.json), the
published Philox4x32-10 known answers, and loop-level invariants."""

import numpy as np
import pytest

from helpers import load_golden, rel

KATS = load_golden("kats.json")
REF = load_golden("ref_vectors.json")


def _two_particle(orc, name, params, r_cut, shift, d):
    L = 2.1 * 2 * (r_cut + 0.4)
    pos4 = np.array([[-0.5 * d, 0, 0, 0], [0.5 * d, 0, 0, 0]], dtype=np.float64)
    rec = orc.pair_params(name, params)
    start, idx = orc.nlist(pos4, np.zeros(2, dtype=np.int32), 1, np.array([L, L, L]), np.array([[(r_cut + 0.4) ** 2]]))
    return orc.pair_forces(pos4, np.zeros(2, dtype=np.int32), 1, np.array([L, L, L]), start, idx, name,
                           rec.reshape(1, 1, 4), np.array([[r_cut * r_cut]]), None, "shift" if shift else "none")


@pytest.mark.parametrize("case", [c for c in KATS["pair"] if c["potential"] != "DPDGeneralWeight"],
                         ids=lambda c: f"{c['potential']}@{c['line']}")
def test_pair_kat(orc, case):
    F, U, W = _two_particle(orc, case["potential"], case["params"], case["r_cut"], case["shift"], case["distance"])
    e, f = case["energy"], case["force"]
    np.testing.assert_array_almost_equal(U, [0.5 * e, 0.5 * e], decimal=4)
    np.testing.assert_array_almost_equal(F, [[-f, 0, 0], [f, 0, 0]], decimal=4)


@pytest.mark.parametrize("case", [c for c in KATS["pair"] if c["potential"] == "DPDGeneralWeight"],
                         ids=lambda c: f"DPD@{c['line']}")
def test_dpd_conservative_kat(orc, case):
    # kT = 0 and zero velocities: only the conservative part acts
    F, U, W = _two_particle(orc, "DPDGeneralWeight", case["params"], case["r_cut"], False, case["distance"])
    e, f = case["energy"], case["force"]
    np.testing.assert_array_almost_equal(U, [0.5 * e, 0.5 * e], decimal=4)
    np.testing.assert_array_almost_equal(F, [[-f, 0, 0], [f, 0, 0]], decimal=4)


@pytest.mark.parametrize("case", KATS["bond"], ids=lambda c: f"{c['potential']}@{c['line']}")
def test_bond_kat(orc, case):
    d = case["distance"]
    L = 20.0
    pos4 = np.array([[-0.5 * d, 0, 0, 0], [0.5 * d, 0, 0, 0]], dtype=np.float64)
    rec = orc.bond_params(case["potential"], dict({"delta": 0.0}, **case["params"]))
    F, U, W = orc.bond_forces(pos4, np.array([L, L, L]), np.array([[0, 1]]), np.array([0]), case["potential"],
                              rec.reshape(1, 8))
    e, f = case["energy"], case["force"]
    np.testing.assert_array_almost_equal(U, [0.5 * e, 0.5 * e], decimal=4)
    np.testing.assert_array_almost_equal(F, [[-f, 0, 0], [f, 0, 0]], decimal=4)


def test_pair_reference_vectors(orc):
    n = 0
    for v in REF["pair"]:
        rec = orc.pair_params(v["name"], v["params"])
        raw = np.array(v["raw"])
        np.testing.assert_allclose(rec[: len(raw)], raw, rtol=1e-15, atol=0)
        ok, f, e = orc.pair_eval(v["name"], rec, v["r"] ** 2, v["rcut"] ** 2, v["shift"])
        assert ok == v["ok"], v
        if ok:
            assert rel(f, v["force_divr"]) < 1e-13 or abs(f - v["force_divr"]) < 1e-13, v
            assert rel(e, v["energy"]) < 1e-13 or abs(e - v["energy"]) < 1e-13, v
            n += 1
    assert n > 200


def test_bond_reference_vectors(orc):
    for v in REF["bond"]:
        rec = orc.bond_params(v["name"], v["params"])
        np.testing.assert_allclose(rec[: len(v["raw"])], v["raw"], rtol=1e-15, atol=0)
        ok, f, e = orc.bond_eval(v["name"], rec, v["r"] ** 2)
        assert ok == v["ok"]
        assert rel(f, v["force_divr"]) < 1e-13 or abs(f - v["force_divr"]) < 1e-12, v
        assert rel(e, v["energy"]) < 1e-13 or abs(e - v["energy"]) < 1e-12, v


def test_flow_reference_vectors(orc):
    for v in REF["flow"]:
        if v["kind"] == "constant":
            u = orc.flow(0, v["U"], v["r"])
        else:
            u = orc.flow(1, [v["mean_velocity"], v["separation"], 0.0], v["r"])
        np.testing.assert_allclose(u, v["u"], rtol=1e-15, atol=1e-15)


# Random123 known-answer vectors for Philox4x32-10 (ctr, key -> out)
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_known_answers(orc, ctr, key, out):
    assert tuple(int(x) for x in orc.philox(ctr, key)) == out


def test_uniform_draws(orc):
    r = np.array([orc.uniform3(202, t, 7, tag, -2.0, 2.0) for t in range(20) for tag in range(50)])
    assert r.min() > -2.0 and r.max() < 2.0
    assert abs(r.mean()) < 0.1
    assert abs(r.var() - 16.0 / 12.0) < 0.1
    # distinct streams for Brownian (201) and Langevin (202)
    assert not np.array_equal(orc.uniform3(201, 5, 7, 3, -1, 1), orc.uniform3(202, 5, 7, 3, -1, 1))


def test_nlist_cell_equals_brute(orc):
    rng = np.random.Generator(np.random.PCG64(5))
    N = 700
    L = np.array([11.0, 12.5, 13.0])
    pos4 = np.zeros((N, 4))
    pos4[:, :3] = rng.uniform(-0.5, 0.5, size=(N, 3)) * L
    types = rng.integers(0, 2, size=N).astype(np.int32)
    pos4[:, 3] = types
    rl = np.array([[1.4, 2.0], [2.0, 0.0]]) ** 2  # type pair (1,1) never listed
    excl = np.array([[i, i + 1] for i in range(0, N - 1, 3)])
    s1, i1 = orc.nlist(pos4, types, 2, L, rl, excl, method="brute")
    s2, i2 = orc.nlist(pos4, types, 2, L, rl, excl, method="cell")
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(i1, i2)
    assert len(i1) > N


def test_pair_loop_invariants(orc):
    rng = np.random.Generator(np.random.PCG64(9))
    N = 400
    L = np.array([9.0, 9.0, 9.0])
    pos4 = np.zeros((N, 4))
    g = np.stack(np.meshgrid(*[np.arange(8)] * 3, indexing="ij"), -1).reshape(-1, 3)[:N]
    pos4[:, :3] = (g + 0.5) * (9.0 / 8) - 4.5 + rng.uniform(-0.1, 0.1, size=(N, 3))
    types = np.zeros(N, dtype=np.int32)
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5))
    s, i = orc.nlist(pos4, types, 1, L, np.array([[3.4 ** 2]]))
    F, U, W = orc.pair_forces(pos4, types, 1, L, s, i, "PerturbedLennardJones", rec.reshape(1, 1, 4),
                              np.array([[9.0]]))
    assert np.abs(F.sum(axis=0)).max() < 1e-9 * np.abs(F).max()
    # pair energy sums twice (half per particle): matches a direct pair sum
    e_direct = 0.0
    for a in range(N):
        for k in range(s[a], s[a + 1]):
            b = i[k]
            if b > a:
                v = pos4[a, :3] - pos4[b, :3]
                v -= L * np.rint(v / L)
                ok, f, e = orc.pair_eval("PerturbedLennardJones", rec, float(v @ v), 9.0, False)
                e_direct += e if ok else 0.0
    assert rel(U.sum(), e_direct) < 1e-12


def test_xplor_smoothing_continuity(orc):
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=1.0))
    L = np.array([20.0, 20.0, 20.0])
    rc, ron = 3.0, 2.0
    vals = []
    for d in (ron - 1e-7, ron + 1e-7, rc - 1e-6):
        pos4 = np.array([[-0.5 * d, 0, 0, 0], [0.5 * d, 0, 0, 0]], dtype=np.float64)
        s, i = orc.nlist(pos4, np.zeros(2, dtype=np.int32), 1, L, np.array([[(rc + 0.4) ** 2]]))
        F, U, W = orc.pair_forces(pos4, np.zeros(2, dtype=np.int32), 1, L, s, i, "PerturbedLennardJones",
                                  rec.reshape(1, 1, 4), np.array([[rc * rc]]), np.array([[ron * ron]]), "xplor")
        vals.append((F[1, 0], U.sum()))
    assert abs(vals[0][0] - vals[1][0]) < 1e-5 and abs(vals[0][1] - vals[1][1]) < 1e-6
    assert abs(vals[2][0]) < 1e-6 and abs(vals[2][1]) < 1e-9


@pytest.mark.parametrize("case", [c for c in KATS["pair"] if c["potential"] == "DPDGeneralWeight"],
                         ids=lambda c: f"DPD-thermostat@{c['line']}")
def test_dpd_thermostat_oracle_kat(orc, case):
    # the full thermostat restatement at kT = 0 with particles at rest reduces to the KAT
    d = case["distance"]
    pos4 = np.array([[-0.5 * d, 0, 0, 0], [0.5 * d, 0, 0, 0]], dtype=np.float64)
    vel4 = np.array([[0, 0, 0, 1.0], [0, 0, 0, 1.0]])
    rec = orc.pair_params("DPDGeneralWeight", case["params"]).reshape(1, 1, 4)
    L = np.array([10.0, 10.0, 10.0])
    F, U, W = orc.dpd_forces(pos4, vel4, [0, 0], [0, 1], 1, L, np.array([0, 1, 2]), np.array([1, 0]), rec,
                             np.array([[case["r_cut"] ** 2]]), 0.0, 0.001, 7, 3)
    np.testing.assert_allclose(F[:, 0], [-case["force"], case["force"]], atol=1e-12)
    np.testing.assert_allclose(U, [0.5 * case["energy"]] * 2, atol=1e-12)


def test_dpd_thermostat_oracle_pair_draw_is_shared(orc):
    # i and j draw the same number (ordered tag counter): the pair forces cancel
    rng = np.random.Generator(np.random.PCG64(2))
    N, L = 300, 6.0
    pos4 = np.concatenate([rng.uniform(-3, 3, size=(N, 3)), np.zeros((N, 1))], axis=1)
    vel4 = np.concatenate([rng.normal(size=(N, 3)), np.ones((N, 1))], axis=1)
    rec = orc.pair_params("DPDGeneralWeight", dict(A=25.0, gamma=4.5, s=0.5)).reshape(1, 1, 4)
    Lv = np.array([L, L, L])
    st, idx = orc.nlist(pos4, np.zeros(N, dtype=np.int32), 1, Lv, np.array([[1.0]]))
    F, U, W = orc.dpd_forces(pos4, vel4, np.zeros(N, dtype=np.int32), np.arange(N, dtype=np.uint32), 1, Lv, st, idx,
                             rec, np.array([[1.0]]), 1.5, 0.01, 11, 4)
    assert np.abs(F.sum(axis=0)).max() < 1e-10 * np.abs(F).sum()
    # the random term is on: a different timestep gives different forces
    F2, _, _ = orc.dpd_forces(pos4, vel4, np.zeros(N, dtype=np.int32), np.arange(N, dtype=np.uint32), 1, Lv, st, idx,
                              rec, np.array([[1.0]]), 1.5, 0.01, 12, 4)
    assert not np.allclose(F, F2)


def test_dpd_md_loop_conserves_momentum_and_thermostats(orc):
    """The oracle's MD loop with DPDGeneralWeight and the drag-free, noiseless
    Langevin step (HOOMD's ConstantVolume): every DPD force is pairwise
    antisymmetric, so the total momentum stays at its start value; the random and
    dissipative terms drive the kinetic temperature of a cold start towards kT
    (src/pytest/test_pair_dpd.py's check, here on the oracle)."""
    rng = np.random.Generator(np.random.PCG64(12))
    n, a, kT = 8, 0.6, 1.5
    g = (np.arange(n) - 0.5 * (n - 1)) * a
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    N = n ** 3
    L = np.full(3, n * a)
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1) + rng.uniform(-0.05, 0.05, size=(N, 3))
    v = rng.normal(0.0, 0.1, size=(N, 3))
    system = dict(pos4=np.concatenate([pos, np.zeros((N, 1))], axis=1),
                  vel4=np.concatenate([v, np.ones((N, 1))], axis=1), accel=np.zeros((N, 3)),
                  image=np.zeros((N, 3), dtype=np.int32), types=np.zeros(N, dtype=np.int32),
                  tags=np.arange(N, dtype=np.uint32), L=L, ntypes=1)
    rec = orc.pair_params("DPDGeneralWeight", dict(A=0.0, gamma=4.5, s=0.5)).reshape(1, 1, 4)
    md = orc.OracleMD(system, pair=dict(name="DPDGeneralWeight", params=rec, rcut=np.array([[1.0]]), kT=kT),
                      method="langevin", gamma=[0.0], kT=0.0, dt=0.01, seed=9, r_buff=0.4, noiseless=True)
    p0 = md.s["vel4"][:, :3].sum(axis=0)
    md.run(150)
    vv = md.s["vel4"][:, :3]
    assert np.abs(vv.sum(axis=0) - p0).max() < 1e-10
    T = float((vv * vv).sum()) / (3 * N - 3)
    assert T == pytest.approx(kT, rel=0.15)
