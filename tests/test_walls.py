"""Wall potentials on the CPU: the oracle against the reference's known answers
(src/pytest/test_wall.py:22-56, extracted into golden/kats.json), the param_type
builders of the C ABI against the oracle's and their asDict round trip
(src/WallEvaluatorLJ93.h:31-52, src/WallEvaluatorColloid.h:31-64), the
extrapolated mode's continuity, and the Python front end (src/wall.py)."""

import ctypes

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import load_golden, oracle_walls

KATS = load_golden("kats.json")["wall"]
PLANE_Z = [[0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 1.0]]  # hoomd.wall.Plane(origin=(0, 0, 0), normal=(0, 0, 1))


@pytest.mark.parametrize("case", KATS, ids=lambda c: f"{c['potential']}@{c['line']}")
def test_oracle_matches_reference_kats(orc, case):
    p = case["params"]
    rec = orc.wall_params(case["potential"], p)
    F, U, W = orc.wall_forces(np.array([[*case["position"], 0.0]]), [0], case["potential"], rec[None], [p["r_cut"]],
                              [p.get("r_extrap", 0.0)], planes=PLANE_Z)
    assert U[0] == pytest.approx(case["energy"], abs=5e-5)
    np.testing.assert_allclose(F[0], [0.0, 0.0, case["force"]], atol=5e-5)


@pytest.mark.parametrize("name", ["LJ93", "Colloid"])
def test_param_builders_match_oracle_and_round_trip(orc, name):
    from azplugins_gb300 import _lib

    L = _lib.load()
    rng = np.random.Generator(np.random.PCG64(3))
    keys = orc.WALL_KEYS[name]
    for _ in range(50):
        d = {k: float(rng.uniform(0.3, 3.0)) for k in keys}
        vals = np.array([d[k] for k in keys])
        rec = np.zeros(4)
        assert L.azp_wall_params_from_values(_lib.WALL_KINDS[name], vals.ctypes.data, rec.ctypes.data) == 0
        np.testing.assert_array_equal(rec, orc.wall_params(name, d))
        back = np.zeros(len(keys))
        assert L.azp_wall_params_to_values(_lib.WALL_KINDS[name], rec.ctypes.data, back.ctypes.data) == 0
        np.testing.assert_allclose(back, vals, rtol=1e-14)
    assert L.azp_wall_params_from_values(7, vals.ctypes.data, rec.ctypes.data) == -1


@pytest.mark.parametrize("name,params", [("LJ93", dict(A=1.3, sigma=0.9)), ("Colloid", dict(A=2.0, a=0.6, sigma=1.0))])
def test_extrapolated_mode(orc, name, params):
    """Linear continuation below r_extrap and on the inactive side: continuous
    energy at r_extrap, constant force towards the active side."""
    rec = orc.wall_params(name, params)
    rc, rx = 3.0, 1.2
    z = np.array([2.0, rx + 1e-9, rx - 1e-9, 0.7, 0.0, -0.5, -2.0])
    pos = np.stack([np.zeros_like(z), np.zeros_like(z), z, np.zeros_like(z)], axis=1)
    F, U, _ = orc.wall_forces(pos, np.zeros(len(z), dtype=np.int32), name, rec[None], [rc], [rx],
                              planes=[[0, 0, 0, 0, 0, 1, 0]])  # closed plane: z = 0 is on the active side
    Fs, Us, _ = orc.wall_forces(pos[:3], np.zeros(3, dtype=np.int32), name, rec[None], [rc], [0.0], planes=PLANE_Z)
    assert U[0] == Us[0] and F[0, 2] == Fs[0, 2]  # beyond r_extrap: the standard form
    assert U[1] == pytest.approx(U[2], rel=1e-6) and F[1, 2] == pytest.approx(F[2, 2], rel=1e-6)
    fx = F[2, 2]
    np.testing.assert_allclose(F[2:, 2], fx)  # constant force below r_extrap, either side
    np.testing.assert_allclose(U[2:], U[2] + fx * (z[2] - z[2:]), rtol=1e-12)
    assert (F[:, :2] == 0).all()


def test_geometry_distances(orc):
    """Sphere and cylinder walls against closed forms of the distance."""
    rec = orc.wall_params("LJ93", dict(A=1.0, sigma=1.0))
    # one particle 1.5 inside a sphere of radius 5 centred at (1, 2, 3), off-axis
    u = np.array([2.0, -1.0, 2.0]) / 3.0
    x = np.array([1.0, 2.0, 3.0]) + 3.5 * u
    F, U, W = orc.wall_forces(np.array([[*x, 0.0]]), [0], "LJ93", rec[None], [3.0], [0.0],
                              spheres=[[5.0, 1.0, 2.0, 3.0, 1.0, 1.0]])
    Fp, Up, _ = orc.wall_forces(np.array([[0, 0, 1.5, 0.0]]), [0], "LJ93", rec[None], [3.0], [0.0], planes=PLANE_Z)
    assert U[0] == pytest.approx(Up[0], rel=1e-12)
    np.testing.assert_allclose(F[0], -u * Fp[0, 2], rtol=1e-12)
    np.testing.assert_allclose(W[0], [F[0, 0] * x[0], F[0, 0] * x[1], F[0, 0] * x[2], F[0, 1] * x[1],
                                      F[0, 1] * x[2], F[0, 2] * x[2]])
    # the same distance outside a cylinder of radius 2 along (1, 1, 0) through the origin
    ax = np.array([1.0, 1.0, 0.0]) / np.sqrt(2.0)
    perp = np.array([0.0, 0.0, 1.0])
    x = 7.0 * ax + 3.5 * perp
    F, U, _ = orc.wall_forces(np.array([[*x, 0.0]]), [0], "LJ93", rec[None], [3.0], [0.0],
                              cylinders=[[2.0, 0, 0, 0, *ax, 0.0, 1.0]])
    assert U[0] == pytest.approx(Up[0], rel=1e-12)
    np.testing.assert_allclose(F[0], perp * Fp[0, 2], rtol=1e-12, atol=1e-15)
    # inside a cylinder: inactive when outside of it and r_extrap = 0
    F, U, _ = orc.wall_forces(np.array([[*x, 0.0]]), [0], "LJ93", rec[None], [3.0], [0.0],
                              cylinders=[[2.0, 0, 0, 0, *ax, 1.0, 1.0]])
    assert U[0] == 0.0 and (F == 0).all()


def test_front_end():
    walls = [az.wall.Plane(origin=(0, 0, 0), normal=(0, 0, 2)), az.wall.Sphere(radius=4.0, inside=False),
             az.wall.Cylinder(radius=3.0, axis=(0, 1, 0), origin=(1, 0, 0))]
    lj = az.wall.LJ93(walls=walls)
    lj.params["A"] = dict(A=1.0, sigma=1.0, r_cut=3.0)
    assert lj.params["A"] == dict(A=1.0, sigma=1.0, r_cut=3.0, r_extrap=0.0)
    lj.params["B"] = dict(A=2.0, sigma=0.5, r_cut=2.0, r_extrap=0.4)
    rec, rc, rx = lj._tables(["A", "B"])
    np.testing.assert_array_equal(rc, [3.0, 2.0])
    np.testing.assert_array_equal(rx, [0.0, 0.4])
    # LJ93 records are 16 bytes (sigma_3, A), as the reference param_type
    np.testing.assert_allclose(rec[1], [0.125, 2.0])
    assert lj.record_to_dict(rec[1]) == pytest.approx(dict(A=2.0, sigma=0.5))
    s, c, p = oracle_walls(lj)
    np.testing.assert_allclose(p[0], [0, 0, 0, 0, 0, 1, 1])
    assert s.shape == (1, 6) and c.shape == (1, 9)
    with pytest.raises(KeyError):
        lj.params["C"] = dict(A=1.0, sigma=1.0)  # r_cut is required
    col = az.wall.Colloid(walls=walls)
    col.params["A"] = dict(A=1.0, a=1.0, sigma=1.0, r_cut=3.0)
    assert col.kind == 1
    with pytest.raises(ValueError):
        az.wall.Plane(origin=(0, 0, 0), normal=(0, 0, 0))
    with pytest.raises(TypeError):
        az.wall.LJ93(walls=[(0, 0, 0)])
    too_many = az.wall.LJ93(walls=[az.wall.Sphere(radius=1.0)] * 21)
    with pytest.raises(ValueError):
        too_many._walls_struct()


def test_c_abi_rejects_bad_walls():
    """Wall checks come before any device work (no GPU needed)."""
    from azplugins_gb300 import _lib

    L = _lib.load()
    s = _lib.System()
    s.N, s.ntypes, s.pos = 4, 1, 1
    for d in range(3):
        s.box.L[d] = 10.0
    out = _lib.Forces()
    out.force, out.precision = 1, _lib.FP64
    pl = (_lib.WallPlane * 1)()
    pl[0].normal[:] = (0.0, 0.0, 0.0)  # zero normal
    w = _lib.Walls()
    w.n_planes, w.planes = 1, ctypes.cast(pl, ctypes.c_void_p)
    one = ctypes.c_void_p(1)
    assert L.azp_wall_forces(ctypes.byref(s), 0, ctypes.byref(w), one, one, one, ctypes.byref(out), None) == -1
    w.n_planes = 61
    assert L.azp_wall_forces(ctypes.byref(s), 0, ctypes.byref(w), one, one, one, ctypes.byref(out), None) == -1
    assert b"more walls" in L.azp_last_error()
