"""Wall potentials on the GPU.

* The reference's known answers (src/pytest/test_wall.py:22-111): one particle at
  (0, 0, z) in a box of 20 above the plane z = 0, the potential in the
  integrator's forces, energies and forces read after run(0) (4 decimals as
  there), in both precisions.
* The drop-in driver azp_wall_forces against the oracle with every geometry at
  once (inside and outside spheres, tilted cylinders, planes; standard and
  extrapolated types): FP64 1e-12 (LJ93) / 1e-11 (Colloid) norm-wise with
  energies and virials, FP32 (FP32 arithmetic) within 1e-5.
* The resident engine with the walls in the integrator's forces (fused into the
  step kernel) against the oracle's MD loop: a Lennard-Jones fluid in a slit
  between two LJ93 planes (Langevin) and in a Colloid-walled cylindrical pore
  (Brownian), FP64 (positions 1e-9) and FP32 forces (1e-3 / 1e-5), plus the
  engine's forces, energy and virial at the final state.
"""

import ctypes

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import force_error, load_golden, oracle_system, oracle_walls, rel

pytestmark = pytest.mark.gpu
KATS = load_golden("kats.json")["wall"]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("case", KATS, ids=lambda c: f"{c['potential']}@{c['line']}")
def test_reference_kats(case, precision):
    s = az.Snapshot(1)
    s.particles.position = np.array([case["position"]], dtype=np.float64)
    s.configuration.box = [20.0, 20.0, 20.0, 0.0, 0.0, 0.0]
    sim = az.Simulation(seed=1, precision=precision)
    sim.create_state_from_snapshot(s)
    wall = az.wall.Plane(origin=(0, 0, 0), normal=(0, 0, 1))
    pot = getattr(az.wall, case["potential"])(walls=[wall])
    pot.params["A"] = case["params"]
    m = az.methods.LangevinFlow("all", kT=0.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=0.0)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[m], forces=[pot])
    sim.run(0)
    for k, v in case["params"].items():
        assert pot.params["A"][k] == v
    np.testing.assert_array_almost_equal(pot.energies, [case["energy"]], decimal=4)
    np.testing.assert_array_almost_equal(pot.forces, [[0.0, 0.0, case["force"]]], decimal=4)
    # the engine's net force at the state carries the wall force too
    sim.run(1)
    f, w = sim._engine.forces()
    np.testing.assert_array_almost_equal(f[:, 3], [case["energy"]], decimal=4)
    np.testing.assert_array_almost_equal(f[:, :3], [[0.0, 0.0, case["force"]]], decimal=4)


def _walls_zoo():
    return [
        az.wall.Sphere(radius=9.0, origin=(0.3, -0.2, 0.1), inside=True),
        az.wall.Sphere(radius=2.5, origin=(-3.0, 2.0, 1.0), inside=False),
        az.wall.Cylinder(radius=7.5, axis=(0.2, 0.1, 1.0), origin=(0.5, 0.0, 0.0), inside=True),
        az.wall.Cylinder(radius=1.5, axis=(1.0, -1.0, 0.3), origin=(2.0, -2.0, -1.0), inside=False),
        az.wall.Plane(origin=(0.0, -8.0, 0.0), normal=(0.0, 1.0, 0.0)),
        az.wall.Plane(origin=(0.0, 8.0, 0.0), normal=(0.1, -1.0, 0.05)),
        az.wall.Plane(origin=(0.0, 0.0, -7.0), normal=(0.0, 0.0, 1.0), open=False),
    ]


@pytest.mark.parametrize("name", ["LJ93", "Colloid"])
def test_driver_matches_oracle(orc, name):
    rng = np.random.Generator(np.random.PCG64(81))
    N = 30011
    L = np.array([20.0, 20.0, 20.0])
    pos = rng.uniform(-0.5, 0.5, size=(N, 3)) * L
    types = rng.integers(0, 3, size=N).astype(np.int32)
    pot = getattr(az.wall, name)(walls=_walls_zoo())
    if name == "LJ93":
        pot.params["A"] = dict(A=1.0, sigma=1.0, r_cut=3.0)
        pot.params["B"] = dict(A=0.5, sigma=1.2, r_cut=2.5, r_extrap=0.8)
        pot.params["C"] = dict(A=2.0, sigma=0.8, r_cut=1.5, r_extrap=0.4)
    else:
        pot.params["A"] = dict(A=1.0, a=0.5, sigma=1.0, r_cut=3.0, r_extrap=0.9)
        pot.params["B"] = dict(A=4.0, a=1.0, sigma=1.0, r_cut=3.5, r_extrap=1.4)
        pot.params["C"] = dict(A=0.3, a=0.3, sigma=0.9, r_cut=2.0, r_extrap=0.5)
    rec, rc, rx = pot._tables(["A", "B", "C"])
    sp, cy, pl = oracle_walls(pot)
    # the standard form diverges at the surface: redraw the few particles whose
    # wall force would leave the FP32 range
    for _ in range(10):
        F, U, W = orc.wall_forces(np.concatenate([pos, types[:, None]], axis=1), types, name, rec, rc, rx, sp, cy,
                                  pl)
        bad = ~(np.abs(F).max(axis=1) < 1e8) | ~(np.abs(U) < 1e8)
        if not bad.any():
            break
        pos[bad] = rng.uniform(-0.5, 0.5, size=(bad.sum(), 3)) * L
    assert not bad.any() and (np.abs(U) > 0).sum() > 1000
    # FP64: the Colloid form subtracts two large terms near the surface, so FMA
    # contraction differences show at 1e-12; LJ93 stays within 1e-12. FP32: FP32
    # arithmetic on FP64 distances (the pair driver's FP32 bound)
    tol64 = 1e-12 if name == "LJ93" else 1e-11
    for prec, tol in (("fp64", tol64), ("fp32", 1e-5)):
        f, w = _driver_forces(pot, (rec, rc, rx), pos, types, L, prec)
        assert force_error(f, F) < tol
        assert np.abs(f[:, 3] - U).max() <= tol * max(np.abs(U).max(), 1.0)
        assert np.abs(w - W).max() <= tol * max(np.abs(W).max(), 1.0)


def _driver_forces(pot, tables, pos, types, L, prec):
    """azp_wall_forces on the GPU: forces + energies [N, 4] and virials [N, 6]
    (outputs filled with NaN beforehand, so that a particle left unwritten shows)."""
    import torch

    from azplugins_gb300 import _lib

    Lib = _lib.load()
    N = len(pos)
    ntypes = len(tables[1])
    dpos = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    dpos[:, :3] = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
    dpos.view(torch.int64)[:, 3] = torch.from_numpy(types.astype(np.int64)).cuda()
    s = _lib.System()
    s.N, s.ntypes, s.pos = N, ntypes, dpos.data_ptr()
    for d in range(3):
        s.box.L[d] = L[d]
    dev = [torch.from_numpy(np.ascontiguousarray(a).reshape(-1).copy()).cuda() for a in tables]
    walls, keep = pot._walls_struct()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dt = torch.float64 if prec == "fp64" else torch.float32
    force = torch.full((N, 4), float("nan"), dtype=dt, device="cuda")
    vir = torch.full((6, N), float("nan"), dtype=dt, device="cuda")
    out = _lib.Forces()
    out.force, out.virial, out.virial_pitch = force.data_ptr(), vir.data_ptr(), N
    out.precision = _lib.FP64 if prec == "fp64" else _lib.FP32
    _lib.check(Lib.azp_wall_forces(ctypes.byref(s), pot.kind, ctypes.byref(walls), dev[0].data_ptr(),
                                   dev[1].data_ptr(), dev[2].data_ptr(), ctypes.byref(out), stream),
               "azp_wall_forces")
    torch.cuda.synchronize()
    del keep
    return force.double().cpu().numpy(), vir.double().cpu().numpy().T


def _at_distance(rng, wall, d, L):
    """Points at signed distance d (positive on the active side) from a wall,
    at the wall's surface point nearest a random point of the box."""
    q = rng.uniform(-0.5, 0.5, size=(len(d), 3)) * L
    if isinstance(wall, az.wall.Plane):
        o = np.asarray(wall.origin, float)
        n = np.asarray(wall.normal, float)
        n = n / np.linalg.norm(n)
        return q - ((q - o) @ n)[:, None] * n + d[:, None] * n
    o = np.asarray(wall.origin, float)
    t = q - o
    if isinstance(wall, az.wall.Cylinder):
        a = np.asarray(wall.axis, float)
        a = a / np.linalg.norm(a)
        along = (t @ a)[:, None] * a
        t = t - along
    else:
        along = 0.0
    u = t / np.linalg.norm(t, axis=1)[:, None]
    rad = wall.radius - d if wall.inside else wall.radius + d
    return o + along + rad[:, None] * u


def test_driver_screen_near_cutoffs(orc):
    """The driver screens particles in FP32 and evaluates in full only those some
    wall may reach: particles within 1e-9 relative of every cutoff and every
    extrapolation distance of walls whose origins lie far outside the box (the
    screen's tolerance grows with them), on both sides of each surface. Every
    particle the oracle gives a force or energy gets one, the others exact zeros;
    FP64 within 5e-11 of the oracle (surfaces of radius 300 and 490 leave the
    distance to the wall, a difference of two numbers near the radius, with a
    rounding of radius x 2^-53 that differs between the GPU's contracted FMAs and
    the oracle's separate roundings, and the steep LJ93 form near the surface
    multiplies it: 5.5e-12 measured), FP32 within 1e-5."""
    rng = np.random.Generator(np.random.PCG64(29))
    L = np.array([40.0, 40.0, 40.0])
    walls = [
        az.wall.Sphere(radius=490.0, origin=(500.0, 0.0, 0.0), inside=False),
        az.wall.Sphere(radius=12.0, origin=(0.0, 0.0, 0.0), inside=True),
        az.wall.Cylinder(radius=300.0, axis=(0.0, 0.1, 1.0), origin=(0.0, 310.0, 0.0), inside=True),
        az.wall.Plane(origin=(1.0e4, -1.0e4, -12.0), normal=(0.0, 0.0, 1.0)),
        az.wall.Plane(origin=(3.0, 14.0, 0.0), normal=(0.2, -1.0, 0.1)),
    ]
    pot = az.wall.LJ93(walls=walls)
    pot.params["A"] = dict(A=1.0, sigma=1.0, r_cut=3.0)
    pot.params["B"] = dict(A=0.5, sigma=1.2, r_cut=2.5, r_extrap=0.8)
    rec, rc, rx = pot._tables(["A", "B"])
    per = 2400
    pos, types = [], []
    for w in walls:
        for t, (cut, ext) in enumerate(((3.0, 0.0), (2.5, 0.8))):
            marks = [cut, ext] if ext > 0 else [cut]
            base = rng.choice(marks, size=per)
            rel_off = rng.choice([-1e-9, 1e-9, -1e-7, 1e-7, -1e-4, 1e-4, -1e-2, 1e-2], size=per)
            d = base * (1.0 + rel_off)
            if ext > 0:  # extrapolated types: the inactive side as well
                d[: per // 4] = -rng.uniform(0.0, 6.0, size=per // 4)
            pos.append(_at_distance(rng, w, d, L))
            types.append(np.full(per, t, np.int32))
    pos.append(rng.uniform(-0.5, 0.5, size=(4000, 3)) * L)
    types.append(rng.integers(0, 2, size=4000).astype(np.int32))
    pos, types = np.concatenate(pos), np.concatenate(types)
    keep = np.all(np.abs(pos) < 0.5 * L, axis=1)
    pos, types = pos[keep], types[keep]
    sp, cy, pl = oracle_walls(pot)
    F, U, W = orc.wall_forces(np.concatenate([pos, types[:, None]], axis=1), types, "LJ93", rec, rc, rx, sp, cy, pl)
    ok = (np.abs(F).max(axis=1) < 1e8) & (np.abs(U) < 1e8)
    pos, types, F, U, W = pos[ok], types[ok], F[ok], U[ok], W[ok]
    acted = (F != 0.0).any(axis=1) | (U != 0.0)
    assert acted.sum() > 5000 and (~acted).sum() > 2000
    for prec, tol in (("fp64", 5e-11), ("fp32", 1e-5)):
        f, w = _driver_forces(pot, (rec, rc, rx), pos, types, L, prec)
        assert force_error(f, F) < tol
        assert np.abs(f[:, 3] - U).max() <= tol * max(np.abs(U).max(), 1.0)
        assert np.abs(w - W).max() <= tol * max(np.abs(W).max(), 1.0)
        if prec == "fp64":
            np.testing.assert_array_equal((f[:, :3] != 0.0).any(axis=1) | (f[:, 3] != 0.0), acted)
        assert np.all(f[~acted] == 0.0) and np.all(w[~acted] == 0.0)


def _slit_fluid(seed, n_xz=8, n_y=10, spacing=1.2):
    """Jittered lattice filling |y| <= 5.4 of a 9.6 x 16 x 9.6 box (walls at y = +-7)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    gx = (np.arange(n_xz) + 0.5) * spacing - 0.5 * n_xz * spacing
    gy = (np.arange(n_y) + 0.5) * spacing - 0.5 * n_y * spacing
    X, Y, Z = np.meshgrid(gx, gy, gx, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1) + rng.uniform(-0.08, 0.08, size=(X.size, 3))
    N = len(pts)
    s = az.Snapshot(N)
    s.particles.types = ["A", "B"]
    s.particles.position = pts
    s.particles.typeid = rng.integers(0, 2, size=N).astype(np.int32)
    s.particles.velocity = rng.normal(size=(N, 3))
    s.particles.velocity -= s.particles.velocity.mean(axis=0)
    s.particles.mass = rng.uniform(0.8, 1.2, size=N)
    s.particles.acceleration = np.zeros((N, 3))
    s.configuration.box = [n_xz * spacing, 16.0, n_xz * spacing, 0.0, 0.0, 0.0]
    return s


def _run(orc, snap, precision, method, pot, steps, dt, seed):
    sim = az.Simulation(seed=seed, precision=precision)
    sim.create_state_from_snapshot(snap)
    lj = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=2.5)
    lj.params[[("A", "A"), ("A", "B"), ("B", "B")]] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5)
    mcls = az.methods.LangevinFlow if method == "langevin" else az.methods.BrownianFlow
    m = mcls("all", kT=1.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=1.0)
    sim.operations.integrator = az.md.Integrator(dt=dt, methods=[m], forces=[lj, pot])
    sim.run(steps // 2)
    sim.run(steps - steps // 2)
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5))
    wrec, wrc, wrx = pot._tables(["A", "B"])
    sp, cy, pl = oracle_walls(pot)
    md = orc.OracleMD(oracle_system(snap, snap.particles.acceleration),
                      pair=dict(name="PerturbedLennardJones", params=np.tile(rec, (2, 2, 1)),
                                rcut=np.full((2, 2), 2.5), mode="none"),
                      method=method, gamma=[1.0, 1.0], kT=1.0, dt=dt, seed=seed,
                      walls=dict(name=pot._name, params=wrec, rcut=wrc, rextrap=wrx, spheres=sp, cylinders=cy,
                                 planes=pl))
    md.run(steps)
    return sim, md


def _unwrapped_err(sim, md, L):
    out = sim.state.get_snapshot().particles
    return float(np.abs((out.position + out.image * L) - (md.s["pos4"][:, :3] + md.s["image"] * L)).max())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-3)])
def test_engine_langevin_slit(orc, precision, tol):
    snap = _slit_fluid(91)
    L = np.array(snap.configuration.box[:3])
    pot = az.wall.LJ93(walls=[az.wall.Plane(origin=(0, -7.0, 0), normal=(0, 1, 0)),
                              az.wall.Plane(origin=(0, 7.0, 0), normal=(0, -1, 0))])
    pot.params["A"] = dict(A=2.0, sigma=1.0, r_cut=3.0)
    pot.params["B"] = dict(A=1.0, sigma=1.2, r_cut=3.0, r_extrap=0.6)
    sim, md = _run(orc, snap, precision, "langevin", pot, 60, 0.004, seed=91)
    F_md, U_md, W_md = md.forces()
    Fw, Uw, _ = orc.wall_forces(md.s["pos4"], md.s["types"], "LJ93", *pot._tables(["A", "B"]),
                                planes=oracle_walls(pot)[2])
    assert (Uw != 0).sum() > 50  # the walls act on the layers next to them
    assert _unwrapped_err(sim, md, L) < tol
    f, w = sim._engine.forces()
    ftol = 1e-12 if precision == "fp64" else 1e-5
    assert force_error(f, F_md) < ftol
    th = sim.thermo()
    assert rel(th["potential_energy"], U_md.sum()) < ftol
    for c in range(6):
        assert abs(th["virial"][c] - W_md[:, c].sum()) <= ftol * max(np.abs(W_md[:, c]).sum(), 1.0)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_engine_brownian_cylindrical_pore(orc, precision, tol):
    snap = _slit_fluid(92)
    L = np.array(snap.configuration.box[:3])
    # a pore of radius 4.2 along y through the slab, and a colloid-walled outer region
    pot = az.wall.Colloid(walls=[az.wall.Cylinder(radius=4.2, axis=(0, 1, 0), inside=True)])
    pot.params["A"] = dict(A=3.0, a=0.4, sigma=1.0, r_cut=2.5, r_extrap=0.7)
    pot.params["B"] = dict(A=5.0, a=0.5, sigma=1.0, r_cut=3.0, r_extrap=0.9)
    sim, md = _run(orc, snap, precision, "brownian", pot, 40, 2e-4, seed=92)
    F_md, U_md, _ = md.forces()
    assert _unwrapped_err(sim, md, L) < tol
    f, _ = sim._engine.forces()
    assert force_error(f, F_md) < (1e-12 if precision == "fp64" else 1e-5)


def test_driver_many_types(orc):
    """1,500 particle types: the FP32-output kernel's per-type float records and
    reaches (9 floats a type, 54 KB with the block's near list) take more than
    the default 48 KB of dynamic shared memory, so the launch raises the limit
    first; both precisions against the oracle, every type with its own
    parameters, cutoff and extrapolation."""
    rng = np.random.Generator(np.random.PCG64(31))
    nt = 1500
    N = 20000
    L = np.array([20.0, 20.0, 20.0])
    pot = az.wall.LJ93(walls=_walls_zoo())
    names = [f"T{k}" for k in range(nt)]
    for k, name in enumerate(names):
        pot.params[name] = dict(A=float(rng.uniform(0.5, 2.0)), sigma=float(rng.uniform(0.8, 1.2)),
                                r_cut=float(rng.uniform(1.5, 3.5)), r_extrap=float(0.5 if k % 3 else 0.0))
    rec, rc, rx = pot._tables(names)
    sp, cy, pl = oracle_walls(pot)
    pos = rng.uniform(-0.5, 0.5, size=(N, 3)) * L
    types = rng.integers(0, nt, size=N).astype(np.int32)
    for _ in range(10):
        F, U, W = orc.wall_forces(np.concatenate([pos, types[:, None]], axis=1), types, "LJ93", rec, rc, rx, sp, cy,
                                  pl)
        bad = ~(np.abs(F).max(axis=1) < 1e8) | ~(np.abs(U) < 1e8)
        if not bad.any():
            break
        pos[bad] = rng.uniform(-0.5, 0.5, size=(bad.sum(), 3)) * L
    assert not bad.any() and (np.abs(U) > 0).sum() > 1000
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
        f, w = _driver_forces(pot, (rec, rc, rx), pos, types, L, prec)
        assert force_error(f, F) < tol
        assert np.abs(f[:, 3] - U).max() <= tol * max(np.abs(U).max(), 1.0)
        assert np.abs(w - W).max() <= tol * max(np.abs(W).max(), 1.0)
