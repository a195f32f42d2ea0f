"""DPD with a general weight function through the drop-in driver (azp_dpd_forces):
the reference's known answers (src/pytest/test_pair.py:75-107), the FP64 oracle
with the random and dissipative terms on (the GPU draws the same Philox numbers),
momentum conservation, and the thermostat check of src/pytest/test_pair_dpd.py
(NVE velocity Verlet with DPD only: the kinetic temperature settles at kT).

Tolerances: FP64 1e-12 relative (forces norm-wise |dF_i| / max(|F_i|, F_rms),
energy, virial); FP32 1e-5 with the same norm."""

import ctypes

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import box_of, force_error, load_golden, pos4_of, rel, two_particle_snapshot

pytestmark = pytest.mark.gpu
KATS = [c for c in load_golden("kats.json")["pair"] if c["potential"] == "DPDGeneralWeight"]


def _attach(snap, pot, precision="fp64", seed=3, dt=0.01):
    sim = az.Simulation(seed=seed, precision=precision)
    sim.create_state_from_snapshot(snap)
    m = az.methods.LangevinFlow("all", kT=0.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=0.0)
    sim.operations.integrator = az.md.Integrator(dt=dt, methods=[m], forces=[pot])
    sim.run(0)
    return sim


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("case", KATS, ids=lambda c: f"DPD@{c['line']}")
def test_dpd_kat(case, precision):
    # kT = 0 and particles at rest: the conservative force alone (the reference's setting)
    r_buff = 0.4
    snap = two_particle_snapshot(case["distance"], 2.1 * 2 * (case["r_cut"] + r_buff))
    pot = az.pair.DPDGeneralWeight(nlist=az.nlist.Cell(buffer=r_buff), kT=0.0, default_r_cut=case["r_cut"])
    pot.params[("A", "A")] = case["params"]
    _attach(snap, pot, precision)
    assert pot.params[("A", "A")] == case["params"]
    e, f = case["energy"], case["force"]
    np.testing.assert_array_almost_equal(pot.energies, [0.5 * e, 0.5 * e], decimal=4)
    np.testing.assert_allclose(pot.forces, [[-f, 0, 0], [f, 0, 0]], rtol=1e-5, atol=1e-6)


def _dpd_system(N=3000, density=3.0, seed=51):
    rng = np.random.Generator(np.random.PCG64(seed))
    L = (N / density) ** (1.0 / 3.0)
    s = az.Snapshot(N)
    s.particles.types = ["A", "B"]
    s.particles.position = rng.uniform(-0.5 * L, 0.5 * L, size=(N, 3))
    s.particles.typeid = rng.integers(0, 2, size=N).astype(np.int32)
    s.particles.velocity = rng.normal(0.0, 1.2, size=(N, 3))
    s.particles.mass = rng.uniform(0.8, 1.2, size=N)
    s.configuration.box = [L, L, L, 0.0, 0.0, 0.0]
    return s


def _dpd_pot(kT=1.5):
    pot = az.pair.DPDGeneralWeight(nlist=az.nlist.Cell(buffer=0.3), kT=kT, default_r_cut=1.0)
    pot.params[("A", "A")] = dict(A=25.0, gamma=4.5, s=0.5)
    pot.params[("A", "B")] = dict(A=40.0, gamma=3.0, s=2.0)
    pot.params[("B", "B")] = dict(A=25.0, gamma=4.5, s=1.0)
    pot.r_cut[("A", "B")] = 1.1
    return pot


def _oracle(orc, snap, pot, kT, dt, timestep, seed):
    p = snap.particles
    types = list(p.types)
    rec, rc, ro = pot._tables(types)
    L = box_of(snap)
    st, idx = orc.nlist(pos4_of(snap), p.typeid, len(types), L, (rc + 0.3) ** 2)
    vel4 = np.concatenate([p.velocity, p.mass[:, None]], axis=1)
    return orc.dpd_forces(pos4_of(snap), vel4, p.typeid, np.arange(p.N, dtype=np.uint32), len(types), L, st, idx,
                          rec, rc * rc, kT, dt, timestep, seed)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_dpd_thermostat_forces_match_oracle(orc, precision, tol):
    snap = _dpd_system()
    pot = _dpd_pot(kT=1.5)
    sim = _attach(snap, pot, precision, seed=77, dt=0.01)
    sim.timestep = 1234
    f = pot.forces
    w = pot.virials
    u = pot.energies
    F, U, W = _oracle(orc, snap, pot, 1.5, 0.01, 1234, 77)
    assert force_error(f, F) < tol
    assert rel(u.sum(), U.sum()) < tol
    for c in range(6):
        assert abs(w[:, c].sum() - W[:, c].sum()) <= tol * max(abs(W[:, c].sum()), np.abs(W[:, c]).sum() * 1e-3)
    # pair draws are shared by i and j: the random and dissipative forces cancel in the sum
    assert np.abs(f.sum(axis=0)).max() <= tol * np.abs(f).sum(axis=0).max()


def test_dpd_draws_change_with_timestep_and_seed(orc):
    snap = _dpd_system(N=1500, seed=52)
    pot = _dpd_pot(kT=1.0)
    sim = _attach(snap, pot, "fp64", seed=5)
    sim.timestep = 10
    f10 = pot.forces
    sim.timestep = 11
    f11 = pot.forces
    assert not np.allclose(f10, f11)
    F11, _, _ = _oracle(orc, snap, pot, 1.0, 0.01, 11, 5)
    assert force_error(f11, F11) < 1e-12


def test_dpd_thermostat_holds_temperature():
    # src/pytest/test_pair_dpd.py: 1000 particles on a 10^3 lattice of spacing 0.6,
    # thermalised at kT = 1.5, DPD with A = 0 (thermostat only), NVE velocity
    # Verlet at dt = 0.01 driven through the drop-in drivers as HOOMD drives them
    import torch

    from azplugins_gb300 import _compute, _lib

    L = _lib.load()
    n, a, kT, dt = 10, 0.6, 1.5, 0.01
    g = (np.arange(n) - 0.5 * (n - 1)) * a
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    N = n ** 3
    snap = az.Snapshot(N)
    snap.particles.position = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    snap.configuration.box = [n * a] * 3 + [0.0, 0.0, 0.0]
    rng = np.random.Generator(np.random.PCG64(53))
    v = rng.normal(0.0, np.sqrt(kT), size=(N, 3))
    v -= v.mean(axis=0)
    pot = az.pair.DPDGeneralWeight(nlist=az.nlist.Cell(buffer=0.4), kT=kT, default_r_cut=1.0)
    pot.params[("A", "A")] = dict(A=0.0, gamma=4.5, s=0.5)
    rec, rc, ro = pot._tables(["A"])
    dev = dict(dtype=torch.float64, device="cuda")
    pos = _compute.device_positions(snap)
    vel = torch.zeros((N, 4), **dev)
    vel[:, :3] = torch.from_numpy(v).cuda()
    vel[:, 3] = 1.0
    acc = torch.zeros((N, 3), **dev)
    img = torch.zeros((N, 3), dtype=torch.int32, device="cuda")
    tags = torch.arange(N, dtype=torch.int32, device="cuda")
    force = torch.zeros((N, 4), **dev)
    params = torch.from_numpy(rec.reshape(-1).copy()).cuda()
    rcut = torch.from_numpy(rc.reshape(-1).copy()).cuda()
    gamma0 = torch.zeros(1, **dev)
    sysd = _compute.make_system(snap, pos, vel=vel.data_ptr(), accel=acc.data_ptr(), image=img.data_ptr(),
                                tag=tags.data_ptr())
    nl = _compute.NeighborList(N, 1, rc, 0.4)
    out = _lib.Forces()
    out.force, out.virial, out.virial_pitch, out.precision = force.data_ptr(), None, N, _lib.FP64
    flow = _lib.Flow()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def forces(t):
        nl.build(sysd)
        _lib.check(L.azp_dpd_forces(ctypes.byref(sysd), nl.handle, params.data_ptr(), rcut.data_ptr(), kT, dt, t, 9,
                                    ctypes.byref(out), stream), "azp_dpd_forces")

    forces(0)
    acc[:] = force[:, :3]
    temps = []
    for t in range(110):
        _lib.check(L.azp_langevin_step1(ctypes.byref(sysd), None, 0, dt, stream), "step1")
        forces(t + 1)
        # step two with no drag and no noise: a = F / m, v += dt a / 2 (NVE)
        _lib.check(L.azp_langevin_step2(ctypes.byref(sysd), None, 0, force.data_ptr(), _lib.FP64, gamma0.data_ptr(),
                                        0, 0.0, flow, dt, 0.0, t + 1, 9, 1, stream), "step2")
        if t >= 10:
            vv = vel[:, :3]
            temps.append(float((vv * vv).sum()) / (3 * N - 3))
    nl.close()
    assert np.mean(temps) == pytest.approx(kT, rel=0.1)


# ---------------------------------------------------------------- DPD inside the resident engine
def _engine_dpd_run(orc, precision, steps=20, seed=77):
    snap = _dpd_system(N=3000, seed=54)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    pot = _dpd_pot(kT=1.5)
    sim = az.Simulation(seed=seed, precision=precision)
    sim.create_state_from_snapshot(snap)
    sim.operations.integrator = az.md.Integrator(dt=0.01, methods=[az.methods.ConstantVolume("all")], forces=[pot])
    sim.run(steps // 2)
    sim.run(steps - steps // 2)
    from helpers import oracle_system

    rec, rc, _ = pot._tables(list(snap.particles.types))
    md = orc.OracleMD(oracle_system(snap, snap.particles.acceleration),
                      pair=dict(name="DPDGeneralWeight", params=rec, rcut=rc, kT=1.5), method="langevin",
                      gamma=[0.0, 0.0], kT=0.0, dt=0.01, seed=seed, r_buff=0.3, noiseless=True)
    md.run(steps)
    return sim, md, box_of(snap)


@pytest.mark.parametrize("precision,ptol,vtol", [("fp64", 1e-9, 1e-8), ("fp32", 2e-4, 2e-3)])
def test_engine_dpd_matches_oracle(orc, precision, ptol, vtol):
    """ConstantVolume + DPDGeneralWeight advanced by the fused engine step against
    the oracle's HOOMD-order loop (forces of t + 1 at the half-step velocities,
    the same per-pair draws): positions, velocities, and the forces and energy
    the engine reports at the end."""
    sim, md, L = _engine_dpd_run(orc, precision)
    snap = sim.state.get_snapshot()
    out = snap.particles
    d = out.position - md.s["pos4"][:, :3]
    d -= L * np.rint(d / L)
    assert np.abs(d).max() < ptol
    assert np.abs(out.velocity - md.s["vel4"][:, :3]).max() < vtol
    # forces and energy at the engine's own end state (same timestep, same draws):
    # the weight (1 - r/r_cut)^(s/2) has an unbounded slope at r_cut, so two
    # trajectories that differ by rounding are not compared force by force
    from helpers import oracle_system

    system = oracle_system(snap)
    system["timestep"] = sim.timestep
    rec, rc, _ = _dpd_pot(kT=1.5)._tables(list(snap.particles.types))
    at_end = orc.OracleMD(system, pair=dict(name="DPDGeneralWeight", params=rec, rcut=rc, kT=1.5), method="langevin",
                          gamma=[0.0, 0.0], kT=0.0, dt=0.01, seed=77, r_buff=0.3, noiseless=True)
    f, _ = sim._engine.forces()
    F, U, _ = at_end.forces()
    assert force_error(f, F) < (1e-12 if precision == "fp64" else 1e-5)
    assert rel(sim.thermo()["potential_energy"], U.sum()) < (1e-12 if precision == "fp64" else 1e-5)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_engine_dpd_thermostat_holds_temperature(precision):
    """src/pytest/test_pair_dpd.py through Simulation.run: 1000 particles on a
    10^3 lattice of spacing 0.6 at kT = 1.5, DPD (A = 0, gamma = 4.5, s = 0.5,
    r_cut 1) with ConstantVolume, dt = 0.01: the kinetic temperature settles at kT."""
    n, a, kT = 10, 0.6, 1.5
    g = (np.arange(n) - 0.5 * (n - 1)) * a
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    N = n ** 3
    snap = az.Snapshot(N)
    snap.particles.position = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    snap.configuration.box = [n * a] * 3 + [0.0, 0.0, 0.0]
    rng = np.random.Generator(np.random.PCG64(55))
    v = rng.normal(0.0, np.sqrt(kT), size=(N, 3))
    snap.particles.velocity = v - v.mean(axis=0)
    pot = az.pair.DPDGeneralWeight(nlist=az.nlist.Cell(buffer=0.4), kT=kT, default_r_cut=1.0)
    pot.params[("A", "A")] = dict(A=0.0, gamma=4.5, s=0.5)
    sim = az.Simulation(seed=9, precision=precision)
    sim.create_state_from_snapshot(snap)
    sim.operations.integrator = az.md.Integrator(dt=0.01, methods=[az.methods.ConstantVolume("all")], forces=[pot])
    sim.run(10)
    temps = []
    for _ in range(10):
        sim.run(10)
        vv = sim.state.get_snapshot().particles.velocity
        temps.append(float((vv * vv).sum()) / (3 * N - 3))
    assert np.mean(temps) == pytest.approx(kT, rel=0.1)
