"""The resident engine (sim.run) against the oracle's HOOMD-order MD loop:
trajectories over 100 steps, run splitting, graph / no-graph equivalence,
thermodynamic sums, FP32-force mode, and Brownian dynamics."""

import os

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import box_of, force_error, oracle_system, pos4_of, random_fluid, rel

pytestmark = pytest.mark.gpu


def _pos_err(a, b, L):
    d = a - b
    d -= L * np.rint(d / L)
    return float(np.abs(d).max())


def _lj_setup(snap, precision="fp64", method="langevin", flow=None, seed=5, kT=1.0, dt=0.005, gamma=1.0,
              lam=0.5, rcut=3.0, mode="none"):
    sim = az.Simulation(seed=seed, precision=precision)
    sim.create_state_from_snapshot(snap)
    nl = az.nlist.Cell(buffer=0.4)
    lj = az.pair.PerturbedLennardJones(nlist=nl, default_r_cut=rcut, mode=mode)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=lam)
    flow = flow or az.flow.ConstantFlow((0.0, 0.0, 0.0))
    cls = az.methods.LangevinFlow if method == "langevin" else az.methods.BrownianFlow
    m = cls("all", kT=kT, flow_field=flow, default_gamma=gamma)
    sim.operations.integrator = az.md.Integrator(dt=dt, methods=[m], forces=[lj])
    return sim, lj


def _oracle_lj(orc, snap, seed=5, kT=1.0, dt=0.005, lam=0.5, rcut=3.0, method="langevin", flow_kind=0,
               flow_p=(0, 0, 0), mode="none", bond=None):
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=lam))
    return orc.OracleMD(oracle_system(snap, snap.particles.acceleration),
                        pair=dict(name="PerturbedLennardJones", params=rec.reshape(1, 1, 4),
                                  rcut=np.array([[rcut]]), mode=mode),
                        bond=bond, method=method, gamma=[1.0], kT=kT, dt=dt, seed=seed, flow_kind=flow_kind,
                        flow_p=flow_p)


def test_lj_fluid_100_steps_fp64(orc):
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=8, density=0.8, seed=21)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    sim, lj = _lj_setup(snap)
    sim.run(100)
    md = _oracle_lj(orc, snap)
    md.run(100)
    out = sim.state.get_snapshot().particles
    L = box_of(snap)
    assert _pos_err(out.position, md.s["pos4"][:, :3], L) < 1e-9
    assert np.abs(out.velocity - md.s["vel4"][:, :3]).max() < 1e-8
    assert np.array_equal(out.image, md.s["image"])
    th = sim.thermo()
    F, U, W = md.forces()
    assert rel(th["potential_energy"], U.sum()) < 1e-10
    assert th["nlist_builds"] >= 2


def _run_chunks(snap, chunks, graphs):
    os.environ["AZP_GRAPHS"] = graphs
    try:
        sim, lj = _lj_setup(snap)
        for c in chunks:
            sim.run(c)
        return sim.state.get_snapshot().particles
    finally:
        os.environ.pop("AZP_GRAPHS", None)


def test_graph_replay_is_bitwise_identical_to_stream_launches():
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=10, density=0.8, seed=22)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    a = _run_chunks(snap, [60, 9], "1")
    b = _run_chunks(snap, [60, 9], "0")
    assert np.array_equal(a.position, b.position)
    assert np.array_equal(a.velocity, b.velocity)
    assert np.array_equal(a.image, b.image)


def test_run_splitting():
    # a run boundary replaces the fused step one by a standalone one: equal to rounding
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=10, density=0.8, seed=22)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    a = _run_chunks(snap, [60], "1")
    b = _run_chunks(snap, [7, 13, 40], "1")
    assert _pos_err(a.position, b.position, box_of(snap)) < 1e-10
    assert np.abs(a.velocity - b.velocity).max() < 1e-9
    assert np.array_equal(a.image, b.image)


def test_forces_at_state_match_oracle(orc):
    snap = random_fluid(1200, 0.8, seed=23)
    sim, lj = _lj_setup(snap)
    sim.run(1)
    s = sim.state.get_snapshot()
    f, w = sim._engine.forces()
    md = _oracle_lj(orc, s)
    F, U, W = md.forces()
    assert force_error(f, F) < 1e-12
    assert rel(f[:, 3].sum(), U.sum()) < 1e-12


def test_fp32_forces_fp64_integration(orc):
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=8, density=0.8, seed=24)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    sim, lj = _lj_setup(snap, precision="fp32")
    sim.run(1)
    s = sim.state.get_snapshot()
    f, w = sim._engine.forces()
    F, U, W = _oracle_lj(orc, s).forces()
    assert force_error(f, F) < 1e-5
    sim.run(99)
    md = _oracle_lj(orc, snap)
    md.run(100)
    # FP32 forces: trajectories stay close over 100 steps (0.5 tau)
    assert _pos_err(sim.state.get_snapshot().particles.position, md.s["pos4"][:, :3], box_of(snap)) < 1e-3


def test_bead_spring_parabolic_flow(orc):
    from azplugins_gb300 import workloads

    snap = workloads.bead_spring_melt(30, 20, density=0.6, seed=25)
    # relax random-walk overlaps with capped Brownian steps first
    sim = az.Simulation(seed=9)
    sim.create_state_from_snapshot(snap)
    wca = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=2 ** (1 / 6))
    wca.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.0)
    qb = az.bond.Quartic()
    qb.params["A-A"] = dict(k=1434.3, r_0=1.5, b_1=-0.7589, b_2=0.0, U_0=67.2234, sigma=1.0, epsilon=1.0)
    relax = az.methods.BrownianFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0, 0, 0)), max_displacement=0.02)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[relax], forces=[wca, qb])
    sim.run(200)
    relaxed = sim.state.get_snapshot()
    relaxed.particles.acceleration = np.zeros((relaxed.particles.N, 3))
    L = box_of(relaxed)
    flow = az.flow.ParabolicFlow(mean_velocity=2.0 / 3.0, separation=L[1])
    sim2 = az.Simulation(seed=10)
    sim2.create_state_from_snapshot(relaxed)
    m = az.methods.LangevinFlow("all", kT=1.0, flow_field=flow, default_gamma=1.0)
    sim2.operations.integrator = az.md.Integrator(dt=0.005, methods=[m], forces=[wca, qb])
    sim2.run(100)
    rec = orc.bond_params("Quartic", qb.params["A-A"])
    md = _oracle_lj(orc, relaxed, seed=10, lam=0.0, rcut=2 ** (1 / 6), flow_kind=1,
                    flow_p=(2.0 / 3.0, L[1], 0.0), bond=dict(name="Quartic", params=rec.reshape(1, 8)))
    md.run(100)
    out = sim2.state.get_snapshot().particles
    assert _pos_err(out.position, md.s["pos4"][:, :3], L) < 1e-8
    assert np.abs(out.velocity - md.s["vel4"][:, :3]).max() < 1e-7


def test_brownian_colloid_like(orc):
    # Brownian steps move by F dt / gamma: keep |F| dt well below the particle size
    snap = random_fluid(800, 0.3, seed=26, min_dist=1.05)
    sim, lj = _lj_setup(snap, method="brownian", flow=az.flow.ConstantFlow((0.1, 0.0, 0.0)), dt=2e-4,
                        lam=1.0, rcut=2.5)
    sim.run(50)
    md = _oracle_lj(orc, snap, method="brownian", dt=2e-4, lam=1.0, rcut=2.5, flow_kind=0, flow_p=(0.1, 0, 0))
    md.run(50)
    out = sim.state.get_snapshot().particles
    assert _pos_err(out.position, md.s["pos4"][:, :3], box_of(snap)) < 1e-10
    assert np.array_equal(out.image, md.s["image"])


# ---------------------------------------------------------------- FP32-force engine state
# FP32-force mode keeps positions as 64-bit fixed point and velocities as float
# pairs (csrc/fixed64.cuh). These tests pin that state: round trips, graph
# equivalence, wrapping and images, and trajectories against the FP64 oracle.


def _unwrapped(p, L):
    return p.position + p.image * L


def _relaxed_melt(n_chains=30, length=20, density=0.6, seed=25):
    from azplugins_gb300 import workloads

    snap = workloads.bead_spring_melt(n_chains, length, density=density, seed=seed)
    sim = az.Simulation(seed=9)
    sim.create_state_from_snapshot(snap)
    wca = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=2 ** (1 / 6))
    wca.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.0)
    qb = az.bond.Quartic()
    qb.params["A-A"] = dict(k=1434.3, r_0=1.5, b_1=-0.7589, b_2=0.0, U_0=67.2234, sigma=1.0, epsilon=1.0)
    relax = az.methods.BrownianFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0, 0, 0)), max_displacement=0.02)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[relax], forces=[wca, qb])
    sim.run(200)
    relaxed = sim.state.get_snapshot()
    relaxed.particles.acceleration = np.zeros((relaxed.particles.N, 3))
    return relaxed, wca, qb


def test_fp32_state_round_trip():
    snap = random_fluid(3000, 0.8, seed=31)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    snap.particles.image = np.random.default_rng(3).integers(-3, 4, size=(snap.particles.N, 3)).astype(np.int32)
    sim, lj = _lj_setup(snap, precision="fp32")
    from azplugins_gb300 import _engine, _lib

    eng = _engine.Engine(sim, sim._attach(), sim.state._arrays())
    eng.push(sim.state._arrays(), 0)
    N = snap.particles.N
    pos, vel = np.empty((N, 4)), np.empty((N, 4))
    img = np.empty((N, 3), dtype=np.int32)
    _lib.check(eng._L.azp_md_get_state(eng._md, pos.ctypes.data, vel.ctypes.data, None, img.ctypes.data, None, 0,
                                       None), "azp_md_get_state")
    L = box_of(snap)
    # 64-bit fixed point holds every FP64 position to within an ulp of the box
    assert np.abs(pos[:, :3] - snap.particles.position).max() <= 4 * np.spacing(L.max() / 2)
    # float pairs hold velocities to 2^-48 relative
    v0 = snap.particles.velocity
    assert np.abs(vel[:, :3] - v0).max() <= 2.0 ** -46 * np.abs(v0).max()
    assert np.array_equal(vel[:, 3], snap.particles.mass)
    assert np.array_equal(pos[:, 3], snap.particles.typeid.astype(float))
    assert np.array_equal(img, snap.particles.image)
    eng.close()


def test_fp32_graph_replay_is_bitwise_identical_to_stream_launches():
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=10, density=0.8, seed=32)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    res = []
    for graphs in ("1", "0"):
        os.environ["AZP_GRAPHS"] = graphs
        try:
            sim, lj = _lj_setup(snap, precision="fp32")
            sim.run(60)
            sim.run(9)
            res.append(sim.state.get_snapshot().particles)
        finally:
            os.environ.pop("AZP_GRAPHS", None)
    a, b = res
    assert np.array_equal(a.position, b.position)
    assert np.array_equal(a.velocity, b.velocity)
    assert np.array_equal(a.image, b.image)


def test_fp32_run_splitting():
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=10, density=0.8, seed=33)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    outs = []
    for chunks in ([60], [7, 13, 40]):
        sim, lj = _lj_setup(snap, precision="fp32")
        for c in chunks:
            sim.run(c)
        outs.append(sim.state.get_snapshot().particles)
    a, b = outs
    L = box_of(snap)
    # a run boundary replaces one fused half-kick pair by two FP32 half kicks
    assert np.abs(_unwrapped(a, L) - _unwrapped(b, L)).max() < 1e-5


def test_fp32_melt_parabolic_flow_vs_oracle(orc):
    relaxed, wca, qb = _relaxed_melt()
    L = box_of(relaxed)
    flow = az.flow.ParabolicFlow(mean_velocity=2.0 / 3.0, separation=L[1])
    sim = az.Simulation(seed=10, precision="fp32")
    sim.create_state_from_snapshot(relaxed)
    m = az.methods.LangevinFlow("all", kT=1.0, flow_field=flow, default_gamma=1.0)
    sim.operations.integrator = az.md.Integrator(dt=0.005, methods=[m], forces=[wca, qb])
    sim.run(100)
    rec = orc.bond_params("Quartic", qb.params["A-A"])
    md = _oracle_lj(orc, relaxed, seed=10, lam=0.0, rcut=2 ** (1 / 6), flow_kind=1,
                    flow_p=(2.0 / 3.0, L[1], 0.0), bond=dict(name="Quartic", params=rec.reshape(1, 8)))
    md.run(100)
    out = sim.state.get_snapshot().particles
    ref_unwrapped = md.s["pos4"][:, :3] + md.s["image"] * L
    # FP32 forces: 100 steps (0.5 tau) of a stiff bead-spring melt stay within 1e-3
    assert np.abs(_unwrapped(out, L) - ref_unwrapped).max() < 1e-3
    assert np.abs(out.velocity - md.s["vel4"][:, :3]).max() < 2e-2
    # wrapped positions lie in the box; images agree with the unwrapped trajectory
    assert (np.abs(out.position) <= L / 2).all()


def test_fp32_brownian_vs_oracle(orc):
    snap = random_fluid(800, 0.3, seed=34, min_dist=1.05)
    sim, lj = _lj_setup(snap, precision="fp32", method="brownian", flow=az.flow.ConstantFlow((0.1, 0.0, 0.0)),
                        dt=2e-4, lam=1.0, rcut=2.5)
    sim.run(50)
    md = _oracle_lj(orc, snap, method="brownian", dt=2e-4, lam=1.0, rcut=2.5, flow_kind=0, flow_p=(0.1, 0, 0))
    md.run(50)
    out = sim.state.get_snapshot().particles
    L = box_of(snap)
    assert np.abs(_unwrapped(out, L) - (md.s["pos4"][:, :3] + md.s["image"] * L)).max() < 1e-6


def test_fp32_images_cross_every_face():
    # a constant drift carries every particle across the +x face and, with a
    # negative y drift, across the -y face: images count the crossings exactly
    snap = random_fluid(500, 0.2, seed=35, min_dist=1.2)
    L = box_of(snap)
    n = 400
    dt = 1e-3
    drift = (L[0] / (n * dt) * 1.3, -L[1] / (n * dt) * 0.6, 0.0)
    sim, lj = _lj_setup(snap, precision="fp32", method="brownian", flow=az.flow.ConstantFlow(drift), dt=dt,
                        lam=0.0, rcut=2 ** (1 / 6), kT=0.0)
    sim.run(n)
    out = sim.state.get_snapshot().particles
    moved = _unwrapped(out, L) - snap.particles.position
    # WCA pushes only at contact (none at this density and spacing); the drift dominates
    assert np.allclose(moved[:, 0], drift[0] * n * dt, rtol=0, atol=0.05)
    assert np.allclose(moved[:, 1], drift[1] * n * dt, rtol=0, atol=0.05)
    assert (out.image[:, 0] >= 1).all() and (out.image[:, 1] <= 0).all()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_large_system_forces_after_run(orc, precision, tol):
    # 40,000 particles: the engine's lists come from the shared-memory staged
    # build; a missing or extra pair would show in the forces
    snap = random_fluid(40000, 0.85, seed=36, min_dist=0.85)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    sim, lj = _lj_setup(snap, precision=precision, lam=0.0, rcut=2 ** (1 / 6), dt=0.002)
    sim.run(40)
    s = sim.state.get_snapshot()
    f, w = sim._engine.forces()
    F, U, W = _oracle_lj(orc, s, lam=0.0, rcut=2 ** (1 / 6)).forces()
    assert force_error(f, F) < tol
    assert rel(f[:, 3].sum(), U.sum()) < max(tol, 1e-12)
    assert sim.thermo()["nlist_builds"] >= 2


# ---------------------------------------------------------------- state set on a running engine
# azp_md_set_state on an engine that holds a state keeps its particle order and
# list, rebuilding only if a particle lies more than r_buff / 2 from its position
# at the last build; a denser state that overflows the list takes the full path.


def _engine_roundtrip(sim):
    s = sim.state.get_snapshot()
    sim.state.set_snapshot(s)


def test_state_round_trip_continues_bitwise_fp64():
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=10, density=0.8, seed=37)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    runs = []
    for roundtrip in (False, True):
        sim, lj = _lj_setup(snap)
        sim.run(30)
        if roundtrip:
            _engine_roundtrip(sim)
        sim.run(30)
        runs.append(sim.state.get_snapshot().particles)
    a, b = runs
    assert np.array_equal(a.position, b.position)
    assert np.array_equal(a.velocity, b.velocity)
    assert np.array_equal(a.image, b.image)


def test_state_set_far_from_last_build_rebuilds(orc):
    snap = random_fluid(3000, 0.8, seed=38)
    sim, lj = _lj_setup(snap, rcut=2.5)
    sim.run(5)
    other = random_fluid(3000, 0.8, seed=39)  # same N and box, unrelated positions
    other.particles.acceleration = np.zeros((3000, 3))
    sim.state.set_snapshot(other)
    sim.run(1)
    s = sim.state.get_snapshot()
    f, w = sim._engine.forces()
    F, U, W = _oracle_lj(orc, s, rcut=2.5).forces()
    assert force_error(f, F) < 1e-12


def test_state_set_denser_overflows_to_full_path(orc):
    import azplugins_gb300 as az

    snap = random_fluid(4000, 0.3, seed=40, min_dist=1.0)
    sim, lj = _lj_setup(snap, rcut=2.5, dt=1e-5)
    sim.run(3)
    # the same particles squeezed into a third of the box: three times the
    # density, more neighbours than the list was sized for
    dense = sim.state.get_snapshot()
    p = dense.particles
    L = box_of(dense)
    p.position = p.position.copy()
    p.position[:, 0] = p.position[:, 0] / 3.0 - L[0] / 3.0
    p.image = np.zeros_like(p.image)
    sim.state.set_snapshot(dense)
    sim.run(1)
    s = sim.state.get_snapshot()
    f, w = sim._engine.forces()
    F, U, W = _oracle_lj(orc, s, rcut=2.5).forces()
    assert force_error(f, F) < 1e-12


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_pinned_and_pageable_state_transfers_agree(precision):
    # page-locked host arrays (read and written in place by the state kernels,
    # full blocks through shared memory, the last block of 232 particles row by
    # row) and pageable ones (staged) give the same state transfers
    import ctypes

    import torch

    from azplugins_gb300 import _lib, workloads

    snap = workloads.lj_fluid(n_side=10, density=0.8, seed=41)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    sim, lj = _lj_setup(snap, precision=precision)
    sim.run(25)
    eng = sim._engine
    N = snap.particles.N
    L = eng._L
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def get(pinned):
        mk = (lambda shape, dt: torch.empty(shape, dtype=dt).pin_memory()) if pinned else \
            (lambda shape, dt: torch.empty(shape, dtype=dt))
        pos, vel, acc, img = mk((N, 4), torch.float64), mk((N, 4), torch.float64), mk((N, 3), torch.float64), \
            mk((N, 3), torch.int32)
        _lib.check(L.azp_md_get_state(eng._md, pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), img.data_ptr(), None, 0,
                                      stream), "azp_md_get_state")
        return pos, vel, acc, img

    a = get(True)
    b = get(False)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    # set the state back through pinned arrays, run, read: equal to the pageable round trip
    outs = []
    for pinned in (True, False):
        src = a if pinned else tuple(t.clone() for t in b)
        _lib.check(L.azp_md_set_state(eng._md, src[0].data_ptr(), src[1].data_ptr(), src[2].data_ptr(),
                                      src[3].data_ptr(), None, 25, 0, stream), "azp_md_set_state")
        _lib.check(L.azp_md_run(eng._md, 7, stream), "azp_md_run")
        outs.append(get(False))
    for x, y in zip(*outs):
        assert torch.equal(x, y)


def _binary_fluid(seed):
    snap = random_fluid(1200, 0.7, seed=seed, ntypes=2)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    return snap


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-4)])
@pytest.mark.parametrize("method", ["langevin", "brownian"])
def test_type_group_and_variant_kT(orc, precision, tol, method):
    """A method on filter.Type(["A"]) (the reference's ParticleGroup: B particles
    feel and exert forces but keep their positions and velocities) with kT a
    ramp of the timestep (the reference's Variant T, evaluated at the timestep of
    step two), against the oracle's loop with the same group and temperatures."""
    from azplugins_gb300 import variant

    snap = _binary_fluid(61)
    ramp = variant.Ramp(0.5, 2.0, 10, 40)
    sim = az.Simulation(seed=13, precision=precision)
    sim.create_state_from_snapshot(snap)
    lj = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=2.5)
    for k in [("A", "A"), ("A", "B"), ("B", "B")]:
        lj.params[k] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5)
    cls = az.methods.LangevinFlow if method == "langevin" else az.methods.BrownianFlow
    m = cls(az.filter.Type(["A"]), kT=ramp, flow_field=az.flow.ConstantFlow((0.1, 0.0, 0.0)), default_gamma=1.0)
    dt = 0.005 if method == "langevin" else 0.0005
    sim.operations.integrator = az.md.Integrator(dt=dt, methods=[m], forces=[lj])
    sim.run(30)
    sim.run(30)
    out = sim.state.get_snapshot().particles
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5))
    md = orc.OracleMD(oracle_system(snap, snap.particles.acceleration),
                      pair=dict(name="PerturbedLennardJones", params=np.tile(rec, (2, 2, 1)),
                                rcut=np.full((2, 2), 2.5)),
                      method=method, gamma=[1.0, 1.0], kT=ramp, dt=dt, seed=13, flow_kind=0, flow_p=(0.1, 0.0, 0.0),
                      group_types=[0])
    md.run(60)
    L = box_of(snap)
    b = snap.particles.typeid == 1
    # B particles did not move (FP32-force mode keeps positions as 64-bit fixed
    # point and velocities as float pairs: equal to the input within that storage)
    still = 0.0 if precision == "fp64" else 1e-12
    assert np.abs(out.position[b] - snap.particles.position[b]).max() <= still
    if method == "langevin":
        assert np.abs(out.velocity[b] - snap.particles.velocity[b]).max() <= (0.0 if precision == "fp64" else 1e-11)
    assert _pos_err(out.position, md.s["pos4"][:, :3], L) < tol
    if method == "langevin":
        assert np.abs(out.velocity - md.s["vel4"][:, :3]).max() < 10 * tol


def _run_tiles(snap, tiles, steps, bonds):
    # tiles need the cell order at every list build: the plain run re-sorts at
    # every build too, so that both keep the same particle order
    os.environ["AZP_TILES"] = "1" if tiles else "0"
    os.environ["AZP_SORT_EVERY"] = "1"
    try:
        sim = az.Simulation(seed=17, precision="fp32")
        sim.create_state_from_snapshot(snap)
        forces = []
        lj = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=2.5 if not bonds else 2 ** (1 / 6))
        lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5 if not bonds else 0.0)
        forces.append(lj)
        if bonds:
            qb = az.bond.Quartic()
            qb.params["A-A"] = dict(k=1434.3, r_0=1.5, b_1=-0.7589, b_2=0.0, U_0=67.2234, sigma=1.0, epsilon=1.0)
            forces.append(qb)
        flow = az.flow.ParabolicFlow(mean_velocity=2.0 / 3.0, separation=snap.configuration.box[1])
        m = az.methods.LangevinFlow("all", kT=1.0, flow_field=flow, default_gamma=1.0)
        sim.operations.integrator = az.md.Integrator(dt=0.005, methods=[m], forces=forces)
        sim.run(steps)
        out = sim.state.get_snapshot().particles
        f, w = sim._engine.forces()
        builds = sim.thermo()["nlist_builds"]
        sim.close()
        return out, f, w, builds
    finally:
        os.environ.pop("AZP_TILES", None)
        os.environ.pop("AZP_SORT_EVERY", None)


@pytest.mark.parametrize("bonds", [False, True])
def test_shared_memory_tiles_match_plain_gathers(bonds):
    """The single-type FP32-force step reading its neighbours from the block's
    shared-memory tile (the neighbour ranges staged once per step) against the
    same step gathering them from global memory: the same list order and the same
    arithmetic, so positions, velocities, forces and virials agree bit for bit
    over a run with several list rebuilds."""
    from azplugins_gb300 import workloads

    if bonds:
        import bench

        snap, _ = bench.relaxed_melt(120, seed=3)
    else:
        snap = workloads.lj_fluid(n_side=24, density=0.8, seed=33)
        snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    a = _run_tiles(snap, True, 60, bonds)
    b = _run_tiles(snap, False, 60, bonds)
    assert a[3] >= 2 and a[3] == b[3]
    assert np.array_equal(a[0].position, b[0].position)
    assert np.array_equal(a[0].velocity, b[0].velocity)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


def test_state_transfers_from_unaligned_device_buffers():
    """Device state buffers that start 8 bytes past a 16-byte boundary (the state
    kernels move positions and velocities as 16-byte pairs) go through aligned
    copies and give the same state as aligned buffers."""
    import ctypes

    import torch

    from azplugins_gb300 import _lib, workloads

    for precision in ("fp64", "fp32"):
        snap = workloads.lj_fluid(n_side=8, density=0.8, seed=43)
        snap.particles.acceleration = np.zeros((snap.particles.N, 3))
        sim, lj = _lj_setup(snap, precision=precision)
        sim.run(10)
        eng = sim._engine
        N = snap.particles.N
        L = eng._L
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def buffers(shift):
            raw = [torch.zeros(N * 4 + 2, dtype=torch.float64, device="cuda") for _ in range(2)]
            pos, vel = (r[shift:shift + 4 * N] for r in raw)
            acc = torch.zeros(N * 3, dtype=torch.float64, device="cuda")
            img = torch.zeros(N * 3, dtype=torch.int32, device="cuda")
            return raw, pos, vel, acc, img

        got = []
        for shift in (0, 1):
            raw, pos, vel, acc, img = buffers(shift)
            assert (pos.data_ptr() % 16 == 0) == (shift == 0)
            _lib.check(L.azp_md_get_state(eng._md, pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), img.data_ptr(), None,
                                          1, stream), "azp_md_get_state")
            torch.cuda.synchronize()
            got.append([t.clone() for t in (pos, vel, acc, img)])
        for x, y in zip(*got):
            assert torch.equal(x, y)
        # set from the unaligned copy, run, read back: equal to the aligned round trip
        outs = []
        for shift in (0, 1):
            raw, pos, vel, acc, img = buffers(shift)
            for t, v in zip((pos, vel, acc, img), got[0]):
                t.copy_(v)
            _lib.check(L.azp_md_set_state(eng._md, pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), img.data_ptr(),
                                          None, 10, 1, stream), "azp_md_set_state")
            _lib.check(L.azp_md_run(eng._md, 5, stream), "azp_md_run")
            o = [torch.zeros_like(t) for t in got[0]]
            _lib.check(L.azp_md_get_state(eng._md, o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), o[3].data_ptr(),
                                          None, 1, stream), "azp_md_get_state")
            torch.cuda.synchronize()
            outs.append(o)
        for x, y in zip(*outs):
            assert torch.equal(x, y)
        sim.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 2e-4)])
def test_order_keeping_builds_match_resorting_builds(precision, tol):
    """List builds that keep the particle order (scanning through the cell member
    table) between the re-sorting ones, against a re-sort at every build: the same
    neighbour sets and the same number of builds, so the trajectories differ only
    by the order of the force sums (FP64 1e-10, FP32 forces 2e-4 in positions
    after 80 steps of a chaotic fluid)."""
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=12, density=0.8, seed=43)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    runs = []
    for every in ("1", "3"):
        # read when the engine is made, at the first run
        os.environ["AZP_SORT_EVERY"] = every
        try:
            sim, lj = _lj_setup(snap, precision=precision)
            sim.run(80)
        finally:
            os.environ.pop("AZP_SORT_EVERY", None)
        p = sim.state.get_snapshot().particles
        runs.append((p.position + p.image * snap.configuration.box[:3], sim.thermo()["nlist_builds"]))
        sim.close()
    (xa, na), (xb, nb) = runs
    assert min(na, nb) >= 4
    # FP64: the same rebuild steps; FP32 forces: a particle at the displacement
    # threshold may tip one build either way
    assert na == nb if precision == "fp64" else abs(na - nb) <= 1
    assert np.abs(xa - xb).max() < tol
