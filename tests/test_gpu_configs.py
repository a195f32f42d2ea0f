"""Parity on the benchmark workloads themselves, at their own sizes.

* PerturbedLJ fluid exactly as the workload states it: N = 4096 on a 16^3
  simple-cubic lattice jittered by +-0.05, density 0.8, epsilon = sigma = 1,
  lambda = 0.5, r_cut = 3, buffer 0.4, Maxwell-Boltzmann velocities at kT = 1;
  LangevinFlow with ConstantFlow 0, gamma = 1, dt = 0.005, 1000 steps with
  forces, energy and virial dumped every 100 steps. The FP64 engine's trajectory
  against the oracle's MD loop (1e-9 in positions after 100 steps), and at every
  dump the engine's own forces, per-particle energies and virials against the
  oracle evaluated at the engine's state: 1e-12 (FP64) and 1e-5 (FP32), forces
  norm-wise max_i |dF_i| / max(|F_i|, F_rms), total energy and each virial
  component relative to the largest component. The contract is the reference's
  pair-loop test (src/pytest/test_pair.py:351-363: U_i = half the pair energies,
  equal and opposite forces).
* The bead-spring melt at N = 1,048,600 (10,486 chains x 100, the headline
  workload after its 200-step relaxation): the resident engine's net forces in
  both precisions against the oracle's pair + bond forces, on a seeded sample of
  20,000 particles (the oracle evaluates every particle; the comparison is over
  the sample), at the same tolerances.
"""

import os

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import box_of, force_error, oracle_system, rel

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-5}


def _pos_err(a, b, L):
    d = a - b
    d -= L * np.rint(d / L)
    return float(np.abs(d).max())


def _check_dump(f, w, F, U, W, tol):
    assert force_error(f, F) < tol
    assert rel(f[:, 3].sum(), U.sum()) < tol
    scale = np.abs(W.sum(axis=0)).max()
    assert np.abs(w.sum(axis=0) - W.sum(axis=0)).max() <= tol * scale
    # per-particle energies and virials, relative to the largest entry
    assert np.abs(f[:, 3] - U).max() <= tol * np.abs(U).max()
    assert np.abs(w - W).max() <= tol * np.abs(W).max()


def _lj_oracle(orc, system, dt=0.005):
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5))
    return orc.OracleMD(system, pair=dict(name="PerturbedLennardJones", params=rec.reshape(1, 1, 4),
                                          rcut=np.array([[3.0]])),
                        gamma=[1.0], kT=1.0, dt=dt, seed=1)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_lj_fluid_workload_as_written(orc, precision):
    from azplugins_gb300 import workloads

    snap = workloads.lj_fluid(n_side=16, density=0.8, jitter=0.05, kT=1.0, seed=1)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    assert snap.particles.N == 4096
    L = box_of(snap)
    sim = az.Simulation(seed=1, precision=precision)
    sim.create_state_from_snapshot(snap)
    lj = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=3.0)
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5)
    m = az.methods.LangevinFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=1.0)
    sim.operations.integrator = az.md.Integrator(dt=0.005, methods=[m], forces=[lj])
    md = _lj_oracle(orc, oracle_system(snap, snap.particles.acceleration))
    dumps = 0
    for block in range(10):
        sim.run(100)
        s = sim.state.get_snapshot()
        if block == 0:
            md.run(100)
            perr = _pos_err(s.particles.position, md.s["pos4"][:, :3], L)
            assert perr < (1e-9 if precision == "fp64" else 1e-4)
        # the dump: forces, energies and virials of the engine at its own state
        f, w = sim._engine.forces()
        ref = _lj_oracle(orc, oracle_system(s, s.particles.acceleration))
        F, U, W = ref.forces()
        _check_dump(f, w, F, U, W, TOL[precision])
        dumps += 1
    assert dumps == 10
    assert sim.thermo()["nlist_builds"] > 10
    sim.close()


@pytest.fixture(scope="module")
def melt_state():
    """The headline melt after its capped relaxation (bench.relaxed_melt, on the host)."""
    import bench

    snap, _ = bench.relaxed_melt(bench.N_CHAINS, seed=1)
    return snap


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_melt_full_size_forces_vs_oracle(orc, melt_state, precision):
    import bench

    snap = melt_state
    N = snap.particles.N
    assert N == 1048600
    L = box_of(snap)
    sim = az.Simulation(seed=7, precision=precision)
    sim.create_state_from_snapshot(snap)
    wca, qb = bench.forces_and_method(az, None)
    flow = az.flow.ParabolicFlow(mean_velocity=2.0 / 3.0, separation=L[1])
    m = az.methods.LangevinFlow("all", kT=bench.KT, flow_field=flow, default_gamma=bench.GAMMA)
    sim.operations.integrator = az.md.Integrator(dt=bench.DT, methods=[m], forces=[wca, qb])
    sim.run(20)
    f, w = sim._engine.forces()
    s = sim.state.get_snapshot()
    sim.close()
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.0))
    brec = orc.bond_params("Quartic", bench.QUARTIC)
    threads = orc.set_threads(os.cpu_count() or 1)
    try:
        md = orc.OracleMD(oracle_system(s, s.particles.acceleration),
                          pair=dict(name="PerturbedLennardJones", params=rec.reshape(1, 1, 4),
                                    rcut=np.array([[bench.RCUT]])),
                          bond=dict(name="Quartic", params=brec.reshape(1, 8)), gamma=[1.0], kT=1.0, dt=bench.DT)
        F, U, W = md.forces()
    finally:
        orc.set_threads(1)
    assert threads >= 1
    rng = np.random.Generator(np.random.PCG64(2024))
    sample = rng.choice(N, size=20000, replace=False)
    # the norm of the whole system (F_rms), the comparison over the sample
    mag = np.sqrt((F ** 2).sum(axis=1))
    den = np.maximum(mag[sample], np.sqrt((mag ** 2).mean()))
    err = float((np.sqrt(((f[sample, :3] - F[sample]) ** 2).sum(axis=1)) / den).max())
    assert err < TOL[precision], err
    assert np.abs(f[sample, 3] - U[sample]).max() <= TOL[precision] * np.abs(U).max()
    assert np.abs(w[sample] - W[sample]).max() <= TOL[precision] * np.abs(W).max()
    assert rel(f[:, 3].sum(), U.sum()) < TOL[precision]


def _colloid_pot(mode="shift"):
    c = az.pair.Colloid(nlist=az.nlist.Cell(buffer=0.4), mode=mode)
    c.params[("S", "S")] = dict(A=144.0, a_1=0.0, a_2=0.0, sigma=1.0)
    c.params[("S", "C")] = dict(A=100.0, a_1=0.0, a_2=2.5, sigma=1.0)
    c.params[("C", "C")] = dict(A=40.0, a_1=2.5, a_2=2.5, sigma=1.0)
    c.r_cut[("S", "S")] = 3.0
    c.r_cut[("S", "C")] = 6.0
    c.r_cut[("C", "C")] = 10.0
    return c


def test_colloid_mixture_fp32_forces_within_budget(orc):
    """The colloid-solvent mixture of the precision workload at 20,000 particles
    (4 % colloids of diameter 5, phi = 0.3, Hamaker 144 / 100 / 40, r_cut 3 / 6 / 10,
    shifted), advanced by the FP32-force engine with BrownianFlow (U = 0.1 x,
    dt = 0.001, gamma = 10 diameter); every 50 steps the FP32 forces of the drop-in
    driver and of the engine against the oracle's FP64 forces at that state: 1e-5
    norm-wise (point-sphere and sphere-sphere forms with the contact difference
    formed exactly, PairEvaluatorColloid.h:125-220), energy and virial 1e-5."""
    from azplugins_gb300 import _compute, workloads
    from helpers import pair_tables, pos4_of

    snap = workloads.colloid_mixture(20000, seed=5)
    pot = _colloid_pot()
    sim = az.Simulation(seed=3, precision="fp32")
    sim.create_state_from_snapshot(snap)
    m = az.methods.BrownianFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0.1, 0.0, 0.0)), alpha=10.0)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[m], forces=[pot])
    types = list(snap.particles.types)
    params = {("S", "S"): dict(A=144.0, a_1=0.0, a_2=0.0, sigma=1.0),
              ("C", "S"): dict(A=100.0, a_1=0.0, a_2=2.5, sigma=1.0),
              ("C", "C"): dict(A=40.0, a_1=2.5, a_2=2.5, sigma=1.0)}
    rcut = {("S", "S"): 3.0, ("C", "S"): 6.0, ("C", "C"): 10.0}
    rec, rc, _ = pair_tables(orc, "Colloid", params, types, rcut)
    worst = 0.0
    for _ in range(4):
        sim.run(50)
        s = sim.state.get_snapshot()
        pos4 = pos4_of(s)
        L = box_of(s)
        st, idx = orc.nlist(pos4, s.particles.typeid, len(types), L, (rc + 0.4) ** 2)
        F, U, W = orc.pair_forces(pos4, s.particles.typeid, len(types), L, st, idx, "Colloid", rec, rc * rc, None,
                                  "shift")
        ref = az.Simulation(precision="fp64")
        ref.create_state_from_snapshot(s)
        f_drv, w_drv = _compute.pair_forces(ref.state, pot, "fp32")
        ref.close()
        f_eng, w_eng = sim._engine.forces()
        for f, w in ((f_drv, w_drv), (f_eng, w_eng)):
            err = force_error(f, F)
            worst = max(worst, err)
            assert err < 1e-5, err
            assert rel(f[:, 3].sum(), U.sum()) < 1e-5
            assert np.abs(w.sum(axis=0) - W.sum(axis=0)).max() <= 1e-5 * np.abs(W.sum(axis=0)).max()
    sim.close()
