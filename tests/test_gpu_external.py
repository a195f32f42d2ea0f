"""Harmonic barriers on the GPU.

* The reference's own sequences (src/pytest/test_external.py:84-223): the barrier
  added as a compute, a moving location, a spring constant switched off between
  runs; forces and energies read after run(1) and run(2) (tolerance 1e-4 as
  there; the FP64 values also equal the oracle's bit for bit).
* The drop-in driver azp_harmonic_barrier_forces against the oracle on a
  three-type system with particles drifted outside the box: FP64 bit-identical,
  FP32 (FP32 arithmetic) within 1e-6 norm-wise; the virial written as zeros.
* The resident engine with the barrier in the integrator's forces (fused into
  the step kernel) against the oracle's HOOMD-order MD loop, Langevin with a
  ramped planar barrier and Brownian with a spherical one: unwrapped positions
  within 1e-9 (FP64) or 1e-3 / 1e-5 (FP32 forces, Langevin / Brownian), and the
  forces (1e-12 / 1e-5 norm-wise) and energy the engine reports at the end.
"""

import ctypes

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import box_of, force_error, load_golden, oracle_system, pos4_of, random_fluid, rel

pytestmark = pytest.mark.gpu
KATS = load_golden("barrier_kats.json")


class _KatVariant(az.variant.Variant):
    """The CustomVariant of src/pytest/test_external.py:11-27."""

    def __init__(self, z):
        self.z = float(z)

    def __call__(self, timestep):
        return self.z if timestep <= 1 else self.z - 1.0


def _kat_snapshot(case):
    s = az.Snapshot(len(case["position"]))
    s.particles.types = list(case["types"])
    s.particles.position = np.array(case["position"], dtype=np.float64)
    s.particles.typeid = np.array(case["typeid"], dtype=np.int32)
    s.configuration.box = [float(x) for x in case["box"]]
    return s


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("geometry", ["planar", "spherical"])
def test_reference_sequence(orc, geometry, precision):
    case = KATS[geometry]
    snap = _kat_snapshot(case)
    sim = az.Simulation(seed=1, precision=precision)
    sim.create_state_from_snapshot(snap)
    # the reference integrates with dt = 0 and no force; particles at rest stay put
    m = az.methods.LangevinFlow("all", kT=0.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=0.0)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[m])
    cls = az.external.PlanarHarmonicBarrier if geometry == "planar" else az.external.SphericalHarmonicBarrier
    barrier = cls(location=_KatVariant(case["variant_z"]))
    first = case["stages"][0]["params"]
    for t in case["types"]:
        barrier.params[t] = first[t]
    sim.operations.add(barrier)
    done = 0
    for stage in case["stages"]:
        for t in case["types"]:
            barrier.params[t] = stage["params"][t]
        sim.run(stage["timestep"] - done)
        done = stage["timestep"]
        assert sim.timestep == stage["timestep"]
        forces, energies = barrier.forces, barrier.energies
        for i, e in stage["energies"].items():
            assert energies[int(i)] == pytest.approx(e, abs=1e-4)
        for i, f in stage["forces"].items():
            np.testing.assert_allclose(forces[int(i)], f, atol=1e-4)
        np.testing.assert_array_equal(barrier.virials, 0.0)
        if precision == "fp64":
            params = np.array([[stage["params"][t]["k"], stage["params"][t]["offset"]] for t in case["types"]])
            F, U = orc.harmonic_barrier(pos4_of(snap), case["typeid"], box_of(snap), geometry,
                                        barrier.location(sim.timestep), params)
            np.testing.assert_array_equal(forces, F)
            np.testing.assert_array_equal(energies, U)


def test_invalid_location_raises():
    case = KATS["planar"]
    sim = az.Simulation(seed=1)
    sim.create_state_from_snapshot(_kat_snapshot(case))
    m = az.methods.LangevinFlow("all", kT=0.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=0.0)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[m])
    barrier = az.external.PlanarHarmonicBarrier(location=10.0)  # box edge 20: y in [-10, 10)
    barrier.params[["A", "B"]] = dict(k=1.0, offset=0.0)
    sim.operations.add(barrier)
    sim.run(0)
    with pytest.raises(RuntimeError, match="Barrier position is invalid"):
        barrier.forces
    # and through the engine: a barrier in the integrator whose ramp leaves the box
    barrier.location = az.variant.Ramp(A=9.0, B=11.0, t_start=0, t_ramp=4)
    sim.operations.integrator.forces.append(barrier)
    with pytest.raises(RuntimeError, match="Barrier position is invalid"):
        sim.run(5)


def _drifted_system(N, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    L = np.array([14.0, 22.0, 18.0])
    pos = rng.uniform(-0.5, 0.5, size=(N, 3)) * L
    # a tenth of the particles drifted up to half a box out (wrapped by the driver)
    out = rng.random(N) < 0.1
    pos[out] += rng.choice([-1.0, 1.0], size=(out.sum(), 3)) * rng.uniform(0.5, 1.0, size=(out.sum(), 3)) * 0.5 * L
    types = rng.integers(0, 3, size=N).astype(np.int32)
    return pos, types, L


@pytest.mark.parametrize("geometry,location", [("planar", 3.25), ("planar", -10.5), ("spherical", 4.0),
                                               ("spherical", 0.0)])
def test_driver_matches_oracle(orc, geometry, location):
    import torch

    from azplugins_gb300 import _lib

    L_ = _lib.load()
    N = 20011
    pos, types, L = _drifted_system(N, seed=61)
    params = np.array([[30.0, 0.2], [0.0, -0.4], [125.0, -1.5]])
    F, U = orc.harmonic_barrier(np.concatenate([pos, types[:, None]], axis=1), types, L, geometry, location, params)
    assert (U > 0).sum() > 100
    dpos = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    dpos[:, :3] = torch.from_numpy(pos).cuda()
    dpos.view(torch.int64)[:, 3] = torch.from_numpy(types.astype(np.int64)).cuda()
    s = _lib.System()
    s.N, s.ntypes, s.pos = N, 3, dpos.data_ptr()
    for d in range(3):
        s.box.L[d] = L[d]
    dpar = torch.from_numpy(params.reshape(-1).copy()).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    geom = _lib.BARRIER_GEOMETRIES[geometry]
    for prec, dt in ((_lib.FP64, torch.float64), (_lib.FP32, torch.float32)):
        force = torch.full((N, 4), float("nan"), dtype=dt, device="cuda")
        vir = torch.full((6, N), float("nan"), dtype=dt, device="cuda")
        out = _lib.Forces()
        out.force, out.virial, out.virial_pitch, out.precision = force.data_ptr(), vir.data_ptr(), N, prec
        _lib.check(L_.azp_harmonic_barrier_forces(ctypes.byref(s), geom, location, dpar.data_ptr(), ctypes.byref(out),
                                                  stream), "azp_harmonic_barrier_forces")
        torch.cuda.synchronize()
        f = force.cpu().numpy()
        assert (vir.cpu().numpy() == 0).all()
        if prec == _lib.FP64:
            np.testing.assert_array_equal(f[:, :3], F)
            np.testing.assert_array_equal(f[:, 3], U)
        else:
            # FP32 arithmetic after the FP64 wrap and cancelling difference
            assert force_error(f, F) < 1e-6
            assert np.abs(f[:, 3] - U).max() <= 1e-6 * np.abs(U).max()


def _barrier_run(orc, precision, method, geometry, location, oracle_location, steps, seed, k=(5.0, 10.0)):
    snap = random_fluid(1500, 0.45, seed=seed, ntypes=2, min_dist=1.0)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    L = box_of(snap)
    sim = az.Simulation(seed=seed, precision=precision)
    sim.create_state_from_snapshot(snap)
    lj = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=2.5)
    lj.params[[("A", "A"), ("A", "B"), ("B", "B")]] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5)
    cls = az.external.PlanarHarmonicBarrier if geometry == "planar" else az.external.SphericalHarmonicBarrier
    barrier = cls(location=location)
    barrier.params["A"] = dict(k=k[0], offset=0.3)
    barrier.params["B"] = dict(k=k[1], offset=-0.5)
    dt = 0.004 if method == "langevin" else 2e-4
    mcls = az.methods.LangevinFlow if method == "langevin" else az.methods.BrownianFlow
    m = mcls("all", kT=1.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=1.0)
    sim.operations.integrator = az.md.Integrator(dt=dt, methods=[m], forces=[lj, barrier])
    # two runs: the second starts from the first's state and timestep
    sim.run(steps // 2)
    sim.run(steps - steps // 2)
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5))
    md = orc.OracleMD(oracle_system(snap, snap.particles.acceleration),
                      pair=dict(name="PerturbedLennardJones", params=np.tile(rec, (2, 2, 1)),
                                rcut=np.full((2, 2), 2.5), mode="none"),
                      method=method, gamma=[1.0, 1.0], kT=1.0, dt=dt, seed=seed,
                      barrier=dict(geometry=geometry, location=oracle_location,
                                   params=np.array([[k[0], 0.3], [k[1], -0.5]])))
    md.run(steps)
    return sim, md, L, barrier


def _unwrapped_err(sim, md, L):
    out = sim.state.get_snapshot().particles
    a = out.position + out.image * L
    b = md.s["pos4"][:, :3] + md.s["image"] * L
    return float(np.abs(a - b).max())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-3)])
def test_engine_langevin_ramped_planar_barrier(orc, precision, tol):
    # the barrier descends from near the top face into the fluid during the run
    L_y = random_fluid(1500, 0.45, seed=71, ntypes=2, min_dist=1.0).configuration.box[1]
    ramp = az.variant.Ramp(A=0.45 * L_y, B=0.3 * L_y, t_start=3, t_ramp=50)
    sim, md, L, barrier = _barrier_run(orc, precision, "langevin", "planar", ramp, ramp, 60, seed=71)
    F_md, U_md, _ = md.forces(md.timestep)
    assert (U_md > 0).sum() > 50  # the barrier acts on many particles
    assert _unwrapped_err(sim, md, L) < tol
    f, _ = sim._engine.forces()
    assert force_error(f, F_md) < (1e-12 if precision == "fp64" else 1e-5)
    assert rel(sim.thermo()["potential_energy"], U_md.sum()) < (1e-12 if precision == "fp64" else 1e-5)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_engine_brownian_spherical_barrier(orc, precision, tol):
    L = random_fluid(1500, 0.45, seed=72, ntypes=2, min_dist=1.0).configuration.box[0]
    R = 0.4 * L
    sim, md, L, barrier = _barrier_run(orc, precision, "brownian", "spherical", R, R, 40, seed=72, k=(2.0, 4.0))
    F_md, U_md, _ = md.forces(md.timestep)
    assert (U_md > 0).sum() > 50
    assert _unwrapped_err(sim, md, L) < tol
    f, _ = sim._engine.forces()
    assert force_error(f, F_md) < (1e-12 if precision == "fp64" else 1e-5)
