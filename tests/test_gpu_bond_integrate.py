"""GPU bond forces (KATs, random chains vs the oracle) and the standalone
integrator drivers: RNG bit-exact with the oracle, Langevin step one / step two
and the Brownian step within FP64 rounding of the oracle."""

import ctypes

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import force_error, load_golden, rel, two_particle_snapshot

pytestmark = pytest.mark.gpu
KATS = load_golden("kats.json")


def _sim(snap, precision="fp64"):
    sim = az.Simulation(seed=1, precision=precision)
    sim.create_state_from_snapshot(snap)
    return sim


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("case", KATS["bond"], ids=lambda c: f"{c['potential']}@{c['line']}")
def test_bond_kat(case, precision):
    snap = two_particle_snapshot(case["distance"], 20.0)
    snap.resize_bonds(1)
    snap.bonds.types = ["A-A"]
    snap.bonds.group = np.array([[0, 1]])
    sim = _sim(snap, precision)
    pot = getattr(az.bond, case["potential"])()
    pot.params["A-A"] = case["params"]
    sim.operations.integrator = az.md.Integrator(
        dt=0.001, methods=[az.methods.LangevinFlow("all", 1.0, az.flow.ConstantFlow((0, 0, 0)))], forces=[pot])
    sim.run(0)
    e, f = case["energy"], case["force"]
    dec = 4 if precision == "fp64" else 3
    np.testing.assert_array_almost_equal(pot.energies, [0.5 * e, 0.5 * e], decimal=dec)
    np.testing.assert_array_almost_equal(pot.forces, [[-f, 0, 0], [f, 0, 0]], decimal=dec)


def test_random_chains_vs_oracle(orc):
    from azplugins_gb300 import workloads

    snap = workloads.bead_spring_melt(40, 25, density=0.5, seed=3)
    params = dict(k=1434.3, r_0=1.5, b_1=-0.7589, b_2=0.0, U_0=67.2234, sigma=1.0, epsilon=1.0, delta=0.0)
    sim = _sim(snap)
    pot = az.bond.Quartic()
    pot.params["A-A"] = params
    sim.operations.integrator = az.md.Integrator(
        dt=0.001, methods=[az.methods.LangevinFlow("all", 1.0, az.flow.ConstantFlow((0, 0, 0)))], forces=[pot])
    sim.run(0)
    from helpers import box_of, pos4_of

    rec = orc.bond_params("Quartic", params)
    F, U, W = orc.bond_forces(pos4_of(snap), box_of(snap), snap.bonds.group, snap.bonds.typeid, "Quartic",
                              rec.reshape(1, 8))
    assert force_error(pot.forces, F) < 1e-12
    assert rel(pot.energies.sum(), U.sum()) < 1e-12
    assert np.allclose(pot.virials.sum(axis=0), W.sum(axis=0), rtol=1e-11, atol=1e-9)


def test_broken_bond_parameters_raise():
    snap = two_particle_snapshot(1.0, 20.0)
    snap.resize_bonds(1)
    snap.bonds.types = ["A-A"]
    snap.bonds.group = np.array([[0, 1]])
    sim = _sim(snap)
    pot = az.bond.DoubleWell()
    pot.params["A-A"] = dict(r_0=1.0, r_1=1.0, U_1=1.0, U_tilt=0.0)  # r_1 == r_0: refused
    sim.operations.integrator = az.md.Integrator(
        dt=0.001, methods=[az.methods.LangevinFlow("all", 1.0, az.flow.ConstantFlow((0, 0, 0)))], forces=[pot])
    sim.run(0)
    with pytest.raises(az._lib.AzpError, match="bond"):
        pot.forces


# ---------------------------------------------------------------- integrators
def _device_system(N, L, seed):
    import torch

    rng = np.random.Generator(np.random.PCG64(seed))
    pos = np.zeros((N, 4))
    pos[:, :3] = rng.uniform(-0.5, 0.5, size=(N, 3)) * L
    types = rng.integers(0, 2, size=N)
    vel = np.zeros((N, 4))
    vel[:, :3] = rng.normal(size=(N, 3))
    vel[:, 3] = rng.uniform(0.5, 2.0, size=N)
    acc = rng.normal(size=(N, 3)) * 10
    img = rng.integers(-2, 3, size=(N, 3)).astype(np.int32)
    force = rng.normal(size=(N, 4)) * 20
    host = dict(pos=pos, types=types, vel=vel, acc=acc, img=img, force=force, L=np.array([L, L, L]))
    d_pos = torch.from_numpy(pos.copy()).cuda()
    d_pos.view(torch.int64)[:, 3] = torch.from_numpy(types.astype(np.int64)).cuda()
    dev = dict(pos=d_pos, vel=torch.from_numpy(vel.copy()).cuda(), acc=torch.from_numpy(acc.copy()).cuda(),
               img=torch.from_numpy(img.copy()).cuda(), tag=torch.arange(N, dtype=torch.int32).cuda(),
               force=torch.from_numpy(force.copy()).cuda())
    s = az._lib.System()
    s.N, s.ntypes = N, 2
    s.pos, s.vel, s.accel, s.image = (dev["pos"].data_ptr(), dev["vel"].data_ptr(), dev["acc"].data_ptr(),
                                      dev["img"].data_ptr())
    s.tag = dev["tag"].data_ptr()
    s.diameter = None
    for d in range(3):
        s.box.L[d] = L
    return host, dev, s


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_uniform_draws_bit_exact(orc):
    import torch

    L = az._lib.load()
    n = 4096
    tags = torch.arange(n, dtype=torch.int32).cuda() * 7919
    out = torch.zeros((n, 3), dtype=torch.float64).cuda()
    for rid, ts, seed in [(202, 0, 0), (202, 123456789, 42), (201, (1 << 35) + 17, 65535 + 9)]:
        az._lib.check(L.azp_uniform3(rid, ts, seed, tags.data_ptr(), n, -1.7, 1.7, out.data_ptr(), _stream()), "u3")
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for k in range(0, n, 97):
            want = orc.uniform3(rid, ts, seed, int(tags[k]), -1.7, 1.7)
            assert np.array_equal(got[k], want), (rid, ts, seed, k)


def test_langevin_steps_vs_oracle(orc):
    import torch

    L = az._lib.load()
    N, Lb = 3000, 20.0
    host, dev, s = _device_system(N, Lb, 11)
    az._lib.check(L.azp_langevin_step1(ctypes.byref(s), None, 0, 0.005, _stream()), "step1")
    p4 = host["pos"].copy()
    v4 = host["vel"].copy()
    img = host["img"].copy()
    orc.langevin_step1(p4, img, v4, host["acc"].copy(), host["L"], 0.005)
    torch.cuda.synchronize()
    gp = dev["pos"].cpu().numpy()
    assert np.allclose(gp[:, :3], p4[:, :3], rtol=0, atol=1e-13)
    assert np.array_equal(dev["img"].cpu().numpy(), img)
    assert np.allclose(dev["vel"].cpu().numpy(), v4, rtol=1e-14, atol=1e-14)
    # the type bits in pos.w survive the update
    assert np.array_equal(dev["pos"].view(torch.int64)[:, 3].cpu().numpy(), host["types"])
    # step two with a parabolic flow and per-type gamma
    gamma = np.array([1.0, 2.5])
    d_gamma = torch.from_numpy(gamma).cuda()
    flow = az.flow.ParabolicFlow(2.0 / 3.0, Lb)._record()
    az._lib.check(L.azp_langevin_step2(ctypes.byref(s), None, 0, dev["force"].data_ptr(), az._lib.FP64,
                                       d_gamma.data_ptr(), 0, 0.0, flow, 0.005, 1.3, 77, 5, 0, _stream()), "step2")
    acc = np.zeros((N, 3))
    p4o = p4.copy()
    p4o[:, 3] = host["types"]
    orc.langevin_step2(p4o, host["types"].astype(np.int32), v4, acc, host["force"][:, :3].copy(),
                       np.arange(N, dtype=np.uint32), gamma, 1, np.array([2.0 / 3.0, Lb, 0.0]), 1.3, 0.005, 77, 5)
    torch.cuda.synchronize()
    assert np.allclose(dev["acc"].cpu().numpy(), acc, rtol=1e-13, atol=1e-12)
    assert np.allclose(dev["vel"].cpu().numpy(), v4, rtol=1e-13, atol=1e-13)


def test_brownian_step_vs_oracle(orc):
    import torch

    L = az._lib.load()
    N, Lb = 2000, 15.0
    host, dev, s = _device_system(N, Lb, 12)
    gamma = np.array([1.0, 3.0])
    d_gamma = torch.from_numpy(gamma).cuda()
    flow = az.flow.ConstantFlow((0.1, 0.0, -0.2))._record()
    az._lib.check(L.azp_brownian_step(ctypes.byref(s), None, 0, dev["force"].data_ptr(), az._lib.FP64,
                                      d_gamma.data_ptr(), 0, 0.0, flow, 0.001, 1.0, 9, 3, 0, 0.0, _stream()), "bd")
    p4 = host["pos"].copy()
    p4[:, 3] = host["types"]
    img = host["img"].copy()
    orc.brownian(p4, img, host["types"].astype(np.int32), host["force"][:, :3].copy(),
                 np.arange(N, dtype=np.uint32), gamma, 0, np.array([0.1, 0.0, -0.2]), host["L"], 1.0, 0.001, 9, 3)
    torch.cuda.synchronize()
    assert np.allclose(dev["pos"].cpu().numpy()[:, :3], p4[:, :3], rtol=0, atol=1e-13)
    assert np.array_equal(dev["img"].cpu().numpy(), img)
    assert np.array_equal(dev["pos"].view(torch.int64)[:, 3].cpu().numpy(), host["types"])
