"""Velocity computes on the GPU (azp_vfield_*).

* The reference's sequences through the Python front end
  (src/pytest/test_compute.py: TestVelocityCompute :15-66, TestVelocityField
  :148-331, TestCartesianVelocityFieldCompute :347-415,
  TestCylindricalVelocityFieldCompute :418-523; the branch without MPCD
  particles), tolerances as there.
* The drop-in compute against the oracle on 200k particles: Cartesian slabs,
  cylindrical bins, a 10^4-bin grid (global-histogram path) and a type group.
  The sums are fixed-point sums of contributions rounded to 2^-40, so each bin's
  mass and momentum are within (members in the bin) x 2^-41 of the oracle's
  FP64 sums; velocities within 1e-9 relative.
* Order independence: the same particles in another order give bit-identical
  sums; a momentum beyond the fixed-point range raises.
"""

import ctypes

import numpy as np
import pytest

import azplugins_gb300 as az

pytestmark = pytest.mark.gpu
L20 = [20.0, 20.0, 20.0, 0.0, 0.0, 0.0]


def _sim(pos, vel, mass, types=("A",), typeid=None):
    s = az.Snapshot(len(pos))
    s.particles.types = list(types)
    s.particles.position = np.asarray(pos, dtype=float)
    s.particles.velocity = np.asarray(vel, dtype=float)
    s.particles.mass = np.asarray(mass, dtype=float)
    if typeid is not None:
        s.particles.typeid = np.asarray(typeid, dtype=np.int32)
    s.configuration.box = L20
    sim = az.Simulation()
    sim.create_state_from_snapshot(s)
    return sim


def test_velocity_compute_reference():
    # TestVelocityCompute.test_attach_detach / test_hoomd_particles
    sim = _sim([[-0.5, 0, 0], [0.5, 0, 0]], np.zeros((2, 3)), [1, 1])
    vel = az.compute.VelocityCompute()
    sim.operations.add(vel)
    sim.run(0)
    np.testing.assert_array_equal(vel.velocity, [0, 0, 0])
    sim = _sim([[0, 0, -1], [0, 0, 1]], [[1, -2, 3], [-2, 4, -6]], [1, 2], types=("A", "B"), typeid=[0, 1])
    sim.run(0)
    vel_all = az.compute.VelocityCompute(filter=az.filter.All())
    sim.operations.add(vel_all)
    np.testing.assert_allclose(vel_all.velocity, [-1, 2, -3])
    vel_a = az.compute.VelocityCompute(filter=az.filter.Type("A"))
    vel_b = az.compute.VelocityCompute(filter=az.filter.Type("B"))
    sim.operations.computes.extend([vel_a, vel_b])
    sim.run(0)
    np.testing.assert_allclose(vel_a.velocity, [1, -2, 3])
    np.testing.assert_allclose(vel_b.velocity, [-2, 4, -6])


@pytest.mark.parametrize("cls,lo,hi", [(az.compute.CartesianVelocityFieldCompute, (-10, -10, -10), (10, 10, 10)),
                                       (az.compute.CylindricalVelocityFieldCompute, (0, 0, -10),
                                        (10, 2 * np.pi, 10))])
def test_field_attach_and_shapes(cls, lo, hi):
    sim = _sim([[-0.5, 0, 0], [0.5, 0, 0]], np.zeros((2, 3)), [1, 1])
    field = cls(num_bins=[2, 0, 1], lower_bounds=lo, upper_bounds=hi)
    sim.operations.add(field)
    sim.run(0)
    v = field.velocities
    assert v.shape == (2, 1, 3)
    assert (v == 0).all()
    for nb, shape in (([2, 3, 4], (2, 3, 4, 3)), ([2, 3, 0], (2, 3, 3)), ([0, 3, 4], (3, 4, 3)), ([2, 0, 0], (2, 3)),
                      ([0, 0, 4], (4, 3)), ([0, 0, 0], (3,))):
        field.num_bins = nb
        assert field.velocities.shape == shape
    sim.operations.remove(field)
    with pytest.raises(az.compute.DataAccessError):
        field.velocities


def test_cartesian_reference():
    sim = _sim([[6, -4, 0.1], [-4, 2, -0.1]], [[1, 2, 3], [-3, -2, -1]], [5, 1])
    field = az.compute.CartesianVelocityFieldCompute(num_bins=[4, 3, 2], lower_bounds=(-10, -6, -5),
                                                     upper_bounds=(10, 3, 5), filter=az.filter.All(),
                                                     include_mpcd_particles=True)
    sim.operations.add(field)
    sim.run(0)
    h, m = [1, 2, 3], [-3, -2, -1]
    v = field.velocities
    np.testing.assert_allclose(v[3, 0, 1], h)
    np.testing.assert_allclose(v[1, 2, 0], m)
    mask = np.ones(v.shape, dtype=bool)
    mask[3, 0, 1] = mask[1, 2, 0] = False
    assert (v[mask] == 0).all()
    field.num_bins = [4, 0, 0]
    np.testing.assert_allclose(field.velocities, [[0, 0, 0], m, [0, 0, 0], h])
    field.num_bins = [0, 3, 0]
    np.testing.assert_allclose(field.velocities, [h, [0, 0, 0], m])
    field.num_bins = [0, 0, 2]
    np.testing.assert_allclose(field.velocities, [m, h])
    field.num_bins = [1, 1, 1]
    field.lower_bounds = [-1, -1, -1]
    field.upper_bounds = [1, 1, 1]
    assert (field.velocities == 0).all()
    field.lower_bounds = [-10, -10, -10]
    field.upper_bounds = [10, 10, 10]
    np.testing.assert_allclose(field.velocities.reshape(3), (5 * np.array(h) + m) / 6, rtol=1e-12)
    # filter None: no particles
    none = az.compute.CylindricalVelocityFieldCompute(num_bins=[1, 1, 1], lower_bounds=(-10, -10, -10),
                                                      upper_bounds=(10, 10, 10))
    sim.operations.add(none)
    sim.run(0)
    assert (none.velocities == 0).all()


def test_cylindrical_reference():
    s = np.sqrt(4.5)
    sim = _sim([[1, 1, 0.1], [-0.5, -0.5, -0.1]], [[-1, 1, 2], [-s, -s, -2]], [5, 1])
    field = az.compute.CylindricalVelocityFieldCompute(num_bins=[2, 3, 4], lower_bounds=(0, 0, -1),
                                                       upper_bounds=(2, 3 * np.pi / 2, 1), filter=az.filter.All())
    sim.operations.add(field)
    sim.run(0)
    h, m = [0, np.sqrt(2), 2], [3, 0, -2]
    v = field.velocities
    np.testing.assert_allclose(v[1, 0, 2], h, atol=1e-11)
    np.testing.assert_allclose(v[0, 2, 1], m, atol=1e-11)
    mask = np.ones(v.shape, dtype=bool)
    mask[1, 0, 2] = mask[0, 2, 1] = False
    assert (v[mask] == 0).all()
    field.num_bins = [2, 0, 0]
    np.testing.assert_allclose(field.velocities, [m, h], atol=1e-11)
    field.num_bins = [0, 3, 0]
    np.testing.assert_allclose(field.velocities, [h, [0, 0, 0], m], atol=1e-11)
    field.num_bins = [0, 0, 4]
    np.testing.assert_allclose(field.velocities, [[0, 0, 0], m, h, [0, 0, 0]], atol=1e-11)
    field.num_bins = [1, 1, 1]
    field.lower_bounds = [1, np.pi, -1]
    field.upper_bounds = [2, 3 * np.pi / 2, 1]
    assert (field.velocities == 0).all()
    field.lower_bounds = [0, 0, -10]
    field.upper_bounds = [10, 2 * np.pi, 10]
    np.testing.assert_allclose(field.velocities.reshape(3), (5 * np.array(h) + m) / 6, atol=1e-11)


def _big_system(N=200_000, seed=101):
    rng = np.random.Generator(np.random.PCG64(seed))
    L = np.array([30.0, 24.0, 36.0])
    pos = rng.uniform(-0.5, 0.5, size=(N, 3)) * L
    # a share drifted out of the box (wrapped by the compute)
    out = rng.random(N) < 0.05
    pos[out] += rng.choice([-1.0, 1.0], size=(out.sum(), 3)) * 0.3 * L
    vel = rng.normal(size=(N, 3)) + np.array([0.3, -0.1, 0.0])
    mass = rng.uniform(0.5, 3.0, size=N)
    types = rng.integers(0, 3, size=N).astype(np.int32)
    return pos, vel, mass, types, L


def _device_run(pos, vel, mass, L, kind, nb, lo, hi, members=None):
    import torch

    from azplugins_gb300 import _lib

    Lib = _lib.load()
    N = len(pos)
    dpos = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    dpos[:, :3] = torch.from_numpy(pos).cuda()
    dvel = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    dvel[:, :3] = torch.from_numpy(vel).cuda()
    dvel[:, 3] = torch.from_numpy(mass).cuda()
    s = _lib.System()
    s.N, s.ntypes, s.pos, s.vel = N, 1, dpos.data_ptr(), dvel.data_ptr()
    for d in range(3):
        s.box.L[d] = L[d]
    st = ctypes.c_int(0)
    nb_ = np.ascontiguousarray(nb, dtype=np.uint32)
    lo_ = np.ascontiguousarray(lo, dtype=np.float64)
    hi_ = np.ascontiguousarray(hi, dtype=np.float64)
    vf = Lib.azp_vfield_create(_lib.BINNING_KINDS[kind], nb_.ctypes.data, lo_.ctypes.data, hi_.ctypes.data,
                               ctypes.byref(st))
    _lib.check(st.value, "azp_vfield_create")
    total = int(Lib.azp_vfield_num_bins(vf))
    mass_o = torch.zeros(total, dtype=torch.float64, device="cuda")
    mom_o = torch.zeros((total, 3), dtype=torch.float64, device="cuda")
    vel_o = torch.zeros((total, 3), dtype=torch.float64, device="cuda")
    grp = None if members is None else torch.from_numpy(np.asarray(members, dtype=np.int32)).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(Lib.azp_vfield_compute(vf, ctypes.byref(s), None if grp is None else grp.data_ptr(),
                                      0 if grp is None else len(members), mass_o.data_ptr(), mom_o.data_ptr(),
                                      vel_o.data_ptr(), stream), "azp_vfield_compute")
    err = ctypes.c_uint32(0)
    _lib.check(Lib.azp_vfield_error(vf, ctypes.byref(err), stream), "azp_vfield_error")
    Lib.azp_vfield_destroy(vf)
    return mass_o.cpu().numpy(), mom_o.cpu().numpy(), vel_o.cpu().numpy(), err.value


CASES = [
    ("cartesian", (0, 12, 0), (0, -12, 0), (0, 12, 0)),
    ("cartesian", (6, 5, 4), (-15, -12, -18), (15, 12, 18)),
    ("cartesian", (100, 100, 0), (-15, -12, 0), (15, 12, 0)),
    ("cylindrical", (5, 8, 3), (0, 0, -18), (12, 2 * np.pi, 18)),
    ("cylindrical", (10, 0, 0), (1.0, 0, 0), (11.0, 0, 0)),
    ("cartesian", (0, 0, 0), (0, 0, 0), (0, 0, 0)),
]


@pytest.mark.parametrize("kind,nb,lo,hi", CASES, ids=[f"{c[0]}{c[1]}" for c in CASES])
def test_matches_oracle(orc, kind, nb, lo, hi):
    pos, vel, mass, types, L = _big_system()
    members = np.flatnonzero(types != 1).astype(np.int32) if kind == "cylindrical" else None
    pos4 = np.concatenate([pos, np.zeros((len(pos), 1))], axis=1)
    vel4 = np.concatenate([vel, mass[:, None]], axis=1)
    M, P, V = orc.velocity_field(pos4, vel4, L, kind, nb, lo, hi, members)
    m, p, v, err = _device_run(pos, vel, mass, L, kind, nb, lo, hi, members)
    assert err == 0
    # per-bin bound: (members in the bin) x 2^-41; the bin's count is at most mass / 0.5
    bound = (M / 0.5 + 1) * 2.0 ** -41
    assert (np.abs(m - M) <= bound).all()
    assert (np.abs(p - P) <= bound[:, None]).all()
    assert np.abs(v - V).max() <= 1e-9 * max(np.abs(V).max(), 1.0)
    assert (M > 0).sum() == (m > 0).sum()


def test_order_independent_and_range():
    pos, vel, mass, types, L = _big_system(N=50_000, seed=102)
    args = ("cylindrical", (4, 6, 2), (0, 0, -18), (14, 2 * np.pi, 18))
    a = _device_run(pos, vel, mass, L, *args)
    perm = np.random.Generator(np.random.PCG64(5)).permutation(len(pos))
    b = _device_run(pos[perm], vel[perm], mass[perm], L, *args)
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)
    vel2 = vel.copy()
    vel2[17] = [3e7, 0, 0]
    *_, err = _device_run(pos, vel2, mass, L, *args)
    from azplugins_gb300 import _lib

    assert err & _lib.EBIT_RANGE
