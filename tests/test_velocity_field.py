"""Velocity computes on the CPU: the oracle against the reference's known
answers (src/pytest/test_compute.py, the branch without MPCD particles:
TestCartesianVelocityFieldCompute :371-400, TestCylindricalVelocityFieldCompute
:448-505, TestVelocityCompute.test_hoomd_particles :47-66), and the front end's
shapes and coordinates (test_binning_shape :243-331) and access rules."""

import numpy as np
import pytest

import azplugins_gb300 as az

L20 = [20.0, 20.0, 20.0]


def _cart_system():
    # src/pytest/test_compute.py:357-368
    pos = np.array([[6, -4, 0.1, 0], [-4, 2, -0.1, 0]], dtype=float)
    vel = np.array([[1, 2, 3, 5], [-3, -2, -1, 1]], dtype=float)
    return pos, vel


def _cyl_system():
    # src/pytest/test_compute.py:434-445
    s = np.sqrt(4.5)
    pos = np.array([[1, 1, 0.1, 0], [-0.5, -0.5, -0.1, 0]], dtype=float)
    vel = np.array([[-1, 1, 2, 5], [-s, -s, -2, 1]], dtype=float)
    return pos, vel


def test_oracle_cartesian_reference(orc):
    pos, vel = _cart_system()
    h, m = np.array([1.0, 2, 3]), np.array([-3.0, -2, -1])

    def field(nb, lo=(-10, -6, -5), hi=(10, 3, 5)):
        _, _, v = orc.velocity_field(pos, vel, L20, "cartesian", nb, lo, hi)
        return v.reshape([n for n in nb if n > 0] + [3])

    v = field([4, 3, 2])
    np.testing.assert_allclose(v[3, 0, 1], h)
    np.testing.assert_allclose(v[1, 2, 0], m)
    mask = np.ones(v.shape, dtype=bool)
    mask[3, 0, 1] = mask[1, 2, 0] = False
    assert (v[mask] == 0).all()
    np.testing.assert_allclose(field([4, 0, 0]), [[0, 0, 0], m, [0, 0, 0], h])
    np.testing.assert_allclose(field([0, 3, 0]), [h, [0, 0, 0], m])
    np.testing.assert_allclose(field([0, 0, 2]), [m, h])
    assert (field([1, 1, 1], (-1, -1, -1), (1, 1, 1)) == 0).all()
    np.testing.assert_array_equal(field([1, 1, 1], (-10, -10, -10), (10, 10, 10)).reshape(3), (5 * h + m) / 6)


def test_oracle_cylindrical_reference(orc):
    pos, vel = _cyl_system()
    h, m = np.array([0.0, np.sqrt(2), 2]), np.array([3.0, 0, -2])

    def field(nb, lo=(0, 0, -1), hi=(2, 3 * np.pi / 2, 1)):
        _, _, v = orc.velocity_field(pos, vel, L20, "cylindrical", nb, lo, hi)
        return v.reshape([n for n in nb if n > 0] + [3])

    v = field([2, 3, 4])
    np.testing.assert_allclose(v[1, 0, 2], h, atol=1e-15)
    np.testing.assert_allclose(v[0, 2, 1], m, atol=1e-15)
    mask = np.ones(v.shape, dtype=bool)
    mask[1, 0, 2] = mask[0, 2, 1] = False
    assert (v[mask] == 0).all()
    np.testing.assert_allclose(field([2, 0, 0]), [m, h], atol=1e-15)
    np.testing.assert_allclose(field([0, 3, 0]), [h, [0, 0, 0], m], atol=1e-15)
    np.testing.assert_allclose(field([0, 0, 4]), [[0, 0, 0], m, h, [0, 0, 0]], atol=1e-15)
    assert (field([1, 1, 1], (1, np.pi, -1), (2, 3 * np.pi / 2, 1)) == 0).all()
    np.testing.assert_allclose(field([1, 1, 1], (0, 0, -10), (10, 2 * np.pi, 10)).reshape(3), (5 * h + m) / 6,
                               atol=1e-15)


def test_oracle_com_velocity(orc):
    # src/pytest/test_compute.py:47-66: two particles of masses 1 and 2
    pos = np.array([[0, 0, -1, 0], [0, 0, 1, 1]], dtype=float)
    vel = np.array([[1, -2, 3, 1], [-2, 4, -6, 2]], dtype=float)
    _, _, v = orc.velocity_field(pos, vel, L20, "cartesian", [0, 0, 0], [0] * 3, [0] * 3)
    np.testing.assert_allclose(v[0], [-1, 2, -3])
    _, _, v = orc.velocity_field(pos, vel, L20, "cartesian", [0, 0, 0], [0] * 3, [0] * 3, members=[0])
    np.testing.assert_allclose(v[0], [1, -2, 3])
    _, _, v = orc.velocity_field(pos, vel, L20, "cartesian", [0, 0, 0], [0] * 3, [0] * 3, members=[])
    np.testing.assert_array_equal(v[0], 0)


@pytest.mark.parametrize("cls,lo,hi", [(az.compute.CartesianVelocityFieldCompute, (-10, -10, -10), (10, 10, 10)),
                                       (az.compute.CylindricalVelocityFieldCompute, (0, 0, -10),
                                        (10, 2 * np.pi, 10))])
def test_front_end_shapes(cls, lo, hi):
    import itertools

    field = cls(num_bins=[2, 0, 1], lower_bounds=lo, upper_bounds=hi)
    assert field.num_bins == (2, 0, 1) and field.filter is None and field.include_mpcd_particles is False
    with pytest.raises(az.compute.DataAccessError):
        field.velocities
    ref = []
    for a, b, n in zip(lo, hi, [2, 3, 4]):
        x, dx = np.linspace(a, b, n, endpoint=False, retstep=True)
        ref.append((x + 0.5 * dx).tolist())

    def shaped(*c):
        return np.reshape(np.array(list(itertools.product(*c))), [len(x) for x in c] + [len(c)])

    field.num_bins = [2, 3, 4]
    np.testing.assert_allclose(field.coordinates, shaped(*ref))
    field.num_bins = [2, 0, 4]
    np.testing.assert_allclose(field.coordinates, shaped(ref[0], ref[2]))
    field.num_bins = [0, 3, 0]
    np.testing.assert_allclose(field.coordinates, ref[1])
    field.num_bins = [0, 0, 0]
    assert field.coordinates is None


def test_compute_attach_rules():
    s = az.Snapshot(2)
    s.configuration.box = L20 + [0, 0, 0]
    sim = az.Simulation()
    sim.create_state_from_snapshot(s)
    vel = az.compute.VelocityCompute()
    with pytest.raises(az.compute.DataAccessError):
        vel.velocity
    sim.operations.add(vel)
    assert len(sim.operations.computes) == 1
    sim.operations.remove(vel)
    assert len(sim.operations.computes) == 0
    with pytest.raises(az.compute.DataAccessError):
        vel.velocity
    with pytest.raises(TypeError):
        az.compute.VelocityCompute(filter="all")
    assert list(az.filter.Type("B").members(_typed())) == [1]
    assert list(az.filter.All().members(_typed())) == [0, 1]


def _typed():
    s = az.Snapshot(2)
    s.particles.types = ["A", "B"]
    s.particles.typeid = np.array([0, 1], dtype=np.int32)
    return s
