"""Harmonic barriers on the CPU: the oracle against the reference's known answers
(src/pytest/test_external.py:84-223, extracted into golden/barrier_kats.json),
the validity rule of the barrier location, the Python front end
(src/external.py:16-155) and the C-ABI location check, which returns before any
device work and so runs without a GPU."""

import ctypes

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import load_golden

KATS = load_golden("barrier_kats.json")


def kat_location(case, timestep):
    """CustomVariant of the reference test (src/pytest/test_external.py:11-27)."""
    z = case["variant_z"]
    return z if timestep <= 1 else z - 1.0


def kat_params(case, stage):
    return np.array([[stage["params"][t]["k"], stage["params"][t]["offset"]] for t in case["types"]])


def kat_pos4(case):
    p = np.array(case["position"], dtype=np.float64)
    return np.concatenate([p, np.array(case["typeid"], dtype=np.float64)[:, None]], axis=1)


@pytest.mark.parametrize("geometry", ["planar", "spherical"])
def test_oracle_matches_reference_kats(orc, geometry):
    case = KATS[geometry]
    L = np.array(case["box"][:3], dtype=np.float64)
    assert len(case["stages"]) == 2
    for stage in case["stages"]:
        F, U = orc.harmonic_barrier(kat_pos4(case), case["typeid"], L, geometry,
                                    kat_location(case, stage["timestep"]), kat_params(case, stage))
        for i, e in stage["energies"].items():
            assert U[int(i)] == pytest.approx(e, abs=1e-10), (stage["line"], i)
        for i, f in stage["forces"].items():
            np.testing.assert_allclose(F[int(i)], f, atol=1e-10)


def test_oracle_wraps_before_evaluating(orc):
    # a particle one box length above the barrier is wrapped back below it
    L = np.array([10.0, 10.0, 10.0])
    pos = np.array([[0.0, 3.0, 0.0, 0.0], [0.0, 3.0 + 10.0, 0.0, 0.0], [0.0, 3.0 - 10.0, 0.0, 0.0]])
    F, U = orc.harmonic_barrier(pos, [0, 0, 0], L, "planar", 2.0, np.array([[4.0, 0.0]]))
    np.testing.assert_allclose(F[0], [0.0, -4.0, 0.0])
    np.testing.assert_allclose(F[1:], F[[0, 0]])
    np.testing.assert_allclose(U, [2.0, 2.0, 2.0])


@pytest.mark.parametrize("geometry,loc,ok", [
    ("planar", -5.0, True), ("planar", 4.999, True), ("planar", 5.0, False), ("planar", -5.001, False),
    ("spherical", 0.0, True), ("spherical", 5.0, True), ("spherical", 5.001, False), ("spherical", -0.1, False),
])
def test_location_validity(orc, geometry, loc, ok):
    # src/PlanarBarrierEvaluator.h:50-56, src/SphericalBarrierEvaluator.h:54-61 in a 10^3 box
    L = np.array([10.0, 10.0, 10.0])
    pos = np.zeros((1, 4))
    if ok:
        orc.harmonic_barrier(pos, [0], L, geometry, loc, np.array([[1.0, 0.0]]))
    else:
        with pytest.raises(ValueError, match="Barrier position is invalid"):
            orc.harmonic_barrier(pos, [0], L, geometry, loc, np.array([[1.0, 0.0]]))
    cls = az.external.PlanarHarmonicBarrier if geometry == "planar" else az.external.SphericalHarmonicBarrier
    b = cls(location=loc)
    assert b._valid(loc, L) == ok


@pytest.mark.parametrize("cls", [az.external.PlanarHarmonicBarrier, az.external.SphericalHarmonicBarrier])
def test_front_end(cls):
    # src/pytest/test_external.py:54-81: constant location, params by update()
    barrier = cls(location=3.0)
    barrier.params["A"].update(dict(k=10.0, offset=0.5))
    assert isinstance(barrier.location, az.variant.Constant)
    assert barrier.location(0) == 3.0
    assert barrier.params["A"] == dict(k=10.0, offset=0.5)
    barrier.params["B"] = dict(k=2.0, offset=-1.0)
    np.testing.assert_array_equal(barrier._table(["A", "B"]), [[10.0, 0.5], [2.0, -1.0]])
    with pytest.raises(KeyError):
        barrier.params["C"] = dict(k=1.0, offset=0.0, extra=1.0)
    with pytest.raises(KeyError):
        barrier._table(["A", "B", "C"])
    ramp = az.variant.Ramp(A=50.0, B=25.0, t_start=100, t_ramp=1000)
    barrier.location = ramp
    assert barrier.location(0) == 50.0 and barrier.location(600) == 37.5 and barrier.location(5000) == 25.0
    np.testing.assert_allclose(ramp.values(90, 2000), [ramp(t) for t in range(90, 2090)])


def test_c_abi_rejects_invalid_location():
    """azp_harmonic_barrier_forces checks the location against the box before any
    device work (no GPU needed): AZP_ERR_INVALID and the reference's message."""
    from azplugins_gb300 import _lib

    L = _lib.load()
    s = _lib.System()
    s.N = 4
    s.ntypes = 1
    s.pos = 1  # never dereferenced: the check comes first
    for d in range(3):
        s.box.L[d] = 10.0
    out = _lib.Forces()
    out.force = 1
    out.precision = _lib.FP64
    for geometry, loc in ((0, 5.0), (0, -5.5), (1, 5.5), (1, -1.0)):
        st = L.azp_harmonic_barrier_forces(ctypes.byref(s), geometry, loc, ctypes.c_void_p(1), ctypes.byref(out), None)
        assert st == -1
        assert b"Barrier position is invalid" in L.azp_last_error()
    assert L.azp_harmonic_barrier_forces(ctypes.byref(s), 2, 0.0, ctypes.c_void_p(1), ctypes.byref(out), None) == -1
