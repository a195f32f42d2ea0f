"""Host-side API semantics mirrored from hoomd.azplugins (no GPU work):
parameter dictionaries and their round trip (src/pytest/test_pair.py:349,
src/pytest/test_bond.py:218), accepted modes, flow-field properties and pickling
(src/pytest/test_flow.py:12-49), snapshot validation."""

import pickle

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import load_golden

KATS = load_golden("kats.json")


@pytest.mark.parametrize("case", [c for c in KATS["pair"] if c["potential"] != "DPDGeneralWeight"],
                         ids=lambda c: f"{c['potential']}@{c['line']}")
def test_pair_params_round_trip(case):
    cls = getattr(az.pair, case["potential"])
    p = cls(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=case["r_cut"], mode="shift" if case["shift"] else "none")
    p.params[("A", "A")] = case["params"]
    assert p.params[("A", "A")] == case["params"]
    rec, rc, ro = p._tables(["A"])
    back = p.record_to_dict(rec[0, 0])
    for k, v in case["params"].items():
        assert back[k] == pytest.approx(v, rel=1e-14, abs=1e-300)
    assert rc[0, 0] == case["r_cut"]


@pytest.mark.parametrize("case", KATS["bond"], ids=lambda c: f"{c['potential']}@{c['line']}")
def test_bond_params_round_trip(case):
    b = getattr(az.bond, case["potential"])()
    b.params["A-A"] = case["params"]
    assert b.params["A-A"] == dict({"delta": 0.0} if case["potential"] == "Quartic" else {}, **case["params"])
    back = b.record_to_dict(b._table(["A-A"])[0])
    for k, v in case["params"].items():
        assert back[k] == pytest.approx(v, rel=1e-14, abs=1e-300)


def test_pair_keys_are_unordered_and_modes_checked():
    p = az.pair.Colloid(nlist=az.nlist.Cell(), default_r_cut=3.0)
    p.params[("S", "C")] = dict(A=100.0, a_1=0.0, a_2=5.0, sigma=1.0)
    assert p.params[("C", "S")]["a_2"] == 5.0
    p.r_cut[("C", "C")] = 10.0
    assert p.r_cut[("C", "C")] == 10.0 and p.r_cut[("S", "S")] == 3.0
    with pytest.raises(ValueError):
        az.pair.Hertz(nlist=az.nlist.Cell(), mode="bogus")
    with pytest.raises(KeyError):
        p.params[("A", "A")] = dict(A=1.0)  # missing keys
    with pytest.raises(KeyError):
        p.params[("A", "A")] = dict(A=1.0, a_1=0, a_2=0, sigma=1, extra=2)


def test_constant_flow_field():
    U = az.flow.ConstantFlow(velocity=(1, 0, 0))
    np.testing.assert_array_almost_equal(U.velocity, (1, 0, 0))
    assert pickle.loads(pickle.dumps(U)) == U
    U.velocity = (1, 2, 3)
    np.testing.assert_array_almost_equal(U.velocity, (1, 2, 3))
    assert pickle.loads(pickle.dumps(U)) == U
    assert U((5.0, 6.0, 7.0)) == (1.0, 2.0, 3.0)


def test_parabolic_flow_field():
    U = az.flow.ParabolicFlow(mean_velocity=4, separation=10)
    assert U.mean_velocity == 4 and U.separation == 10
    assert pickle.loads(pickle.dumps(U)) == U
    U.mean_velocity = 10
    U.separation = 20
    np.testing.assert_array_almost_equal((U.mean_velocity, U.separation), (10, 20))
    assert pickle.loads(pickle.dumps(U)) == U
    # centreline speed 1.5 U, zero at the plates, gradient along y
    assert U((0.0, 0.0, 3.0))[0] == pytest.approx(15.0)
    assert U((0.0, 10.0, 0.0))[0] == pytest.approx(0.0)


def test_flow_reference_values():
    for v in load_golden("ref_vectors.json")["flow"]:
        if v["kind"] == "constant":
            u = az.flow.ConstantFlow(v["U"])(v["r"])
        else:
            f = az.flow.ParabolicFlow(v["mean_velocity"], v["separation"])
            u = f(v["r"])
            assert f.mean_velocity == pytest.approx(v["get_mean_velocity"])
            assert f.separation == pytest.approx(v["get_separation"])
        np.testing.assert_allclose(u, v["u"], rtol=1e-15, atol=1e-15)


def test_snapshot_validation():
    s = az.Snapshot(2)
    s.configuration.box = [5, 5, 5, 0.1, 0, 0]
    with pytest.raises(ValueError):
        s.validate()
    s.configuration.box = [5, 5, 5, 0, 0, 0]
    s.particles.typeid[:] = [0, 3]
    with pytest.raises(ValueError):
        s.validate()


def test_methods_and_integrator_config():
    m = az.methods.LangevinFlow("all", kT=1.0, flow_field=az.flow.ParabolicFlow(2 / 3, 10.0), default_gamma=2.0)
    m.gamma["B"] = 3.0
    assert m._gamma_table(["A", "B"]) == [2.0, 3.0]
    with pytest.raises(TypeError):
        az.methods.BrownianFlow("all", kT=1.0, flow_field=(0, 0, 0))
    with pytest.raises(ValueError):
        az.nlist.Cell(exclusions=("angle",))
