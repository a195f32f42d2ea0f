"""ImageHarmonic bond on the CPU: the oracle against the reference test's cases
(src/pytest/test_bond.py:240-309, golden/kats.json "image_bond": box 5, k = 2,
r0 = 1, energy (d - 1)^2 split in halves, force -2 (d - 1) along the unwrapped
bond), and the parameter builders of the C ABI."""

import numpy as np
import pytest

from helpers import load_golden

CASES = load_golden("kats.json")["image_bond"]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['image_1']}-{c['image_2']}")
def test_oracle_matches_reference(orc, case):
    L = np.array([5.0, 5.0, 5.0])
    p1, p2 = np.array(case["position_1"], float), np.array(case["position_2"], float)
    i1, i2 = np.array(case["image_1"]), np.array(case["image_2"])
    rec = np.zeros(8)
    rec[:2] = [2.0, 1.0]
    pos = np.array([[*p1, 0.0], [*p2, 0.0]])
    F, U, W = orc.image_bond_forces(pos, np.array([i1, i2], dtype=np.int32), L, [[0, 1]], [0], "ImageHarmonic",
                                    rec[None])
    u1, u2 = p1 + i1 * L, p2 + i2 * L
    d = np.linalg.norm(u2 - u1)
    e = (d - 1) ** 2
    np.testing.assert_allclose(U, [0.5 * e, 0.5 * e], rtol=1e-12)
    fv = -2 * (d - 1) * (-(u2 - u1) / d)
    np.testing.assert_allclose(F, [fv, -fv], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(W[0], W[1])


def test_param_builders(orc):
    from azplugins_gb300 import _lib

    L = _lib.load()
    vals = np.array([25.0, 1.2])
    rec = np.zeros(8)
    assert L.azp_bond_params_from_values(2, vals.ctypes.data, rec.ctypes.data) == 0
    np.testing.assert_array_equal(rec, orc.bond_params("ImageHarmonic", dict(k=25.0, r0=1.2)))
    back = np.zeros(2)
    assert L.azp_bond_params_to_values(2, rec.ctypes.data, back.ctypes.data) == 0
    np.testing.assert_array_equal(back, vals)
    assert L.azp_bond_num_values(2) == 2


def test_front_end():
    import azplugins_gb300 as az

    ih = az.bond.ImageHarmonic()
    ih.params["A-A"] = dict(k=25.0, r0=1.0)
    assert ih.kind == 2
    np.testing.assert_array_equal(ih._table(["A-A"])[0, :2], [25.0, 1.0])
    assert ih.record_to_dict(ih._table(["A-A"])[0]) == dict(k=25.0, r0=1.0)
    with pytest.raises(KeyError):
        ih.params["B-B"] = dict(k=1.0)
