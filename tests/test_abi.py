"""The C-ABI library loads and exports every function include/azplugins_gb300.h
declares; host-only entry points (the param_type dict constructors and asDict)
agree with the oracle and the reference's own vectors. No device compute."""

import ctypes

import numpy as np
import pytest

from helpers import load_golden

REF = load_golden("ref_vectors.json")


@pytest.fixture(scope="module")
def lib():
    from azplugins_gb300 import _lib

    return _lib.load()


def test_exports_every_header_symbol(lib):
    from azplugins_gb300 import _lib

    syms = _lib.header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert missing == []
    declared = {name for name, _, _ in _lib._SIGNATURES}
    assert set(syms) == declared


def test_abi_version_and_device_count(lib):
    assert lib.azp_abi_version() == 1
    assert lib.azp_device_count() >= 0


@pytest.mark.parametrize("v", REF["pair"][::2], ids=lambda v: v["name"])
def test_pair_param_builders_match_reference(lib, v):
    from azplugins_gb300 import _lib, pair

    cls = getattr(pair, v["name"])
    vals = np.array([v["params"][k] for k in cls._keys], dtype=np.float64)
    rec = np.zeros(4)
    assert lib.azp_pair_params_from_values(_lib.PAIR_KINDS[v["name"]], vals.ctypes.data, rec.ctypes.data) == 0
    np.testing.assert_allclose(rec[: len(v["raw"])], v["raw"], rtol=1e-15, atol=0)
    back = np.zeros(len(vals))
    assert lib.azp_pair_params_to_values(_lib.PAIR_KINDS[v["name"]], rec.ctypes.data, back.ctypes.data) == 0
    np.testing.assert_allclose(back, [v["asdict"][k] for k in cls._keys], rtol=1e-15, atol=1e-300)


@pytest.mark.parametrize("v", REF["bond"], ids=lambda v: v["name"])
def test_bond_param_builders_match_reference(lib, v):
    from azplugins_gb300 import _lib, bond

    cls = getattr(bond, v["name"])
    vals = np.array([v["params"][k] for k in cls._keys], dtype=np.float64)
    rec = np.zeros(8)
    assert lib.azp_bond_params_from_values(_lib.BOND_KINDS[v["name"]], vals.ctypes.data, rec.ctypes.data) == 0
    np.testing.assert_allclose(rec[: len(v["raw"])], v["raw"], rtol=1e-15, atol=0)
    back = np.zeros(len(vals))
    assert lib.azp_bond_params_to_values(_lib.BOND_KINDS[v["name"]], rec.ctypes.data, back.ctypes.data) == 0
    np.testing.assert_allclose(back, [v["asdict"][k] for k in cls._keys], rtol=1e-15, atol=1e-300)


def test_invalid_arguments_are_rejected(lib):
    assert lib.azp_pair_params_from_values(99, None, None) == -1
    assert lib.azp_pair_num_values(0) == 3 and lib.azp_bond_num_values(0) == 8
    st = ctypes.c_int(0)
    # ntypes == 0 is refused before any device work
    assert not lib.azp_nlist_create(10, 0, 8, ctypes.byref(st))
    assert st.value == -1
