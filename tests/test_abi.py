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
    assert lib.azp_abi_version() == 2
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
    # particle indices must stay below 2^31 (list entries carry a mark in bit 31)
    st.value = 0
    assert not lib.azp_nlist_create(0x80000000, 1, 8, ctypes.byref(st))
    assert st.value == -1


# sizeof(param_type) of the reference's evaluators, printed by oracle/ref_sizes.cpp
# compiled from the reference headers (double- and single-precision HOOMD builds)
SIZES = REF["record_bytes"]
_CLASSES = {"pair": (0, {"PerturbedLennardJones": 0, "ExpandedYukawa": 1, "Hertz": 2, "Colloid": 3,
                         "DPDGeneralWeight": 4}),
            "bond": (1, {"Quartic": 0, "DoubleWell": 1}),
            "wall": (2, {"LJ93": 0, "Colloid": 1})}


@pytest.mark.parametrize("prec", ["double", "single"])
def test_record_sizes_match_reference_sizeof(lib, prec):
    assert SIZES[prec]["scalar_bytes"] == (8 if prec == "double" else 4)
    for cls, (code, kinds) in _CLASSES.items():
        for name, kind in kinds.items():
            assert lib.azp_record_size(code, kind, prec == "single") == SIZES[prec][cls][name], (cls, name)
    # HOOMD's harmonic bond {k, r_0} (ImageHarmonic) is not in the azplugins tree:
    # two Scalars, aligned(16) / aligned(8)
    assert lib.azp_record_size(1, 2, prec == "single") == (16 if prec == "double" else 8)
    assert lib.azp_record_size(0, 99, 0) == -1 and lib.azp_record_size(7, 0, 0) == -1


def test_header_structs_have_reference_size():
    from azplugins_gb300 import _lib

    L = _lib.load()
    d = ctypes.c_double
    # the header's typedefs as ctypes structures: field count x 8 bytes
    fields = {(0, 0): 4, (0, 1): 4, (0, 2): 1, (0, 3): 4, (0, 4): 4, (1, 0): 8, (1, 1): 4, (1, 2): 2,
              (2, 0): 2, (2, 1): 4}
    for (cls, kind), n in fields.items():
        st = type("R", (ctypes.Structure,), {"_fields_": [(f"f{i}", d) for i in range(n)]})
        assert ctypes.sizeof(st) == L.azp_record_size(cls, kind, 0)


@pytest.mark.parametrize("cls,kind,nvals", [(0, 0, 3), (0, 1, 3), (0, 2, 1), (0, 3, 4), (0, 4, 3),
                                            (1, 0, 8), (1, 1, 4), (1, 2, 2), (2, 0, 2), (2, 1, 3)])
def test_builders_write_one_record(lib, cls, kind, nvals):
    """The dict constructors write exactly one record of the reference size: a
    table of several records can be filled in place."""
    size = lib.azp_record_size(cls, kind, 0) // 8
    buf = np.full(size + 4, 12345.0)
    vals = np.linspace(0.5, 1.5, nvals)
    if cls == 1 and kind == 1:
        vals = np.array([0.8, 1.2, 2.0, 0.5])  # DoubleWell r_0 < r_1
    fn = {0: lib.azp_pair_params_from_values, 1: lib.azp_bond_params_from_values,
          2: lib.azp_wall_params_from_values}[cls]
    assert fn(kind, vals.ctypes.data, buf.ctypes.data) == 0
    assert np.all(buf[size:] == 12345.0)
    assert np.all(np.isfinite(buf[:size]))


@pytest.mark.parametrize("cls,kind", [(0, 0), (0, 1), (0, 2), (0, 3), (0, 4), (1, 0), (1, 1), (1, 2), (2, 0), (2, 1)])
def test_params_from_single(lib, cls, kind):
    """A single-precision HOOMD table (Scalar = float, records padded to their
    alignment) widens to the double layout field by field."""
    sb = lib.azp_record_size(cls, kind, 1)
    db = lib.azp_record_size(cls, kind, 0)
    nf = {(0, 0): 4, (0, 1): 3, (0, 2): 1, (0, 3): 4, (0, 4): 3, (1, 0): 8, (1, 1): 4, (1, 2): 2,
          (2, 0): 2, (2, 1): 3}[(cls, kind)]
    n = 5
    rng = np.random.default_rng(3)
    raw = np.zeros(n * sb, dtype=np.uint8)
    vals = rng.uniform(-3, 3, size=(n, nf)).astype(np.float32)
    for r in range(n):
        raw[r * sb: r * sb + 4 * nf] = vals[r].view(np.uint8)
        raw[r * sb + 4 * nf: (r + 1) * sb] = 0xFF  # alignment padding: ignored
    out = np.full(n * db // 8, np.nan)
    assert lib.azp_params_from_single(cls, kind, raw.ctypes.data, n, out.ctypes.data) == 0
    out = out.reshape(n, db // 8)
    np.testing.assert_array_equal(out[:, :nf], vals.astype(np.float64))
    assert np.all(out[:, nf:] == 0.0)
    assert lib.azp_params_from_single(cls, 99, raw.ctypes.data, n, out.ctypes.data) == -1

