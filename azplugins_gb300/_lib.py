"""Loader of the native library ``libazplugins_gb300.so`` (the C ABI in
``include/azplugins_gb300.h``).

There is no fallback: if the library is missing, importing the compute path
raises, and every device call checks its status and raises ``AzpError``.
"""

from __future__ import annotations

import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libazplugins_gb300.so")
HEADER_PATH = os.path.join(_HERE, "..", "include", "azplugins_gb300.h")

STATUS = {
    0: "ok",
    -1: "invalid argument",
    -2: "CUDA runtime error",
    -3: "neighbour list overflow",
    -4: "bond evaluator refused a bond (bond out of bounds)",
    -5: "box too small for r_cut + r_buff (minimum image)",
    -6: "bounded device wait timed out",
    -7: "non-finite position",
    -8: "unsupported combination",
    -9: "cell list overflow",
    -10: "no CUDA device",
    -11: "size above the entry point's fixed limit",
}

# header enums
PAIR_KINDS = {"PerturbedLennardJones": 0, "ExpandedYukawa": 1, "Hertz": 2, "Colloid": 3, "DPDGeneralWeight": 4}
BOND_KINDS = {"Quartic": 0, "DoubleWell": 1, "ImageHarmonic": 2}
MODES = {"none": 0, "shift": 1, "xplor": 2}
FP64, FP32 = 0, 1
FLOW_CONSTANT, FLOW_PARABOLIC = 0, 1
METHOD_LANGEVIN, METHOD_BROWNIAN = 0, 1
BARRIER_GEOMETRIES = {"planar": 0, "spherical": 1}
WALL_KINDS = {"LJ93": 0, "Colloid": 1}
# record classes of azp_record_size / azp_params_from_single
RECORD_PAIR, RECORD_BOND, RECORD_WALL = 0, 1, 2


def record_doubles(record_class: int, kind: int) -> int:
    """Doubles per param_type record of (class, kind) in the layout every table
    argument of the C ABI takes: the reference's sizeof in a double-precision
    HOOMD build, divided by 8."""
    n = load().azp_record_size(record_class, kind, 0)
    if n <= 0:
        raise ValueError(f"unknown record class {record_class} / kind {kind}")
    return n // 8
EBIT_NLIST_OVERFLOW, EBIT_BOND, EBIT_NONFINITE, EBIT_TIMEOUT = 0x1, 0x2, 0x4, 0x8
EBIT_RANGE = 0x20
BINNING_KINDS = {"cartesian": 0, "cylindrical": 1}


class AzpError(RuntimeError):
    """A non-zero status from the native library."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = STATUS.get(status, f"status {status}")
        detail = ""
        if status in (-2, -11) and _lib is not None:
            detail = _lib.azp_last_error().decode(errors="replace")
        super().__init__(f"{what}: {msg}" + (f" ({detail})" if detail else ""))


class Box(ctypes.Structure):
    _fields_ = [("L", ctypes.c_double * 3)]


class Flow(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("pad_", ctypes.c_int32), ("p", ctypes.c_double * 3)]


class System(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_uint32),
        ("ntypes", ctypes.c_uint32),
        ("pos", ctypes.c_void_p),
        ("vel", ctypes.c_void_p),
        ("accel", ctypes.c_void_p),
        ("image", ctypes.c_void_p),
        ("tag", ctypes.c_void_p),
        ("diameter", ctypes.c_void_p),
        ("box", Box),
    ]


class Forces(ctypes.Structure):
    _fields_ = [
        ("force", ctypes.c_void_p),
        ("virial", ctypes.c_void_p),
        ("virial_pitch", ctypes.c_uint32),
        ("precision", ctypes.c_int32),
    ]


class WallSphere(ctypes.Structure):
    _fields_ = [("r", ctypes.c_double), ("origin", ctypes.c_double * 3), ("inside", ctypes.c_int32),
                ("open", ctypes.c_int32)]


class WallCylinder(ctypes.Structure):
    _fields_ = [("r", ctypes.c_double), ("origin", ctypes.c_double * 3), ("axis", ctypes.c_double * 3),
                ("inside", ctypes.c_int32), ("open", ctypes.c_int32)]


class WallPlane(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("normal", ctypes.c_double * 3), ("open", ctypes.c_int32),
                ("pad_", ctypes.c_int32)]


class Walls(ctypes.Structure):
    _fields_ = [("n_spheres", ctypes.c_uint32), ("n_cylinders", ctypes.c_uint32), ("n_planes", ctypes.c_uint32),
                ("pad_", ctypes.c_uint32), ("spheres", ctypes.c_void_p), ("cylinders", ctypes.c_void_p),
                ("planes", ctypes.c_void_p)]


class MDConfig(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_uint32),
        ("ntypes", ctypes.c_uint32),
        ("box", Box),
        ("precision", ctypes.c_int32),
        ("pair_kind", ctypes.c_int32),
        ("shift_mode", ctypes.c_int32),
        ("pair_params", ctypes.c_void_p),
        ("r_cut", ctypes.c_void_p),
        ("r_on", ctypes.c_void_p),
        ("r_buff", ctypes.c_double),
        ("bond_kind", ctypes.c_int32),
        ("nbondtypes", ctypes.c_uint32),
        ("bond_params", ctypes.c_void_p),
        ("nbonds", ctypes.c_uint32),
        ("bonds", ctypes.c_void_p),
        ("bond_types", ctypes.c_void_p),
        ("exclude_bonds", ctypes.c_int32),
        ("method", ctypes.c_int32),
        ("dt", ctypes.c_double),
        ("kT", ctypes.c_double),
        ("seed", ctypes.c_uint32),
        ("noiseless", ctypes.c_int32),
        ("gamma", ctypes.c_void_p),
        ("use_lambda", ctypes.c_int32),
        ("lambda_", ctypes.c_double),
        ("flow", Flow),
        ("max_displacement", ctypes.c_double),
        ("pair_force_cap", ctypes.c_double),
        ("barrier_geometry", ctypes.c_int32),
        ("barrier_params", ctypes.c_void_p),
        ("wall_kind", ctypes.c_int32),
        ("walls", ctypes.c_void_p),
        ("wall_params", ctypes.c_void_p),
        ("wall_r_cut", ctypes.c_void_p),
        ("wall_r_extrap", ctypes.c_void_p),
        ("dpd_kT", ctypes.c_double),
        ("group_types", ctypes.c_uint32),
    ]


class BatchConfig(ctypes.Structure):
    _fields_ = [
        ("nsys", ctypes.c_uint32),
        ("N", ctypes.c_void_p),
        ("L", ctypes.c_void_p),
        ("precision", ctypes.c_int32),
        ("pair_kind", ctypes.c_int32),
        ("shift_mode", ctypes.c_int32),
        ("pair_params", ctypes.c_void_p),
        ("r_cut", ctypes.c_void_p),
        ("r_buff", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("kT", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("seeds", ctypes.c_void_p),
        ("noiseless", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("flow", Flow),
    ]


_lib = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_u32 = ctypes.c_uint32
_u64 = ctypes.c_uint64
_d = ctypes.c_double

# (name, restype, argtypes)
_SIGNATURES = [
    ("azp_abi_version", _i, []),
    ("azp_device_count", _i, []),
    ("azp_last_error", ctypes.c_char_p, []),
    ("azp_pair_params_from_values", _i, [_i, _vp, _vp]),
    ("azp_pair_params_to_values", _i, [_i, _vp, _vp]),
    ("azp_bond_params_from_values", _i, [_i, _vp, _vp]),
    ("azp_bond_params_to_values", _i, [_i, _vp, _vp]),
    ("azp_pair_num_values", _i, [_i]),
    ("azp_bond_num_values", _i, [_i]),
    ("azp_record_size", _i, [_i, _i, _i]),
    ("azp_params_from_single", _i, [_i, _i, _vp, _u32, _vp]),
    ("azp_nlist_create", _vp, [_u32, _u32, _u32, ctypes.POINTER(_i)]),
    ("azp_nlist_destroy", None, [_vp]),
    ("azp_nlist_set_cutoffs", _i, [_vp, _vp, _d]),
    ("azp_nlist_set_exclusions", _i, [_vp, _vp, _vp]),
    ("azp_nlist_build", _i, [_vp, ctypes.POINTER(System), _vp]),
    ("azp_nlist_view", _i, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_u32), ctypes.POINTER(_u32)]),
    ("azp_nlist_set_tpp", _i, [_vp, _i]),
    ("azp_nlist_download", _i, [_vp, _vp, _vp, _vp]),
    ("azp_pair_forces", _i, [ctypes.POINTER(System), _vp, _i, _vp, _vp, _vp, _i, ctypes.POINTER(Forces), _vp]),
    ("azp_pair_forces_static", _i, [ctypes.POINTER(System), _vp, _vp, _u32, _i, _vp, _vp, _vp, _i,
                                    ctypes.POINTER(Forces), _vp]),
    ("azp_dpd_forces", _i, [ctypes.POINTER(System), _vp, _vp, _vp, _d, _d, _u64, _u32, ctypes.POINTER(Forces), _vp]),
    ("azp_harmonic_barrier_forces", _i, [ctypes.POINTER(System), _i, _d, _vp, ctypes.POINTER(Forces), _vp]),
    ("azp_wall_params_from_values", _i, [_i, _vp, _vp]),
    ("azp_wall_params_to_values", _i, [_i, _vp, _vp]),
    ("azp_wall_forces", _i, [ctypes.POINTER(System), _i, ctypes.POINTER(Walls), _vp, _vp, _vp, ctypes.POINTER(Forces),
                             _vp]),
    ("azp_vfield_create", _vp, [_i, _vp, _vp, _vp, ctypes.POINTER(_i)]),
    ("azp_vfield_destroy", None, [_vp]),
    ("azp_vfield_num_bins", _u32, [_vp]),
    ("azp_vfield_compute", _i, [_vp, ctypes.POINTER(System), _vp, _u32, _vp, _vp, _vp, _vp]),
    ("azp_vfield_error", _i, [_vp, ctypes.POINTER(_u32), _vp]),
    ("azp_bond_forces", _i, [ctypes.POINTER(System), _vp, _vp, _u32, _i, _vp, _u32, ctypes.POINTER(Forces), _vp, _vp]),
    ("azp_pair_adjoint", _i, [ctypes.POINTER(System), _vp, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp]),
    ("azp_bond_adjoint", _i, [ctypes.POINTER(System), _vp, _vp, _i, _vp, _u32, _vp, _vp, _vp, _vp, _vp]),
    ("azp_langevin_step1", _i, [ctypes.POINTER(System), _vp, _u32, _d, _vp]),
    ("azp_langevin_step2", _i, [ctypes.POINTER(System), _vp, _u32, _vp, _i, _vp, _i, _d, Flow, _d, _d, _u64, _u32, _i, _vp]),
    ("azp_brownian_step", _i, [ctypes.POINTER(System), _vp, _u32, _vp, _i, _vp, _i, _d, Flow, _d, _d, _u64, _u32, _i, _d, _vp]),
    ("azp_uniform3", _i, [_u32, _u64, _u32, _vp, _u32, _d, _d, _vp, _vp]),
    ("azp_md_create", _vp, [ctypes.POINTER(MDConfig), ctypes.POINTER(_i)]),
    ("azp_md_destroy", None, [_vp]),
    ("azp_md_set_state", _i, [_vp, _vp, _vp, _vp, _vp, _vp, _u64, _i, _vp]),
    ("azp_md_get_state", _i, [_vp, _vp, _vp, _vp, _vp, ctypes.POINTER(_u64), _i, _vp]),
    ("azp_md_set_barrier_locations", _i, [_vp, _u64, _u32, _vp, _vp]),
    ("azp_md_set_temperatures", _i, [_vp, _u64, _u32, _vp, _vp]),
    ("azp_md_run", _i, [_vp, _u64, _vp]),
    ("azp_md_run_checked", _i, [_vp, _u64, _vp]),
    ("azp_md_forces", _i, [_vp, _vp, _vp, _i, _vp]),
    ("azp_md_thermo", _i, [_vp, _vp, _vp]),
    ("azp_md_error", _i, [_vp, ctypes.POINTER(_u32), _vp]),
    ("azp_md_last_launches", _u64, [_vp]),
    ("azp_md_time_step_kernel", _i, [_vp, _i, ctypes.POINTER(ctypes.c_float), _vp]),
    ("azp_batch_create", _vp, [ctypes.POINTER(BatchConfig), ctypes.POINTER(_i)]),
    ("azp_batch_destroy", None, [_vp]),
    ("azp_batch_set_state", _i, [_vp, _vp, _vp, _vp, _vp, _u64, _vp]),
    ("azp_batch_get_state", _i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    ("azp_batch_run", _i, [_vp, _u64, _vp]),
    ("azp_batch_error", _i, [_vp, ctypes.POINTER(_u32), ctypes.POINTER(_u32), _vp]),
    ("azp_batch_set_tpp", _i, [_vp, _i]),
    ("azp_batch_set_block", _i, [_vp, _i]),
    ("azp_batch_last_launches", _u64, [_vp]),
]


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    with open(HEADER_PATH) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(azp_[a-z0-9_]+)\s*\(", text)))


def load():
    """Load the native library (no fallback: raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"azplugins_gb300: native library not built ({LIB_PATH}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` or `python azplugins_gb300/build.py`"
        )
    L = ctypes.CDLL(LIB_PATH)
    for name, res, args in _SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int, what: str) -> None:
    if status != 0:
        raise AzpError(status, what)


def require_gpu() -> None:
    """Raise unless a CUDA device is visible to the native library."""
    if load().azp_device_count() < 1:
        raise AzpError(-10, "azplugins_gb300 needs a CUDA GPU (there is no CPU path)")
