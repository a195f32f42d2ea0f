"""ctypes front end of the CPU oracle (``azp_oracle.cpp``).

TEST INFRASTRUCTURE ONLY. The tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use it to check and time the GPU results; the product package
``azplugins_gb300`` never imports it.

The oracle restates, in FP64, the azplugins short-range force-and-integrate
path (evaluators from ``src/PairEvaluator*.h`` / ``src/BondEvaluator*.h``,
flow fields ``src/ConstantFlow.h`` / ``src/ParabolicFlow.h``, the legacy flow
integrators ``src/TwoStepLangevinFlow.h:128-245`` and
``src/TwoStepBrownianFlow.h:136-178``) plus HOOMD's pair / bond / neighbour
list loops, which are not in the azplugins tree. Every function of the C file
cites the reference line it follows.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libazp_oracle.so")

PAIR_KINDS = {
    "PerturbedLennardJones": 0,
    "ExpandedYukawa": 1,
    "Hertz": 2,
    "Colloid": 3,
    "DPDGeneralWeight": 4,
}
BOND_KINDS = {"Quartic": 0, "DoubleWell": 1, "ImageHarmonic": 2}

# dict keys in the order the C parameter builders read them
PAIR_KEYS = {
    "PerturbedLennardJones": ("epsilon", "sigma", "attraction_scale_factor"),
    "ExpandedYukawa": ("epsilon", "kappa", "delta"),
    "Hertz": ("epsilon",),
    "Colloid": ("A", "a_1", "a_2", "sigma"),
    "DPDGeneralWeight": ("A", "gamma", "s"),
}
BOND_KEYS = {
    "Quartic": ("k", "r_0", "b_1", "b_2", "U_0", "sigma", "epsilon", "delta"),
    "DoubleWell": ("r_0", "r_1", "U_1", "U_tilt"),
    "ImageHarmonic": ("k", "r0"),
}
PAIR_STRIDE = 4
BOND_STRIDE = 8
MODES = {"none": 0, "shift": 1, "xplor": 2}

_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def build():
    """Compile the oracle library with its recipe (g++, a second or two)."""
    subprocess.run(["bash", os.path.join(_HERE, "build_oracle.sh")], check=True)


def lib():
    """Load (building on first use) the oracle shared library."""
    global _lib
    if _lib is not None:
        return _lib
    src = os.path.join(_HERE, "azp_oracle.cpp")
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        build()
    L = ctypes.CDLL(_LIB_PATH)
    c_int, c_long, c_double, c_u32, c_u64 = (
        ctypes.c_int,
        ctypes.c_long,
        ctypes.c_double,
        ctypes.c_uint32,
        ctypes.c_uint64,
    )
    vp = ctypes.c_void_p
    L.orc_version.restype = c_int
    L.orc_set_threads.argtypes = [c_int]
    L.orc_set_threads.restype = c_int
    L.orc_pair_params.argtypes = [c_int, _dp, _dp]
    L.orc_bond_params.argtypes = [c_int, _dp, _dp]
    L.orc_pair_eval.argtypes = [c_int, _dp, c_double, c_double, c_int, ctypes.POINTER(c_double), ctypes.POINTER(c_double)]
    L.orc_bond_eval.argtypes = [c_int, _dp, c_double, ctypes.POINTER(c_double), ctypes.POINTER(c_double)]
    L.orc_flow.argtypes = [c_int, _dp, _dp, _dp]
    L.orc_philox4x32_10.argtypes = [_up, _up, _up]
    L.orc_uniform3.argtypes = [c_int, c_u64, c_u32, c_u32, c_double, c_double, _dp]
    for fn in (L.orc_nlist_brute, L.orc_nlist_cell):
        fn.argtypes = [c_int, _dp, _ip, c_int, _dp, _dp, vp, vp, _ip, _ip, c_long]
        fn.restype = c_long
    L.orc_pair_forces.argtypes = [c_int, _dp, _ip, c_int, _dp, _ip, _ip, c_int, _dp, c_int, _dp, vp, c_int, _dp, _dp, vp, c_double]
    L.orc_dpd_forces.argtypes = [c_int, _dp, _dp, _ip, _up, c_int, _dp, _ip, _ip, _dp, _dp, c_double, c_double, c_u64,
                                 c_u32, _dp, _dp, vp]
    L.orc_bond_forces.argtypes = [c_int, _dp, _dp, c_long, _ip, _ip, c_int, _dp, c_int, _dp, _dp, vp]
    L.orc_bond_forces.restype = c_long
    L.orc_bond_forces_pp.argtypes = [c_int, _dp, _dp, _ip, _ip, _ip, c_int, _dp, c_int, _dp, _dp, vp]
    L.orc_bond_forces_pp.restype = c_long
    L.orc_langevin_step1.argtypes = [c_int, _dp, _ip, _dp, _dp, _dp, c_double]
    L.orc_langevin_step2.argtypes = [c_int, _dp, _ip, _dp, _dp, _dp, _up, vp, _dp, c_int, c_double, c_int, _dp, c_double, c_double, c_u64, c_u32, c_int]
    L.orc_brownian.argtypes = [c_int, _dp, _ip, _ip, _dp, _up, vp, _dp, c_int, c_double, c_int, _dp, _dp, c_double, c_double, c_u64, c_u32, c_int, c_double]
    L.orc_max_disp2.argtypes = [c_int, _dp, _dp, _dp]
    L.orc_max_disp2.restype = c_double
    L.orc_wall_forces.argtypes = [c_int, _dp, _ip, c_int, _dp, _dp, _dp, c_int, _dp, c_int, _dp, c_int, _dp, _dp, _dp,
                                  vp]
    L.orc_wall_params.argtypes = [c_int, _dp, _dp]
    L.orc_wall_params.restype = c_int
    L.orc_velocity_field.argtypes = [c_int, _dp, _dp, _dp, vp, c_int, c_int, _up, _dp, _dp, _dp, _dp, _dp]
    L.orc_image_bond_forces.argtypes = [c_int, _dp, _ip, _dp, c_long, _ip, _ip, c_int, _dp, c_int, _dp, _dp, vp]
    L.orc_image_bond_forces.restype = c_long
    L.orc_image_bond_forces_pp.argtypes = [c_int, _dp, _ip, _dp, _ip, _ip, _ip, c_int, _dp, c_int, _dp, _dp, vp]
    L.orc_image_bond_forces_pp.restype = c_long
    L.orc_barrier_valid.argtypes = [c_int, c_double, _dp]
    L.orc_harmonic_barrier.argtypes = [c_int, _dp, _ip, _dp, c_int, c_double, _dp, _dp, _dp]
    _lib = L
    return L


def set_threads(n: int) -> int:
    """Threads for every parallel phase; returns the count in effect."""
    return lib().orc_set_threads(int(n))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


# ------------------------------------------------------------------ evaluators
def _records(params, width):
    """A parameter table as the oracle's flat array: the last axis padded with
    zeros to ``width`` values per record (4 for pair and wall records, 8 for
    bonds), so tables at the reference's param_type strides and the oracle's
    own padded ones are both accepted."""
    a = np.asarray(params, dtype=np.float64)
    if a.ndim == 0:
        a = a.reshape(1)
    if a.shape[-1] < width:
        pad = np.zeros(a.shape[:-1] + (width - a.shape[-1],))
        a = np.concatenate([a, pad], axis=-1)
    return np.ascontiguousarray(a).reshape(-1)


def pair_params(name: str, d: dict) -> np.ndarray:
    """The reference param_type fields built from a parameter dict (padded to 4)."""
    vals = np.array([float(d[k]) for k in PAIR_KEYS[name]], dtype=np.float64)
    out = np.zeros(PAIR_STRIDE, dtype=np.float64)
    lib().orc_pair_params(PAIR_KINDS[name], np.ascontiguousarray(vals), out)
    return out


def bond_params(name: str, d: dict) -> np.ndarray:
    vals = np.array([float(d[k]) for k in BOND_KEYS[name]], dtype=np.float64)
    out = np.zeros(BOND_STRIDE, dtype=np.float64)
    lib().orc_bond_params(BOND_KINDS[name], np.ascontiguousarray(vals), out)
    return out


def pair_eval(name: str, p: np.ndarray, rsq: float, rcutsq: float, shift: bool):
    f, e = ctypes.c_double(), ctypes.c_double()
    ok = lib().orc_pair_eval(PAIR_KINDS[name], np.ascontiguousarray(p, dtype=np.float64), rsq, rcutsq, int(shift), ctypes.byref(f), ctypes.byref(e))
    return bool(ok), f.value, e.value


def bond_eval(name: str, p: np.ndarray, rsq: float):
    f, e = ctypes.c_double(), ctypes.c_double()
    ok = lib().orc_bond_eval(BOND_KINDS[name], np.ascontiguousarray(p, dtype=np.float64), rsq, ctypes.byref(f), ctypes.byref(e))
    return bool(ok), f.value, e.value


def flow(kind: int, fp, r):
    out = np.zeros(3)
    lib().orc_flow(kind, np.ascontiguousarray(fp, dtype=np.float64), np.ascontiguousarray(r, dtype=np.float64), out)
    return out


def philox(ctr, key):
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(np.ascontiguousarray(ctr, dtype=np.uint32), np.ascontiguousarray(key, dtype=np.uint32), out)
    return out


def uniform3(rng_id: int, timestep: int, seed: int, tag: int, lo: float, hi: float):
    out = np.zeros(3)
    lib().orc_uniform3(rng_id, timestep, seed, tag, lo, hi, out)
    return out


# ------------------------------------------------------------------ neighbour list
def _excl_csr(N, exclusions):
    """exclusions: iterable of (i, j) pairs -> CSR arrays (both directions)."""
    if exclusions is None or len(exclusions) == 0:
        return None, None
    ex = np.asarray(exclusions, dtype=np.int64).reshape(-1, 2)
    a = np.concatenate([ex[:, 0], ex[:, 1]])
    b = np.concatenate([ex[:, 1], ex[:, 0]])
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    start = np.zeros(N + 1, dtype=np.int32)
    np.add.at(start, a + 1, 1)
    start = np.cumsum(start).astype(np.int32)
    return start, np.ascontiguousarray(b, dtype=np.int32)


def nlist(pos4, types, ntypes, L, rlistsq, exclusions=None, method="cell"):
    """Full neighbour list as CSR (start[N+1], idx) with ascending rows."""
    N = pos4.shape[0]
    pos4 = np.ascontiguousarray(pos4, dtype=np.float64)
    types = np.ascontiguousarray(types, dtype=np.int32)
    L = np.ascontiguousarray(L, dtype=np.float64)
    rlistsq = np.ascontiguousarray(rlistsq, dtype=np.float64).reshape(-1)
    es, ei = _excl_csr(N, exclusions)
    fn = lib().orc_nlist_brute if method == "brute" else lib().orc_nlist_cell
    cap = max(64 * N, 1024)
    while True:
        start = np.zeros(N + 1, dtype=np.int32)
        idx = np.zeros(cap, dtype=np.int32)
        n = fn(N, pos4, types, ntypes, L, rlistsq, _ptr(es), _ptr(ei), start, idx, cap)
        if n >= 0:
            return start, idx[:n].copy()
        cap = -n + 16


# ------------------------------------------------------------------ forces
def pair_forces(pos4, types, ntypes, L, start, idx, name, params, rcutsq, ronsq=None, mode="none", fcap=0.0):
    """Pair force, per-particle energy (half per pair) and virial (xx,xy,xz,yy,yz,zz)."""
    N = pos4.shape[0]
    F = np.zeros((N, 3))
    U = np.zeros(N)
    W = np.zeros((N, 6))
    ron = None if ronsq is None else np.ascontiguousarray(ronsq, dtype=np.float64).reshape(-1)
    lib().orc_pair_forces(
        N,
        np.ascontiguousarray(pos4, dtype=np.float64),
        np.ascontiguousarray(types, dtype=np.int32),
        ntypes,
        np.ascontiguousarray(L, dtype=np.float64),
        np.ascontiguousarray(start, dtype=np.int32),
        np.ascontiguousarray(idx, dtype=np.int32),
        PAIR_KINDS[name],
        _records(params, 4),
        PAIR_STRIDE,
        np.ascontiguousarray(rcutsq, dtype=np.float64).reshape(-1),
        _ptr(ron),
        MODES[mode],
        F,
        U,
        _ptr(W),
        float(fcap),
    )
    return F, U, W


def dpd_forces(pos4, vel4, types, tags, ntypes, L, start, idx, params, rcutsq, kT, dt, timestep, seed):
    """DPDGeneralWeight thermostat forces (conservative + dissipative + random),
    per-particle energy (conservative, half per pair) and conservative virial.
    params [ntypes, ntypes, 4] records (A, gamma, s, -)."""
    N = pos4.shape[0]
    F = np.zeros((N, 3))
    U = np.zeros(N)
    W = np.zeros((N, 6))
    lib().orc_dpd_forces(
        N,
        np.ascontiguousarray(pos4, dtype=np.float64),
        np.ascontiguousarray(vel4, dtype=np.float64),
        np.ascontiguousarray(types, dtype=np.int32),
        np.ascontiguousarray(tags, dtype=np.uint32),
        ntypes,
        np.ascontiguousarray(L, dtype=np.float64),
        np.ascontiguousarray(start, dtype=np.int32),
        np.ascontiguousarray(idx, dtype=np.int32),
        _records(params, 4),
        np.ascontiguousarray(rcutsq, dtype=np.float64).reshape(-1),
        float(kT),
        float(dt),
        int(timestep),
        int(seed),
        F,
        U,
        _ptr(W),
    )
    return F, U, W


WALL_KINDS = {"LJ93": 0, "Colloid": 1}
WALL_KEYS = {"LJ93": ("A", "sigma"), "Colloid": ("A", "a", "sigma")}


def wall_params(name, d):
    """param_type record (4 doubles) of a wall potential from its dict."""
    out = np.zeros(4)
    vals = np.array([d[k] for k in WALL_KEYS[name]], dtype=np.float64)
    assert lib().orc_wall_params(WALL_KINDS[name], vals, out) == 0
    return out


def wall_forces(pos4, types, name, params, rcut, rextrap, spheres=(), cylinders=(), planes=()):
    """Wall force [N,3], energy [N], virial [N,6] (HOOMD EvaluatorWalls semantics).
    params [ntypes, 4] records; rcut, rextrap [ntypes]; spheres rows (r, ox, oy, oz,
    inside, open); cylinders (r, ox, oy, oz, ax, ay, az, inside, open) with a unit
    axis; planes (ox, oy, oz, nx, ny, nz, open) with a unit normal."""
    N = pos4.shape[0]
    F = np.zeros((N, 3))
    U = np.zeros(N)
    W = np.zeros((N, 6))
    sp = np.ascontiguousarray(np.asarray(spheres, dtype=np.float64).reshape(-1, 6))
    cy = np.ascontiguousarray(np.asarray(cylinders, dtype=np.float64).reshape(-1, 9))
    pl = np.ascontiguousarray(np.asarray(planes, dtype=np.float64).reshape(-1, 7))
    lib().orc_wall_forces(
        N,
        np.ascontiguousarray(pos4, dtype=np.float64),
        np.ascontiguousarray(types, dtype=np.int32),
        WALL_KINDS[name],
        _records(params, 4),
        np.ascontiguousarray(rcut, dtype=np.float64).reshape(-1),
        np.ascontiguousarray(rextrap, dtype=np.float64).reshape(-1),
        len(sp), sp.reshape(-1) if len(sp) else np.zeros(1),
        len(cy), cy.reshape(-1) if len(cy) else np.zeros(1),
        len(pl), pl.reshape(-1) if len(pl) else np.zeros(1),
        F, U, _ptr(W),
    )
    return F, U, W


def velocity_field(pos4, vel4, L, kind, num_bins, lower, upper, members=None):
    """Per-bin mass, momentum and mass-averaged velocity (src/VelocityFieldCompute.h);
    kind "cartesian" or "cylindrical"; members an index list or None for all.
    Returns arrays shaped [total bins], [total bins, 3], [total bins, 3] in the
    reference's ravel order (z fastest)."""
    nb = [max(int(n), 1) for n in num_bins]
    total = nb[0] * nb[1] * nb[2]
    mass = np.zeros(total)
    mom = np.zeros((total, 3))
    vel = np.zeros((total, 3))
    mem = None if members is None else np.ascontiguousarray(members, dtype=np.int32)
    lib().orc_velocity_field(
        pos4.shape[0],
        np.ascontiguousarray(pos4, dtype=np.float64),
        np.ascontiguousarray(vel4, dtype=np.float64),
        np.ascontiguousarray(L, dtype=np.float64),
        None if mem is None else mem.ctypes.data,
        0 if mem is None else len(mem),
        {"cartesian": 0, "cylindrical": 1}[kind],
        np.ascontiguousarray(num_bins, dtype=np.uint32),
        np.ascontiguousarray(lower, dtype=np.float64),
        np.ascontiguousarray(upper, dtype=np.float64),
        mass,
        mom,
        vel,
    )
    return mass, mom, vel


BARRIER_GEOMETRIES = {"planar": 0, "spherical": 1}


def harmonic_barrier(pos4, types, L, geometry, location, params):
    """Harmonic barrier force [N,3] and energy [N] (src/HarmonicBarrier.h:149-180);
    geometry "planar" or "spherical", params [ntypes, 2] = (k, offset). Raises
    ValueError("Barrier position is invalid") like the reference's makeEvaluator."""
    N = pos4.shape[0]
    F = np.zeros((N, 3))
    U = np.zeros(N)
    st = lib().orc_harmonic_barrier(
        N,
        np.ascontiguousarray(pos4, dtype=np.float64),
        np.ascontiguousarray(types, dtype=np.int32),
        np.ascontiguousarray(L, dtype=np.float64),
        BARRIER_GEOMETRIES[geometry],
        float(location),
        np.ascontiguousarray(params, dtype=np.float64).reshape(-1),
        F,
        U,
    )
    if st:
        raise ValueError("Barrier position is invalid")
    return F, U


def image_bond_forces(pos4, image, L, bonds, btypes, name, params):
    """Image-unwrapped bond forces (src/ImagePotentialBond.h:57-204): F [N,3],
    U [N], W [N,6] from the bond list (B,2) and per-bond types."""
    N = pos4.shape[0]
    F = np.zeros((N, 3))
    U = np.zeros(N)
    W = np.zeros((N, 6))
    bonds = np.ascontiguousarray(bonds, dtype=np.int32).reshape(-1, 2)
    bad = lib().orc_image_bond_forces(
        N, np.ascontiguousarray(pos4, dtype=np.float64), np.ascontiguousarray(image, dtype=np.int32).reshape(-1),
        np.ascontiguousarray(L, dtype=np.float64), len(bonds), bonds.reshape(-1),
        np.ascontiguousarray(btypes, dtype=np.int32), BOND_KINDS[name],
        _records(params, 8), BOND_STRIDE, F, U, _ptr(W))
    if bad:
        raise ValueError(f"bond {bad - 1} refused")
    return F, U, W


def bond_forces(pos4, L, bonds, btypes, name, params, F=None, U=None, W=None):
    """Bond forces (accumulated into F/U/W if given). Raises on a refused bond."""
    N = pos4.shape[0]
    F = np.zeros((N, 3)) if F is None else F
    U = np.zeros(N) if U is None else U
    W = np.zeros((N, 6)) if W is None else W
    bonds = np.ascontiguousarray(bonds, dtype=np.int32).reshape(-1, 2)
    rc = lib().orc_bond_forces(
        N,
        np.ascontiguousarray(pos4, dtype=np.float64),
        np.ascontiguousarray(L, dtype=np.float64),
        bonds.shape[0],
        bonds,
        np.ascontiguousarray(btypes, dtype=np.int32),
        BOND_KINDS[name],
        _records(params, 8),
        BOND_STRIDE,
        F,
        U,
        _ptr(W),
    )
    if rc:
        raise RuntimeError(f"bond.{name}: bond out of bounds (bond {rc - 1})")
    return F, U, W


def bond_table(N, bonds, btypes):
    """Per-particle bond table (each bond on both ends): start[N+1], partner, type."""
    bonds = np.asarray(bonds, dtype=np.int64).reshape(-1, 2)
    bt = np.asarray(btypes, dtype=np.int64)
    a = np.concatenate([bonds[:, 0], bonds[:, 1]])
    b = np.concatenate([bonds[:, 1], bonds[:, 0]])
    t = np.concatenate([bt, bt])
    order = np.argsort(a, kind="stable")
    start = np.zeros(N + 1, dtype=np.int64)
    np.add.at(start, a + 1, 1)
    start = np.cumsum(start)
    return start.astype(np.int32), b[order].astype(np.int32), t[order].astype(np.int32)


def bond_forces_pp(pos4, L, table, name, params, F, U, W=None):
    start, partner, btype = table
    rc = lib().orc_bond_forces_pp(
        pos4.shape[0],
        pos4,
        np.ascontiguousarray(L, dtype=np.float64),
        start,
        partner,
        btype,
        BOND_KINDS[name],
        _records(params, 8),
        BOND_STRIDE,
        F,
        U,
        _ptr(W),
    )
    if rc:
        raise RuntimeError(f"bond.{name}: bond out of bounds (particle {rc - 1})")


def image_bond_forces_pp(pos4, image, L, table, name, params, F, U, W=None):
    """Image-unwrapped bond forces from the per-particle table, accumulated into
    F/U/W: the MD loop's form of ``image_bond_forces``."""
    start, partner, btype = table
    rc = lib().orc_image_bond_forces_pp(
        pos4.shape[0],
        pos4,
        np.ascontiguousarray(image, dtype=np.int32).reshape(-1),
        np.ascontiguousarray(L, dtype=np.float64),
        start,
        partner,
        btype,
        BOND_KINDS[name],
        _records(params, 8),
        BOND_STRIDE,
        F,
        U,
        _ptr(W),
    )
    if rc:
        raise RuntimeError(f"bond.{name}: bond refused (particle {rc - 1})")


# ------------------------------------------------------------------ integrators
FLOW_CONSTANT, FLOW_PARABOLIC = 0, 1


def langevin_step1(pos4, image, vel4, accel, L, dt):
    lib().orc_langevin_step1(pos4.shape[0], pos4, image, vel4, accel, np.ascontiguousarray(L, dtype=np.float64), dt)


def langevin_step2(pos4, types, vel4, accel, net_force, tags, gamma, flow_kind, flow_p, kT, dt, timestep, seed,
                   noiseless=False, diameter=None, use_lambda=False, lam=0.0):
    lib().orc_langevin_step2(
        pos4.shape[0], pos4, types, vel4, accel, np.ascontiguousarray(net_force, dtype=np.float64), tags,
        _ptr(diameter), np.ascontiguousarray(gamma, dtype=np.float64), int(use_lambda), lam, flow_kind,
        np.ascontiguousarray(flow_p, dtype=np.float64), kT, dt, timestep, seed, int(noiseless))


def brownian(pos4, image, types, net_force, tags, gamma, flow_kind, flow_p, L, kT, dt, timestep, seed,
             noiseless=False, diameter=None, use_lambda=False, lam=0.0, max_disp=0.0):
    lib().orc_brownian(
        pos4.shape[0], pos4, image, types, np.ascontiguousarray(net_force, dtype=np.float64), tags, _ptr(diameter),
        np.ascontiguousarray(gamma, dtype=np.float64), int(use_lambda), lam, flow_kind,
        np.ascontiguousarray(flow_p, dtype=np.float64), np.ascontiguousarray(L, dtype=np.float64), kT, dt, timestep,
        seed, int(noiseless), float(max_disp))


def max_disp2(pos4, pos_build, L):
    return lib().orc_max_disp2(pos4.shape[0], pos4, pos_build, np.ascontiguousarray(L, dtype=np.float64))


class OracleMD:
    """HOOMD-order MD loop on the oracle: step one, list check, forces, step two.

    ``system`` is a dict of numpy arrays in tag order (see tests/systems.py):
    pos4 (N,4: x,y,z,type), vel4 (N,4: v, mass), accel (N,3), image (N,3),
    types (N,), tags (N,), L (3,), bonds (B,2), btypes (B,).
    """

    def __init__(self, system, pair=None, bond=None, method="langevin", gamma=(1.0,), flow_kind=0,
                 flow_p=(0.0, 0.0, 0.0), kT=1.0, dt=0.005, seed=0, r_buff=0.4, noiseless=False, exclude_bonds=True,
                 max_disp=0.0, force_cap=0.0, barrier=None, walls=None, group_types=None):
        self.s = {k: (np.ascontiguousarray(v).copy() if isinstance(v, np.ndarray) else v) for k, v in system.items()}
        s = self.s
        self.N = s["pos4"].shape[0]
        self.pair = pair  # dict(name, params[ntypes,ntypes,4], rcut[ntypes,ntypes], ron, mode)
        self.bond = bond  # dict(name, params[nbt,8])
        self.method = method
        self.gamma = np.asarray(gamma, dtype=np.float64)
        self.flow_kind = flow_kind
        self.flow_p = np.asarray(flow_p, dtype=np.float64)
        # kT: a float or a function of the timestep (the reference evaluates its
        # Variant at the timestep of step two, src/TwoStepLangevinFlow.h:194-219)
        self.kT, self.dt, self.seed = kT, dt, seed
        # the method's group as the integrated type ids (None: every particle);
        # the reference's kernels visit the group's members only
        # (src/TwoStepLangevinFlowGPU.cuh:25-55), so the others keep their state
        self.group_types = None if group_types is None else np.asarray(group_types, dtype=np.int32)
        self.r_buff = r_buff
        self.noiseless = noiseless
        self.max_disp = max_disp
        self.force_cap = force_cap
        # dict(geometry, location: float or callable(timestep), params [ntypes, 2])
        self.barrier = barrier
        # dict(name, params [ntypes, 4], rcut [ntypes], rextrap [ntypes], spheres, cylinders, planes)
        self.walls = walls
        self.timestep = int(s.get("timestep", 0))
        self.ntypes = int(s.get("ntypes", int(s["types"].max()) + 1))
        self.exclusions = s["bonds"] if (exclude_bonds and s.get("bonds") is not None and len(s["bonds"])) else None
        self.table = None
        if bond is not None and s.get("bonds") is not None and len(s["bonds"]):
            self.table = bond_table(self.N, s["bonds"], s["btypes"])
        self.pos_build = None
        self.nlist_csr = None
        self.builds = 0

    def _rlistsq(self):
        rc = np.asarray(self.pair["rcut"], dtype=np.float64)
        rl = np.where(rc > 0, rc + self.r_buff, 0.0)
        return rl * rl

    def _check_build(self):
        s = self.s
        if self.pos_build is not None:
            if max_disp2(s["pos4"], self.pos_build, s["L"]) <= (0.5 * self.r_buff) ** 2:
                return
        self.nlist_csr = nlist(s["pos4"], s["types"], self.ntypes, s["L"], self._rlistsq(), self.exclusions)
        self.pos_build = s["pos4"].copy()
        self.builds += 1

    def forces(self, timestep=None):
        """Net force, energy and virial at the current positions; ``timestep`` is the
        one the positions belong to (the barrier location's argument)."""
        s = self.s
        N = self.N
        F = np.zeros((N, 3))
        U = np.zeros(N)
        W = np.zeros((N, 6))
        if self.pair is not None and self.pair["name"] == "DPDGeneralWeight":
            # velocity-dependent: the current (half-step) velocities, the draw of
            # the timestep the positions belong to
            self._check_build()
            rc = np.asarray(self.pair["rcut"], dtype=np.float64)
            t = self.timestep if timestep is None else timestep
            F, U, W = dpd_forces(s["pos4"], s["vel4"], s["types"], s["tags"], self.ntypes, s["L"], *self.nlist_csr,
                                 self.pair["params"], rc * rc, self.pair["kT"], self.dt, t, self.seed)
        elif self.pair is not None:
            self._check_build()
            rc = np.asarray(self.pair["rcut"], dtype=np.float64)
            ron = self.pair.get("ron")
            ronsq = None if ron is None else np.asarray(ron, dtype=np.float64) ** 2
            F, U, W = pair_forces(s["pos4"], s["types"], self.ntypes, s["L"], *self.nlist_csr, self.pair["name"],
                                  self.pair["params"], rc * rc, ronsq, self.pair.get("mode", "none"), self.force_cap)
        if self.bond is not None and self.table is not None:
            if self.bond["name"] == "ImageHarmonic":
                # the bond measured between the unwrapped positions (x + img L)
                image_bond_forces_pp(s["pos4"], s["image"], s["L"], self.table, self.bond["name"],
                                     self.bond["params"], F, U, W)
            else:
                bond_forces_pp(s["pos4"], s["L"], self.table, self.bond["name"], self.bond["params"], F, U, W)
        if self.walls is not None:
            w = self.walls
            Fw, Uw, Ww = wall_forces(s["pos4"], s["types"], w["name"], w["params"], w["rcut"], w["rextrap"],
                                     w.get("spheres", ()), w.get("cylinders", ()), w.get("planes", ()))
            F = F + Fw
            U = U + Uw
            W = W + Ww
        if self.barrier is not None:
            loc = self.barrier["location"]
            t = self.timestep if timestep is None else timestep
            Fb, Ub = harmonic_barrier(s["pos4"], s["types"], s["L"], self.barrier["geometry"],
                                      loc(t) if callable(loc) else loc, self.barrier["params"])
            F = F + Fb
            U = U + Ub
        return F, U, W

    def _kT_at(self, t):
        return float(self.kT(t)) if callable(self.kT) else self.kT

    def step(self):
        s = self.s
        t = self.timestep
        keep = None
        if self.group_types is not None:
            out = ~np.isin(s["types"], self.group_types)
            keep = (out, s["pos4"][out].copy(), s["image"][out].copy(), s["vel4"][out].copy(), s["accel"][out].copy())
        if self.method == "langevin":
            langevin_step1(s["pos4"], s["image"], s["vel4"], s["accel"], s["L"], self.dt)
            if keep is not None:
                s["pos4"][keep[0]], s["image"][keep[0]], s["vel4"][keep[0]] = keep[1], keep[2], keep[3]
            F, U, W = self.forces(t + 1)
            langevin_step2(s["pos4"], s["types"], s["vel4"], s["accel"], F, s["tags"], self.gamma, self.flow_kind,
                           self.flow_p, self._kT_at(t), self.dt, t, self.seed, self.noiseless)
        else:
            F, U, W = self.forces(t)
            brownian(s["pos4"], s["image"], s["types"], F, s["tags"], self.gamma, self.flow_kind, self.flow_p,
                     s["L"], self._kT_at(t), self.dt, t, self.seed, self.noiseless, max_disp=self.max_disp)
        if keep is not None:
            out = keep[0]
            s["pos4"][out], s["image"][out], s["vel4"][out], s["accel"][out] = keep[1], keep[2], keep[3], keep[4]
        self.timestep = t + 1
        self.last = (F, U, W)

    def run(self, steps):
        for _ in range(int(steps)):
            self.step()
