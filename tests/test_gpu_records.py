"""Parameter tables at the reference's param_type strides, handed straight to the
drop-in drivers: a HOOMD caller passes its GPUArray<param_type> through
unchanged. Records are built as ctypes structures mirroring the header typedefs
(azp_params_hertz: 8 bytes, azp_params_double_well: 32, azp_params_wall_lj93: 16;
src/PairEvaluatorHertz.h:41-47, src/BondEvaluatorDoubleWell.h:52-61,
src/WallEvaluatorLJ93.h:50-58), with different values for every type pair or
type, so a wrong stride reads the wrong record. Forces are checked against the
oracle at 1e-12 (FP64). A single-precision HOOMD table widened by
azp_params_from_single gives the forces of the same values in double layout."""

import ctypes

import numpy as np
import pytest

import azplugins_gb300 as az
from azplugins_gb300 import _compute, _lib
from helpers import force_error, pos4_of, random_fluid, rel

pytestmark = pytest.mark.gpu

_d = ctypes.c_double


class HertzRecord(ctypes.Structure):
    _fields_ = [("epsilon", _d)]


class DoubleWellRecord(ctypes.Structure):
    _fields_ = [("r_1", _d), ("r_diff", _d), ("U_1", _d), ("U_tilt", _d)]


class LJ93Record(ctypes.Structure):
    _fields_ = [("sigma_3", _d), ("A", _d)]


def _device(buf):
    import torch

    raw = np.frombuffer(bytes(buf), dtype=np.float64).copy()
    return torch.from_numpy(raw).cuda()


def _pair_call(snap, kind, table_d, rc, r_buff=0.4):
    import torch

    L = _lib.load()
    N, nt = snap.particles.N, len(snap.particles.types)
    pos = _compute.device_positions(snap)
    sysd = _compute.make_system(snap, pos)
    nl = _compute.NeighborList(N, nt, rc, r_buff)
    nl.build(sysd)
    rc_d = torch.from_numpy(np.ascontiguousarray(rc, dtype=np.float64).reshape(-1)).cuda()
    force = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    vir = torch.zeros((6, N), dtype=torch.float64, device="cuda")
    out = _lib.Forces()
    out.force, out.virial, out.virial_pitch, out.precision = force.data_ptr(), vir.data_ptr(), N, _lib.FP64
    _lib.check(L.azp_pair_forces(ctypes.byref(sysd), nl.handle, kind, table_d.data_ptr(), rc_d.data_ptr(), None,
                                 0, ctypes.byref(out), _compute._stream()), "azp_pair_forces")
    torch.cuda.synchronize()
    nl.close()
    return force.cpu().numpy(), vir.cpu().numpy().T


def _oracle_pair(orc, snap, name, rec4, rc, r_buff=0.4):
    nt = len(snap.particles.types)
    pos4 = pos4_of(snap)
    Lb = np.array(snap.configuration.box[:3])
    s, i = orc.nlist(pos4, snap.particles.typeid, nt, Lb, (rc + r_buff) ** 2)
    return orc.pair_forces(pos4, snap.particles.typeid, nt, Lb, s, i, name, rec4, rc * rc)


def test_hertz_two_type_table_in_reference_layout(orc):
    snap = random_fluid(2000, 0.9, seed=5, ntypes=2)
    eps = np.array([[2.0, 0.7], [0.7, 5.0]])
    table = (HertzRecord * 4)(*[HertzRecord(eps[a, b]) for a in range(2) for b in range(2)])
    assert ctypes.sizeof(table) == 4 * _lib.load().azp_record_size(0, 2, 0) == 32
    rc = np.array([[1.5, 1.3], [1.3, 1.1]])
    f, w = _pair_call(snap, 2, _device(table), rc)
    rec4 = np.zeros((2, 2, 4))
    rec4[:, :, 0] = eps
    F, U, W = _oracle_pair(orc, snap, "Hertz", rec4, rc)
    assert force_error(f, F) < 1e-12
    assert rel(f[:, 3].sum(), U.sum()) < 1e-12
    assert np.abs(w - W).max() <= 1e-12 * np.abs(W).max()


def test_double_well_two_bond_types_in_reference_layout(orc):
    import torch

    L = _lib.load()
    rng = np.random.Generator(np.random.PCG64(8))
    n_chain, length = 200, 10
    N = n_chain * length
    Lb = np.array([15.0, 16.0, 14.0])
    pos = np.zeros((N, 3))
    bonds, btypes = [], []
    for c in range(n_chain):
        x = rng.uniform(-Lb / 2, Lb / 2)
        for k in range(length):
            i = c * length + k
            if k:
                d = rng.normal(size=3)
                x = x + d / np.linalg.norm(d) * rng.uniform(0.7, 1.6)
                bonds.append((i - 1, i))
                btypes.append(k % 2)
            pos[i] = x - Lb * np.rint(x / Lb)
    bonds, btypes = np.array(bonds), np.array(btypes)
    # (r_0, r_1, U_1, U_tilt) per bond type; record (r_1, r_1 - r_0, U_1, U_tilt)
    vals = [(0.8, 1.3, 2.0, 0.3), (1.0, 1.5, 4.0, -0.5)]
    table = (DoubleWellRecord * 2)(*[DoubleWellRecord(r1, r1 - r0, u1, ut) for r0, r1, u1, ut in vals])
    assert ctypes.sizeof(table) == 2 * L.azp_record_size(1, 1, 0) == 64
    snap = az.Snapshot(N)
    snap.configuration.box = [*Lb, 0, 0, 0]
    snap.particles.position = pos
    snap.particles.typeid = np.zeros(N, dtype=np.int32)
    n, tab, h = _compute.bond_table(N, bonds, btypes)
    posd = _compute.device_positions(snap)
    sysd = _compute.make_system(snap, posd)
    force = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    vir = torch.zeros((6, N), dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = _lib.Forces()
    out.force, out.virial, out.virial_pitch, out.precision = force.data_ptr(), vir.data_ptr(), N, _lib.FP64
    n_d = torch.from_numpy(n.astype(np.int32)).cuda()
    t_d = torch.from_numpy(tab.view(np.int32).reshape(-1).copy()).cuda()
    p_d = _device(table)
    _lib.check(L.azp_bond_forces(ctypes.byref(sysd), n_d.data_ptr(), t_d.data_ptr(), h, 1, p_d.data_ptr(), 2,
                                 ctypes.byref(out), err.data_ptr(), _compute._stream()), "azp_bond_forces")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    rec8 = np.zeros((2, 8))
    for t, (r0, r1, u1, ut) in enumerate(vals):
        rec8[t, :4] = (r1, r1 - r0, u1, ut)
    pos4 = np.concatenate([pos, np.zeros((N, 1))], axis=1)
    F, U, W = orc.bond_forces(pos4, Lb, bonds, btypes, "DoubleWell", rec8)
    f = force.cpu().numpy()
    assert force_error(f, F) < 1e-12
    assert rel(f[:, 3].sum(), U.sum()) < 1e-12


def test_lj93_wall_records_in_reference_layout(orc):
    import torch

    L = _lib.load()
    snap = random_fluid(3000, 0.7, seed=12, ntypes=2)
    Lb = np.array(snap.configuration.box[:3])
    # (A, sigma) per type; record (sigma^3, A)
    vals = [(1.0, 1.0), (2.5, 1.3)]
    table = (LJ93Record * 2)(*[LJ93Record(s ** 3, a) for a, s in vals])
    assert ctypes.sizeof(table) == 2 * L.azp_record_size(2, 0, 0) == 32
    planes = (_lib.WallPlane * 2)()
    for k, sgn in enumerate((1.0, -1.0)):
        planes[k].origin[1] = -sgn * 0.4 * Lb[1]
        planes[k].normal[1] = sgn
    walls = _lib.Walls()
    walls.n_planes = 2
    walls.planes = ctypes.cast(planes, ctypes.c_void_p)
    rc = np.array([3.0, 2.5])
    rx = np.zeros(2)
    pos = _compute.device_positions(snap)
    sysd = _compute.make_system(snap, pos)
    force = torch.zeros((snap.particles.N, 4), dtype=torch.float64, device="cuda")
    out = _lib.Forces()
    out.force, out.virial, out.virial_pitch, out.precision = force.data_ptr(), None, 0, _lib.FP64
    p_d = _device(table)
    rc_d, rx_d = torch.from_numpy(rc).cuda(), torch.from_numpy(rx).cuda()
    _lib.check(L.azp_wall_forces(ctypes.byref(sysd), 0, ctypes.byref(walls), p_d.data_ptr(), rc_d.data_ptr(),
                                 rx_d.data_ptr(), ctypes.byref(out), _compute._stream()), "azp_wall_forces")
    torch.cuda.synchronize()
    rec4 = np.zeros((2, 4))
    rec4[:, 0] = [s ** 3 for _, s in vals]
    rec4[:, 1] = [a for a, _ in vals]
    prow = np.array([[0.0, -0.4 * Lb[1], 0.0, 0.0, 1.0, 0.0, 0.0], [0.0, 0.4 * Lb[1], 0.0, 0.0, -1.0, 0.0, 0.0]])
    F, U, W = orc.wall_forces(pos4_of(snap), snap.particles.typeid, "LJ93", rec4, rc, rx, planes=prow)
    f = force.cpu().numpy()
    assert np.abs(F).max() > 0
    assert force_error(f[:, :3], F) < 1e-12
    assert rel(f[:, 3].sum(), U.sum()) < 1e-12


def test_single_precision_table_widened(orc):
    """An FP32 HOOMD build's PerturbedLJ table (16-byte records) through
    azp_params_from_single gives the forces of its float values exactly."""
    L = _lib.load()
    snap = random_fluid(1500, 0.8, seed=21, ntypes=2)
    # float32 fields sigma_6, epsilon_x_4, attraction_scale_factor, rwcasq per type pair
    rec = np.zeros((2, 2, 4), dtype=np.float32)
    for a, b, eps, sig, lam in [(0, 0, 1.0, 1.0, 0.5), (0, 1, 0.8, 1.1, 0.3), (1, 0, 0.8, 1.1, 0.3),
                                (1, 1, 1.3, 0.9, 0.0)]:
        rec[a, b] = (sig ** 6, 4 * eps, lam, 2 ** (1 / 3) * sig * sig)
    assert rec.nbytes == 4 * L.azp_record_size(0, 0, 1)
    wide = np.zeros(16)
    assert L.azp_params_from_single(0, 0, rec.ctypes.data, 4, wide.ctypes.data) == 0
    np.testing.assert_array_equal(wide.reshape(2, 2, 4), rec.astype(np.float64))
    import torch

    rc = np.full((2, 2), 2.5)
    f, w = _pair_call(snap, 0, torch.from_numpy(wide).cuda(), rc)
    F, U, W = _oracle_pair(orc, snap, "PerturbedLennardJones", rec.astype(np.float64), rc)
    assert force_error(f, F) < 1e-12
