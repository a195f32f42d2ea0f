"""Per-force evaluation through the drop-in drivers (``azp_nlist_*``,
``azp_pair_forces``, ``azp_bond_forces``): what HOOMD's PotentialPairGPU /
PotentialBondGPU ``computeForces`` does for one force object. Used for the
``forces`` / ``energies`` / ``virials`` properties of pair and bond objects.
Device buffers are torch CUDA tensors; the kernels are this package's own.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _torch():
    import torch

    return torch


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def device_positions(snap):
    """(N, 4) float64 CUDA tensor: x, y, z and the type in the low bits of w."""
    torch = _torch()
    p = snap.particles
    N = p.N
    pos = torch.zeros((max(N, 1), 4), dtype=torch.float64, device="cuda")
    if N:
        pos[:N, :3] = torch.from_numpy(np.ascontiguousarray(p.position, dtype=np.float64)).cuda()
        pos.view(torch.int64)[:N, 3] = torch.from_numpy(np.asarray(p.typeid, dtype=np.int64)).cuda()
    return pos


def make_system(snap, pos, **extra):
    s = _lib.System()
    s.N = snap.particles.N
    s.ntypes = len(snap.particles.types)
    s.pos = pos.data_ptr()
    for d in range(3):
        s.box.L[d] = snap.configuration.box[d]
    for k, v in extra.items():
        setattr(s, k, v)
    return s


def exclusions_csr(N, group):
    group = np.asarray(group, dtype=np.int64).reshape(-1, 2)
    a = np.concatenate([group[:, 0], group[:, 1]])
    b = np.concatenate([group[:, 1], group[:, 0]])
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    start = np.zeros(N + 1, dtype=np.uint32)
    np.add.at(start, a + 1, 1)
    return np.cumsum(start).astype(np.uint32), b.astype(np.uint32)


class NeighborList:
    """Owner of an ``azp_nlist`` workspace."""

    def __init__(self, N, ntypes, r_cut, r_buff, exclusions=None, max_neighbors=64, tpp=4):
        L = _lib.load()
        self._L = L
        st = ctypes.c_int(0)
        self._nl = L.azp_nlist_create(N, ntypes, max_neighbors, ctypes.byref(st))
        _lib.check(st.value, "azp_nlist_create")
        rc = np.ascontiguousarray(r_cut, dtype=np.float64).reshape(-1)
        _lib.check(L.azp_nlist_set_cutoffs(self._nl, rc.ctypes.data, float(r_buff)), "azp_nlist_set_cutoffs")
        if exclusions is not None:
            start, partners = exclusions
            _lib.check(L.azp_nlist_set_exclusions(self._nl, start.ctypes.data, partners.ctypes.data),
                       "azp_nlist_set_exclusions")
        _lib.check(L.azp_nlist_set_tpp(self._nl, int(tpp)), "azp_nlist_set_tpp")
        self.N = N

    @property
    def handle(self):
        return self._nl

    def build(self, system):
        _lib.check(self._L.azp_nlist_build(self._nl, ctypes.byref(system), _stream()), "azp_nlist_build")

    def to_csr(self):
        """The list as host CSR (start[N+1], idx) with ascending rows."""
        max_nn, nb = ctypes.c_uint32(), ctypes.c_uint32()
        _lib.check(self._L.azp_nlist_view(self._nl, None, None, ctypes.byref(max_nn), ctypes.byref(nb)),
                   "azp_nlist_view")
        N = self.N
        counts = np.zeros(max(N, 1), dtype=np.uint32)
        nbrs = np.zeros((max(max_nn.value, 1), max(N, 1)), dtype=np.uint32)
        _lib.check(self._L.azp_nlist_download(self._nl, counts.ctypes.data, nbrs.ctypes.data, _stream()),
                   "azp_nlist_download")
        start = np.zeros(N + 1, dtype=np.int64)
        start[1:] = np.cumsum(counts[:N])
        idx = np.zeros(start[-1], dtype=np.int64)
        for i in range(N):
            idx[start[i]:start[i + 1]] = np.sort(nbrs[: counts[i], i])
        return start, idx

    def counts(self):
        """Per-particle list lengths (host uint32 [N])."""
        max_nn, nb = ctypes.c_uint32(), ctypes.c_uint32()
        _lib.check(self._L.azp_nlist_view(self._nl, None, None, ctypes.byref(max_nn), ctypes.byref(nb)),
                   "azp_nlist_view")
        counts = np.zeros(max(self.N, 1), dtype=np.uint32)
        nbrs = np.zeros((max(max_nn.value, 1), max(self.N, 1)), dtype=np.uint32)
        _lib.check(self._L.azp_nlist_download(self._nl, counts.ctypes.data, nbrs.ctypes.data, _stream()),
                   "azp_nlist_download")
        return counts[: self.N]

    def close(self):
        if getattr(self, "_nl", None):
            self._L.azp_nlist_destroy(self._nl)
            self._nl = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pair_forces(state, pair, precision="fp64", tpp=4):
    """(force4 [N,4] fx,fy,fz,energy ; virial [N,6]) of one pair potential at the state."""
    torch = _torch()
    _lib.require_gpu()
    L = _lib.load()
    snap = state._arrays()
    p = snap.particles
    N = p.N
    types = list(p.types)
    nt = len(types)
    rec, rc, ro = pair._tables(types)
    excl = None
    if pair.nlist.exclude_bonds and snap.bonds.N:
        excl = exclusions_csr(N, snap.bonds.group)
    pos = device_positions(snap)
    sysd = make_system(snap, pos)
    nl = NeighborList(N, nt, rc, pair.nlist.buffer, excl, tpp=tpp)
    nl.build(sysd)
    prec = _lib.FP32 if precision == "fp32" else _lib.FP64
    dt = torch.float32 if prec == _lib.FP32 else torch.float64
    params_d = torch.from_numpy(rec.reshape(-1).copy()).cuda()
    rc_d = torch.from_numpy(rc.reshape(-1).copy()).cuda()
    ro_d = torch.from_numpy(ro.reshape(-1).copy()).cuda()
    force = torch.zeros((max(N, 1), 4), dtype=dt, device="cuda")
    vir = torch.zeros((6, max(N, 1)), dtype=dt, device="cuda")
    out = _lib.Forces()
    out.force = force.data_ptr()
    out.virial = vir.data_ptr()
    out.virial_pitch = max(N, 1)
    out.precision = prec
    _lib.check(L.azp_pair_forces(ctypes.byref(sysd), nl.handle, pair.kind, params_d.data_ptr(), rc_d.data_ptr(),
                                 ro_d.data_ptr(), _lib.MODES[pair.mode], ctypes.byref(out), _stream()),
               "azp_pair_forces")
    torch.cuda.synchronize()
    f = force[:N].double().cpu().numpy()
    w = vir[:, :N].double().cpu().numpy().T.copy()
    nl.close()
    return f, w


def dpd_forces(state, pair, precision, dt, timestep, seed, tpp=2):
    """(force4 [N,4], virial [N,6]) of a DPDGeneralWeight potential at the state:
    conservative + dissipative + random forces, conservative energy and virial."""
    torch = _torch()
    _lib.require_gpu()
    L = _lib.load()
    snap = state._arrays()
    p = snap.particles
    N = p.N
    types = list(p.types)
    nt = len(types)
    rec, rc, ro = pair._tables(types)
    excl = None
    if pair.nlist.exclude_bonds and snap.bonds.N:
        excl = exclusions_csr(N, snap.bonds.group)
    pos = device_positions(snap)
    vel = torch.zeros((max(N, 1), 4), dtype=torch.float64, device="cuda")
    tags = torch.arange(max(N, 1), dtype=torch.int32, device="cuda")
    if N:
        vel[:N, :3] = torch.from_numpy(np.ascontiguousarray(p.velocity, dtype=np.float64)).cuda()
        vel[:N, 3] = torch.from_numpy(np.ascontiguousarray(p.mass, dtype=np.float64)).cuda()
    sysd = make_system(snap, pos, vel=vel.data_ptr(), tag=tags.data_ptr())
    nl = NeighborList(N, nt, rc, pair.nlist.buffer, excl, tpp=tpp)
    nl.build(sysd)
    prec = _lib.FP32 if precision == "fp32" else _lib.FP64
    dt_ = torch.float32 if prec == _lib.FP32 else torch.float64
    params_d = torch.from_numpy(rec.reshape(-1).copy()).cuda()
    rc_d = torch.from_numpy(rc.reshape(-1).copy()).cuda()
    force = torch.zeros((max(N, 1), 4), dtype=dt_, device="cuda")
    vir = torch.zeros((6, max(N, 1)), dtype=dt_, device="cuda")
    out = _lib.Forces()
    out.force = force.data_ptr()
    out.virial = vir.data_ptr()
    out.virial_pitch = max(N, 1)
    out.precision = prec
    _lib.check(L.azp_dpd_forces(ctypes.byref(sysd), nl.handle, params_d.data_ptr(), rc_d.data_ptr(), float(pair.kT),
                                float(dt), int(timestep), int(seed), ctypes.byref(out), _stream()), "azp_dpd_forces")
    torch.cuda.synchronize()
    f = force[:N].double().cpu().numpy()
    w = vir[:, :N].double().cpu().numpy().T.copy()
    nl.close()
    return f, w


def bond_table(N, group, typeid):
    """Per-particle table: n_bonds[N], table [height][N][2] (partner, type)."""
    group = np.asarray(group, dtype=np.int64).reshape(-1, 2)
    typeid = np.asarray(typeid, dtype=np.int64)
    n = np.zeros(N, dtype=np.uint32)
    for a, b in group:
        n[a] += 1
        n[b] += 1
    h = int(n.max()) if N and len(group) else 0
    table = np.zeros((max(h, 1), N, 2), dtype=np.uint32)
    fill = np.zeros(N, dtype=np.int64)
    for (a, b), t in zip(group, typeid):
        table[fill[a], a] = (b, t)
        fill[a] += 1
        table[fill[b], b] = (a, t)
        fill[b] += 1
    return n, table, max(h, 1)


def bond_forces(state, bond, precision="fp64"):
    torch = _torch()
    _lib.require_gpu()
    L = _lib.load()
    snap = state._arrays()
    N = snap.particles.N
    b = snap.bonds
    prec = _lib.FP32 if precision == "fp32" else _lib.FP64
    dt = torch.float32 if prec == _lib.FP32 else torch.float64
    force = torch.zeros((max(N, 1), 4), dtype=dt, device="cuda")
    vir = torch.zeros((6, max(N, 1)), dtype=dt, device="cuda")
    if b.N:
        n, table, h = bond_table(N, b.group, b.typeid)
        pos = device_positions(snap)
        extra = {}
        if bond.kind == _lib.BOND_KINDS["ImageHarmonic"]:
            img = torch.from_numpy(np.ascontiguousarray(snap.particles.image, dtype=np.int32).reshape(-1)).cuda()
            extra["image"] = img.data_ptr()
        sysd = make_system(snap, pos, **extra)
        n_d = torch.from_numpy(n.view(np.int32)).cuda()
        t_d = torch.from_numpy(table.reshape(-1).view(np.int32)).cuda()
        params_d = torch.from_numpy(bond._table(b.types).reshape(-1)).cuda()
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        out = _lib.Forces()
        out.force = force.data_ptr()
        out.virial = vir.data_ptr()
        out.virial_pitch = max(N, 1)
        out.precision = prec
        _lib.check(L.azp_bond_forces(ctypes.byref(sysd), n_d.data_ptr(), t_d.data_ptr(), h, bond.kind,
                                     params_d.data_ptr(), len(b.types), ctypes.byref(out), err.data_ptr(),
                                     _stream()), "azp_bond_forces")
        torch.cuda.synchronize()
        if int(err.item()) & _lib.EBIT_BOND:
            raise _lib.AzpError(-4, f"bond.{bond._name}")
    f = force[:N].double().cpu().numpy()
    w = vir[:, :N].double().cpu().numpy().T.copy()
    return f, w


def barrier_forces(state, barrier, precision, timestep):
    """(force4 [N,4], virial [N,6]) of a harmonic barrier at the state: the
    barrier's force and energy per particle; the virial is zero, as the
    reference leaves it (src/HarmonicBarrier.h:177-179)."""
    torch = _torch()
    _lib.require_gpu()
    L = _lib.load()
    snap = state._arrays()
    p = snap.particles
    N = p.N
    types = list(p.types)
    location = barrier._location_at(timestep, snap.configuration.box[:3])
    pos = device_positions(snap)
    sysd = make_system(snap, pos)
    prec = _lib.FP32 if precision == "fp32" else _lib.FP64
    dt_ = torch.float32 if prec == _lib.FP32 else torch.float64
    params_d = torch.from_numpy(barrier._table(types).reshape(-1).copy()).cuda()
    force = torch.zeros((max(N, 1), 4), dtype=dt_, device="cuda")
    vir = torch.full((6, max(N, 1)), float("nan"), dtype=dt_, device="cuda")
    out = _lib.Forces()
    out.force = force.data_ptr()
    out.virial = vir.data_ptr()
    out.virial_pitch = max(N, 1)
    out.precision = prec
    _lib.check(L.azp_harmonic_barrier_forces(ctypes.byref(sysd), barrier.geometry, float(location),
                                             params_d.data_ptr(), ctypes.byref(out), _stream()),
               "azp_harmonic_barrier_forces")
    torch.cuda.synchronize()
    f = force[:N].double().cpu().numpy()
    w = vir[:, :N].double().cpu().numpy().T.copy()
    return f, w


def wall_forces(state, pot, precision):
    """(force4 [N,4], virial [N,6]) of a wall potential at the state."""
    torch = _torch()
    _lib.require_gpu()
    L = _lib.load()
    snap = state._arrays()
    p = snap.particles
    N = p.N
    types = list(p.types)
    rec, rc, rx = pot._tables(types)
    walls, keep = pot._walls_struct()
    pos = device_positions(snap)
    sysd = make_system(snap, pos)
    prec = _lib.FP32 if precision == "fp32" else _lib.FP64
    dt_ = torch.float32 if prec == _lib.FP32 else torch.float64
    dev = [torch.from_numpy(np.ascontiguousarray(a).reshape(-1).copy()).cuda() for a in (rec, rc, rx)]
    force = torch.zeros((max(N, 1), 4), dtype=dt_, device="cuda")
    vir = torch.zeros((6, max(N, 1)), dtype=dt_, device="cuda")
    out = _lib.Forces()
    out.force = force.data_ptr()
    out.virial = vir.data_ptr()
    out.virial_pitch = max(N, 1)
    out.precision = prec
    _lib.check(L.azp_wall_forces(ctypes.byref(sysd), pot.kind, ctypes.byref(walls), dev[0].data_ptr(),
                                 dev[1].data_ptr(), dev[2].data_ptr(), ctypes.byref(out), _stream()),
               "azp_wall_forces")
    torch.cuda.synchronize()
    del keep
    f = force[:N].double().cpu().numpy()
    w = vir[:, :N].double().cpu().numpy().T.copy()
    return f, w


def velocity_field(snap, kind, num_bins, lower, upper, members):
    """(mass [nb], momentum [nb, 3], velocity [nb, 3]) through ``azp_vfield_*``;
    members: uint32 index array, or None for every particle."""
    torch = _torch()
    _lib.require_gpu()
    L = _lib.load()
    p = snap.particles
    N = p.N
    nb = np.ascontiguousarray(num_bins, dtype=np.uint32)
    lo = np.ascontiguousarray(lower, dtype=np.float64)
    hi = np.ascontiguousarray(upper, dtype=np.float64)
    st = ctypes.c_int(0)
    vf = L.azp_vfield_create(int(kind), nb.ctypes.data, lo.ctypes.data, hi.ctypes.data, ctypes.byref(st))
    _lib.check(st.value, "azp_vfield_create")
    try:
        total = int(L.azp_vfield_num_bins(vf))
        pos = device_positions(snap)
        vel = torch.zeros((max(N, 1), 4), dtype=torch.float64, device="cuda")
        if N:
            vel[:N, :3] = torch.from_numpy(np.ascontiguousarray(p.velocity, dtype=np.float64)).cuda()
            vel[:N, 3] = torch.from_numpy(np.ascontiguousarray(p.mass, dtype=np.float64)).cuda()
        sysd = make_system(snap, pos, vel=vel.data_ptr())
        group = None
        n_group = 0
        if members is not None:
            group = torch.from_numpy(np.ascontiguousarray(members, dtype=np.int32).reshape(-1)).cuda()
            n_group = int(group.numel())
            group = torch.cat([group, torch.zeros(1, dtype=torch.int32, device="cuda")])  # never empty
        out = torch.zeros((total, 7), dtype=torch.float64, device="cuda")
        mass, mom, velo = out[:, 0].contiguous(), out[:, 1:4].contiguous(), out[:, 4:7].contiguous()
        _lib.check(L.azp_vfield_compute(vf, ctypes.byref(sysd), None if group is None else group.data_ptr(), n_group,
                                        mass.data_ptr(), mom.data_ptr(), velo.data_ptr(), _stream()),
                   "azp_vfield_compute")
        err = ctypes.c_uint32(0)
        _lib.check(L.azp_vfield_error(vf, ctypes.byref(err), _stream()), "azp_vfield_error")
        if err.value & _lib.EBIT_RANGE:
            raise _lib.AzpError(-11, "azp_vfield_compute (a momentum above the fixed-point range)")
        return mass.cpu().numpy(), mom.cpu().numpy(), velo.cpu().numpy()
    finally:
        L.azp_vfield_destroy(vf)
