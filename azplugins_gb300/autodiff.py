"""Differentiable forces and Langevin rollouts on the hand-written adjoint kernels.

``pair_forces(pos, values, pair, ...)`` is a ``torch.autograd.Function`` whose
forward runs the FP64 pair driver (``azp_pair_forces``) and whose backward runs
the adjoint kernel (``azp_pair_adjoint``): gradients with respect to positions
and to the pair potential's parameter dict values (epsilon, sigma,
attraction_scale_factor for PerturbedLennardJones; epsilon, kappa, delta for
ExpandedYukawa; ...). ``bond_forces`` does the same for bonds (e.g. Quartic k).

``langevin_rollout`` advances K LangevinFlow steps (HOOMD order: step one,
forces, step two; Philox noise from the device stream of the integrator, fixed
by seed / timestep / tag) in FP64 torch arithmetic around those Functions, with
``torch.utils.checkpoint`` every ``checkpoint_every`` steps so that memory stays
O(N K / m) and the backward pass recomputes each segment.

Scope: one type pair carries learnable parameters (systems of one particle type,
as the gradient workload); the neighbour list is a non-differentiable input,
rebuilt when a particle has moved more than r_buff / 2.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _compute, _lib

_POW_2_13 = 2.0 ** (1.0 / 3.0)
RNG_LANGEVIN_FLOW = 202  # src/RNGIdentifiers.h:25


def _torch():
    import torch

    return torch


def _stream():
    return ctypes.c_void_p(_torch().cuda.current_stream().cuda_stream)


# d(param_type record fields) / d(dict values), per evaluator: rows = record fields
def record_jacobian(name, values):
    v = [float(x) for x in values]
    if name == "PerturbedLennardJones":
        eps, sig, lam = v
        return np.array([[0.0, 6.0 * sig ** 5, 0.0], [4.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, 2.0 * _POW_2_13 * sig, 0.0]])
    if name == "ExpandedYukawa":
        return np.vstack([np.eye(3), np.zeros((1, 3))])
    if name == "Hertz":
        return np.array([[1.0], [0.0], [0.0], [0.0]])
    if name == "Colloid":
        A, a1, a2, sig = v
        J = np.eye(4)
        J[3, 3] = 3.0 * sig * sig
        return J
    if name == "Quartic":
        k, r0, b1, b2, U0, sig, eps, dl = v
        J = np.zeros((8, 8))
        for m in (0, 1, 2, 3, 4, 7):
            J[m, m] = 1.0
        J[5, 5] = 6.0 * sig ** 5
        J[6, 6] = 4.0
        return J
    if name == "DoubleWell":
        # record (r_1, r_1 - r_0, U_1, U_tilt) from values (r_0, r_1, U_1, U_tilt)
        return np.array([[0, 1, 0, 0], [-1, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1.0], [0, 0, 0, 0], [0, 0, 0, 0],
                         [0, 0, 0, 0], [0, 0, 0, 0]], dtype=np.float64)
    raise KeyError(name)


def record_jacobian_t(name, values):
    """record_jacobian on the device: the same matrix built with torch from the
    values tensor (no host round trip inside a backward pass)."""
    torch = _torch()
    v = values.detach().to(torch.float64)
    dev = v.device
    if name == "PerturbedLennardJones":
        J = torch.zeros((4, 3), dtype=torch.float64, device=dev)
        J[0, 1] = 6.0 * v[1] ** 5
        J[1, 0] = 4.0
        J[2, 2] = 1.0
        J[3, 1] = 2.0 * _POW_2_13 * v[1]
        return J
    if name == "Colloid":
        J = torch.eye(4, dtype=torch.float64, device=dev)
        J[3, 3] = 3.0 * v[3] * v[3]
        return J
    if name == "Quartic":
        J = torch.zeros((8, 8), dtype=torch.float64, device=dev)
        for m in (0, 1, 2, 3, 4, 7):
            J[m, m] = 1.0
        J[5, 5] = 6.0 * v[5] ** 5
        J[6, 6] = 4.0
        return J
    # constant Jacobians
    return torch.from_numpy(record_jacobian(name, [0.0] * len(v))).to(dev)


class Context:
    """Static inputs of a differentiable force: types, box, list parameters."""

    def __init__(self, pair, types, typeid, box, r_cut, r_buff=0.4, exclusions=None, bond=None, bond_group=None,
                 bond_typeid=None, bond_types=None, r_on=0.0):
        torch = _torch()
        self.pair = pair
        self.types = list(types)
        self.typeid = torch.as_tensor(np.asarray(typeid, dtype=np.int64)).cuda()
        self.box = [float(x) for x in box[:3]]
        self.r_cut = float(r_cut)
        self.r_on = float(r_on)
        self.r_buff = float(r_buff)
        self.N = int(len(typeid))
        self.exclusions = exclusions
        self.nl = None
        self.x_build = None
        self.bond = bond
        if bond is not None:
            n, table, h = _compute.bond_table(self.N, bond_group, bond_typeid)
            self.bond_n = torch.from_numpy(n.view(np.int32)).cuda()
            self.bond_table = torch.from_numpy(table.reshape(-1).view(np.int32)).cuda()
            self.bond_h = h
            self.bond_types = list(bond_types)

    def system(self, pos4):
        s = _lib.System()
        s.N = self.N
        s.ntypes = len(self.types)
        s.pos = pos4.data_ptr()
        for d in range(3):
            s.box.L[d] = self.box[d]
        return s

    def pos4(self, x):
        torch = _torch()
        p = torch.empty((self.N, 4), dtype=torch.float64, device="cuda")
        p[:, :3] = x.detach()
        p.view(torch.int64)[:, 3] = self.typeid
        return p

    def neighbor_list(self, x):
        """The list at x (rebuilt when a particle moved more than r_buff / 2)."""
        torch = _torch()
        if self.nl is not None:
            d = x.detach() - self.x_build
            L = torch.tensor(self.box, dtype=torch.float64, device="cuda")
            d = d - L * torch.round(d / L)
            if float((d * d).sum(dim=1).max()) <= (0.5 * self.r_buff) ** 2:
                return self.nl
        # a replaced list stays alive while an autograd node still refers to it
        nt = len(self.types)
        rc = np.full((nt, nt), self.r_cut)
        self.nl = _compute.NeighborList(self.N, nt, rc, self.r_buff, self.exclusions)
        self.nl.build(self.system(self.pos4(x)))
        self.x_build = x.detach().clone()
        return self.nl


def _pair_tables(ctx, values):
    torch = _torch()
    L = _lib.load()
    rec = np.zeros(_lib.record_doubles(_lib.RECORD_PAIR, ctx.pair.kind))
    vals = np.ascontiguousarray([float(v) for v in values], dtype=np.float64)
    _lib.check(L.azp_pair_params_from_values(ctx.pair.kind, vals.ctypes.data, rec.ctypes.data), "params")
    nt = len(ctx.types)
    params = torch.from_numpy(np.tile(rec, nt * nt)).cuda()
    rc = torch.full((nt * nt,), ctx.r_cut, dtype=torch.float64, device="cuda")
    ro = torch.full((nt * nt,), ctx.r_on, dtype=torch.float64, device="cuda")
    return params, rc, ro


def _make_pair_fn():
    torch = _torch()

    class PairFn(torch.autograd.Function):
        @staticmethod
        def forward(fctx, x, values, ctx):
            L = _lib.load()
            nl = ctx.neighbor_list(x)
            pos4 = ctx.pos4(x)
            sysd = ctx.system(pos4)
            params, rc, ro = _pair_tables(ctx, values)
            force = torch.zeros((ctx.N, 4), dtype=torch.float64, device="cuda")
            out = _lib.Forces()
            out.force, out.virial, out.virial_pitch, out.precision = force.data_ptr(), None, ctx.N, _lib.FP64
            _lib.check(L.azp_pair_forces(ctypes.byref(sysd), nl.handle, ctx.pair.kind, params.data_ptr(), rc.data_ptr(),
                                         ro.data_ptr(), _lib.MODES[ctx.pair.mode], ctypes.byref(out), _stream()),
                       "azp_pair_forces")
            fctx.save_for_backward(pos4, params, rc, ro, values)
            fctx.ctx = ctx
            fctx.nl = nl
            return force[:, :3].clone(), force[:, 3].clone()

        @staticmethod
        def backward(fctx, gF, gU):
            L = _lib.load()
            pos4, params, rc, ro, values = fctx.saved_tensors
            ctx = fctx.ctx
            grad = torch.zeros((ctx.N, 4), dtype=torch.float64, device="cuda")
            if gF is not None:
                grad[:, :3] = gF
            if gU is not None:
                grad[:, 3] = gU
            gpos = torch.empty((ctx.N, 3), dtype=torch.float64, device="cuda")
            grec = torch.empty((ctx.N, 4), dtype=torch.float64, device="cuda")
            sysd = ctx.system(pos4)
            _lib.check(L.azp_pair_adjoint(ctypes.byref(sysd), fctx.nl.handle, ctx.pair.kind, params.data_ptr(),
                                          rc.data_ptr(), ro.data_ptr(), _lib.MODES[ctx.pair.mode], grad.data_ptr(),
                                          gpos.data_ptr(), grec.data_ptr(), _stream()), "azp_pair_adjoint")
            J = record_jacobian_t(ctx.pair._name, values)
            gvals = J.T @ grec.sum(dim=0)
            return gpos, gvals.to(values.dtype), None

    return PairFn


_PairFn = None


def pair_forces(x, values, ctx):
    """(F [N,3], U_i [N]) at positions x for parameter dict values (differentiable)."""
    global _PairFn
    if _PairFn is None:
        _PairFn = _make_pair_fn()
    return _PairFn.apply(x, values, ctx)


def _make_bond_fn():
    torch = _torch()

    class BondFn(torch.autograd.Function):
        @staticmethod
        def forward(fctx, x, values, ctx):
            L = _lib.load()
            pos4 = ctx.pos4(x)
            sysd = ctx.system(pos4)
            rec = np.zeros(_lib.record_doubles(_lib.RECORD_BOND, ctx.bond.kind))
            vals = np.ascontiguousarray([float(v) for v in values], dtype=np.float64)
            _lib.check(L.azp_bond_params_from_values(ctx.bond.kind, vals.ctypes.data, rec.ctypes.data), "params")
            params = torch.from_numpy(np.tile(rec, len(ctx.bond_types))).cuda()
            force = torch.zeros((ctx.N, 4), dtype=torch.float64, device="cuda")
            err = torch.zeros(1, dtype=torch.int32, device="cuda")
            out = _lib.Forces()
            out.force, out.virial, out.virial_pitch, out.precision = force.data_ptr(), None, ctx.N, _lib.FP64
            _lib.check(L.azp_bond_forces(ctypes.byref(sysd), ctx.bond_n.data_ptr(), ctx.bond_table.data_ptr(),
                                         ctx.bond_h, ctx.bond.kind, params.data_ptr(), len(ctx.bond_types),
                                         ctypes.byref(out), err.data_ptr(), _stream()), "azp_bond_forces")
            fctx.save_for_backward(pos4, params, values)
            fctx.ctx = ctx
            return force[:, :3].clone(), force[:, 3].clone()

        @staticmethod
        def backward(fctx, gF, gU):
            L = _lib.load()
            pos4, params, values = fctx.saved_tensors
            ctx = fctx.ctx
            grad = torch.zeros((ctx.N, 4), dtype=torch.float64, device="cuda")
            if gF is not None:
                grad[:, :3] = gF
            if gU is not None:
                grad[:, 3] = gU
            gpos = torch.empty((ctx.N, 3), dtype=torch.float64, device="cuda")
            grec = torch.empty((ctx.N, 8), dtype=torch.float64, device="cuda")
            sysd = ctx.system(pos4)
            _lib.check(L.azp_bond_adjoint(ctypes.byref(sysd), ctx.bond_n.data_ptr(), ctx.bond_table.data_ptr(),
                                          ctx.bond.kind, params.data_ptr(), len(ctx.bond_types), grad.data_ptr(),
                                          gpos.data_ptr(), grec.data_ptr(), None, _stream()), "azp_bond_adjoint")
            J = record_jacobian_t(ctx.bond._name, values)
            gvals = J.T @ grec.sum(dim=0)
            return gpos, gvals.to(values.dtype), None

    return BondFn


_BondFn = None


def bond_forces(x, values, ctx):
    """(F [N,3], U_i [N]) of the context's bond potential (differentiable)."""
    global _BondFn
    if _BondFn is None:
        _BondFn = _make_bond_fn()
    return _BondFn.apply(x, values, ctx)


def langevin_noise(N, timestep, seed, c):
    """The integrator's uniform noise in [-c, c]^3 for tags 0..N-1 (device draws)."""
    torch = _torch()
    L = _lib.load()
    tags = torch.arange(N, dtype=torch.int32, device="cuda")
    out = torch.empty((N, 3), dtype=torch.float64, device="cuda")
    _lib.check(L.azp_uniform3(RNG_LANGEVIN_FLOW, int(timestep), int(seed), tags.data_ptr(), N, -c, c, out.data_ptr(),
                              _stream()), "azp_uniform3")
    return out


def langevin_rollout(x0, v0, values, ctx, steps, dt, kT=1.0, gamma=1.0, seed=0, timestep=0, mass=None,
                     checkpoint_every=10, flow_velocity=(0.0, 0.0, 0.0)):
    """K LangevinFlow steps from (x0, v0); returns (x, v, F, U_i) at the end.

    Differentiable with respect to x0, v0 and the pair parameter values."""
    torch = _torch()
    from torch.utils.checkpoint import checkpoint

    N = x0.shape[0]
    m = torch.ones(N, 1, dtype=torch.float64, device="cuda") if mass is None else mass.view(N, 1)
    u = torch.tensor(flow_velocity, dtype=torch.float64, device="cuda")
    c = float(np.sqrt(6.0 * gamma * kT / dt))
    noise = [langevin_noise(N, timestep + t, seed, c) for t in range(steps)]

    def segment(x, v, a, t0, t1):
        F = U = None
        for t in range(t0, t1):
            x = x + (v + 0.5 * dt * a) * dt
            v = v + 0.5 * dt * a
            F, U = pair_forces(x, values, ctx)
            a = (F + (noise[t] - gamma * (v - u))) / m
            v = v + 0.5 * dt * a
        return x, v, a, F, U

    F, U = pair_forces(x0, values, ctx)
    a = F / m
    x, v = x0, v0
    t = 0
    while t < steps:
        t1 = min(steps, t + checkpoint_every)
        x, v, a, F, U = checkpoint(segment, x, v, a, t, t1, use_reentrant=False)
        t = t1
    return x, v, F, U
