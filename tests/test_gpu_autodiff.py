"""The hand-written adjoint kernels: gradients of a force/energy loss with
respect to positions and to the potential parameters, checked against FP64
central finite differences through the forward driver and against a dense FP64
all-pairs torch reference; and through short Langevin rollouts with
checkpointing. Tolerance 1e-6 relative (the gradient workload's bar)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    import torch

    return torch


def _fluid(N, density, seed):
    from helpers import random_fluid

    return random_fluid(N, density, seed=seed, min_dist=0.9)


def _ctx(snap, pair, r_cut):
    from azplugins_gb300 import autodiff

    return autodiff.Context(pair, snap.particles.types, snap.particles.typeid, snap.configuration.box, r_cut)


def _loss(F, U, Ft, Ut):
    return ((F - Ft) ** 2).sum(dim=1).mean() + (U.sum() - Ut) ** 2


def _dense_plj(x, L, eps, sig, lam, rc, shift):
    """All-pairs FP64 PerturbedLJ (torch), forces by autograd of the energy."""
    torch = _torch()
    x = x.detach().clone().requires_grad_(True)
    N = x.shape[0]
    d = x[:, None, :] - x[None, :, :]
    d = d - L * torch.round(d / L)
    s = (d * d).sum(-1) + torch.eye(N, dtype=x.dtype, device=x.device)  # no self term
    mask = (s < rc * rc) & ~torch.eye(N, dtype=torch.bool, device=x.device)

    def e_of(s):
        r6 = (sig * sig / s) ** 3
        elj = 4 * eps * (r6 * r6 - r6)
        wca = s < 2 ** (1 / 3) * sig * sig
        return torch.where(wca, elj + eps * (1 - lam), lam * elj)

    e = e_of(s)
    if shift:
        e = e - e_of(torch.tensor(rc * rc, dtype=x.dtype, device=x.device))
    e = torch.where(mask, e, torch.zeros_like(e))
    Ui = 0.5 * e.sum(dim=1)
    F = -torch.autograd.grad(Ui.sum(), x, create_graph=True)[0]
    return F, Ui, x


@pytest.mark.parametrize("shift", [False, True])
def test_single_call_matches_dense_fp64_reference(shift):
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff

    snap = _fluid(512, 0.8, seed=41)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="shift" if shift else "none")
    ctx = _ctx(snap, pot, 2.5)
    x = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda", requires_grad=True)
    vals = torch.tensor([1.0, 1.0, 0.5], dtype=torch.float64, device="cuda", requires_grad=True)
    valst = torch.tensor([1.1, 0.98, 0.4], dtype=torch.float64, device="cuda")
    with torch.no_grad():
        Ft, Ut = autodiff.pair_forces(x, valst, ctx)
    F, U = autodiff.pair_forces(x, vals, ctx)
    loss = _loss(F, U, Ft, Ut.sum())
    gx, gv = torch.autograd.grad(loss, (x, vals))
    # dense reference with parameters as tensors
    L = torch.tensor(snap.configuration.box[:3], dtype=torch.float64, device="cuda")
    p = vals.detach().clone().requires_grad_(True)
    Fd, Ud, xd = _dense_plj(x.detach(), L, p[0], p[1], p[2], 2.5, shift)
    assert torch.allclose(Fd, F, rtol=1e-10, atol=1e-9)
    loss_d = _loss(Fd, Ud, Ft, Ut.sum())
    gxd, gvd = torch.autograd.grad(loss_d, (xd, p))
    scale = gxd.abs().max()
    assert float((gx - gxd).abs().max() / scale) < 1e-6
    assert float(((gv - gvd).abs() / gvd.abs().clamp_min(1e-12)).max()) < 1e-6


def test_parameter_gradient_matches_finite_differences():
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff

    snap = _fluid(4096, 0.8, seed=42)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="shift")
    ctx = _ctx(snap, pot, 3.0)
    x = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda")
    valst = torch.tensor([1.1, 0.98, 0.4], dtype=torch.float64, device="cuda")
    with torch.no_grad():
        Ft, Ut = autodiff.pair_forces(x, valst, ctx)
        Ut = Ut.sum()
    vals = torch.tensor([1.0, 1.0, 0.5], dtype=torch.float64, device="cuda", requires_grad=True)
    F, U = autodiff.pair_forces(x, vals, ctx)
    (gv,) = torch.autograd.grad(_loss(F, U, Ft, Ut), (vals,))
    h = 1e-6
    for k in range(3):
        with torch.no_grad():
            vp = vals.detach().clone()
            vm = vals.detach().clone()
            vp[k] += h
            vm[k] -= h
            Fp, Up = autodiff.pair_forces(x, vp, ctx)
            Fm, Um = autodiff.pair_forces(x, vm, ctx)
            fd = (_loss(Fp, Up, Ft, Ut) - _loss(Fm, Um, Ft, Ut)) / (2 * h)
        assert abs(float(gv[k]) - float(fd)) <= 1e-6 * abs(float(fd)), (k, float(gv[k]), float(fd))


def test_position_gradient_matches_finite_differences():
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff

    snap = _fluid(1000, 0.8, seed=43)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="shift")
    ctx = _ctx(snap, pot, 2.5)
    vals = torch.tensor([1.0, 1.0, 0.5], dtype=torch.float64, device="cuda")
    x = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda", requires_grad=True)
    F, U = autodiff.pair_forces(x, vals, ctx)
    w = torch.linspace(-1, 1, 3 * x.shape[0], dtype=torch.float64, device="cuda").view(-1, 3)
    loss = (F * w).sum() + 0.1 * U.sum()
    (gx,) = torch.autograd.grad(loss, (x,))
    h = 1e-6
    rng = np.random.Generator(np.random.PCG64(1))
    for i in rng.integers(0, x.shape[0], size=5):
        for d in range(3):
            with torch.no_grad():
                xp = x.detach().clone()
                xm = x.detach().clone()
                xp[i, d] += h
                xm[i, d] -= h
                Fp, Up = autodiff.pair_forces(xp, vals, ctx)
                Fm, Um = autodiff.pair_forces(xm, vals, ctx)
                fd = (((Fp * w).sum() + 0.1 * Up.sum()) - ((Fm * w).sum() + 0.1 * Um.sum())) / (2 * h)
            assert abs(float(gx[i, d]) - float(fd)) <= 1e-6 * max(abs(float(fd)), 1e-3), (i, d)


@pytest.mark.parametrize("name,vals", [("ExpandedYukawa", [1.0, 1.5, 0.3]), ("Hertz", [2.0])])
def test_dual_number_adjoint_other_potentials(name, vals):
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff

    snap = _fluid(2000, 0.5, seed=44)
    pot = getattr(az.pair, name)(nlist=az.nlist.Cell(buffer=0.4), mode="shift")
    ctx = _ctx(snap, pot, 2.2)
    x = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda")
    v = torch.tensor(vals, dtype=torch.float64, device="cuda", requires_grad=True)
    F, U = autodiff.pair_forces(x, v, ctx)
    loss = (F ** 2).sum() + U.sum()
    (gv,) = torch.autograd.grad(loss, (v,))
    h = 1e-6
    for k in range(len(vals)):
        with torch.no_grad():
            vp, vm = v.detach().clone(), v.detach().clone()
            vp[k] += h
            vm[k] -= h
            Fp, Up = autodiff.pair_forces(x, vp, ctx)
            Fm, Um = autodiff.pair_forces(x, vm, ctx)
            fd = (((Fp ** 2).sum() + Up.sum()) - ((Fm ** 2).sum() + Um.sum())) / (2 * h)
        assert abs(float(gv[k]) - float(fd)) <= 1e-6 * abs(float(fd))


def test_quartic_bond_k_gradient():
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff, workloads

    snap = workloads.bead_spring_melt(50, 10, density=0.3, seed=45)
    qb = az.bond.Quartic()
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4))
    ctx = autodiff.Context(pot, snap.particles.types, snap.particles.typeid, snap.configuration.box, 1.12,
                           bond=qb, bond_group=snap.bonds.group, bond_typeid=snap.bonds.typeid,
                           bond_types=snap.bonds.types)
    x = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor([1434.3, 1.5, -0.7589, 0.0, 67.2234, 1.0, 1.0, 0.0], dtype=torch.float64, device="cuda",
                     requires_grad=True)
    F, U = autodiff.bond_forces(x, v, ctx)
    loss = (F ** 2).sum() + U.sum()
    gx, gv = torch.autograd.grad(loss, (x, v))
    h = 1e-3  # k is O(1e3)
    with torch.no_grad():
        vp, vm = v.detach().clone(), v.detach().clone()
        vp[0] += h
        vm[0] -= h
        Fp, Up = autodiff.bond_forces(x, vp, ctx)
        Fm, Um = autodiff.bond_forces(x, vm, ctx)
        fd = (((Fp ** 2).sum() + Up.sum()) - ((Fm ** 2).sum() + Um.sum())) / (2 * h)
    assert abs(float(gv[0]) - float(fd)) <= 1e-6 * abs(float(fd))


def test_xplor_single_call_gradient():
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff

    snap = _fluid(3000, 0.8, seed=47)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="xplor")
    ctx = autodiff.Context(pot, snap.particles.types, snap.particles.typeid, snap.configuration.box, 3.0, r_on=2.5)
    x = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda", requires_grad=True)
    v = torch.tensor([1.0, 1.0, 0.5], dtype=torch.float64, device="cuda", requires_grad=True)
    F, U = autodiff.pair_forces(x, v, ctx)
    loss = (F ** 2).sum() + U.sum()
    (gv,) = torch.autograd.grad(loss, (v,))
    h = 1e-6
    for k in range(3):
        with torch.no_grad():
            vp, vm = v.detach().clone(), v.detach().clone()
            vp[k] += h
            vm[k] -= h
            Fp, Up = autodiff.pair_forces(x, vp, ctx)
            Fm, Um = autodiff.pair_forces(x, vm, ctx)
            fd = (((Fp ** 2).sum() + Up.sum()) - ((Fm ** 2).sum() + Um.sum())) / (2 * h)
        assert abs(float(gv[k]) - float(fd)) <= 1e-6 * abs(float(fd)), k


def test_rollout_gradient_matches_finite_differences():
    # forces smoothed to zero at r_cut (xplor): the loss is C1 along trajectories,
    # so central differences through the dynamics are meaningful
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff, workloads

    snap = workloads.lj_fluid(n_side=8, density=0.8, seed=46)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="xplor")
    ctx = autodiff.Context(pot, snap.particles.types, snap.particles.typeid, snap.configuration.box, 3.0, r_on=2.5)
    x0 = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda")
    v0 = torch.tensor(snap.particles.velocity, dtype=torch.float64, device="cuda")
    vals = torch.tensor([1.0, 1.0, 0.5], dtype=torch.float64, device="cuda", requires_grad=True)
    K = 20

    def loss_of(v):
        x, vel, F, U = autodiff.langevin_rollout(x0, v0, v, ctx, K, 0.005, seed=9, checkpoint_every=5)
        return (F ** 2).sum(dim=1).mean() + (U.sum() / x.shape[0]) ** 2

    (gv,) = torch.autograd.grad(loss_of(vals), (vals,))
    h = 1e-6
    for k in range(3):
        with torch.no_grad():
            vp, vm = vals.detach().clone(), vals.detach().clone()
            vp[k] += h
            vm[k] -= h
            fd = (loss_of(vp) - loss_of(vm)) / (2 * h)
        assert abs(float(gv[k]) - float(fd)) <= 1e-6 * abs(float(fd)), (k, float(gv[k]), float(fd))


def test_rollout_gradient_matches_dense_autograd():
    # PerturbedLJ with its force jump at r_cut: the exact gradient of the same
    # discrete dynamics, taken by torch autograd through a dense FP64 all-pairs
    # implementation, is the reference (finite differences see the cutoff jumps)
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff, workloads

    # N = 512, K = 100 Langevin steps with checkpoints every 10 (the gradient
    # workload's dense check)
    snap = workloads.lj_fluid(n_side=8, density=0.8, seed=48)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="shift")
    ctx = _ctx(snap, pot, 2.5)
    L = torch.tensor(snap.configuration.box[:3], dtype=torch.float64, device="cuda")
    x0 = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda")
    v0 = torch.tensor(snap.particles.velocity, dtype=torch.float64, device="cuda")
    K, dt, seed = 100, 0.005, 9
    vals = torch.tensor([1.0, 1.0, 0.5], dtype=torch.float64, device="cuda", requires_grad=True)
    x, v, F, U = autodiff.langevin_rollout(x0, v0, vals, ctx, K, dt, seed=seed, checkpoint_every=10)
    loss = (F ** 2).sum(dim=1).mean() + (U.sum() / x.shape[0]) ** 2
    (gv,) = torch.autograd.grad(loss, (vals,))
    # dense
    p = vals.detach().clone().requires_grad_(True)
    c = float(np.sqrt(6.0 * 1.0 * 1.0 / dt))

    def dense_forces(xx):
        d = xx[:, None, :] - xx[None, :, :]
        d = d - L * torch.round(d / L)
        N = xx.shape[0]
        eye = torch.eye(N, dtype=torch.bool, device="cuda")
        s = (d * d).sum(-1) + eye.double()
        mask = (s < 2.5 * 2.5) & ~eye
        eps, sig, lam = p[0], p[1], p[2]

        def e_of(s):
            r6 = (sig * sig / s) ** 3
            elj = 4 * eps * (r6 * r6 - r6)
            return torch.where(s < 2 ** (1 / 3) * sig * sig, elj + eps * (1 - lam), lam * elj)

        r6 = (sig * sig / s) ** 3
        fdr = 24 * eps * (2 * r6 * r6 - r6) / s
        fdr = torch.where(s < 2 ** (1 / 3) * sig * sig, fdr, lam * fdr)
        fdr = torch.where(mask, fdr, torch.zeros_like(fdr))
        e = torch.where(mask, e_of(s) - e_of(torch.tensor(6.25, dtype=torch.float64, device="cuda")),
                        torch.zeros_like(s))
        return (fdr[:, :, None] * d).sum(1), 0.5 * e.sum(1)

    xx, vv = x0, v0
    FF, UU = dense_forces(xx)
    a = FF
    for t in range(K):
        xx = xx + (vv + 0.5 * dt * a) * dt
        vv = vv + 0.5 * dt * a
        FF, UU = dense_forces(xx)
        a = FF + (autodiff.langevin_noise(xx.shape[0], t, seed, c) - vv)
        vv = vv + 0.5 * dt * a
    assert torch.allclose(xx, x, rtol=0, atol=1e-9)
    loss_d = (FF ** 2).sum(dim=1).mean() + (UU.sum() / xx.shape[0]) ** 2
    (gd,) = torch.autograd.grad(loss_d, (p,))
    assert bool(((gv - gd).abs() <= 1e-6 * gd.abs() + 1e-10).all()), (gv, gd)


def test_rollout_gradient_at_workload_size():
    """The gradient workload at its own size: PerturbedLJ fluid, N = 65,536 at
    density 0.8, (epsilon, sigma, lambda) = (1, 1, 0.5), loss on forces and energy
    against targets at (1.1, 0.98, 0.4), K = 100 Langevin steps (dt = 0.005,
    fixed seed) with checkpoints every 10, against FP64 central differences
    (h = 1e-6). Forces smoothed to zero at r_cut (xplor, r_on = 2.5, r_cut = 3)
    so that no pair crossing r_cut makes the loss jump. epsilon and lambda meet
    1e-6. sigma moves the kink of the WCA split at r^2 = 2^(1/3) sigma^2
    (PairEvaluatorPerturbedLennardJones.h:131-145: the force's derivative jumps
    there), so over 100 steps pairs straddle the kink inside [sigma - h, sigma + h]
    and the central difference itself carries an error; sigma is held to 1e-4
    here and to 1e-6 against the exact dense gradient of the same dynamics
    (test_rollout_gradient_matches_dense_autograd)."""
    torch = _torch()
    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff

    snap = _fluid(65536, 0.8, seed=5)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="xplor")
    ctx = autodiff.Context(pot, snap.particles.types, snap.particles.typeid, snap.configuration.box, 3.0, r_on=2.5)
    x0 = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda")
    v0 = torch.tensor(snap.particles.velocity, dtype=torch.float64, device="cuda")
    vals = torch.tensor([1.0, 1.0, 0.5], dtype=torch.float64, device="cuda", requires_grad=True)
    with torch.no_grad():
        Ft, Ut = autodiff.pair_forces(x0, torch.tensor([1.1, 0.98, 0.4], dtype=torch.float64, device="cuda"), ctx)
        Ut = Ut.sum()

    def roll(v):
        x, vel, F, U = autodiff.langevin_rollout(x0, v0, v, ctx, 100, 0.005, seed=9, checkpoint_every=10)
        return ((F - Ft) ** 2).sum(dim=1).mean() + (U.sum() - Ut) ** 2

    (g,) = torch.autograd.grad(roll(vals), (vals,))
    h = 1e-6
    err = []
    for k in range(3):
        with torch.no_grad():
            vp, vm = vals.detach().clone(), vals.detach().clone()
            vp[k] += h
            vm[k] -= h
            fd = (roll(vp) - roll(vm)) / (2 * h)
        err.append(abs(float(g[k]) - float(fd)) / abs(float(fd)))
    print("rollout FD relative errors (eps, sigma, lambda):", err)
    assert err[0] <= 1e-6 and err[2] <= 1e-6, err
    assert err[1] <= 1e-4, err

