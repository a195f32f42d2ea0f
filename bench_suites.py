"""Measurements of the workloads beside the headline melt (``bench.py --suite ...``).

Each suite prints one JSON line:

* ``lj``: the PerturbedLennardJones fluid (N = 4096 on a jittered 16^3 lattice,
  density 0.8, epsilon = sigma = 1, lambda = 0.5, r_cut = 3, buffer 0.4;
  LangevinFlow, ConstantFlow 0, gamma = 1, dt = 0.005, 1000 steps; forces,
  energy and virial every 100 steps) on the GPU next to the CPU oracle.
* ``batched``: 256 ExpandedYukawa replicas (N log-uniform in [500, 20000],
  density U(0.3, 0.8), kappa U(0.5, 3), delta U(0, 1), r_cut = delta + 5 / kappa,
  LangevinFlow kT = 1, dt = 0.002) in one fused launch per step (graph-replayed,
  autotuned threads per particle) against the same replicas advanced one after
  the other through per-replica engines with plain stream launches.
* ``adjoint``: gradients on the PerturbedLJ fluid (N = 65,536, density 0.8,
  learnable epsilon, sigma, lambda; loss on forces and energy against targets at
  (1.1, 0.98, 0.4)): adjoint / forward cost, agreement with FP64 central finite
  differences (h = 1e-6), for one force call and through K Langevin steps with
  checkpoints every 10.
* ``precision``: the colloid-solvent mixture (N = 262,144, 4 % colloids of
  diameter 5, phi = 0.3, Hamaker A_SS = 144, A_CS = 100, A_CC = 40, r_cut 3 / 6 / 10;
  BrownianFlow, ConstantFlow U = 0.1 x, dt = 0.001, drag gamma = 10 diameter) --
  FP32-compensated against FP64 forces, energy and virial every 500 steps along the
  FP32-force Brownian trajectory.
* ``nlist``: the neighbour-list drop-in driver (``azp_nlist_build``: cell binning,
  scan, scatter, per-cell sort and the list kernel) on the relaxed headline melt
  (N = 1,048,600, WCA r_cut 2^(1/6), buffer 0.4, bonded pairs excluded), positions
  resident; in the melt's chain order and in cell order (the order the resident
  engine keeps its particles in).
* ``drivers``: the drop-in drivers of the rows beside the headline path
  (DPDGeneralWeight, HarmonicBarrier, LJ93 walls, velocity fields, ImageHarmonic)
  on about 10^6 particles: time per call, algorithmic bytes, fraction of the
  measured HBM bandwidth, and the oracle's host time on a sample; and the DPD
  fluid advanced by the resident engine (ConstantVolume + DPDGeneralWeight).
"""

from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np


def _cuda_ms(fn, reps=1):
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


# ---------------------------------------------------------------- LJ fluid
def suite_lj(args):
    import azplugins_gb300 as az
    from azplugins_gb300 import workloads
    from oracle import oracle as orc
    from tests.helpers import force_error, oracle_system

    snap = workloads.lj_fluid(16, 0.8, 0.05, 1.0, seed=1)
    snap.particles.acceleration = np.zeros((snap.particles.N, 3))
    steps = 1000
    out = {}
    for prec in ("fp64", "fp32"):
        sim = az.Simulation(seed=1, precision=prec)
        sim.create_state_from_snapshot(snap)
        lj = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=3.0)
        lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5)
        m = az.methods.LangevinFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0, 0, 0)), default_gamma=1.0)
        sim.operations.integrator = az.md.Integrator(dt=0.005, methods=[m], forces=[lj])
        sim.run(10)
        t0 = time.perf_counter()
        logs = []
        for _ in range(steps // 100):
            sim.run(100)
            logs.append(sim.thermo())
        dt = time.perf_counter() - t0
        out[prec] = {"timesteps_per_s": steps / dt, "final_pe": logs[-1]["potential_energy"],
                     "list_builds": logs[-1]["nlist_builds"]}
        if prec == "fp32":
            s = sim.state.get_snapshot()
            f32, _ = sim._engine.forces()
        sim.close()
    # FP32 force error against the FP64 oracle at the final FP32 state
    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.5))
    md = orc.OracleMD(oracle_system(s, s.particles.acceleration),
                      pair=dict(name="PerturbedLennardJones", params=rec.reshape(1, 1, 4), rcut=np.array([[3.0]])),
                      gamma=[1.0], kT=1.0, dt=0.005, seed=1)
    F, U, W = md.forces()
    cores = orc.set_threads(os.cpu_count() or 1)
    md2 = orc.OracleMD(oracle_system(snap, snap.particles.acceleration),
                       pair=dict(name="PerturbedLennardJones", params=rec.reshape(1, 1, 4), rcut=np.array([[3.0]])),
                       gamma=[1.0], kT=1.0, dt=0.005, seed=1)
    t0 = time.perf_counter()
    md2.run(200)
    cpu = 200 / (time.perf_counter() - t0)
    line = {"suite": "lj", "workload": "PerturbedLJ fluid N=4096 rho=0.8 lambda=0.5 r_cut=3 LangevinFlow 1000 steps",
            "gpu": out, "fp32_force_error_vs_fp64_oracle": force_error(f32, F),
            "fp32_energy_rel_error": abs(f32[:, 3].sum() - U.sum()) / abs(U.sum()),
            "cpu_oracle": {"timesteps_per_s": cpu, "cores": cores, "sample": "200 steps, OpenMP"}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- batched replicas
def suite_batched(args):
    import torch

    import azplugins_gb300 as az
    from azplugins_gb300 import workloads
    from azplugins_gb300.batch import ReplicaBatch

    snaps, params, redraws = workloads.yukawa_replicas(256, seed=4)
    seeds = list(range(1000, 1256))
    yk = [dict(epsilon=p["epsilon"], kappa=p["kappa"], delta=p["delta"]) for p in params]
    rc = [p["r_cut"] for p in params]
    b = ReplicaBatch(snaps, az.pair.ExpandedYukawa, yk, rc, seeds, dt=0.002, precision="fp32")
    tune = b.autotune(candidates=(1, 2, 4, 8), steps=20, blocks=(128, 256, 512))
    b.run(50)  # warm-up
    steps = args.steps if args.steps != 2000 else 500
    ms = _cuda_ms(lambda: b.run(steps, check=False))
    launches = b.last_launches
    b.run(0)
    batched = 256 * steps / (ms * 1e-3)
    b.close()
    # the same replicas one after the other, plain stream launches
    os.environ["AZP_GRAPHS"] = "0"
    sims = []
    try:
        for s, p, sd in zip(snaps, params, seeds):
            sim = az.Simulation(seed=sd, precision="fp32")
            sim.create_state_from_snapshot(s)
            pot = az.pair.ExpandedYukawa(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=p["r_cut"])
            pot.params[("A", "A")] = dict(epsilon=p["epsilon"], kappa=p["kappa"], delta=p["delta"])
            m = az.methods.LangevinFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0, 0, 0)))
            sim.operations.integrator = az.md.Integrator(dt=0.002, methods=[m], forces=[pot])
            sim.run(2)
            sims.append(sim)
    finally:
        os.environ.pop("AZP_GRAPHS", None)
    sep_steps = 20

    def sweep():
        for _ in range(sep_steps):
            for sim in sims:
                sim._engine.run_async(1)

    ms_sep = _cuda_ms(sweep)
    separate = 256 * sep_steps / (ms_sep * 1e-3)
    for sim in sims:
        sim.close()
    line = {"suite": "batched", "workload": "256 ExpandedYukawa replicas, N log-uniform [500, 20000], LangevinFlow",
            "total_particles": int(sum(s.particles.N for s in snaps)), "redraws_for_min_image": redraws,
            "batched_replica_steps_per_s": batched, "separate_replica_steps_per_s": separate,
            "speedup": batched / separate, "autotune_ms_per_step": {str(k): v for k, v in tune.items()},
            "tpp": int(min(tune, key=tune.get)[0]), "block": int(min(tune, key=tune.get)[1]),
            "batched_launches_in_timed_region": launches,
            "steps_batched": steps, "steps_separate": sep_steps, "forces": "fp32",
            "integration": "f64 positions and velocities"}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- adjoint
def suite_adjoint(args):
    import torch

    import azplugins_gb300 as az
    from azplugins_gb300 import autodiff
    from tests.helpers import random_fluid

    snap = random_fluid(65536, 0.8, seed=5, min_dist=0.9)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="shift")
    ctx = autodiff.Context(pot, snap.particles.types, snap.particles.typeid, snap.configuration.box, 3.0)
    x = torch.tensor(snap.particles.position, dtype=torch.float64, device="cuda", requires_grad=True)
    vals = torch.tensor([1.0, 1.0, 0.5], dtype=torch.float64, device="cuda", requires_grad=True)
    valst = torch.tensor([1.1, 0.98, 0.4], dtype=torch.float64, device="cuda")
    with torch.no_grad():
        Ft, Ut = autodiff.pair_forces(x, valst, ctx)
        Ut = Ut.sum()

    def loss_fn(F, U):
        return ((F - Ft) ** 2).sum(dim=1).mean() + (U.sum() - Ut) ** 2

    # cost through torch autograd (Python, table set-up and reductions included)
    F, U = autodiff.pair_forces(x, vals, ctx)
    loss = loss_fn(F, U)
    gF, gU = torch.autograd.grad(loss, (F, U), retain_graph=True)
    # one untimed call of each first (library handles, first use of torch ops)
    autodiff.pair_forces(x.detach(), vals.detach(), ctx)
    torch.autograd.grad((F, U), (x, vals), (gF, gU), retain_graph=True)
    fwd = _cuda_ms(lambda: autodiff.pair_forces(x.detach(), vals.detach(), ctx), reps=20)
    bwd = _cuda_ms(lambda: torch.autograd.grad((F, U), (x, vals), (gF, gU), retain_graph=True), reps=20)
    # cost of the kernels alone through the C ABI: the forward pair driver and
    # the adjoint driver on the same list, CUDA events on the launching stream
    from azplugins_gb300 import _lib

    L = _lib.load()
    nl = ctx.neighbor_list(x)
    pos4 = ctx.pos4(x)
    sysd = ctx.system(pos4)
    params, rc, ro = autodiff._pair_tables(ctx, vals.detach())
    force = torch.empty((ctx.N, 4), dtype=torch.float64, device="cuda")
    out = _lib.Forces()
    out.force, out.virial, out.virial_pitch, out.precision = force.data_ptr(), None, ctx.N, _lib.FP64
    grad = torch.cat([gF, gU[:, None]], dim=1).contiguous()
    gpos = torch.empty((ctx.N, 3), dtype=torch.float64, device="cuda")
    grec = torch.empty((ctx.N, 4), dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    mode = _lib.MODES[pot.mode]
    k_fwd = _cuda_ms(lambda: L.azp_pair_forces(ctypes.byref(sysd), nl.handle, pot.kind, params.data_ptr(), rc.data_ptr(),
                                                ro.data_ptr(), mode, ctypes.byref(out), stream), reps=50)
    k_adj = _cuda_ms(lambda: L.azp_pair_adjoint(ctypes.byref(sysd), nl.handle, pot.kind, params.data_ptr(),
                                                 rc.data_ptr(), ro.data_ptr(), mode, grad.data_ptr(), gpos.data_ptr(),
                                                 grec.data_ptr(), stream), reps=50)
    gx, gv = torch.autograd.grad(loss, (x, vals))
    h = 1e-6
    fd_err = []
    for k in range(3):
        with torch.no_grad():
            vp, vm = vals.detach().clone(), vals.detach().clone()
            vp[k] += h
            vm[k] -= h
            fd = (loss_fn(*autodiff.pair_forces(x.detach(), vp, ctx)) - loss_fn(*autodiff.pair_forces(x.detach(), vm, ctx))) / (2 * h)
        fd_err.append(abs(float(gv[k]) - float(fd)) / abs(float(fd)))
    # through K Langevin steps with checkpoints every 10. Finite differences of
    # a trajectory loss are only meaningful when the forces are continuous in
    # r: the rollout uses the xplor form (forces smoothed to zero between
    # r_on = 2.5 and r_cut = 3), so no pair crossing r_cut makes the loss jump.
    K = 100
    x0 = x.detach()
    v0 = torch.tensor(snap.particles.velocity, dtype=torch.float64, device="cuda")
    pot_s = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), mode="xplor")
    ctx_s = autodiff.Context(pot_s, snap.particles.types, snap.particles.typeid, snap.configuration.box, 3.0,
                             r_on=2.5)
    with torch.no_grad():
        Fts, Uts = autodiff.pair_forces(x0, valst, ctx_s)
        Uts = Uts.sum()

    def roll(v):
        xx, vv, FF, UU = autodiff.langevin_rollout(x0, v0, v, ctx_s, K, 0.005, seed=9, checkpoint_every=10)
        return ((FF - Fts) ** 2).sum(dim=1).mean() + (UU.sum() - Uts) ** 2

    t0 = time.perf_counter()
    lossK = roll(vals)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    (gK,) = torch.autograd.grad(lossK, (vals,))
    torch.cuda.synchronize()
    t_bwd = time.perf_counter() - t0
    roll_err, roll_err_small = [], []
    for k in range(3):
        for hh, errs in ((h, roll_err), (0.1 * h, roll_err_small)):
            with torch.no_grad():
                vp, vm = vals.detach().clone(), vals.detach().clone()
                vp[k] += hh
                vm[k] -= hh
                fd = (roll(vp) - roll(vm)) / (2 * hh)
            errs.append(abs(float(gK[k]) - float(fd)) / abs(float(fd)))
    line = {"suite": "adjoint", "workload": "PerturbedLJ fluid N=65536 rho=0.8 r_cut=3 shift; learn (eps, sigma, lambda)",
            "forward_ms": fwd, "adjoint_ms": bwd, "adjoint_over_forward": bwd / fwd,
            "kernel_forward_ms": k_fwd, "kernel_adjoint_ms": k_adj, "kernel_adjoint_over_forward": k_adj / k_fwd,
            "single_call_fd_rel_error": fd_err, "rollout_steps": K, "checkpoint_every": 10,
            "rollout_forward_s": t_fwd, "rollout_backward_s": t_bwd, "rollout_fd_rel_error": roll_err, "rollout_fd_rel_error_h_1e-7": roll_err_small,
            "fd_step": h, "precision": "f64"}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- precision study
def suite_precision(args):
    import azplugins_gb300 as az
    from azplugins_gb300 import _compute, workloads
    from tests.helpers import force_error

    snap = workloads.colloid_mixture(262144, seed=3)
    N = snap.particles.N

    def colloid(mode="shift"):
        c = az.pair.Colloid(nlist=az.nlist.Cell(buffer=0.4), mode=mode)
        c.params[("S", "S")] = dict(A=144.0, a_1=0.0, a_2=0.0, sigma=1.0)
        c.params[("S", "C")] = dict(A=100.0, a_1=0.0, a_2=2.5, sigma=1.0)
        c.params[("C", "C")] = dict(A=40.0, a_1=2.5, a_2=2.5, sigma=1.0)
        c.r_cut[("S", "S")] = 3.0
        c.r_cut[("S", "C")] = 6.0
        c.r_cut[("C", "C")] = 10.0
        return c

    # the trajectory: FP32 compensated forces, 64-bit integration; Stokes-like
    # drag gamma = 10 diameter (the reference's use_lambda with lambda = 10): a
    # solvent bead's Brownian step sqrt(2 kT dt / gamma) = 0.014 stays well inside
    # its repulsive core (at gamma = 1 the kicks drive beads into the cores and
    # the trajectory blows up at this dt)
    sim = az.Simulation(seed=3, precision="fp32")
    sim.create_state_from_snapshot(snap)
    pot = colloid()
    m = az.methods.BrownianFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0.1, 0.0, 0.0)), alpha=10.0)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[m], forces=[pot])
    total = 5000 if args.steps == 2000 else args.steps
    every = max(total // 10, 1)
    rows = []
    done = 0
    t_run = 0.0
    while True:
        s = sim.state.get_snapshot()
        st = az.Simulation(precision="fp64")
        st.create_state_from_snapshot(s)
        f64, w64 = _compute.pair_forces(st.state, pot, "fp64")
        f32, w32 = _compute.pair_forces(st.state, pot, "fp32")
        typ = s.particles.typeid
        rows.append({"step": done, "force_error": force_error(f32, f64),
                     "force_error_solvent": force_error(f32[typ == 0], f64[typ == 0]),
                     "force_error_colloid": force_error(f32[typ == 1], f64[typ == 1]),
                     "energy_rel_error": abs(f32[:, 3].sum() - f64[:, 3].sum()) / abs(f64[:, 3].sum()),
                     "virial_rel_error": float(np.abs(w32.sum(axis=0) - w64.sum(axis=0)).max() /
                                               np.abs(w64.sum(axis=0)).max()),
                     "max_force": float(np.sqrt((f64[:, :3] ** 2).sum(axis=1)).max())})
        if done >= total:
            break
        t0 = time.perf_counter()
        sim.run(every)
        t_run += time.perf_counter() - t0
        done += every
    sim.close()
    # trajectory deviation: the same start, seed and random draws advanced 100
    # steps with FP32 forces and with FP64 forces; RMS and largest difference of
    # the unwrapped positions
    Lbox = np.array(snap.configuration.box[:3])
    traj = {}
    for prec in ("fp32", "fp64"):
        t = az.Simulation(seed=11, precision=prec)
        t.create_state_from_snapshot(snap)
        tm = az.methods.BrownianFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0.1, 0.0, 0.0)), alpha=10.0)
        t.operations.integrator = az.md.Integrator(dt=0.001, methods=[tm], forces=[colloid()])
        t.run(100)
        p = t.state.get_snapshot().particles
        traj[prec] = p.position + p.image * Lbox
        t.close()
    dev = traj["fp32"] - traj["fp64"]
    dev2 = (dev * dev).sum(axis=1)
    finite = all(np.isfinite([r["force_error"], r["energy_rel_error"], r["virial_rel_error"]]).all() for r in rows)
    line = {"suite": "precision", "workload": f"colloid mixture N={N}, 4% colloids (d=5), phi=0.3, BrownianFlow "
                                              f"U=0.1x dt=0.001 gamma=10 diameter, {total} steps (FP32-force trajectory)",
            "samples": rows, "all_finite": bool(finite),
            "max_force_error": max(r["force_error"] for r in rows),
            "max_energy_rel_error": max(r["energy_rel_error"] for r in rows),
            "max_virial_rel_error": max(r["virial_rel_error"] for r in rows),
            "reference": "FP64 drivers (equal to the FP64 oracle to 1e-12, tests/test_gpu_pair.py)",
            "trajectory_100_steps": {"rms_position_deviation": float(np.sqrt(dev2.mean())),
                                     "max_position_deviation": float(np.sqrt(dev2.max())),
                                     "compared": "FP32-force vs FP64-force engine, same start, seed and draws"},
            "fp32_brownian_timesteps_per_s": total / t_run if t_run else None}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- drop-in drivers of the widened rows
def _sys_struct(N, ntypes, L, **ptrs):
    from azplugins_gb300 import _lib

    s = _lib.System()
    s.N, s.ntypes = N, ntypes
    for k, v in ptrs.items():
        setattr(s, k, v)
    for d in range(3):
        s.box.L[d] = L[d]
    return s


def _forces_out(N, precision, torch):
    from azplugins_gb300 import _lib

    dt = torch.float32 if precision == "fp32" else torch.float64
    force = torch.zeros((N, 4), dtype=dt, device="cuda")
    vir = torch.zeros((6, N), dtype=dt, device="cuda")
    out = _lib.Forces()
    out.force, out.virial, out.virial_pitch = force.data_ptr(), vir.data_ptr(), N
    out.precision = _lib.FP32 if precision == "fp32" else _lib.FP64
    return force, vir, out


def suite_drivers(args):
    """Each drop-in driver of the rows beyond the headline path (DPDGeneralWeight,
    HarmonicBarrier, walls, velocity field, ImageHarmonic) on about 10^6 particles:
    CUDA-event time per call (inputs resident in HBM, 20 calls after 3 warm-up
    calls; every call's inputs exceed the L2), algorithmic bytes per call (what the
    caller's arrays and the outputs hold: the caller's FP64 position and velocity
    records, list indices, outputs in the output precision; neighbour gathers are
    cache traffic and not counted, as for the pair force) and the fraction of the
    measured HBM copy bandwidth; beside each, the oracle's time on a sample of the
    same inputs on the host cores (one thread), scaled to the full size."""
    import torch

    import azplugins_gb300 as az
    from azplugins_gb300 import _compute, _lib
    from bench import measured_peak
    from oracle import oracle as orc

    L_ = _lib.load()
    peak, peak_kind = measured_peak()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.Generator(np.random.PCG64(17))
    reps = max(1, min(20, args.steps))  # --steps 1: one timed call per driver (profiling runs)
    rows = {}

    def record(name, ms, nbytes, cpu_s, sample, **extra):
        gbs = nbytes / (ms * 1e-3) / 1e9
        rows[name] = {"ms_per_call": ms, "bytes_per_call": nbytes, "achieved_gbs": gbs, "frac": gbs / peak,
                      "cpu_oracle_ms_per_call_scaled": None if cpu_s is None else cpu_s * 1e3,
                      "cpu_sample": sample, **extra}

    def cpu_time(fn, frac):
        t0 = time.perf_counter()
        fn()
        return (time.perf_counter() - t0) / frac

    # -- a 2-type fluid of 2^20 particles at the melt's density, positions in FP64
    N = 1 << 20
    L = np.full(3, (N / 0.85) ** (1.0 / 3.0))
    pos = (rng.uniform(-0.5, 0.5, size=(N, 3)) * L)
    types = rng.integers(0, 2, size=N).astype(np.int32)
    vel = rng.normal(size=(N, 3))
    mass = rng.uniform(0.8, 1.2, size=N)
    dpos = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    dpos[:, :3] = torch.from_numpy(pos).cuda()
    dpos.view(torch.int64)[:, 3] = torch.from_numpy(types.astype(np.int64)).cuda()
    dvel = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    dvel[:, :3] = torch.from_numpy(vel).cuda()
    dvel[:, 3] = torch.from_numpy(mass).cuda()
    sysd = _sys_struct(N, 2, L, pos=dpos.data_ptr(), vel=dvel.data_ptr())
    pos4 = np.concatenate([pos, types[:, None].astype(float)], axis=1)
    sample = N // 16
    # HarmonicBarrier, planar at 0.3 L: read 32 B, write force and virial
    bpar = torch.tensor([[50.0, 0.1], [200.0, -0.1]], dtype=torch.float64, device="cuda")
    for prec in ("fp64", "fp32"):
        force, vir, out = _forces_out(N, prec, torch)

        def call():
            _lib.check(L_.azp_harmonic_barrier_forces(ctypes.byref(sysd), 0, 0.3 * L[1], bpar.data_ptr(),
                                                      ctypes.byref(out), stream), "barrier")

        for _ in range(3):
            call()
        ms = _cuda_ms(call, reps)
        wb = 8 if prec == "fp64" else 4
        cpu = cpu_time(lambda: orc.harmonic_barrier(pos4[:sample], types[:sample], L, "planar", 0.3 * L[1],
                                                    np.array([[50.0, 0.1], [200.0, -0.1]])), sample / N)
        record(f"harmonic_barrier_{prec}", ms, N * (32 + 4 * wb + 6 * wb), cpu, f"{sample} particles")
    # walls: LJ93 slit (two planes) and a cylinder, 2 types
    pot = az.wall.LJ93(walls=[az.wall.Plane(origin=(0, -0.45 * L[1], 0), normal=(0, 1, 0)),
                              az.wall.Plane(origin=(0, 0.45 * L[1], 0), normal=(0, -1, 0)),
                              az.wall.Cylinder(radius=0.4 * L[0], axis=(0, 0, 1), inside=True)])
    pot.params["A"] = dict(A=1.0, sigma=1.0, r_cut=3.0)
    pot.params["B"] = dict(A=2.0, sigma=1.2, r_cut=3.0, r_extrap=0.5)
    rec, rc, rx = pot._tables(["A", "B"])
    walls, keep = pot._walls_struct()
    wdev = [torch.from_numpy(np.ascontiguousarray(a).reshape(-1).copy()).cuda() for a in (rec, rc, rx)]
    from tests.helpers import oracle_walls

    sp, cy, pl = oracle_walls(pot)
    for prec in ("fp64", "fp32"):
        force, vir, out = _forces_out(N, prec, torch)

        def call():
            _lib.check(L_.azp_wall_forces(ctypes.byref(sysd), pot.kind, ctypes.byref(walls), wdev[0].data_ptr(),
                                          wdev[1].data_ptr(), wdev[2].data_ptr(), ctypes.byref(out), stream),
                       "walls")

        for _ in range(3):
            call()
        ms = _cuda_ms(call, reps)
        wb = 8 if prec == "fp64" else 4
        cpu = cpu_time(lambda: orc.wall_forces(pos4[:sample], types[:sample], "LJ93", rec, rc, rx, sp, cy, pl),
                       sample / N)
        record(f"walls_lj93_{prec}", ms, N * (32 + 4 * wb + 6 * wb), cpu, f"{sample} particles", walls="2 planes + 1 cylinder")
    del keep
    # velocity fields: 100 slabs along y; cylindrical 20 x 16 x 10 bins; both read pos and vel (64 B)
    vel4 = np.concatenate([vel, mass[:, None]], axis=1)
    for kind, nb, lo, hi in (("cartesian", (0, 100, 0), (0, -L[1] / 2, 0), (0, L[1] / 2, 0)),
                             ("cylindrical", (20, 16, 10), (0, 0, -L[2] / 2), (L[0] / 2, 2 * np.pi, L[2] / 2))):
        nb_ = np.ascontiguousarray(nb, dtype=np.uint32)
        lo_, hi_ = np.ascontiguousarray(lo, dtype=np.float64), np.ascontiguousarray(hi, dtype=np.float64)
        st = ctypes.c_int(0)
        vf = L_.azp_vfield_create(_lib.BINNING_KINDS[kind], nb_.ctypes.data, lo_.ctypes.data, hi_.ctypes.data,
                                  ctypes.byref(st))
        _lib.check(st.value, "azp_vfield_create")
        total = int(L_.azp_vfield_num_bins(vf))
        vout = torch.zeros((total, 7), dtype=torch.float64, device="cuda")

        def call():
            _lib.check(L_.azp_vfield_compute(vf, ctypes.byref(sysd), None, 0, vout.data_ptr(), None, None, stream),
                       "vfield")

        for _ in range(3):
            call()
        ms = _cuda_ms(call, reps)
        cpu = cpu_time(lambda: orc.velocity_field(pos4[:sample], vel4[:sample], L, kind, nb, lo, hi), sample / N)
        L_.azp_vfield_destroy(vf)
        record(f"velocity_field_{kind}", ms, N * 64, cpu, f"{sample} particles", bins=total)
    # ImageHarmonic on 10,486 chains x 100 beads (random walks, 1 in 25 bonds longer than half the box)
    n_chains, length = 10486, 100
    Nc = n_chains * length
    Lc = np.full(3, (Nc / 0.85) ** (1.0 / 3.0))
    steps = rng.normal(size=(n_chains, length, 3))
    steps *= 0.97 / np.linalg.norm(steps, axis=2, keepdims=True)
    un = np.cumsum(steps, axis=1).reshape(Nc, 3) + np.repeat(rng.uniform(-0.5, 0.5, size=(n_chains, 3)) * Lc, length, 0)
    img = np.floor((un + 0.5 * Lc) / Lc).astype(np.int32)
    cpos = un - img * Lc
    bonds = (np.arange(Nc).reshape(n_chains, length)[:, :-1].reshape(-1, 1) + np.array([0, 1])).astype(np.int64)
    n, table, h = _compute.bond_table(Nc, bonds, np.zeros(len(bonds), dtype=np.int32))
    cd = torch.zeros((Nc, 4), dtype=torch.float64, device="cuda")
    cd[:, :3] = torch.from_numpy(cpos).cuda()
    dimg = torch.from_numpy(img.reshape(-1)).cuda()
    csys = _sys_struct(Nc, 1, Lc, pos=cd.data_ptr(), image=dimg.data_ptr())
    n_d = torch.from_numpy(n.view(np.int32)).cuda()
    t_d = torch.from_numpy(table.reshape(-1).view(np.int32)).cuda()
    bp = np.zeros(8)
    bp[:2] = [30.0, 1.0]
    bp_d = torch.from_numpy(bp).cuda()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    nbm = float(n.mean())
    for prec in ("fp64", "fp32"):
        force, vir, out = _forces_out(Nc, prec, torch)

        def call():
            _lib.check(L_.azp_bond_forces(ctypes.byref(csys), n_d.data_ptr(), t_d.data_ptr(), h, 2, bp_d.data_ptr(), 1,
                                          ctypes.byref(out), err.data_ptr(), stream), "image bond")

        for _ in range(3):
            call()
        ms = _cuda_ms(call, reps)
        wb = 8 if prec == "fp64" else 4
        cs = Nc // 16
        cb = bonds[(bonds < cs).all(axis=1)]
        cpu = cpu_time(lambda: orc.image_bond_forces(np.concatenate([cpos[:cs], np.zeros((cs, 1))], axis=1), img[:cs],
                                                     Lc, cb, np.zeros(len(cb), dtype=np.int32), "ImageHarmonic",
                                                     bp[None]), cs / Nc)
        # own position and image, bond count and table; force and virial accumulated (read + write)
        record(f"image_harmonic_{prec}", ms, int(Nc * (32 + 12 + 4 + 8 * nbm + 2 * 4 * wb + 2 * 6 * wb)), cpu,
               f"{cs} particles", bonds_per_particle=nbm)
    # DPDGeneralWeight at density 3, r_cut 1, buffer 0.3, 2 types, thermostat on
    Nd = 1 << 20
    Ld = np.full(3, (Nd / 3.0) ** (1.0 / 3.0))
    snap = az.Snapshot(Nd)
    snap.particles.types = ["A", "B"]
    snap.particles.position = rng.uniform(-0.5, 0.5, size=(Nd, 3)) * Ld
    snap.particles.typeid = rng.integers(0, 2, size=Nd).astype(np.int32)
    snap.particles.velocity = rng.normal(size=(Nd, 3))
    snap.particles.mass = np.ones(Nd)
    snap.configuration.box = [*Ld, 0, 0, 0]
    dpd = az.pair.DPDGeneralWeight(nlist=az.nlist.Cell(buffer=0.3), kT=1.0, default_r_cut=1.0)
    dpd.params[("A", "A")] = dict(A=25.0, gamma=4.5, s=0.5)
    dpd.params[("A", "B")] = dict(A=30.0, gamma=4.5, s=1.0)
    dpd.params[("B", "B")] = dict(A=25.0, gamma=4.5, s=2.0)
    drec, drc, _ = dpd._tables(["A", "B"])
    ppos = _compute.device_positions(snap)
    pvel = torch.zeros((Nd, 4), dtype=torch.float64, device="cuda")
    pvel[:, :3] = torch.from_numpy(snap.particles.velocity).cuda()
    pvel[:, 3] = 1.0
    tags = torch.arange(Nd, dtype=torch.int32, device="cuda")
    dsys = _compute.make_system(snap, ppos, vel=pvel.data_ptr(), tag=tags.data_ptr())
    nl = _compute.NeighborList(Nd, 2, drc, 0.3, tpp=4)
    nl.build(dsys)
    counts, didx = nl.to_csr()
    nbar = float(np.diff(counts).mean())
    # the oracle (OpenMP, all host cores) on the first 1/16 of the rows
    Sd = Nd // 16
    dcores = orc.set_threads(os.cpu_count() or 1)
    dvel4 = np.concatenate([snap.particles.velocity, np.ones((Nd, 1))], axis=1)
    dpos4 = np.concatenate([snap.particles.position, snap.particles.typeid[:, None].astype(float)], axis=1)
    dcpu = cpu_time(lambda: orc.dpd_forces(dpos4, dvel4, snap.particles.typeid,
                                           np.arange(Nd, dtype=np.uint32), 2, Ld, np.minimum(counts, counts[Sd]),
                                           didx[:counts[Sd]], drec, drc * drc, 1.0, 0.01, 5, 77), Sd / Nd)
    dparams = torch.from_numpy(drec.reshape(-1).copy()).cuda()
    drc_d = torch.from_numpy(drc.reshape(-1).copy()).cuda()
    for prec, tpp in (("fp64", 4), ("fp32", 1), ("fp32", 2), ("fp32", 4)):
        force, vir, out = _forces_out(Nd, prec, torch)
        _lib.check(L_.azp_nlist_set_tpp(nl.handle, tpp), "azp_nlist_set_tpp")

        def call():
            _lib.check(L_.azp_dpd_forces(ctypes.byref(dsys), nl.handle, dparams.data_ptr(), drc_d.data_ptr(), 1.0, 0.01,
                                         77, 5, ctypes.byref(out), stream), "dpd")

        for _ in range(3):
            call()
        ms = _cuda_ms(call, reps)
        wb = 8 if prec == "fp64" else 4
        record(f"dpd_{prec}_tpp{tpp}", ms, int(Nd * (32 + 32 + 4 + 4 + 4 * nbar + 4 * wb + 6 * wb)), dcpu,
               f"{Sd} particles' rows", cpu_cores=dcores, mean_neighbours=nbar, density=3.0,
               pairs_per_s=float(np.diff(counts).sum()) / (ms * 1e-3))
    nl.close()
    # the same fluid advanced by the resident engine: ConstantVolume + DPDGeneralWeight,
    # one fused launch per step (forces of t + 1 at the half-step velocities, both
    # velocity-Verlet halves) after a velocity snapshot; wall clock around run(K)
    # with the device synchronised on both sides (one host check per run call).
    # Bytes per particle and step: FP32 forces read and write the fixed-point words
    # (2 x 16 B), the float-float velocity (2 x 32 B) and the snapshot (16 B written,
    # 16 B read); FP64 the position (2 x 32 B), fixed words (16 B), velocity (2 x 32 B)
    # and snapshot (2 x 32 B); both the list row (4 B count, 4 B per neighbour)
    steps = 10 * reps
    for prec in ("fp32", "fp64"):
        pot = az.pair.DPDGeneralWeight(nlist=az.nlist.Cell(buffer=0.3), kT=1.0, default_r_cut=1.0)
        pot.params[("A", "A")] = dict(A=25.0, gamma=4.5, s=0.5)
        pot.params[("A", "B")] = dict(A=30.0, gamma=4.5, s=1.0)
        pot.params[("B", "B")] = dict(A=25.0, gamma=4.5, s=2.0)
        sim = az.Simulation(seed=5, precision=prec)
        sim.create_state_from_snapshot(snap)
        sim.operations.integrator = az.md.Integrator(dt=0.01, methods=[az.methods.ConstantVolume("all")],
                                                     forces=[pot])
        sim.run(20)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.run(steps)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / steps
        per = (2 * 16 + 2 * 32 + 2 * 16) if prec == "fp32" else (2 * 32 + 16 + 2 * 32 + 2 * 32)
        record(f"dpd_engine_step_{prec}", ms, int(Nd * (per + 4 + 4 * nbar)), None, None, steps=steps,
               timesteps_per_s=1e3 / ms, pairs_per_s=float(np.diff(counts).sum()) / (ms * 1e-3), density=3.0)
        sim.close()
    line = {"suite": "drivers", "n_particles": N, "peak_gbs": peak, "peak_kind": peak_kind, "reps": reps,
            "drivers": rows}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- list build
def suite_nlist(args):
    import torch

    import bench
    from azplugins_gb300 import _compute

    snap, _ = bench.relaxed_melt(args.chains, seed=1)
    N = snap.particles.N
    L = np.array(snap.configuration.box[:3])
    r_list = bench.RCUT + bench.R_BUFF
    # cell order: particles sorted by the index of a cell of width >= r_list
    dims = np.floor(L / r_list).astype(np.int64)
    cell = np.floor((snap.particles.position + L / 2) / L * dims).astype(np.int64) % dims
    order = np.argsort((cell[:, 2] * dims[1] + cell[:, 1]) * dims[0] + cell[:, 0], kind="stable")
    rank = np.empty(N, dtype=np.int64)
    rank[order] = np.arange(N)
    out = {"suite": "nlist", "workload": "bead-spring melt N=1048600 after relaxation, WCA r_cut 2^(1/6), "
           "buffer 0.4, bonded pairs excluded", "N": N}
    for name, perm in (("chain_order", None), ("cell_order", order)):
        pos = snap.particles.position if perm is None else snap.particles.position[perm]
        group = snap.bonds.group if perm is None else rank[snap.bonds.group]
        ex = _compute.exclusions_csr(N, group)
        sub = type(snap)(N)
        sub.configuration.box = list(snap.configuration.box)
        sub.particles.position = pos
        sub.particles.typeid = np.zeros(N, dtype=np.int32)
        posd = _compute.device_positions(sub)
        sysd = _compute.make_system(sub, posd)
        nl = _compute.NeighborList(N, 1, np.array([[bench.RCUT]]), bench.R_BUFF, ex)
        nl.build(sysd)  # sizes the list
        for _ in range(3):
            nl.build(sysd)
        ms = _cuda_ms(lambda: nl.build(sysd), reps=20)
        torch.cuda.nvtx.range_push(f"nlist_build_{name}")
        nl.build(sysd)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        counts = nl.counts()
        out[name] = {"ms_per_build": ms, "mean_listed": float(counts.mean()), "max_listed": int(counts.max())}
        nl.close()
    out["note"] = ("one azp_nlist_build = cell binning + scan + scatter + per-cell sort + list kernel; CUDA events "
                   "over 20 builds after 4")
    print(json.dumps(out), flush=True)


def run(args):
    import torch

    torch.cuda.set_device(0)
    {"lj": suite_lj, "batched": suite_batched, "adjoint": suite_adjoint, "precision": suite_precision,
     "drivers": suite_drivers, "nlist": suite_nlist}[args.suite](args)
