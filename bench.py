"""Benchmark of the short-range force-and-integrate path on one GB300.

Workload (the headline metric's configuration): a bead-spring melt of 10,486
linear chains x 100 beads (N = 1,048,600) at number density 0.85, seeded random
walks with bond length 0.97 relaxed by 200 displacement-capped Brownian steps;
PerturbedLennardJones with lambda = 0, r_cut = 2^(1/6) (WCA), buffer 0.4, bonded
pairs excluded; Quartic bonds k = 1434.3, b_1 = -0.7589, b_2 = 0, r_0 = 1.5,
U_0 = 67.2234, sigma = epsilon = 1; LangevinFlow with ParabolicFlow
(mean_velocity = 2/3, separation = L: centreline speed 1.0 along x, gradient
along y as in the reference functor), gamma = 1, kT = 1, dt = 0.005. FP32 pair
and bond arithmetic (compensated sums) with FP64 integration.

A "step" is one MD timestep (forces + Langevin step two + step one of the next
timestep, list rebuilds amortised as they happen). ``value`` is timesteps/s
with the state resident in HBM; ``e2e`` is the same metric through the public
C ABI with a full host snapshot round trip every step (pinned host buffers:
positions, velocities, accelerations, images in; the same out, plus the
thermodynamic sums). The working set (about 0.6 GB) is larger than L2.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
For N > 1 (torchrun, one rank per GPU) every rank advances an independent
replica (replicas only: the single-system path has no exchange-free sharding).
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "timesteps/s & HBM GB/s vs peak at N=1M; batched & adjoint vs plain at 1e-5 err"
N_CHAINS, CHAIN_LEN, DENSITY = 10486, 100, 0.85
QUARTIC = dict(k=1434.3, r_0=1.5, b_1=-0.7589, b_2=0.0, U_0=67.2234, sigma=1.0, epsilon=1.0, delta=0.0)
DT, KT, GAMMA, R_BUFF = 0.005, 1.0, 1.0, 0.4
RCUT = 2.0 ** (1.0 / 6.0)
# overlap relaxation: 200 Brownian steps in four stages whose per-pair force cap
# rises 20 -> 1000 (bonds hold while overlaps are pushed apart), displacements
# capped at 0.02 per component; then extra uncapped-force stages only while the
# largest force is still above RELAX_FMAX
RELAX_STEPS, RELAX_DT, RELAX_MAX_DISP = 200, 0.002, 0.02
RELAX_CAPS = (20.0, 50.0, 200.0, 1000.0)
RELAX_FMAX = 2000.0
# reference arm (the oracle on the host cores): warm-up cap and time box of the timed steps
REF_MAX_WARMUP, REF_TIME_BOX_S = 10, 60.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chains", type=int, default=N_CHAINS)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--suite", default="melt", choices=["melt", "batched", "adjoint", "precision", "lj", "drivers", "nlist"],
                    help="melt: the headline line; the others measure the remaining workloads")
    return ap.parse_args()


def log(msg):
    """Stage marker on stderr (flushed), so a slow stage can be located."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_melt(n_chains, seed):
    from azplugins_gb300 import workloads

    return workloads.bead_spring_melt(n_chains, CHAIN_LEN, DENSITY, 0.97, KT, seed=seed)


def forces_and_method(az, flow, precision_unused=None):
    wca = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=R_BUFF), default_r_cut=RCUT)
    wca.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.0)
    qb = az.bond.Quartic()
    qb.params["A-A"] = QUARTIC
    return wca, qb


def _melt_oracle(orc, snap, method, dt, seed, **kw):
    """The melt's forces (WCA pair, Quartic bonds, bonded pairs excluded) on the
    oracle, as an OracleMD loop on a copy of ``snap``."""
    from tests.helpers import oracle_system

    rec = orc.pair_params("PerturbedLennardJones", dict(epsilon=1.0, sigma=1.0, attraction_scale_factor=0.0))
    brec = orc.bond_params("Quartic", QUARTIC)
    return orc.OracleMD(oracle_system(snap, snap.particles.acceleration),
                        pair=dict(name="PerturbedLennardJones", params=rec.reshape(1, 1, 4), rcut=np.array([[RCUT]])),
                        bond=dict(name="Quartic", params=brec.reshape(1, 8)), method=method, gamma=[GAMMA], kT=KT,
                        dt=dt, seed=seed, r_buff=R_BUFF, **kw)


def state_hash(snap):
    """First 16 hex digits of the SHA-256 of the positions, images and velocities."""
    import hashlib

    p = snap.particles
    h = hashlib.sha256()
    for a in (p.position, p.image, p.velocity):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def relaxed_melt(n_chains, seed):
    """Random-walk melt with overlaps removed by capped Brownian steps, on the
    host with the FP64 oracle (deterministic for any thread count), so that both
    arms of the benchmark start from the same state: four stages of 50 steps with
    the per-pair force capped at 20, 50, 200, 1000 and displacements at 0.02, then
    up to four uncapped 50-step stages while the largest force exceeds
    RELAX_FMAX. Velocities Maxwell-Boltzmann at kT (zero momentum), accelerations
    zero. Returns (snapshot, relaxation summary)."""
    from oracle import oracle as orc

    snap = make_melt(n_chains, seed)
    p = snap.particles
    p.acceleration = np.zeros((p.N, 3))
    threads = orc.set_threads(os.cpu_count() or 1)
    try:
        stages = [(cap, RELAX_STEPS // len(RELAX_CAPS)) for cap in RELAX_CAPS]
        k, extra, fmax = 0, 0, None
        while k < len(stages):
            cap, n = stages[k]
            md = _melt_oracle(orc, snap, "brownian", RELAX_DT, seed + k, max_disp=RELAX_MAX_DISP, force_cap=cap)
            md.run(n)
            p.position = md.s["pos4"][:, :3].copy()
            p.image = md.s["image"].copy()
            k += 1
            if k == len(stages):
                F, _, _ = _melt_oracle(orc, snap, "brownian", RELAX_DT, seed).forces()
                fmax = float(np.sqrt((F * F).sum(axis=1)).max())
                if extra < 4 and fmax > RELAX_FMAX:
                    stages.append((0.0, 50))
                    extra += 1
    finally:
        orc.set_threads(threads)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    v = rng.normal(0.0, np.sqrt(KT), size=(p.N, 3))
    p.velocity = v - v.mean(axis=0)
    # broken bonds (stretched past r_0 by the relaxation), reported
    g = np.asarray(snap.bonds.group)
    L = np.array(snap.configuration.box[:3])
    d = p.position[g[:, 0]] - p.position[g[:, 1]]
    d -= L * np.rint(d / L)
    broken = int((np.sqrt((d * d).sum(axis=1)) >= QUARTIC["r_0"]).sum())
    info = {"steps": RELAX_STEPS + 50 * extra, "dt": RELAX_DT, "pair_force_caps": list(RELAX_CAPS),
            "uncapped_stages": extra, "max_displacement": RELAX_MAX_DISP, "max_force_after": fmax,
            "broken_bonds": broken, "engine": "oracle (host, FP64)", "state_sha256_16": state_hash(snap)}
    log(f"relaxation: {info['steps']} steps, max |F| {fmax:.1f}, {broken} stretched bonds, "
        f"state {info['state_sha256_16']}")
    return snap, info


def melt_config(N, n_chains, relax, precision):
    """The ``config`` dict both arms print for the melt workload."""
    return {"workload": f"bead-spring melt N={N} PLJ(WCA)+Quartic LangevinFlow(Parabolic)", "N": N,
            "chains": n_chains, "chain_length": CHAIN_LEN, "density": DENSITY, "dt": DT, "r_buff": R_BUFF,
            "relax": relax, "l2": "working set > L2 (no flush needed)",
            "forces": precision,
            "integration": ("64-bit fixed-point positions, float-pair velocities, FP32 kicks"
                            if precision == "fp32" else "f64")}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix=f"azp_clocks_{index}_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        try:
            os.unlink(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


CLOCK_ROLL_S = 0.6


def _roll(eng, seconds):
    """Untimed steps of the workload for about `seconds` (clock sampling under load)."""
    import torch

    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        eng.run_async(20)
        torch.cuda.synchronize()
        n += 20
    return n


def algorithmic_bytes(n_nbr_mean, n_bond_mean, precision="fp32"):
    """Bytes per particle of one fused step launch.

    FP32 forces (64-bit fixed positions, float-pair velocities): reads high
    words 16, low words 16, count 4, list 4 n, bond count 4 + table 8 n_b,
    velocity record 32, tag 4, build shadow 16; writes high words 16, low words
    16, velocity record 32.
    FP64: reads fixed_i 16, count 4, list 4 n, bond count 4 + table 8 n_b, pos 32,
    vel 32, tag 4, build shadow 16; writes pos_next 32, vel 32, fixed_next 16."""
    if precision == "fp32":
        return 16 + 16 + 4 + 4 * n_nbr_mean + 4 + 8 * n_bond_mean + 32 + 4 + 16 + 16 + 16 + 32
    return 16 + 4 + 4 * n_nbr_mean + 4 + 8 * n_bond_mean + 32 + 32 + 4 + 16 + 32 + 32 + 16


def step_bytes(n_particles, n_nbr_mean, n_bond_mean, builds_per_step, precision="fp32"):
    """Algorithmic bytes of one whole timestep: the fused step launch plus the
    list build amortised over the steps between builds, N (16 + 4 n) per build
    (the fixed-point record read once and the list written)."""
    return n_particles * (algorithmic_bytes(n_nbr_mean, n_bond_mean, precision)
                          + builds_per_step * (16 + 4 * n_nbr_mean))


# DRAM traffic of one FP32-force fused step per particle, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum) of the same kernel on the melt at
# N = 700,000, whose step traffic and resident set exceed L2
# (profiles/k_md_step_fx_melt700k.md); scaled to a launch by N
TRAFFIC_BYTES_PER_PARTICLE_FP32 = 183.0


def measured_peak():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline(snap, seconds=15.0):
    """The oracle port (OpenMP, all host cores) on a bounded sample of the same
    workload: the state after the GPU's timed run, full N, one untimed step, then
    full-N steps for about ``seconds`` with the list rebuilt whenever a particle
    moved more than r_buff / 2 (the rebuilds inside the sample are counted); then
    two steps on one thread."""
    from oracle import oracle as orc

    cores = orc.set_threads(os.cpu_count() or 1)
    L = np.array(snap.configuration.box[:3])
    md = _melt_oracle(orc, snap, "langevin", DT, 7, flow_kind=1, flow_p=(2.0 / 3.0, L[1], 0.0))
    md.step()  # includes the first list build
    builds0 = md.builds
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds or steps < 2:
        md.step()
        steps += 1
    per_step = (time.perf_counter() - t0) / steps
    builds = md.builds - builds0
    one = cpu_single_thread(orc, md)
    return {"value": 1.0 / per_step, "unit": "timesteps/s", "cores": cores, "kind": "port",
            "sample": f"N={snap.particles.N} full system from the state after the timed run, {steps} FP64 steps "
                      f"after one untimed step, {builds} list builds inside them; oracle/azp_oracle.cpp, "
                      f"OpenMP {cores} threads",
            "single_thread": {"value": 1.0 / one, "unit": "timesteps/s", "cores": 1,
                              "sample": "2 full-N steps on one thread after the sample"}}


def cpu_single_thread(orc, md, steps=2):
    """Seconds per full-N oracle step on one thread (HOOMD's CPU model: serial per
    MPI rank), over ``steps`` steps of the loop as it stands."""
    threads = orc.set_threads(1)
    try:
        t0 = time.perf_counter()
        md.run(steps)
        return (time.perf_counter() - t0) / steps
    finally:
        orc.set_threads(threads)


def run_reference(args):
    """The reference arm: the CPU oracle port of the path on all host cores."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    import azplugins_gb300 as az  # noqa: F401  (snapshot types only, no GPU work)
    from oracle import oracle as orc

    snap, relax = relaxed_melt(args.chains, seed=1)
    cores = orc.set_threads(os.cpu_count() or 1)
    L = np.array(snap.configuration.box[:3])
    md = _melt_oracle(orc, snap, "langevin", DT, 7, flow_kind=1, flow_p=(2.0 / 3.0, L[1], 0.0))
    # bounded sample: a full-N oracle step takes about 0.1 s on 16 cores, so the
    # warm-up is capped at REF_MAX_WARMUP steps and the timed steps stop after
    # REF_TIME_BOX_S seconds (the rate of full-N steps is what is reported)
    warm = min(args.warmup, REF_MAX_WARMUP)
    md.run(warm)
    builds0 = md.builds
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        md.step()
        done += 1
        if time.perf_counter() - t0 > REF_TIME_BOX_S:
            break
    t = time.perf_counter() - t0
    builds = md.builds - builds0
    v = done / t
    one = cpu_single_thread(orc, md)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "timesteps/s", "n_gpus": args.gpus,
        "steps": done, "warmup": warm, "ms_per_step": 1e3 * t / done, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random-walk melt, "
                                                                        "capped-Brownian relaxed)",
        "config": melt_config(snap.particles.N, args.chains, relax, args.precision),
        "nlist_builds_in_timed_steps": builds,
        "cpu_baseline": {"value": v, "unit": "timesteps/s", "cores": cores, "kind": "port",
                         "sample": f"{done} full-N FP64 steps timed ({args.steps} requested, time box "
                                   f"{REF_TIME_BOX_S:.0f} s) after {warm} warm-up steps, {builds} list builds "
                                   "inside them; oracle/azp_oracle.cpp OpenMP",
                         "single_thread": {"value": 1.0 / one, "unit": "timesteps/s", "cores": 1,
                                           "sample": "2 full-N steps on one thread after the timed steps"}},
        "e2e": {"value": v, "unit": "timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import azplugins_gb300 as az
    from azplugins_gb300 import _lib

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    _lib.load()
    log("relaxing the melt")
    snap, relax = relaxed_melt(args.chains, seed=1 + rank)
    N = snap.particles.N
    L = snap.configuration.box[:3]
    flow = az.flow.ParabolicFlow(mean_velocity=2.0 / 3.0, separation=L[1])
    wca, qb = forces_and_method(az, flow)
    sim = az.Simulation(seed=7 + rank, precision=args.precision)
    sim.create_state_from_snapshot(snap)
    m = az.methods.LangevinFlow("all", kT=KT, flow_field=flow, default_gamma=GAMMA)
    sim.operations.integrator = az.md.Integrator(dt=DT, methods=[m], forces=[wca, qb])
    sim.run(args.warmup)
    log("warm-up done")
    eng = sim._engine
    stream = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        # nvidia-smi polls every 200 ms, longer than a short timed region: the
        # sampler also runs over CLOCK_ROLL_S of the same steps on each side of it
        roll = roll_before = _roll(eng, CLOCK_ROLL_S)
        builds0 = sim.thermo()["nlist_builds"]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("timed")
        start.record(stream)
        eng.run_async(args.steps)
        end.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        if world > 1:
            torch.distributed.barrier()
        ms = start.elapsed_time(end)
        launches = eng.last_launches
        err = eng.error_word()
        if err:
            raise RuntimeError(f"timed region raised device error word 0x{err:x}: measurement invalid")
        builds = sim.thermo()["nlist_builds"] - builds0
        roll += _roll(eng, CLOCK_ROLL_S)
    sim._timestep += args.steps + roll
    sim.state._host_valid = False
    t_max, value = reduce_over_ranks(ms, args.steps, world, "cuda")

    log(f"timed region done: {ms:.1f} ms")
    state_after = sim.state.get_snapshot()
    n_nbr, n_bond, n_cut = neighbour_stats(state_after)
    log("neighbour statistics done")
    accuracy = force_accuracy(eng, state_after, args.precision)
    log("force accuracy done")
    # end to end through the public C ABI with pinned host buffers
    torch.cuda.nvtx.range_push("e2e")
    e2e = e2e_measure(eng, state_after, args.e2e_steps)
    torch.cuda.nvtx.range_pop()
    log("e2e done")
    # dominant kernel alone (last: it advances the state without list checks);
    # its own NVTX range lets a profiler pick these plain launches
    torch.cuda.nvtx.range_push("step_kernel")
    kernel_ms = time_step_kernel(eng, reps=200)
    torch.cuda.nvtx.range_pop()
    log("kernel timing done")
    bytes_per_launch = algorithmic_bytes(n_nbr, n_bond, args.precision) * N
    peak, peak_kind = measured_peak()
    achieved = bytes_per_launch / (kernel_ms * 1e-3) / 1e9

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "timesteps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64",
            "data": "synthetic (seeded random-walk melt, capped-Brownian relaxed)",
            "config": dict(melt_config(N, args.chains, relax, args.precision),
                           parallelism="replicas" if world > 1 else "single GPU"),
            "gpu_launches": int(launches),
            "nlist_builds_in_timed_steps": builds,
            "nlist_builds_per_step": builds / args.steps,
            "step_gbs": step_bytes(N, n_nbr, n_bond, builds / args.steps, args.precision)
            / (t_max / args.steps * 1e-3) / 1e9,
            "pair_interactions_per_s": N * n_cut / (t_max / args.steps * 1e-3),
            "mean_neighbours_in_cut": n_cut,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": (TRAFFIC_BYTES_PER_PARTICLE_FP32 * N if args.precision == "fp32" else None),
                         "traffic_source": "ncu capture at N=700,000 scaled by N (profiles/k_md_step_fx_melt700k.md)",
                         "kernel": ("k_md_step_fx" if args.precision == "fp32" else "k_md_step") + " (fused forces + Langevin step)",
                         "kernel_ms": kernel_ms, "bytes_per_launch": bytes_per_launch,
                         "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", "mean_neighbours": n_nbr,
                         "mean_bonds": n_bond},
            "clocks": dict(clk.summary(), window=f"nvidia-smi every 200 ms over the timed region and {CLOCK_ROLL_S} s "
                           "of the same steps on each side of it"),
            "untimed_steps_before_timed_region": {"warmup": args.warmup, "clock_window": roll_before},
            "accuracy": accuracy,
            "e2e": e2e,
        }
        if not args.no_cpu_baseline:
            log("cpu baseline")
            line["cpu_baseline"] = cpu_baseline(state_after)
        print(json.dumps(line), flush=True)
    sim.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def reduce_over_ranks(ms, steps, world, device="cpu"):
    """Slowest rank's time and the whole-job rate (replicas: every rank advanced
    `steps` timesteps of its own system)."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * steps / (ms * 1e-3)


def neighbour_stats(s):
    from azplugins_gb300 import _compute

    N = s.particles.N
    ex = _compute.exclusions_csr(N, s.bonds.group)
    pos = _compute.device_positions(s)
    sysd = _compute.make_system(s, pos)
    nl = _compute.NeighborList(N, 1, np.array([[RCUT]]), R_BUFF, ex)
    nl.build(sysd)
    n_list = float(nl.counts().astype(np.float64).sum()) / N
    nl.close()
    # the same list without the buffer: the full-list count inside r_cut (pair interactions)
    nl = _compute.NeighborList(N, 1, np.array([[RCUT]]), 0.0, ex)
    nl.build(sysd)
    n_cut = float(nl.counts().astype(np.float64).sum()) / N
    nl.close()
    return n_list, 2.0 * s.bonds.N / N, n_cut


def force_accuracy(eng, snap, precision):
    """The engine's forces (pair + bond, its own precision and list) at the state
    after the timed run against the FP64 oracle at the same positions (all host
    cores): max_i |dF_i| / max(|F_i|, F_rms) over all particles and the relative
    error of the total energy."""
    from oracle import oracle as orc
    from tests.helpers import force_error

    f_eng, _ = eng.forces()
    threads = orc.set_threads(os.cpu_count() or 1)
    try:
        F, U, _ = _melt_oracle(orc, snap, "langevin", DT, 7).forces()
    finally:
        orc.set_threads(threads)
    return {"forces": precision, "reference": "FP64 oracle (oracle/azp_oracle.cpp) at the same state",
            "force_error": force_error(f_eng, F),
            "energy_rel_error": abs(f_eng[:, 3].sum() - U.sum()) / abs(U.sum()),
            "norm": "max_i |dF_i| / max(|F_i|, F_rms), all particles"}


def time_step_kernel(eng, reps):
    import torch

    from azplugins_gb300 import _lib

    L = _lib.load()
    stream = torch.cuda.current_stream()
    s = ctypes.c_void_p(stream.cuda_stream)
    ms = ctypes.c_float(0.0)
    _lib.check(L.azp_md_time_step_kernel(eng._md, reps, ctypes.byref(ms), s), "azp_md_time_step_kernel")
    return ms.value


def e2e_measure(eng, s, steps):
    """Per step: pinned host snapshot -> device, one timestep, device -> pinned host, thermo sums."""
    import torch

    from azplugins_gb300 import _lib

    L = _lib.load()
    p = s.particles
    N = p.N
    pos = torch.empty((N, 4), dtype=torch.float64).pin_memory()
    vel = torch.empty((N, 4), dtype=torch.float64).pin_memory()
    acc = torch.empty((N, 3), dtype=torch.float64).pin_memory()
    img = torch.empty((N, 3), dtype=torch.int32).pin_memory()
    pos[:, :3] = torch.from_numpy(p.position)
    pos[:, 3] = torch.from_numpy(p.typeid.astype(np.float64))
    vel[:, :3] = torch.from_numpy(p.velocity)
    vel[:, 3] = torch.from_numpy(p.mass)
    acc[:] = torch.from_numpy(p.acceleration)
    img[:] = torch.from_numpy(p.image)
    thermo = np.zeros(9)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ts = ctypes.c_uint64(0)

    def one(t):
        _lib.check(L.azp_md_set_state(eng._md, pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), img.data_ptr(), None,
                                      t, 0, stream), "set_state")
        _lib.check(L.azp_md_run(eng._md, 1, stream), "run")
        _lib.check(L.azp_md_get_state(eng._md, pos.data_ptr(), vel.data_ptr(), acc.data_ptr(), img.data_ptr(),
                                      ctypes.byref(ts), 0, stream), "get_state")
        _lib.check(L.azp_md_thermo(eng._md, thermo.ctypes.data, stream), "thermo")

    for t in range(3):
        one(t)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in range(steps):
        one(3 + t)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    h2d = N * (32 + 32 + 24 + 12)
    # where an end-to-end step goes: each call timed alone, synchronised
    parts = {"set_state": 0.0, "run": 0.0, "get_state": 0.0, "thermo": 0.0}
    reps = max(2, min(steps, 10))
    for t in range(reps):
        for name, fn in (("set_state", lambda: L.azp_md_set_state(eng._md, pos.data_ptr(), vel.data_ptr(),
                                                                  acc.data_ptr(), img.data_ptr(), None,
                                                                  1000 + t, 0, stream)),
                         ("run", lambda: L.azp_md_run(eng._md, 1, stream)),
                         ("get_state", lambda: L.azp_md_get_state(eng._md, pos.data_ptr(), vel.data_ptr(),
                                                                  acc.data_ptr(), img.data_ptr(), ctypes.byref(ts),
                                                                  0, stream)),
                         ("thermo", lambda: L.azp_md_thermo(eng._md, thermo.ctypes.data, stream))):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            _lib.check(fn(), name)
            torch.cuda.synchronize()
            parts[name] += (time.perf_counter() - t1) / reps
    breakdown = {f"{k}_ms": 1e3 * v for k, v in parts.items()}
    breakdown["set_state_h2d_gbs"] = h2d / parts["set_state"] / 1e9
    breakdown["get_state_d2h_gbs"] = h2d / parts["get_state"] / 1e9
    return {"value": steps / dt, "unit": "timesteps/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": h2d + 72, "api": "azp_md_set_state / azp_md_run(1) / azp_md_get_state / azp_md_thermo",
            "steps": steps, "breakdown": breakdown,
            "note": "set_state reads the pinned host state in place and rebuilds the list only when a particle lies more than r_buff / 2 from its position at the last build; get_state writes the pinned outputs in place; rates include that"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.suite == "melt":
        run_ours(args)
    else:
        import bench_suites

        bench_suites.run(args)


if __name__ == "__main__":
    main()
