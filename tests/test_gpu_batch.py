"""Batched replicas (one fused launch per step for all replicas) against the
oracle's MD loop run replica by replica, against the same replicas run one by one
through the single-system engine, and the autotuner keeping the state intact."""

import numpy as np
import pytest

import azplugins_gb300 as az

pytestmark = pytest.mark.gpu


def _replicas(n, seed, n_max=2500):
    from azplugins_gb300 import workloads

    return workloads.yukawa_replicas(n, seed=seed, n_min=300, n_max=n_max)


def _single(snap, prm, seed, steps, precision, dt=0.002):
    sim = az.Simulation(seed=seed, precision=precision)
    sim.create_state_from_snapshot(snap)
    pot = az.pair.ExpandedYukawa(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=prm["r_cut"])
    pot.params[("A", "A")] = dict(epsilon=prm["epsilon"], kappa=prm["kappa"], delta=prm["delta"])
    m = az.methods.LangevinFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0, 0, 0)), default_gamma=1.0)
    sim.operations.integrator = az.md.Integrator(dt=dt, methods=[m], forces=[pot])
    sim.run(steps)
    out = sim.state.get_snapshot().particles
    sim.close()
    return out


def _pos_err(a, b, L):
    d = a - b
    d -= L * np.rint(d / L)
    return float(np.abs(d).max())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-4)])
def test_batch_equals_separate_runs(precision, tol):
    from azplugins_gb300.batch import ReplicaBatch

    snaps, params, _ = _replicas(6, seed=51)
    seeds = [100 + r for r in range(len(snaps))]
    b = ReplicaBatch(snaps, az.pair.ExpandedYukawa, [dict(epsilon=p["epsilon"], kappa=p["kappa"], delta=p["delta"])
                                                     for p in params],
                     [p["r_cut"] for p in params], seeds, dt=0.002, precision=precision)
    b.run(40)
    arrays = b.get_arrays()
    for r, (s, p) in enumerate(zip(snaps, params)):
        one = _single(s, p, seeds[r], 40, precision)
        pos, vel, acc, img = b.replica(r, arrays)
        L = np.array(s.configuration.box[:3])
        assert _pos_err(pos, one.position, L) < tol, r
        assert np.abs(vel - one.velocity).max() < 10 * tol, r
    assert b.last_launches > 0
    b.close()


def test_autotune_restores_state():
    from azplugins_gb300.batch import ReplicaBatch

    snaps, params, _ = _replicas(12, seed=52)
    b = ReplicaBatch(snaps, az.pair.ExpandedYukawa, [dict(epsilon=p["epsilon"], kappa=p["kappa"], delta=p["delta"])
                                                     for p in params],
                     [p["r_cut"] for p in params], list(range(12)), dt=0.002)
    before = b.get_arrays()
    res = b.autotune(candidates=(1, 2, 4), steps=5, repeats=1)
    assert set(res) == {1, 2, 4} and all(v > 0 for v in res.values())
    after = b.get_arrays()
    for x, y in zip(before, after):
        assert np.array_equal(np.sort(x, axis=0), np.sort(y, axis=0))
    b.run(10)
    b.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-4)])
def test_batch_replicas_match_oracle(orc, precision, tol):
    """Every replica of the batch against the oracle's HOOMD-order Langevin loop
    (ExpandedYukawa, its own box, parameters and seed; 40 steps at dt = 0.002):
    positions to 1e-9 (FP64 forces) or 1e-4 (FP32 forces), velocities to 10x
    that, the same list builds decided the same way."""
    from azplugins_gb300.batch import ReplicaBatch
    from helpers import oracle_system

    snaps, params, _ = _replicas(6, seed=53)
    seeds = [200 + r for r in range(len(snaps))]
    b = ReplicaBatch(snaps, az.pair.ExpandedYukawa, [dict(epsilon=p["epsilon"], kappa=p["kappa"], delta=p["delta"])
                                                     for p in params],
                     [p["r_cut"] for p in params], seeds, dt=0.002, precision=precision)
    b.run(40)
    arrays = b.get_arrays()
    for r, (s, p) in enumerate(zip(snaps, params)):
        rec = orc.pair_params("ExpandedYukawa", dict(epsilon=p["epsilon"], kappa=p["kappa"], delta=p["delta"]))
        acc = s.particles.acceleration if s.particles.acceleration is not None else np.zeros((s.particles.N, 3))
        md = orc.OracleMD(oracle_system(s, acc),
                          pair=dict(name="ExpandedYukawa", params=rec.reshape(1, 1, 4), rcut=np.array([[p["r_cut"]]])),
                          gamma=[1.0], kT=1.0, dt=0.002, seed=seeds[r])
        md.run(40)
        pos, vel, _, img = b.replica(r, arrays)
        L = np.array(s.configuration.box[:3])
        assert _pos_err(pos, md.s["pos4"][:, :3], L) < tol, r
        assert np.abs(vel - md.s["vel4"][:, :3]).max() < 10 * tol, r
        if precision == "fp64":
            assert np.array_equal(img, md.s["image"]), r
    b.close()



def test_autotune_over_block_sizes():
    """The autotuner's second knob: every (threads per particle, block size)
    pair is timed and the best one is kept; the block size does not change any
    particle's arithmetic, so fresh runs at 128, 256 and 512 threads per block
    agree to the FP64 tolerance of the batch tests (not bit for bit: cells of more
    than 512 particles, which the large-cutoff replicas have, keep the order in
    which the binning atomics placed their members, so the list order can differ
    between runs)."""
    from azplugins_gb300.batch import ReplicaBatch

    snaps, params, _ = _replicas(8, seed=54)
    args = ([dict(epsilon=p["epsilon"], kappa=p["kappa"], delta=p["delta"]) for p in params],
            [p["r_cut"] for p in params], list(range(8)))
    b = ReplicaBatch(snaps, az.pair.ExpandedYukawa, *args, dt=0.002, precision="fp64")
    res = b.autotune(candidates=(1, 2), steps=4, repeats=1, blocks=(128, 512))
    assert set(res) == {(1, 128), (2, 128), (1, 512), (2, 512)} and all(v > 0 for v in res.values())
    assert (b.tpp, b.block) == min(res, key=res.get)
    b.close()
    out = []
    for block in (128, 256, 512):
        r = ReplicaBatch(snaps, az.pair.ExpandedYukawa, *args, dt=0.002, precision="fp64")
        r.set_tpp(2)
        r.set_block(block)
        r.run(20)
        out.append(r.get_arrays())
        r.close()
    for other in out[1:]:
        assert np.abs(other[0][:, :3] - out[0][0][:, :3]).max() < 1e-9
        assert np.abs(other[1][:, :3] - out[0][1][:, :3]).max() < 1e-8
