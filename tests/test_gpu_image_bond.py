"""ImageHarmonic bond on the GPU (azp_bond_forces with AZP_BOND_IMAGE_HARMONIC):
the reference test's cases through the Python front end
(src/pytest/test_bond.py:240-309, 4 decimals as there) in both precisions, and
random chains whose bonds span more than half the box against the oracle's
image-unwrapped bond loop (FP64 1e-12, FP32 1e-5 norm-wise, energies and
virials), and the same chains advanced by the resident engine (Langevin with
noise, with and without a Hertz pair force that excludes bonded pairs) against
the oracle's MD loop: unwrapped positions and velocities after 30 steps
(FP64 1e-9 / 1e-8, FP32 2e-4 / 2e-3) and forces at the engine's end state
(FP64 1e-12, FP32 1e-5)."""

import numpy as np
import pytest

import azplugins_gb300 as az
from helpers import force_error, image_chains, load_golden, oracle_system

pytestmark = pytest.mark.gpu
CASES = load_golden("kats.json")["image_bond"]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['image_1']}-{c['image_2']}")
def test_reference_cases(case, precision):
    s = az.Snapshot(2)
    s.configuration.box = [5, 5, 5, 0, 0, 0]
    s.particles.position = np.array([case["position_1"], case["position_2"]], dtype=float)
    s.particles.image = np.array([case["image_1"], case["image_2"]], dtype=np.int32)
    s.resize_bonds(1)
    s.bonds.group = np.array([[0, 1]], dtype=np.int64)
    s.bonds.typeid = np.array([0], dtype=np.int32)
    s.bonds.types = ["A-A"]
    sim = az.Simulation(precision=precision)
    sim.create_state_from_snapshot(s)
    harmonic = az.bond.ImageHarmonic()
    harmonic.params["A-A"] = dict(k=2.0, r0=1.0)
    m = az.methods.LangevinFlow("all", kT=0.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=0.0)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[m], forces=[harmonic])
    sim.run(0)
    box = np.array([5.0, 5.0, 5.0])
    u1 = np.array(case["position_1"]) + np.array(case["image_1"]) * box
    u2 = np.array(case["position_2"]) + np.array(case["image_2"]) * box
    d = np.linalg.norm(u2 - u1)
    e = (d - 1) ** 2
    np.testing.assert_array_almost_equal(harmonic.energies, [0.5 * e, 0.5 * e], decimal=4)
    fv = -2 * (d - 1) * (-(u2 - u1) / d)
    np.testing.assert_array_almost_equal(harmonic.forces, [fv, -fv], decimal=4)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_chains_match_oracle(orc, precision, tol):
    rng = np.random.Generator(np.random.PCG64(111))
    n_chains, length = 300, 12
    L = np.array([6.0, 7.0, 5.0])
    N = n_chains * length
    # random walks with steps of 0.9-1.4 in unwrapped space, then wrapped
    steps = rng.normal(size=(n_chains, length, 3))
    steps *= rng.uniform(0.9, 1.4, size=(n_chains, length, 1)) / np.linalg.norm(steps, axis=2, keepdims=True)
    # some bonds longer than half the box
    steps[:, ::4] *= 3.5
    un = np.cumsum(steps, axis=1).reshape(N, 3) + rng.uniform(-20, 20, size=(n_chains, 1, 3)).repeat(length, 1).reshape(N, 3)
    img = np.floor((un + 0.5 * L) / L).astype(np.int32)
    pos = un - img * L
    bonds = np.array([[c * length + k, c * length + k + 1] for c in range(n_chains) for k in range(length - 1)])
    btypes = rng.integers(0, 2, size=len(bonds)).astype(np.int32)
    s = az.Snapshot(N)
    s.configuration.box = [*L, 0, 0, 0]
    s.particles.position = pos
    s.particles.image = img
    s.resize_bonds(len(bonds))
    s.bonds.group = bonds
    s.bonds.typeid = btypes
    s.bonds.types = ["A-A", "A-B"]
    sim = az.Simulation(precision=precision)
    sim.create_state_from_snapshot(s)
    ih = az.bond.ImageHarmonic()
    ih.params["A-A"] = dict(k=30.0, r0=1.0)
    ih.params["A-B"] = dict(k=5.0, r0=1.5)
    m = az.methods.LangevinFlow("all", kT=0.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=0.0)
    sim.operations.integrator = az.md.Integrator(dt=0.001, methods=[m], forces=[ih])
    sim.run(0)
    rec = np.zeros((2, 8))
    rec[0, :2] = [30.0, 1.0]
    rec[1, :2] = [5.0, 1.5]
    F, U, W = orc.image_bond_forces(np.concatenate([pos, np.zeros((N, 1))], axis=1), img, L, bonds, btypes,
                                    "ImageHarmonic", rec)
    assert (np.linalg.norm(un[bonds[:, 1]] - un[bonds[:, 0]], axis=1) > 0.5 * L.min()).sum() > 100
    f = np.concatenate([ih.forces, ih.energies[:, None]], axis=1)
    w = ih.virials
    assert force_error(f, F) < tol
    assert np.abs(f[:, 3] - U).max() <= tol * np.abs(U).max()
    assert np.abs(w - W).max() <= tol * np.abs(W).max()


def _engine_chains(orc, precision, with_pair, steps=30):
    pos, img, un, bonds, btypes, L = image_chains(n_chains=200, L=(9.0, 10.0, 8.0))
    N = len(pos)
    rng = np.random.Generator(np.random.PCG64(7))
    s = az.Snapshot(N)
    s.configuration.box = [*L, 0, 0, 0]
    s.particles.position = pos
    s.particles.image = img
    s.particles.velocity = rng.normal(0.0, 1.0, size=(N, 3))
    s.particles.acceleration = np.zeros((N, 3))
    s.resize_bonds(len(bonds))
    s.bonds.group = bonds
    s.bonds.typeid = btypes
    s.bonds.types = ["A-A", "A-B"]
    ih = az.bond.ImageHarmonic()
    ih.params["A-A"] = dict(k=30.0, r0=1.0)
    ih.params["A-B"] = dict(k=5.0, r0=1.5)
    forces = [ih]
    pair = None
    if with_pair:
        # a soft repulsion between non-bonded beads (bonded pairs excluded, as
        # HOOMD's nlist exclusions=("bond",)): Hertz stays finite at r = 0, so
        # the randomly placed chains start without a blow-up
        pair = az.pair.Hertz(nlist=az.nlist.Cell(buffer=0.4, exclusions=("bond",)), default_r_cut=0.8)
        pair.params[("A", "A")] = dict(epsilon=5.0)
        forces.append(pair)
    m = az.methods.LangevinFlow("all", kT=1.0, flow_field=az.flow.ConstantFlow((0.0, 0.0, 0.0)), default_gamma=1.0)
    sim = az.Simulation(seed=21, precision=precision)
    sim.create_state_from_snapshot(s)
    sim.operations.integrator = az.md.Integrator(dt=0.002, methods=[m], forces=forces)
    sim.run(steps // 2)
    sim.run(steps - steps // 2)
    rec = np.zeros((2, 8))
    rec[0, :2] = [30.0, 1.0]
    rec[1, :2] = [5.0, 1.5]
    kw = dict(bond=dict(name="ImageHarmonic", params=rec), method="langevin", gamma=[1.0], kT=1.0, dt=0.002, seed=21)
    if pair is not None:
        prec, prc, _ = pair._tables(["A"])
        kw["pair"] = dict(name="Hertz", params=prec, rcut=prc, mode="none")
        kw["r_buff"] = 0.4
    md = orc.OracleMD(oracle_system(s, s.particles.acceleration), **kw)
    md.run(steps)
    return sim, md, L, kw, img


@pytest.mark.parametrize("with_pair", [False, True], ids=["bonds", "bonds+hertz"])
@pytest.mark.parametrize("precision,ptol,vtol,ftol", [("fp64", 1e-9, 1e-8, 1e-12), ("fp32", 2e-4, 2e-3, 1e-5)])
def test_engine_chains_match_oracle(orc, precision, ptol, vtol, ftol, with_pair):
    sim, md, L, kw, img0 = _engine_chains(orc, precision, with_pair)
    snap = sim.state.get_snapshot()
    out = snap.particles
    ue = out.position + out.image * L
    uo = md.s["pos4"][:, :3] + md.s["image"] * L
    assert np.abs(ue - uo).max() < ptol
    assert np.abs(out.velocity - md.s["vel4"][:, :3]).max() < vtol
    assert np.abs(out.image - img0).sum() > 10  # particles crossed the faces during the run
    # forces at the engine's own end state (its positions and images)
    at_end = orc.OracleMD(oracle_system(snap), **kw)
    f, _ = sim._engine.forces()
    F, U, _ = at_end.forces()
    assert force_error(f, F) < ftol
    assert np.abs(f[:, 3].sum() - U.sum()) <= ftol * np.abs(U).sum()
