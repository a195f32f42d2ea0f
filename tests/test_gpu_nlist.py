"""GPU neighbour lists are bit-exact against the oracle's brute-force FP64 list
at r_cut + r_buff, compared as sorted sets; exclusions, multi-type cutoffs with
an unlisted type pair, thin boxes (fewer than three cells) and list overflow."""

import numpy as np
import pytest

from helpers import box_of, pos4_of, random_fluid

pytestmark = pytest.mark.gpu


def _gpu_list(snap, rcut, r_buff, exclusions=None, max_neighbors=64):
    from azplugins_gb300 import _compute

    N = snap.particles.N
    ex = None if exclusions is None else _compute.exclusions_csr(N, exclusions)
    pos = _compute.device_positions(snap)
    sysd = _compute.make_system(snap, pos)
    nl = _compute.NeighborList(N, len(snap.particles.types), rcut, r_buff, ex, max_neighbors=max_neighbors)
    nl.build(sysd)
    s, i = nl.to_csr()
    nl.close()
    return s, i


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_single_type_bit_exact(orc, seed):
    snap = random_fluid(3000, 0.8, seed=seed, min_dist=0.7)
    rc = np.array([[2.5]])
    s, i = _gpu_list(snap, rc, 0.4)
    so, io = orc.nlist(pos4_of(snap), snap.particles.typeid, 1, box_of(snap), (rc + 0.4) ** 2, method="brute")
    np.testing.assert_array_equal(s, so)
    np.testing.assert_array_equal(i, io)


def test_boundary_pairs_decided_exactly(orc):
    # pairs placed at |dx| within a few ulps of r_list: FP32 cannot decide them
    rng = np.random.Generator(np.random.PCG64(4))
    import azplugins_gb300 as az

    N = 400
    L = 12.0
    r_list = 1.5
    base = rng.uniform(-0.45, 0.45, size=(N // 2, 3)) * L
    d = rng.normal(size=(N // 2, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    eps = rng.choice([-1, 1], size=(N // 2, 1)) * rng.uniform(0, 4e-16, size=(N // 2, 1)) * r_list
    other = base + d * (r_list + eps)
    pos = np.concatenate([base, other])
    pos -= L * np.floor((pos + 0.5 * L) / L)
    snap = az.Snapshot(N)
    snap.particles.position = pos
    snap.configuration.box = [L, L, L, 0, 0, 0]
    rc = np.array([[1.1]])
    s, i = _gpu_list(snap, rc, 0.4)
    so, io = orc.nlist(pos4_of(snap), snap.particles.typeid, 1, box_of(snap), (rc + 0.4) ** 2, method="brute")
    np.testing.assert_array_equal(s, so)
    np.testing.assert_array_equal(i, io)


def test_multitype_and_exclusions(orc):
    snap = random_fluid(2500, 0.6, seed=5, ntypes=3, min_dist=0.6)
    rc = np.array([[1.2, 2.0, 0.0], [2.0, 3.0, 1.5], [0.0, 1.5, 2.2]])
    N = snap.particles.N
    ex = np.array([[k, k + 1] for k in range(0, N - 1, 2)] + [[k, k + 7] for k in range(0, N - 7, 11)])
    s, i = _gpu_list(snap, rc, 0.3, ex)
    rl = np.where(rc > 0, rc + 0.3, 0.0) ** 2
    so, io = orc.nlist(pos4_of(snap), snap.particles.typeid, 3, box_of(snap), rl, ex, method="brute")
    np.testing.assert_array_equal(s, so)
    np.testing.assert_array_equal(i, io)


@pytest.mark.parametrize("seed", [6, 7])
def test_disparate_cutoffs_subdivided_grid(orc, seed):
    """List radii 1.2 and 4.6 (ratio above 3): the grid is cut to cells of a third
    of the largest radius with a stencil of three cells each way; the sets stay
    those of the brute-force oracle."""
    snap = random_fluid(6000, 0.5, seed=seed, ntypes=2, min_dist=0.6)
    rc = np.array([[0.8, 3.0], [3.0, 4.2]])
    s, i = _gpu_list(snap, rc, 0.4, max_neighbors=256)
    rl = (rc + 0.4) ** 2
    so, io = orc.nlist(pos4_of(snap), snap.particles.typeid, 2, box_of(snap), rl, method="brute")
    np.testing.assert_array_equal(s, so)
    np.testing.assert_array_equal(i, io)


def test_thin_box_and_overflow_regrow(orc):
    import azplugins_gb300 as az

    rng = np.random.Generator(np.random.PCG64(6))
    N = 600
    L = np.array([30.0, 5.2, 6.0])  # y and z hold fewer than three cells
    snap = az.Snapshot(N)
    snap.particles.position = (rng.uniform(-0.5, 0.5, size=(N, 3)) * L)
    snap.configuration.box = [L[0], L[1], L[2], 0, 0, 0]
    rc = np.array([[2.0]])
    s, i = _gpu_list(snap, rc, 0.5, max_neighbors=4)  # far too small: the build grows it
    so, io = orc.nlist(pos4_of(snap), snap.particles.typeid, 1, box_of(snap), (rc + 0.5) ** 2, method="brute")
    np.testing.assert_array_equal(s, so)
    np.testing.assert_array_equal(i, io)


@pytest.mark.parametrize("cells", [(3, 3, 3), (4, 3, 5), (6, 4, 3), (3, 7, 4), (5, 5, 5), (12, 3, 4)])
def test_small_grids_bit_exact(orc, cells):
    """Boxes of 3-12 cells per axis: the stencil's periodic wrap at the faces,
    and axes whose whole extent the stencil covers (every neighbour cell also
    a periodic image of another), against the oracle's brute-force sets."""
    import azplugins_gb300 as az

    rng = np.random.Generator(np.random.PCG64(sum(cells)))
    rc, r_buff = 2.5, 0.4
    rl = rc + r_buff
    L = np.array([c * rl * 1.07 for c in cells])
    N = int(0.6 * np.prod(L))
    snap = az.Snapshot(N)
    snap.particles.position = rng.uniform(-0.5, 0.5, size=(N, 3)) * L
    snap.configuration.box = [L[0], L[1], L[2], 0, 0, 0]
    s, i = _gpu_list(snap, np.array([[rc]]), r_buff, max_neighbors=96)
    so, io = orc.nlist(pos4_of(snap), snap.particles.typeid, 1, box_of(snap), np.array([[rl * rl]]), method="brute")
    np.testing.assert_array_equal(s, so)
    np.testing.assert_array_equal(i, io)


# ---------------------------------------------------------------- melt-density systems
# Larger grids at the bead-spring melt's density, several types, exclusions,
# boundary pairs and crowded clumps. The same bit-exact bar.


def _check(orc, snap, rc, r_buff, ex=None, ntypes=1):
    s, i = _gpu_list(snap, rc, r_buff, ex)
    rl = np.where(rc > 0, rc + r_buff, 0.0) ** 2
    so, io = orc.nlist(pos4_of(snap), snap.particles.typeid, ntypes, box_of(snap), rl, ex)
    np.testing.assert_array_equal(s, so)
    np.testing.assert_array_equal(i, io)


@pytest.mark.parametrize("seed", [7, 8])
def test_melt_density_bit_exact(orc, seed):
    # WCA list radius at melt density: 21 cells per axis
    snap = random_fluid(30000, 0.85, seed=seed, min_dist=0.8)
    _check(orc, snap, np.array([[2 ** (1 / 6)]]), 0.4)


def test_melt_multitype_and_exclusions(orc):
    snap = random_fluid(30000, 0.6, seed=9, ntypes=3, min_dist=0.6)
    rc = np.array([[1.1, 1.3, 0.0], [1.3, 1.5, 1.2], [0.0, 1.2, 1.0]])
    N = snap.particles.N
    ex = np.array([[k, k + 1] for k in range(0, N - 1, 2)] + [[k, k + 13] for k in range(0, N - 13, 7)])
    _check(orc, snap, rc, 0.3, ex, ntypes=3)


def test_melt_boundary_pairs(orc):
    import azplugins_gb300 as az

    rng = np.random.Generator(np.random.PCG64(10))
    N = 20000
    L = 40.0
    r_list = 1.5
    base = rng.uniform(-0.5, 0.5, size=(N // 2, 3)) * L
    d = rng.normal(size=(N // 2, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    eps = rng.choice([-1, 1], size=(N // 2, 1)) * rng.uniform(0, 2e-5, size=(N // 2, 1)) * r_list
    other = base + d * (r_list + eps)
    pos = np.concatenate([base, other])
    pos -= L * np.floor((pos + 0.5 * L) / L)
    snap = az.Snapshot(N)
    snap.particles.position = pos
    snap.configuration.box = [L, L, L, 0, 0, 0]
    _check(orc, snap, np.array([[1.1]]), 0.4)


def test_crowded_clumps(orc):
    # a dense clump overflows the shared-memory staging of its chunks
    import azplugins_gb300 as az

    rng = np.random.Generator(np.random.PCG64(11))
    L = 30.0
    bulk = rng.uniform(-0.5, 0.5, size=(16000, 3)) * L
    clump = rng.normal(scale=1.5, size=(1500, 3)) + np.array([3.0, -2.0, 5.0])
    pos = np.concatenate([bulk, clump])
    pos -= L * np.floor((pos + 0.5 * L) / L)
    snap = az.Snapshot(len(pos))
    snap.particles.position = pos
    snap.configuration.box = [L, L, L, 0, 0, 0]
    s, i = _gpu_list(snap, np.array([[1.0]]), 0.3)
    so, io = orc.nlist(pos4_of(snap), snap.particles.typeid, 1, box_of(snap), np.array([[1.3 ** 2]]))
    np.testing.assert_array_equal(s, so)
    np.testing.assert_array_equal(i, io)
