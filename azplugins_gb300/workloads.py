"""Seeded synthetic configurations with the shapes of the benchmark workloads.

No dataset is involved anywhere: every configuration is generated from a seed
with ``numpy.random.Generator(PCG64(seed))``.
"""

from __future__ import annotations

import numpy as np

from .simulation import Snapshot


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def _wrap(x, L):
    """Wrap positions into [-L/2, L/2) and return the image counts."""
    img = np.floor((x + 0.5 * L) / L).astype(np.int64)
    x = x - img * L
    for d in range(3):
        hi = x[:, d] >= 0.5 * L[d]
        x[hi, d] -= L[d]
        img[hi, d] += 1
        lo = x[:, d] < -0.5 * L[d]
        x[lo, d] += L[d]
        img[lo, d] -= 1
    return x, img.astype(np.int32)


def maxwell_boltzmann(rng, N, kT, mass=1.0):
    v = rng.normal(0.0, np.sqrt(kT / mass), size=(N, 3))
    v -= v.mean(axis=0)
    return v


def lj_fluid(n_side=16, density=0.8, jitter=0.05, kT=1.0, seed=1):
    """Simple-cubic lattice of n_side^3 particles, jittered by U(-jitter, jitter),
    at number density ``density``, Maxwell-Boltzmann velocities (zero momentum)."""
    rng = _rng(seed)
    N = n_side ** 3
    L = (N / density) ** (1.0 / 3.0)
    a = L / n_side
    g = (np.arange(n_side) + 0.5) * a - 0.5 * L
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    pos += rng.uniform(-jitter, jitter, size=pos.shape)
    box = np.array([L, L, L])
    pos, img = _wrap(pos, box)
    s = Snapshot(N)
    p = s.particles
    p.types = ["A"]
    p.position = pos
    p.image = img
    p.velocity = maxwell_boltzmann(rng, N, kT)
    s.configuration.box = [L, L, L, 0.0, 0.0, 0.0]
    return s


def bead_spring_melt(n_chains, chain_length=100, density=0.85, bond_length=0.97, kT=1.0, seed=2):
    """Linear chains as seeded random walks with fixed bond length, at total
    number density ``density``; chain starts uniform in the box. Overlaps are
    expected and must be relaxed (capped Brownian steps) before dynamics."""
    rng = _rng(seed)
    N = n_chains * chain_length
    L = (N / density) ** (1.0 / 3.0)
    box = np.array([L, L, L])
    walk = np.empty((n_chains, chain_length, 3))
    walk[:, 0] = rng.uniform(-0.5 * L, 0.5 * L, size=(n_chains, 3))
    for k in range(1, chain_length):
        d = rng.normal(size=(n_chains, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        walk[:, k] = walk[:, k - 1] + bond_length * d
    pos, img = _wrap(walk.reshape(N, 3), box)
    s = Snapshot(N)
    p = s.particles
    p.types = ["A"]
    p.position = pos
    p.image = img
    p.velocity = maxwell_boltzmann(rng, N, kT)
    s.configuration.box = [L, L, L, 0.0, 0.0, 0.0]
    idx = np.arange(N).reshape(n_chains, chain_length)
    group = np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], axis=1)
    s.resize_bonds(len(group))
    s.bonds.types = ["A-A"]
    s.bonds.group = group
    s.bonds.typeid = np.zeros(len(group), dtype=np.int32)
    return s


def _jittered_lattice(rng, N, L, jitter_frac=0.1):
    """N points on a jittered simple-cubic lattice filling a cube of side L."""
    n = int(np.ceil(N ** (1.0 / 3.0)))
    a = L / n
    g = (np.arange(n) + 0.5) * a - 0.5 * L
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    pts = pts[rng.permutation(len(pts))[:N]]
    pts += rng.uniform(-jitter_frac * a, jitter_frac * a, size=pts.shape)
    box = np.array([L, L, L])
    pts, img = _wrap(pts, box)
    return pts


def yukawa_replicas(n_replicas=256, seed=4, n_min=500, n_max=20000, rho=(0.3, 0.8), kappa=(0.5, 3.0),
                    delta=(0.0, 1.0), r_buff=0.4, kT=1.0):
    """Independent ExpandedYukawa systems of uneven size: N log-uniform in
    [n_min, n_max], density uniform in rho, kappa and delta uniform, r_cut =
    delta + 5 / kappa. A draw whose box is smaller than 2 (r_cut + r_buff), or
    whose delta comes within 0.25 of the closest starting separation (0.9 of the
    jittered lattice spacing; the potential diverges at r = delta), is redrawn
    (kappa, delta) from the same stream; the number of redraws is returned.

    Returns (snapshots, params) with params[r] = dict(epsilon, kappa, delta, r_cut)."""
    rng = _rng(seed)
    snaps, params = [], []
    redraws = 0
    for _ in range(n_replicas):
        N = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        density = rng.uniform(*rho)
        L = (N / density) ** (1.0 / 3.0)
        closest = 0.9 * L / int(np.ceil(N ** (1.0 / 3.0)))
        while True:
            k = rng.uniform(*kappa)
            d = rng.uniform(*delta)
            rc = d + 5.0 / k
            if L >= 2.0 * (rc + r_buff) and d <= closest - 0.25:
                break
            redraws += 1
        s = Snapshot(N)
        s.particles.types = ["A"]
        s.particles.position = _jittered_lattice(rng, N, L, 0.05)
        s.particles.velocity = maxwell_boltzmann(rng, N, kT)
        s.particles.acceleration = np.zeros((N, 3))
        s.configuration.box = [L, L, L, 0.0, 0.0, 0.0]
        snaps.append(s)
        params.append(dict(epsilon=1.0, kappa=k, delta=d, r_cut=rc))
    return snaps, params, redraws


def colloid_mixture(N=262144, colloid_fraction=0.04, colloid_diameter=5.0, solvent_diameter=1.0, phi=0.3, seed=3,
                    kT=1.0):
    """Binary colloid (type C) / solvent (type S) mixture at total volume fraction
    phi, placed without overlaps: colloids on randomly chosen sites of a simple
    cubic lattice, each jittered so that surface gaps stay at least 0.4 solvent
    diameters (colloids at contact would start at a diverging colloid-colloid
    force), then solvent on a jittered grid of spacing 1.1 solvent diameters
    outside the colloids' exclusion shells."""
    rng = _rng(seed)
    nc = int(round(colloid_fraction * N))
    ns = N - nc
    ac, as_ = 0.5 * colloid_diameter, 0.5 * solvent_diameter
    vol = (4.0 / 3.0) * np.pi * (nc * ac ** 3 + ns * as_ ** 3)
    L = (vol / phi) ** (1.0 / 3.0)
    box = np.array([L, L, L])
    cols = np.zeros((0, 3))
    if nc:
        m = int(np.ceil(nc ** (1.0 / 3.0)))
        a = L / m
        gap = a - colloid_diameter
        if gap < 0.4 * solvent_diameter:
            raise ValueError("colloid lattice too tight for this volume fraction")
        jit = 0.5 * (gap - 0.4 * solvent_diameter)
        site = (np.arange(m) + 0.5) * a - 0.5 * L
        X, Y, Z = np.meshgrid(site, site, site, indexing="ij")
        sites = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        cols = sites[rng.permutation(len(sites))[:nc]] + rng.uniform(-jit, jit, size=(nc, 3))
    cols = np.array(cols).reshape(-1, 3)
    # solvent: jittered grid points outside the colloid shells
    sp = 1.1 * solvent_diameter
    n = int(L // sp)
    g = (np.arange(n) + 0.5) * (L / n) - 0.5 * L
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    keep = np.ones((n, n, n), dtype=bool)
    excl = ac + solvent_diameter
    h = L / n
    reach = int(np.ceil(excl / h)) + 1
    off = np.arange(-reach, reach + 1)
    for c in cols:
        # grid cells around the colloid only
        ic = np.floor((c + 0.5 * L) / h - 0.5).astype(int)
        ix = (ic[0] + off) % n
        iy = (ic[1] + off) % n
        iz = (ic[2] + off) % n
        dx = g[ix] - c[0]
        dy = g[iy] - c[1]
        dz = g[iz] - c[2]
        dx -= L * np.rint(dx / L)
        dy -= L * np.rint(dy / L)
        dz -= L * np.rint(dz / L)
        inside = (dx[:, None, None] ** 2 + dy[None, :, None] ** 2 + dz[None, None, :] ** 2) < excl * excl
        sub = keep[np.ix_(ix, iy, iz)]
        keep[np.ix_(ix, iy, iz)] = sub & ~inside
    pts = pts[keep.ravel()]
    if len(pts) < ns:
        raise ValueError("not enough room for the solvent at this volume fraction")
    pts = pts[rng.permutation(len(pts))[:ns]]
    pts += rng.uniform(-0.04, 0.04, size=pts.shape) * (L / n)
    pos, img = _wrap(np.concatenate([pts, cols]), box)
    s = Snapshot(N)
    p = s.particles
    p.types = ["S", "C"]
    p.position = pos
    p.image = img
    p.typeid = np.array([0] * ns + [1] * nc, dtype=np.int32)
    p.diameter = np.where(p.typeid == 1, colloid_diameter, solvent_diameter).astype(np.float64)
    p.velocity = maxwell_boltzmann(rng, N, kT)
    s.configuration.box = [L, L, L, 0.0, 0.0, 0.0]
    return s
