"""Shared helpers of the test suite: systems, oracle adapters, error norms."""

from __future__ import annotations

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def two_particle_snapshot(d, L, types=("A",)):
    """HOOMD's two_particle_snapshot_factory: particles at (-d/2,0,0), (d/2,0,0)."""
    import azplugins_gb300 as az

    s = az.Snapshot(2)
    s.particles.types = list(types)
    s.particles.position = np.array([[-0.5 * d, 0.0, 0.0], [0.5 * d, 0.0, 0.0]])
    s.configuration.box = [L, L, L, 0.0, 0.0, 0.0]
    return s


def pos4_of(snap):
    p = snap.particles
    return np.ascontiguousarray(np.concatenate([p.position, np.asarray(p.typeid, dtype=float)[:, None]], axis=1))


def box_of(snap):
    return np.array(snap.configuration.box[:3], dtype=np.float64)


def force_error(F, Fref):
    """max_i |F_i - Fref_i| / max(|Fref_i|, F_rms)."""
    F = np.asarray(F)[:, :3]
    Fref = np.asarray(Fref)[:, :3]
    mag = np.sqrt((Fref ** 2).sum(axis=1))
    rms = np.sqrt((mag ** 2).mean()) if len(mag) else 1.0
    den = np.maximum(mag, max(rms, 1e-300))
    return float((np.sqrt(((F - Fref) ** 2).sum(axis=1)) / den).max()) if len(F) else 0.0


def rel(a, b):
    a, b = float(a), float(b)
    return abs(a - b) / max(abs(b), 1e-300)


def random_fluid(N, density, seed, ntypes=1, min_dist=0.85):
    """Random positions with a minimum separation (grid rejection), tag order."""
    import azplugins_gb300 as az

    rng = np.random.Generator(np.random.PCG64(seed))
    L = (N / density) ** (1.0 / 3.0)
    # jittered lattice is the robust way to a dense, overlap-free start
    n = int(np.ceil(N ** (1.0 / 3.0)))
    a = L / n
    g = (np.arange(n) + 0.5) * a - 0.5 * L
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    pts = pts[rng.permutation(len(pts))[:N]]
    jit = max(0.0, 0.5 * (a - min_dist))
    pts = pts + rng.uniform(-jit, jit, size=pts.shape)
    pts = pts - L * np.floor((pts + 0.5 * L) / L)
    s = az.Snapshot(N)
    s.particles.types = [chr(ord("A") + t) for t in range(ntypes)]
    s.particles.position = pts
    s.particles.typeid = rng.integers(0, ntypes, size=N).astype(np.int32)
    s.particles.velocity = rng.normal(size=(N, 3))
    s.particles.velocity -= s.particles.velocity.mean(axis=0)
    s.particles.mass = rng.uniform(0.8, 1.5, size=N)
    s.configuration.box = [L, L, L, 0.0, 0.0, 0.0]
    return s


def oracle_system(snap, accel=None):
    p = snap.particles
    N = p.N
    b = snap.bonds
    return dict(
        pos4=pos4_of(snap),
        vel4=np.ascontiguousarray(np.concatenate([p.velocity, p.mass[:, None]], axis=1)),
        accel=np.zeros((N, 3)) if accel is None else np.array(accel, dtype=np.float64),
        image=np.ascontiguousarray(p.image, dtype=np.int32),
        types=np.ascontiguousarray(p.typeid, dtype=np.int32),
        tags=np.arange(N, dtype=np.uint32),
        L=box_of(snap),
        ntypes=len(p.types),
        bonds=np.asarray(b.group, dtype=np.int32) if b.N else None,
        btypes=np.asarray(b.typeid, dtype=np.int32) if b.N else None,
    )


def pair_tables(orc, name, params_by_pair, types, rcut_by_pair, ron_by_pair=None):
    nt = len(types)
    rec = np.zeros((nt, nt, 4))
    rc = np.zeros((nt, nt))
    ro = np.zeros((nt, nt))
    for a in range(nt):
        for b in range(nt):
            key = tuple(sorted((types[a], types[b])))
            rec[a, b] = orc.pair_params(name, params_by_pair[key])
            rc[a, b] = rcut_by_pair[key]
            if ron_by_pair is not None:
                ro[a, b] = ron_by_pair[key]
    return rec, rc, ro


def image_chains(seed=111, n_chains=300, length=12, L=(6.0, 7.0, 5.0)):
    """Random bead chains drawn in unwrapped space (bond lengths 0.9-1.4, every
    fourth bond 3.5x longer, so that many bonds span more than half the box),
    wrapped into the box with image counts, two bond types.

    Returns (pos [N,3], img [N,3] int32, unwrapped [N,3], bonds [B,2], btypes [B], L [3])."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = np.asarray(L, dtype=np.float64)
    N = n_chains * length
    steps = rng.normal(size=(n_chains, length, 3))
    steps *= rng.uniform(0.9, 1.4, size=(n_chains, length, 1)) / np.linalg.norm(steps, axis=2, keepdims=True)
    steps[:, ::4] *= 3.5
    un = np.cumsum(steps, axis=1).reshape(N, 3) + rng.uniform(-20, 20, size=(n_chains, 1, 3)).repeat(length, 1).reshape(
        N, 3)
    img = np.floor((un + 0.5 * L) / L).astype(np.int32)
    pos = un - img * L
    bonds = np.array([[c * length + k, c * length + k + 1] for c in range(n_chains) for k in range(length - 1)])
    btypes = rng.integers(0, 2, size=len(bonds)).astype(np.int32)
    return pos, img, un, bonds, btypes, L


def oracle_walls(pot):
    """Rows of a wall potential's walls in the oracle's layout: spheres [n, 6],
    cylinders [n, 9], planes [n, 7]."""
    from azplugins_gb300.wall import Cylinder, Plane, Sphere

    return (np.array([w._row() for w in pot.walls if isinstance(w, Sphere)]).reshape(-1, 6),
            np.array([w._row() for w in pot.walls if isinstance(w, Cylinder)]).reshape(-1, 9),
            np.array([w._row() for w in pot.walls if isinstance(w, Plane)]).reshape(-1, 7))
