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
