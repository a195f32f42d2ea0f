"""Particle filters (the part of ``hoomd.filter`` the computes take):
``All()`` and ``Type(types)``; a filter maps a snapshot to member indices."""

from __future__ import annotations

import numpy as np


class ParticleFilter:
    def members(self, snap):
        raise NotImplementedError


class All(ParticleFilter):
    def members(self, snap):
        return np.arange(snap.particles.N, dtype=np.uint32)

    def __eq__(self, other):
        return isinstance(other, All)

    def __hash__(self):
        return hash("All")

    def __repr__(self):
        return "All()"


class Type(ParticleFilter):
    def __init__(self, types):
        self.types = tuple([types] if isinstance(types, str) else types)

    def members(self, snap):
        names = list(snap.particles.types)
        ids = [names.index(t) for t in self.types if t in names]
        return np.flatnonzero(np.isin(snap.particles.typeid, ids)).astype(np.uint32)

    def __eq__(self, other):
        return isinstance(other, Type) and set(other.types) == set(self.types)

    def __hash__(self):
        return hash(("Type", frozenset(self.types)))

    def __repr__(self):
        return f"Type({list(self.types)!r})"
