"""Timestep-dependent scalars (the part of ``hoomd.variant`` that azplugins'
moving barriers take: ``location`` is ``variant_like``, src/external.py:52-57).

A float becomes a :class:`Constant`; any object with ``__call__(timestep)`` is
accepted as a variant. :class:`Ramp` follows HOOMD's linear ramp.
"""

from __future__ import annotations

import numpy as np


class Variant:
    """Base class: ``variant(timestep) -> float``."""

    def __call__(self, timestep):
        raise NotImplementedError

    def values(self, t0, n):
        """Values at timesteps t0, t0 + 1, ..., t0 + n - 1 (float64 array)."""
        return np.array([float(self(t0 + k)) for k in range(int(n))], dtype=np.float64)


class Constant(Variant):
    def __init__(self, value):
        self.value = float(value)

    def __call__(self, timestep):
        return self.value

    def values(self, t0, n):
        return np.full(int(n), self.value)

    def __repr__(self):
        return f"Constant({self.value!r})"


class Ramp(Variant):
    """A until t_start, then linear to B over t_ramp steps, then B."""

    def __init__(self, A, B, t_start, t_ramp):
        self.A, self.B = float(A), float(B)
        self.t_start, self.t_ramp = int(t_start), int(t_ramp)

    def __call__(self, timestep):
        t = int(timestep)
        if t < self.t_start:
            return self.A
        if t < self.t_start + self.t_ramp:
            s = (t - self.t_start) / self.t_ramp
            return (1.0 - s) * self.A + s * self.B
        return self.B

    def values(self, t0, n):
        t = np.arange(int(t0), int(t0) + int(n), dtype=np.int64)
        s = np.clip((t - self.t_start) / max(self.t_ramp, 1), 0.0, 1.0)
        out = (1.0 - s) * self.A + s * self.B
        out[t < self.t_start] = self.A
        out[t >= self.t_start + self.t_ramp] = self.B
        return out

    def __repr__(self):
        return f"Ramp({self.A!r}, {self.B!r}, {self.t_start!r}, {self.t_ramp!r})"


def as_variant(value):
    """A float becomes Constant; a Variant or any callable of the timestep stays."""
    if isinstance(value, Variant):
        return value
    if callable(value):
        return value
    return Constant(value)
