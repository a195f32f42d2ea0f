"""Computes (mirror of ``hoomd.azplugins.compute``, ``src/compute.py``):
:class:`VelocityCompute` (centre-of-mass velocity of a group) and the binned
mass-averaged velocity fields :class:`CartesianVelocityFieldCompute` and
:class:`CylindricalVelocityFieldCompute`, with the reference's constructor
arguments, properties and array shapes.

They are added with ``sim.operations.add`` and evaluated on the GPU by the
drop-in compute ``azp_vfield_*`` at the current state. MPCD particles do not
exist in this package: ``include_mpcd_particles`` is accepted and reported but
adds nothing.
"""

from __future__ import annotations

import ctypes
import itertools

import numpy as np

from . import _lib
from .filter import ParticleFilter


class DataAccessError(RuntimeError):
    """A computed quantity read before the compute is attached and run."""

    def __init__(self, name):
        super().__init__(f"{name} is not available before the compute is attached to a simulation that has run")


class _Compute:
    def __init__(self, filter, include_mpcd_particles):  # noqa: A002
        if filter is not None and not isinstance(filter, ParticleFilter):
            raise TypeError("filter must be a ParticleFilter or None")
        self._filter = filter
        self._include_mpcd = bool(include_mpcd_particles)
        self._sim = None

    @property
    def filter(self):
        return self._filter

    @property
    def include_mpcd_particles(self):
        return self._include_mpcd

    def _state(self, name):
        sim = self._sim
        if sim is None or sim.state is None or not sim._has_run:
            raise DataAccessError(name)
        return sim.state

    def _evaluate(self, kind, num_bins, lower, upper, name):
        """(mass [nb], momentum [nb, 3], velocity [nb, 3]) of the members on the GPU."""
        from . import _compute

        state = self._state(name)
        snap = state._arrays()
        members = None if self._filter is None else self._filter.members(snap)
        if self._filter is None:
            members = np.zeros(0, dtype=np.uint32)  # no HOOMD particles selected
        return _compute.velocity_field(snap, kind, num_bins, lower, upper, members)


class VelocityCompute(_Compute):
    """Centre-of-mass velocity sum(m v) / sum(m) of a group (``src/VelocityCompute.h``)."""

    def __init__(self, filter=None, include_mpcd_particles=False):  # noqa: A002
        super().__init__(filter, include_mpcd_particles)

    @property
    def velocity(self):
        _, _, v = self._evaluate(_lib.BINNING_KINDS["cartesian"], (0, 0, 0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0),
                                 "velocity")
        return tuple(float(x) for x in v[0])


class VelocityFieldCompute(_Compute):
    """Binned mass-averaged velocity (base class; use a derived type)."""

    _kind = None

    def __init__(self, num_bins, lower_bounds, upper_bounds, filter=None, include_mpcd_particles=False):  # noqa: A002
        super().__init__(filter, include_mpcd_particles)
        self.num_bins = num_bins
        self.lower_bounds = lower_bounds
        self.upper_bounds = upper_bounds

    @property
    def num_bins(self):
        return self._num_bins

    @num_bins.setter
    def num_bins(self, v):
        v = tuple(int(x) for x in v)
        if len(v) != 3 or any(x < 0 for x in v):
            raise ValueError("num_bins is three non-negative integers")
        self._num_bins = v

    @property
    def lower_bounds(self):
        return self._lower

    @lower_bounds.setter
    def lower_bounds(self, v):
        v = tuple(float(x) for x in v)
        if len(v) != 3:
            raise ValueError("lower_bounds is three numbers")
        self._lower = v

    @property
    def upper_bounds(self):
        return self._upper

    @upper_bounds.setter
    def upper_bounds(self, v):
        v = tuple(float(x) for x in v)
        if len(v) != 3:
            raise ValueError("upper_bounds is three numbers")
        self._upper = v

    def _shape(self):
        return [n for n in self._num_bins if n > 0]

    @property
    def coordinates(self):
        """Bin centres (src/compute.py:202-230): None without binned coordinates,
        a 1-D array for one, else an array [n_1, ..., n_k, k]."""
        coords, shape = [], []
        for n, lo, hi in zip(self._num_bins, self._lower, self._upper):
            if n > 0:
                x, dx = np.linspace(lo, hi, n, endpoint=False, retstep=True)
                coords.append(x + 0.5 * dx)
                shape.append(n)
        if not shape:
            return None
        if len(shape) > 1:
            shape.append(len(shape))
        return np.reshape(list(itertools.product(*coords)), shape)

    @property
    def velocities(self):
        """Mass-averaged velocity per bin, shaped [n_1, ..., n_k, 3]."""
        _, _, v = self._evaluate(_lib.BINNING_KINDS[self._kind], self._num_bins, self._lower, self._upper,
                                 "velocities")
        return v.reshape(self._shape() + [3])


class CartesianVelocityFieldCompute(VelocityFieldCompute):
    """Velocity field binned in (x, y, z) (``src/CartesianBinningOperation.h``)."""

    _kind = "cartesian"


class CylindricalVelocityFieldCompute(VelocityFieldCompute):
    """Velocity field binned in (r, theta, z), 0 <= theta < 2 pi, velocities as
    (v_r, v_theta, v_z) (``src/CylindricalBinningOperation.h``)."""

    _kind = "cylindrical"
