"""External potentials (mirror of ``hoomd.azplugins.external``, ``src/external.py``).

:class:`PlanarHarmonicBarrier` and :class:`SphericalHarmonicBarrier` take the
reference's constructor (``location``: a float or a variant of the timestep) and
per-type ``params`` with the keys ``k`` and ``offset``. Like any HOOMD force they
may sit in ``Integrator.forces`` (the resident engine adds them to the net force
inside its fused step) or be added with ``sim.operations.add`` as a compute whose
``forces`` / ``energies`` / ``virials`` are read. Those properties are evaluated
at ``sim.timestep`` by the drop-in driver (``azp_harmonic_barrier_forces``). The
virial is zero: the reference does not compute it (src/HarmonicBarrier.h:177-179).
"""

from __future__ import annotations

import numpy as np

from . import _lib
from .typeparam import TypeParameterDict
from .variant import as_variant


class HarmonicBarrier:
    """Repulsive harmonic barrier (base class; use a derived type)."""

    _geometry = None

    def __init__(self, location):
        self.location = location
        self.params = TypeParameterDict(1, required=("k", "offset"), name="params")
        self._sim = None

    @property
    def location(self):
        return self._location

    @location.setter
    def location(self, value):
        self._location = as_variant(value)

    @property
    def geometry(self) -> int:
        return _lib.BARRIER_GEOMETRIES[self._geometry]

    def _table(self, types):
        """Host table [ntypes, 2] of (k, offset)."""
        t = np.zeros((len(types), 2))
        for a, name in enumerate(types):
            if name not in self.params:
                raise KeyError(f"{type(self).__name__}.params[{name!r}] is not set")
            d = self.params[name]
            t[a] = (d["k"], d["offset"])
        return t

    def _valid(self, location, L):
        """The evaluator's valid(box) (src/PlanarBarrierEvaluator.h:50-56,
        src/SphericalBarrierEvaluator.h:54-61) for an orthorhombic box."""
        if self._geometry == "planar":
            return -0.5 * L[1] <= location < 0.5 * L[1]
        return location >= 0.0 and all(Ld >= 2.0 * location for Ld in L)

    def _location_at(self, timestep, L):
        """The location at ``timestep``; raises like HarmonicBarrier::makeEvaluator
        (src/HarmonicBarrier.h:121-130) when it is outside the box."""
        loc = float(self._location(int(timestep)))
        if not self._valid(loc, L):
            raise RuntimeError("Barrier position is invalid")
        return loc

    # ------------------------------------------------------------------ results
    def _compute(self):
        if self._sim is None:
            raise RuntimeError("attach the force to a Simulation (sim.run(0)) before reading results")
        from . import _compute

        return _compute.barrier_forces(self._sim.state, self, self._sim.precision, self._sim.timestep)

    @property
    def forces(self):
        return self._compute()[0][:, :3].copy()

    @property
    def energies(self):
        return self._compute()[0][:, 3].copy()

    @property
    def energy(self):
        return float(self._compute()[0][:, 3].sum())

    @property
    def virials(self):
        return self._compute()[1].copy()


class PlanarHarmonicBarrier(HarmonicBarrier):
    """Planar barrier with normal +y (src/PlanarBarrierEvaluator.h): particles above
    y = H + offset are pushed in -y with U = k/2 (y - H - offset)^2; H = ``location``."""

    _geometry = "planar"


class SphericalHarmonicBarrier(HarmonicBarrier):
    """Spherical barrier (src/SphericalBarrierEvaluator.h): particles beyond
    r = R + offset are pushed inward with U = k/2 (r - R - offset)^2; R = ``location``."""

    _geometry = "spherical"
