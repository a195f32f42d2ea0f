"""Flow fields (mirror of ``hoomd.azplugins.flow``, ``src/flow.py:13-92``).

``ConstantFlow(velocity)``: u(r) = U (``src/ConstantFlow.h:48-51``).
``ParabolicFlow(mean_velocity, separation)``: u_x(y) = 1.5 U [1 - (y / H)^2]
with H = separation / 2, gradient along y (``src/ParabolicFlow.h:69-93``).
Both are plain value objects, picklable, and are passed by value to the
integrator kernels as an ``azp_flow`` record.
"""

from __future__ import annotations

from . import _lib


class FlowField:
    """Base flow field."""

    def _record(self):
        raise NotImplementedError

    def __eq__(self, other):
        return type(self) is type(other) and self.__dict__ == other.__dict__

    def __repr__(self):
        args = ", ".join(f"{k.lstrip('_')}={v!r}" for k, v in self.__dict__.items())
        return f"{type(self).__name__}({args})"


class ConstantFlow(FlowField):
    """Constant flow profile, independent of position."""

    def __init__(self, velocity):
        self.velocity = velocity

    @property
    def velocity(self):
        return self._velocity

    @velocity.setter
    def velocity(self, v):
        v = tuple(float(x) for x in v)
        if len(v) != 3:
            raise ValueError("velocity must have three components")
        self._velocity = v

    def __call__(self, r):
        return self._velocity

    def _record(self):
        f = _lib.Flow()
        f.kind = _lib.FLOW_CONSTANT
        for d in range(3):
            f.p[d] = self._velocity[d]
        return f


class ParabolicFlow(FlowField):
    """Parabolic (plane Poiseuille) flow along x between plates at y = +/- separation/2."""

    def __init__(self, mean_velocity, separation):
        self.mean_velocity = mean_velocity
        self.separation = separation

    @property
    def mean_velocity(self):
        return self._mean_velocity

    @mean_velocity.setter
    def mean_velocity(self, v):
        self._mean_velocity = float(v)

    @property
    def separation(self):
        return self._separation

    @separation.setter
    def separation(self, v):
        self._separation = float(v)

    def __call__(self, r):
        umax = 1.5 * self._mean_velocity
        yr = r[1] / (0.5 * self._separation)
        return (umax * (1.0 - yr * yr), 0.0, 0.0)

    def _record(self):
        f = _lib.Flow()
        f.kind = _lib.FLOW_PARABOLIC
        f.p[0] = self._mean_velocity
        f.p[1] = self._separation
        f.p[2] = 0.0
        return f
