"""Integration methods in a flow field.

The reference keeps Langevin and Brownian dynamics in a flow field as legacy,
unbuilt C++ classes (``src/TwoStepLangevinFlow.h:30-273``,
``src/TwoStepBrownianFlow.h:30-206``; constructor arguments group, kT, flow
field, seed, use_lambda / lambda, noiseless) whose Python front end was removed
(``CHANGELOG.rst:300-303`` records the v0 ``flow.langevin`` / ``flow.brownian``).
These classes give that integrator a HOOMD-v4-style front end:

* ``filter``: the particles the method integrates, ``"all"`` / ``filter.All()``
  or ``filter.Type(types)`` (the reference's ParticleGroup, src/TwoStepLangevinFlow.h:35;
  particles outside it feel and exert forces but do not move);
* ``gamma[type]`` per-type drag (``default_gamma``), or ``alpha`` for
  gamma = alpha * diameter (the reference's use_lambda / lambda);
* ``kT`` is a float or a variant of the timestep (the reference's
  ``std::shared_ptr<Variant> T``, evaluated at the timestep of step two,
  src/TwoStepLangevinFlow.h:194-219);
* the RNG seed is the Simulation's seed.
"""

from __future__ import annotations

from . import filter as _filter
from .flow import FlowField
from .typeparam import TypeParameterDict
from .variant import Constant, as_variant


class _FlowMethod:
    def __init__(self, filter, kT, flow_field, default_gamma=1.0, alpha=None, noiseless=False):
        if filter in (None, "all"):
            filter = _filter.All()
        if not isinstance(filter, (_filter.All, _filter.Type)):
            raise ValueError("the method's group is filter.All() or filter.Type(types)")
        if not isinstance(flow_field, FlowField):
            raise TypeError("flow_field must be an azplugins_gb300.flow.FlowField")
        self.filter = filter
        self.kT = as_variant(kT)
        self.flow_field = flow_field
        self.noiseless = bool(noiseless)
        self.alpha = None if alpha is None else float(alpha)
        self.gamma = TypeParameterDict(1, scalar=True, name="gamma")
        self.gamma.set_default(default_gamma)

    def _gamma_table(self, types):
        return [self.gamma[t] for t in types]

    def _group_types(self, types):
        """Bit mask of the integrated types (0: every particle)."""
        if isinstance(self.filter, _filter.All):
            return 0
        if len(types) > 32:
            raise ValueError("filter.Type groups need at most 32 particle types")
        mask = 0
        for k, t in enumerate(types):
            if t in self.filter.types:
                mask |= 1 << k
        return mask

    @property
    def kT_constant(self):
        """The temperature when it does not vary, else None."""
        return self.kT.value if isinstance(self.kT, Constant) else None


class LangevinFlow(_FlowMethod):
    """Langevin dynamics relative to a flow field u(r) (velocity Verlet, uniform noise).

    a = (F + R - gamma (v - u(r))) / m with R uniform in [-c, c]^3,
    c = sqrt(6 gamma kT / dt) (``src/TwoStepLangevinFlow.h:194-245``).
    """

    method_id = 0


class BrownianFlow(_FlowMethod):
    """Overdamped Brownian dynamics in a flow field:
    x += (u(x) + (F + R) / gamma) dt (``src/TwoStepBrownianFlow.h:136-178``).

    ``max_displacement`` (default 0 = off) caps each displacement component and
    ``force_cap`` (default 0 = off) caps the magnitude of every pair force; both
    exist for the overlap relaxation of generated configurations.
    """

    method_id = 1

    def __init__(self, filter, kT, flow_field, default_gamma=1.0, alpha=None, noiseless=False, max_displacement=0.0,
                 force_cap=0.0):
        super().__init__(filter, kT, flow_field, default_gamma, alpha, noiseless)
        self.max_displacement = float(max_displacement)
        self.force_cap = float(force_cap)


class ConstantVolume(LangevinFlow):
    """Constant-volume, constant-energy integration (HOOMD ``md.methods.ConstantVolume``
    without a thermostat): velocity Verlet, i.e. the Langevin step above with no
    drag and no noise. A DPDGeneralWeight pair force thermostats it, as in
    ``src/pytest/test_pair_dpd.py``."""

    def __init__(self, filter):
        from .flow import ConstantFlow

        super().__init__(filter, kT=0.0, flow_field=ConstantFlow((0.0, 0.0, 0.0)), default_gamma=0.0, noiseless=True)


__all__ = ["LangevinFlow", "BrownianFlow", "ConstantVolume"]
