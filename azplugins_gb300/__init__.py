"""azplugins_gb300 -- GB300-native (sm_103a) short-range force-and-integrate path
with azplugins' operator API.

Submodules mirror ``hoomd.azplugins``: :mod:`pair`, :mod:`bond`, :mod:`flow`,
plus :mod:`methods` (Langevin / Brownian dynamics in a flow field), :mod:`nlist`
and the small HOOMD-style host layer in :mod:`simulation`. All compute runs in
hand-written CUDA kernels through the C ABI declared in
``include/azplugins_gb300.h``; there is no CPU path.
"""

from . import bond, compute, external, filter, flow, methods, nlist, pair, variant, wall
from .simulation import Integrator, Simulation, Snapshot, State

__version__ = "0.1.0"

# ``azplugins_gb300.md.Integrator`` reads like ``hoomd.md.Integrator``
class md:  # noqa: N801
    Integrator = Integrator
    methods = methods
    nlist = nlist


__all__ = ["bond", "compute", "external", "filter", "flow", "variant", "wall", "methods", "nlist", "pair", "md", "Integrator", "Simulation", "Snapshot", "State"]
