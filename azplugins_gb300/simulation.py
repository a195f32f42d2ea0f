"""Minimal HOOMD-style host objects around the engine: ``Snapshot``,
``State``, ``md.Integrator`` and ``Simulation``.

HOOMD-blue itself (the ``Simulation`` / ``Operations`` layer above azplugins) is
not part of this project; these classes carry only what the azplugins
force-and-integrate path needs, with HOOMD's attribute names so that scripts
written against ``hoomd.azplugins`` port by changing imports.
"""

from __future__ import annotations

import numpy as np

from . import _lib


class _Particles:
    def __init__(self, N=0):
        self.types = ["A"]
        self._resize(N)

    def _resize(self, N):
        self.N = int(N)
        self.position = np.zeros((N, 3))
        self.velocity = np.zeros((N, 3))
        self.acceleration = None
        self.mass = np.ones(N)
        self.typeid = np.zeros(N, dtype=np.int32)
        self.image = np.zeros((N, 3), dtype=np.int32)
        self.diameter = np.ones(N)


class _Bonds:
    def __init__(self):
        self.types = []
        self._resize(0)

    def _resize(self, N):
        self.N = int(N)
        self.group = np.zeros((N, 2), dtype=np.int64)
        self.typeid = np.zeros(N, dtype=np.int32)


class _Configuration:
    def __init__(self):
        self.box = [1.0, 1.0, 1.0, 0.0, 0.0, 0.0]
        self.dimensions = 3


class Snapshot:
    """Particle, bond and box data in tag order (HOOMD ``Snapshot`` names).

    ``particles.N`` / ``bonds.N`` are set through :meth:`resize` /
    :meth:`resize_bonds`, which allocate the arrays.
    """

    def __init__(self, N=0):
        self.particles = _Particles(N)
        self.bonds = _Bonds()
        self.configuration = _Configuration()

    def resize(self, N):
        self.particles._resize(N)

    def resize_bonds(self, N):
        self.bonds._resize(N)

    def copy(self):
        import copy

        return copy.deepcopy(self)

    def validate(self):
        p = self.particles
        box = self.configuration.box
        if any(x != 0 for x in box[3:]):
            raise ValueError("only orthorhombic boxes are supported (tilts must be 0)")
        if min(box[:3]) <= 0:
            raise ValueError("box lengths must be positive")
        if p.N and (p.typeid.min() < 0 or p.typeid.max() >= len(p.types)):
            raise ValueError("typeid out of range")
        if self.bonds.N:
            if self.bonds.group.min() < 0 or self.bonds.group.max() >= p.N:
                raise ValueError("bond group references a particle that does not exist")
            if len(self.bonds.types) == 0 or self.bonds.typeid.max() >= len(self.bonds.types):
                raise ValueError("bond typeid out of range")


class State:
    """The simulation state; host copies are refreshed from the engine lazily."""

    def __init__(self, sim, snapshot: Snapshot):
        snapshot.validate()
        self._sim = sim
        self._snap = snapshot.copy()
        self._host_valid = True

    @property
    def N(self):
        return self._snap.particles.N

    @property
    def types(self):
        return list(self._snap.particles.types)

    @property
    def box(self):
        return list(self._snap.configuration.box)

    def _pull(self):
        if not self._host_valid and self._sim._engine is not None:
            self._sim._engine.pull(self._snap)
            self._host_valid = True

    def get_snapshot(self) -> Snapshot:
        self._pull()
        return self._snap.copy()

    def set_snapshot(self, snapshot: Snapshot):
        snapshot.validate()
        self._snap = snapshot.copy()
        self._host_valid = True
        self._sim._state_changed = True

    # arrays used by the drop-in compute path (tag order, host)
    def _arrays(self):
        self._pull()
        return self._snap


class _Operations:
    def __init__(self, sim=None):
        self.integrator = None
        self.computes = []
        self._sim = sim

    def add(self, op):
        """Add a compute, or a force as a compute (HOOMD ``Operations.add``): it
        is not integrated; its quantities are read at the current state. On a
        simulation that has run it attaches at once."""
        if op not in self.computes:
            self.computes.append(op)
        if self._sim is not None and self._sim._has_run:
            op._sim = self._sim

    def remove(self, op):
        """Detach a compute (HOOMD ``Operations.remove``)."""
        self.computes.remove(op)
        op._sim = None


class Integrator:
    """Velocity-Verlet style integrator holding methods and forces (HOOMD ``md.Integrator``)."""

    def __init__(self, dt, methods=(), forces=()):
        self.dt = float(dt)
        self.methods = list(methods)
        self.forces = list(forces)


class Simulation:
    """One system on one GPU.

    Args:
        seed (int): Seed of the counter-based RNG streams (uniform noise of the
            flow integrators); combined with the RNG id, timestep and tag.
        precision (str): ``"fp64"`` -- FP64 forces; ``"fp32"`` -- FP32 pair and bond
            arithmetic with compensated sums on exact fixed-point displacements;
            positions, velocities and the integration stay FP64 in both.
        device (int): CUDA device ordinal (the current torch device by default).
    """

    def __init__(self, seed=0, precision="fp64", device=None):
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.seed = int(seed) & 0xFFFFFFFF
        self.precision = precision
        self.device = device
        self.operations = _Operations(self)
        self.state = None
        self._engine = None
        self._engine_key = None
        self._state_changed = False
        self._timestep = 0
        self._has_run = False

    @property
    def timestep(self):
        return self._timestep

    @timestep.setter
    def timestep(self, t):
        if self._engine is not None and self._timestep != int(t):
            self._state_changed = True
        self._timestep = int(t)

    def create_state_from_snapshot(self, snapshot: Snapshot):
        if self.state is not None:
            raise RuntimeError("the state already exists")
        self.state = State(self, snapshot)
        self._state_changed = True

    # ------------------------------------------------------------------ run
    def _attach(self):
        integ = self.operations.integrator
        for f in list(integ.forces if integ is not None else []) + list(self.operations.computes):
            f._sim = self
        return integ

    def run(self, steps):
        """Advance ``steps`` timesteps on the GPU (``run(0)`` only attaches)."""
        if self.state is None:
            raise RuntimeError("create the state first")
        integ = self._attach()
        self._has_run = True
        steps = int(steps)
        if steps == 0:
            return
        if integ is None:
            raise RuntimeError("set sim.operations.integrator first")
        from . import _engine

        key = _engine.Engine.config_key(self, integ)
        if self._engine is None or self._engine_key != key:
            snap = self.state._arrays()
            if self._engine is not None:
                self._engine.close()
            self._engine = _engine.Engine(self, integ, snap)
            self._engine_key = key
            self._state_changed = True
        if self._state_changed:
            self._engine.push(self.state._arrays(), self._timestep)
            self._state_changed = False
        self._engine.run(steps)
        self._timestep += steps
        self.state._host_valid = False

    def thermo(self):
        """Potential energy, kinetic energy and virial sums (FP64) at the current state."""
        if self._engine is None:
            raise RuntimeError("run the simulation first")
        if self._state_changed:
            self._engine.push(self.state._arrays(), self._timestep)
            self._state_changed = False
        return self._engine.thermo()

    def close(self):
        if self._engine is not None:
            self._engine.close()
            self._engine = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["Snapshot", "State", "Integrator", "Simulation"]
