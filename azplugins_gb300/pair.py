"""Pair potentials (mirror of ``hoomd.azplugins.pair``, ``src/pair.py``).

Same class names, constructor arguments (``nlist, default_r_cut, default_r_on,
mode``), accepted modes and ``params`` keys as the reference; the parameter
records are built by the native library's ports of the reference ``param_type``
dict constructors, so ``params[(a, b)]`` round-trips exactly as
``src/pytest/test_pair.py:349`` requires. After ``Simulation.run`` the
per-particle ``forces``, ``energies`` and ``virials`` are evaluated on the GPU
by the drop-in pair driver (``azp_pair_forces``).
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .typeparam import TypeParameterDict


class Pair:
    """Base class of the isotropic pair potentials (HOOMD ``md.pair.Pair``)."""

    _name = None
    _keys = ()
    _accepted_modes = ("none", "shift", "xplor")

    def __init__(self, nlist, default_r_cut=None, default_r_on=0.0, mode="none"):
        if mode not in self._accepted_modes:
            raise ValueError(f"mode {mode!r} not in {self._accepted_modes}")
        self.nlist = nlist
        self.mode = mode
        self.params = TypeParameterDict(2, required=self._keys, name="params")
        self.r_cut = TypeParameterDict(2, scalar=True, name="r_cut")
        self.r_on = TypeParameterDict(2, scalar=True, name="r_on")
        if default_r_cut is not None:
            self.r_cut.set_default(default_r_cut)
        self.r_on.set_default(default_r_on if default_r_on is not None else 0.0)
        self._sim = None

    @property
    def kind(self) -> int:
        return _lib.PAIR_KINDS[self._name]

    def _tables(self, types):
        """Host tables for ``types``: records [nt, nt, d] (d doubles per record, the
        reference's param_type size), r_cut [nt, nt], r_on [nt, nt]."""
        L = _lib.load()
        nt = len(types)
        d_rec = _lib.record_doubles(_lib.RECORD_PAIR, self.kind)
        rec = np.zeros((nt, nt, d_rec))
        rc = np.zeros((nt, nt))
        ro = np.zeros((nt, nt))
        for a in range(nt):
            for b in range(nt):
                key = (types[a], types[b])
                if key not in self.params:
                    raise KeyError(f"{type(self).__name__}.params{key} is not set")
                d = self.params[key]
                vals = np.ascontiguousarray([d[k] for k in self._keys], dtype=np.float64)
                out = np.zeros(d_rec)
                _lib.check(L.azp_pair_params_from_values(self.kind, vals.ctypes.data, out.ctypes.data), "params")
                rec[a, b] = out
                rc[a, b] = self.r_cut[key] if key in self.r_cut else 0.0
                ro[a, b] = self.r_on[key] if key in self.r_on else 0.0
        return rec, rc, ro

    def record_to_dict(self, rec):
        """asDict() of a param_type record (the reference round trip)."""
        L = _lib.load()
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        vals = np.zeros(len(self._keys))
        _lib.check(L.azp_pair_params_to_values(self.kind, rec.ctypes.data, vals.ctypes.data), "asDict")
        return dict(zip(self._keys, (float(v) for v in vals)))

    # ------------------------------------------------------------------ results
    def _compute(self):
        if self._sim is None:
            raise RuntimeError("attach the force to a Simulation (sim.run(0)) before reading results")
        from . import _compute

        return _compute.pair_forces(self._sim.state, self, self._sim.precision)

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


class Colloid(Pair):
    """Colloid pair potential (``src/PairEvaluatorColloid.h``)."""

    _name = "Colloid"
    _keys = ("A", "a_1", "a_2", "sigma")


class DPDGeneralWeight(Pair):
    """DPD with a general weight function (``src/DPDPairEvaluatorGeneralWeight.h``,
    ``src/pair.py:121-239``): conservative A (1 - r / r_cut), dissipative
    -gamma w(r) (v_ij . r_hat) r_hat and random sqrt(gamma w(r)) theta r_hat forces
    with w = (1 - r / r_cut)^s. ``params`` keys: ``A``, ``gamma``, ``s``; mode
    ``"none"`` only; ``kT`` the thermostat temperature (a constant here).

    The forces depend on the velocities, the timestep and the Simulation's seed:
    ``forces`` / ``energies`` / ``virials`` are evaluated by the drop-in driver
    (``azp_dpd_forces``) at the current state, timestep and integrator ``dt``.
    ``Simulation.run`` advances it inside the resident engine's fused step with a
    Langevin-type method (``methods.ConstantVolume`` for the plain DPD
    thermostat): the forces of timestep t + 1 from the half-step velocities, the
    same per-pair draws as the driver."""

    _name = "DPDGeneralWeight"
    _keys = ("A", "gamma", "s")
    _accepted_modes = ("none",)

    def __init__(self, nlist, kT, default_r_cut=None):
        super().__init__(nlist=nlist, default_r_cut=default_r_cut, default_r_on=0.0, mode="none")
        self.kT = float(kT)

    def _compute(self):
        if self._sim is None:
            raise RuntimeError("attach the force to a Simulation (sim.run(0)) before reading results")
        from . import _compute

        integ = self._sim.operations.integrator
        return _compute.dpd_forces(self._sim.state, self, self._sim.precision, integ.dt, self._sim.timestep,
                                   self._sim.seed)


class ExpandedYukawa(Pair):
    """Expanded Yukawa pair potential (``src/PairEvaluatorExpandedYukawa.h``)."""

    _name = "ExpandedYukawa"
    _keys = ("epsilon", "kappa", "delta")


class Hertz(Pair):
    """Hertz pair potential (``src/PairEvaluatorHertz.h``)."""

    _name = "Hertz"
    _keys = ("epsilon",)


class PerturbedLennardJones(Pair):
    """Perturbed Lennard-Jones pair potential (``src/PairEvaluatorPerturbedLennardJones.h``)."""

    _name = "PerturbedLennardJones"
    _keys = ("epsilon", "sigma", "attraction_scale_factor")


__all__ = ["Pair", "Colloid", "DPDGeneralWeight", "ExpandedYukawa", "Hertz", "PerturbedLennardJones"]
