"""Bond potentials (mirror of ``hoomd.azplugins.bond``, ``src/bond.py``).

``params["A-A"]`` keys follow the reference schemas (``src/bond.py:45-49`` for
DoubleWell, ``:141-156`` for Quartic, whose ``delta`` defaults to 0 as in the
reference, ``:160-192`` for ImageHarmonic's ``k``, ``r0``); records are built by
the native ports of the reference dict constructors.
"""

from __future__ import annotations

import numpy as np

from . import _lib
from .typeparam import TypeParameterDict


class Bond:
    """Base class of the bond potentials (HOOMD ``md.bond.Bond``)."""

    _name = None
    _keys = ()
    _defaults = {}

    def __init__(self):
        self.params = TypeParameterDict(1, required=tuple(k for k in self._keys if k not in self._defaults),
                                        defaults=self._defaults, name="params")
        self._sim = None

    @property
    def kind(self) -> int:
        return _lib.BOND_KINDS[self._name]

    def _table(self, bond_types):
        L = _lib.load()
        d_rec = _lib.record_doubles(_lib.RECORD_BOND, self.kind)
        rec = np.zeros((len(bond_types), d_rec))
        for t, name in enumerate(bond_types):
            if name not in self.params:
                raise KeyError(f"{type(self).__name__}.params[{name!r}] is not set")
            d = self.params[name]
            vals = np.ascontiguousarray([d[k] for k in self._keys], dtype=np.float64)
            out = np.zeros(d_rec)
            _lib.check(L.azp_bond_params_from_values(self.kind, vals.ctypes.data, out.ctypes.data), "params")
            rec[t] = out
        return rec

    def record_to_dict(self, rec):
        L = _lib.load()
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        vals = np.zeros(len(self._keys))
        _lib.check(L.azp_bond_params_to_values(self.kind, rec.ctypes.data, vals.ctypes.data), "asDict")
        return dict(zip(self._keys, (float(v) for v in vals)))

    def _compute(self):
        if self._sim is None:
            raise RuntimeError("attach the force to a Simulation (sim.run(0)) before reading results")
        from . import _compute

        return _compute.bond_forces(self._sim.state, self, self._sim.precision)

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


class DoubleWell(Bond):
    """Double-well bond potential (``src/BondEvaluatorDoubleWell.h``)."""

    _name = "DoubleWell"
    _keys = ("r_0", "r_1", "U_1", "U_tilt")


class Quartic(Bond):
    """Quartic (breakable) bond potential with a WCA core (``src/BondEvaluatorQuartic.h``)."""

    _name = "Quartic"
    _keys = ("k", "r_0", "b_1", "b_2", "U_0", "sigma", "epsilon", "delta")
    _defaults = {"delta": 0.0}


__all__ = ["Bond", "DoubleWell", "Quartic"]


class ImageHarmonic(Bond):
    """Harmonic bond U = k/2 (r - r0)^2 on the image-unwrapped distance
    (``src/ImagePotentialBond.h``, ``src/bond.py:160-192``): the bond vector is
    (x_j + img_j L) - (x_i + img_i L), so a bond may span more than half the box.
    Evaluated by the drop-in driver (``azp_bond_forces``, reading the images) and
    inside the resident engine's step (``Simulation.run``), which measures each
    bond from the image counts of the step's start."""

    _name = "ImageHarmonic"
    _keys = ("k", "r0")
