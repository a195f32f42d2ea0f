"""Wall potentials (mirror of ``hoomd.azplugins.wall``, ``src/wall.py``) and the
wall geometries they take (the part of ``hoomd.wall`` they need).

``LJ93(walls)`` and ``Colloid(walls)`` take a list of :class:`Sphere`,
:class:`Cylinder` and :class:`Plane` objects (HOOMD's constructors and defaults)
and per-type ``params`` with the reference's keys: LJ93 ``A``, ``sigma``,
``r_cut`` (and ``r_extrap``, default 0); Colloid ``A``, ``a``, ``sigma``,
``r_cut`` (and ``r_extrap``). ``forces`` / ``energies`` / ``virials`` are
evaluated by the drop-in driver (``azp_wall_forces``) at the current state; the
resident engine (``Simulation.run``) adds them to the net force inside its fused
step when the potential is in the integrator's forces.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .typeparam import TypeParameterDict


def _vec3(v, name):
    a = np.asarray(v, dtype=np.float64).reshape(-1)
    if a.shape != (3,) or not np.isfinite(a).all():
        raise ValueError(f"{name} must be three finite numbers")
    return tuple(float(x) for x in a)


class Sphere:
    """Spherical wall (``hoomd.wall.Sphere``): active side inside (``inside=True``)
    or outside; ``open=True`` leaves the surface itself out of the active side."""

    def __init__(self, radius, origin=(0.0, 0.0, 0.0), inside=True, open=True):  # noqa: A002
        self.radius = float(radius)
        if not self.radius >= 0.0:
            raise ValueError("radius must be >= 0")
        self.origin = _vec3(origin, "origin")
        self.inside = bool(inside)
        self.open = bool(open)

    def _struct(self):
        w = _lib.WallSphere()
        w.r = self.radius
        w.origin[:] = self.origin
        w.inside, w.open = int(self.inside), int(self.open)
        return w

    def _row(self):
        return [self.radius, *self.origin, float(self.inside), float(self.open)]

    def __repr__(self):
        return f"Sphere(radius={self.radius}, origin={self.origin}, inside={self.inside}, open={self.open})"


class Cylinder:
    """Cylindrical wall (``hoomd.wall.Cylinder``) of infinite length along ``axis``."""

    def __init__(self, radius, axis, origin=(0.0, 0.0, 0.0), inside=True, open=True):  # noqa: A002
        self.radius = float(radius)
        if not self.radius >= 0.0:
            raise ValueError("radius must be >= 0")
        self.axis = _vec3(axis, "axis")
        if not np.linalg.norm(self.axis) > 0.0:
            raise ValueError("axis must be non-zero")
        self.origin = _vec3(origin, "origin")
        self.inside = bool(inside)
        self.open = bool(open)

    def _struct(self):
        w = _lib.WallCylinder()
        w.r = self.radius
        w.origin[:] = self.origin
        w.axis[:] = self.axis
        w.inside, w.open = int(self.inside), int(self.open)
        return w

    def _row(self):
        a = np.asarray(self.axis) / np.linalg.norm(self.axis)
        return [self.radius, *self.origin, *a, float(self.inside), float(self.open)]

    def __repr__(self):
        return (f"Cylinder(radius={self.radius}, axis={self.axis}, origin={self.origin}, inside={self.inside}, "
                f"open={self.open})")


class Plane:
    """Planar wall (``hoomd.wall.Plane``): the active side is the one ``normal``
    points into."""

    def __init__(self, origin, normal, open=True):  # noqa: A002
        self.origin = _vec3(origin, "origin")
        self.normal = _vec3(normal, "normal")
        if not np.linalg.norm(self.normal) > 0.0:
            raise ValueError("normal must be non-zero")
        self.open = bool(open)

    def _struct(self):
        w = _lib.WallPlane()
        w.origin[:] = self.origin
        w.normal[:] = self.normal
        w.open = int(self.open)
        return w

    def _row(self):
        n = np.asarray(self.normal) / np.linalg.norm(self.normal)
        return [*self.origin, *n, float(self.open)]

    def __repr__(self):
        return f"Plane(origin={self.origin}, normal={self.normal}, open={self.open})"


class WallPotential:
    """Base class of the wall potentials (HOOMD ``md.external.wall.WallPotential``)."""

    _name = None
    _keys = ()

    def __init__(self, walls):
        self.walls = list(walls)
        for w in self.walls:
            if not isinstance(w, (Sphere, Cylinder, Plane)):
                raise TypeError(f"walls are Sphere, Cylinder or Plane objects, got {type(w).__name__}")
        self.params = TypeParameterDict(1, required=self._keys + ("r_cut",), defaults={"r_extrap": 0.0},
                                        name="params")
        self._sim = None

    @property
    def kind(self) -> int:
        return _lib.WALL_KINDS[self._name]

    def _tables(self, types):
        """Host tables for ``types``: records [nt, d] (the reference's param_type
        size in doubles), r_cut [nt], r_extrap [nt]."""
        L = _lib.load()
        nt = len(types)
        d_rec = _lib.record_doubles(_lib.RECORD_WALL, self.kind)
        rec = np.zeros((nt, d_rec))
        rc = np.zeros(nt)
        rx = np.zeros(nt)
        for a, name in enumerate(types):
            if name not in self.params:
                raise KeyError(f"{type(self).__name__}.params[{name!r}] is not set")
            d = self.params[name]
            vals = np.ascontiguousarray([d[k] for k in self._keys], dtype=np.float64)
            out = np.zeros(d_rec)
            _lib.check(L.azp_wall_params_from_values(self.kind, vals.ctypes.data, out.ctypes.data), "wall params")
            rec[a] = out
            rc[a] = d["r_cut"]
            rx[a] = d.get("r_extrap", 0.0)
        return rec, rc, rx

    def _counts(self):
        ns = sum(isinstance(w, Sphere) for w in self.walls)
        nc = sum(isinstance(w, Cylinder) for w in self.walls)
        npl = sum(isinstance(w, Plane) for w in self.walls)
        if ns > 20 or nc > 20 or npl > 60:
            raise ValueError("at most 20 spheres, 20 cylinders and 60 planes")
        return ns, nc, npl

    def _walls_struct(self):
        """(azp_walls, keep-alive arrays) for the C ABI."""
        self._counts()
        sp = [w._struct() for w in self.walls if isinstance(w, Sphere)]
        cy = [w._struct() for w in self.walls if isinstance(w, Cylinder)]
        pl = [w._struct() for w in self.walls if isinstance(w, Plane)]
        keep = [(_lib.WallSphere * max(len(sp), 1))(*sp), (_lib.WallCylinder * max(len(cy), 1))(*cy),
                (_lib.WallPlane * max(len(pl), 1))(*pl)]
        w = _lib.Walls()
        w.n_spheres, w.n_cylinders, w.n_planes = len(sp), len(cy), len(pl)
        w.spheres, w.cylinders, w.planes = (ctypes.cast(k, ctypes.c_void_p) for k in keep)
        return w, keep

    def record_to_dict(self, rec):
        """asDict() of a param_type record (the reference round trip)."""
        L = _lib.load()
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        vals = np.zeros(len(self._keys))
        _lib.check(L.azp_wall_params_to_values(self.kind, rec.ctypes.data, vals.ctypes.data), "asDict")
        return dict(zip(self._keys, (float(v) for v in vals)))

    # ------------------------------------------------------------------ results
    def _compute(self):
        if self._sim is None:
            raise RuntimeError("attach the force to a Simulation (sim.run(0)) before reading results")
        from . import _compute

        return _compute.wall_forces(self._sim.state, self, self._sim.precision)

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


class LJ93(WallPotential):
    """Lennard-Jones 9-3 wall potential (``src/WallEvaluatorLJ93.h``):
    U(r) = A [(2/15) (sigma/r)^9 - (sigma/r)^3], shifted to zero at r_cut."""

    _name = "LJ93"
    _keys = ("A", "sigma")


class Colloid(WallPotential):
    """Lennard-Jones colloid wall potential (``src/WallEvaluatorColloid.h``) for a
    sphere of radius a against a half space, shifted to zero at r_cut."""

    _name = "Colloid"
    _keys = ("A", "a", "sigma")
