"""Python handle of the resident engine (``azp_md_*`` in the C ABI)."""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .bond import Bond
from .external import HarmonicBarrier
from .methods import BrownianFlow, LangevinFlow
from .pair import Pair
from .variant import Constant
from .wall import WallPotential

# rows of the engine's barrier-location table (AZP_MD_BARRIER_ROWS)
BARRIER_ROWS = 65536


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def split_forces(integ):
    """(pair, bond, barrier, wall) of the integrator's forces, each None when absent."""
    kinds = (Pair, Bond, HarmonicBarrier, WallPotential)
    found = [[f for f in integ.forces if isinstance(f, k)] for k in kinds]
    other = [f for f in integ.forces if not isinstance(f, kinds)]
    if other:
        raise NotImplementedError(f"unsupported force objects: {other}")
    if any(len(x) > 1 for x in found):
        raise NotImplementedError("the engine advances at most one pair, one bond, one barrier and one wall potential")
    return tuple(x[0] if x else None for x in found)


class Engine:
    """Owns one ``azp_md`` object."""

    @staticmethod
    def config_key(sim, integ):
        pair, bond, barrier, wall = split_forces(integ)
        if len(integ.methods) != 1 or not isinstance(integ.methods[0], (LangevinFlow, BrownianFlow)):
            raise NotImplementedError("exactly one LangevinFlow or BrownianFlow method is required")
        m = integ.methods[0]
        parts = [sim.precision, sim.seed, integ.dt, type(m).__name__, m.kT, repr(m.filter), m.noiseless, m.alpha,
                 getattr(m, "max_displacement", 0.0), getattr(m, "force_cap", 0.0), repr(m.flow_field), sorted(m.gamma.items()),
                 m.gamma.default]
        if pair is not None:
            parts += [type(pair).__name__, pair.mode, sorted(pair.params.items()), sorted(pair.r_cut.items()),
                      pair.r_cut.default, sorted(pair.r_on.items()), pair.r_on.default, pair.nlist.buffer,
                      pair.nlist.exclusions, getattr(pair, "kT", None)]
        if bond is not None:
            parts += [type(bond).__name__, sorted((k, sorted(v.items())) for k, v in bond.params.items())]
        if barrier is not None:
            # the location is not part of the key: it is tabulated run by run
            parts += [type(barrier).__name__, sorted((k, sorted(v.items())) for k, v in barrier.params.items())]
        if wall is not None:
            parts += [type(wall).__name__, repr(wall.walls), sorted((k, sorted(v.items())) for k, v in wall.params.items())]
        return repr(parts)

    def __init__(self, sim, integ, snap):
        L = _lib.load()
        _lib.require_gpu()
        import torch  # noqa: F401  (initialises the CUDA context used by torch streams)

        self._L = L
        pair, bond, barrier, wall = split_forces(integ)
        m = integ.methods[0]
        p = snap.particles
        types = list(p.types)
        nt = len(types)
        c = _lib.MDConfig()
        c.N = p.N
        c.ntypes = nt
        for d in range(3):
            c.box.L[d] = snap.configuration.box[d]
        c.precision = _lib.FP32 if sim.precision == "fp32" else _lib.FP64
        self._keep = []

        def arr(a, dt=np.float64):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a.ctypes.data

        if pair is not None:
            rec, rc, ro = pair._tables(types)
            c.pair_kind = pair.kind
            c.shift_mode = _lib.MODES[pair.mode]
            c.pair_params = arr(rec.reshape(-1))
            c.r_cut = arr(rc.reshape(-1))
            c.r_on = arr(ro.reshape(-1))
            c.r_buff = pair.nlist.buffer
            c.exclude_bonds = int(pair.nlist.exclude_bonds)
            if pair._name == "DPDGeneralWeight":
                if isinstance(m, BrownianFlow):
                    raise NotImplementedError("DPDGeneralWeight needs velocities: use ConstantVolume or LangevinFlow")
                c.dpd_kT = float(pair.kT)
        else:
            c.pair_kind = -1
            c.r_buff = 0.4
            c.exclude_bonds = 0
        b = snap.bonds
        if bond is not None and b.N > 0:
            c.bond_kind = bond.kind
            c.nbondtypes = len(b.types)
            c.bond_params = arr(bond._table(b.types).reshape(-1))
            c.nbonds = b.N
            c.bonds = arr(np.asarray(b.group).reshape(-1), np.uint32)
            c.bond_types = arr(b.typeid, np.uint32)
        else:
            c.bond_kind = -1
        c.method = _lib.METHOD_BROWNIAN if isinstance(m, BrownianFlow) else _lib.METHOD_LANGEVIN
        c.dt = integ.dt
        # a varying temperature is tabulated run by run (azp_md_set_temperatures)
        self._kT = m.kT
        c.kT = m.kT_constant if m.kT_constant is not None else float(m.kT(0))
        c.group_types = m._group_types(types)
        c.seed = sim.seed
        c.noiseless = int(m.noiseless)
        c.gamma = arr(m._gamma_table(types))
        c.use_lambda = int(m.alpha is not None)
        c.lambda_ = m.alpha or 0.0
        c.flow = m.flow_field._record()
        c.max_displacement = getattr(m, "max_displacement", 0.0)
        c.pair_force_cap = getattr(m, "force_cap", 0.0)
        self._barrier = barrier
        self._box = tuple(snap.configuration.box[:3])
        self._brownian = isinstance(m, BrownianFlow)
        if barrier is not None:
            c.barrier_geometry = barrier.geometry
            c.barrier_params = arr(barrier._table(types).reshape(-1))
        else:
            c.barrier_geometry = 0
            c.barrier_params = None
        if wall is not None:
            rec_w, rc_w, rx_w = wall._tables(types)
            walls, keep = wall._walls_struct()
            self._keep += [walls, keep]
            c.wall_kind = wall.kind
            c.walls = ctypes.addressof(walls)
            c.wall_params = arr(rec_w.reshape(-1))
            c.wall_r_cut = arr(rc_w)
            c.wall_r_extrap = arr(rx_w)
        else:
            c.wall_kind = 0
            c.walls = None
        st = ctypes.c_int(0)
        self._md = L.azp_md_create(ctypes.byref(c), ctypes.byref(st))
        _lib.check(st.value, "azp_md_create")
        self.N = p.N
        self.has_accel = p.acceleration is not None
        self.last_launches = 0
        self.timestep = 0

    def push(self, snap, timestep):
        p = snap.particles
        N = p.N
        pos = np.empty((N, 4))
        pos[:, :3] = p.position
        pos[:, 3] = p.typeid
        vel = np.empty((N, 4))
        vel[:, :3] = p.velocity
        vel[:, 3] = p.mass
        img = np.ascontiguousarray(p.image, dtype=np.int32)
        diam = np.ascontiguousarray(p.diameter, dtype=np.float64)
        acc = None if p.acceleration is None else np.ascontiguousarray(p.acceleration, dtype=np.float64)
        s = _stream()
        _lib.check(
            self._L.azp_md_set_state(self._md, pos.ctypes.data, vel.ctypes.data,
                                     None if acc is None else acc.ctypes.data, img.ctypes.data, diam.ctypes.data,
                                     int(timestep), 0, s),
            "azp_md_set_state")
        self.timestep = int(timestep)

    def pull(self, snap):
        p = snap.particles
        N = p.N
        pos = np.empty((N, 4))
        vel = np.empty((N, 4))
        acc = np.empty((N, 3))
        img = np.empty((N, 3), dtype=np.int32)
        ts = ctypes.c_uint64(0)
        _lib.check(self._L.azp_md_get_state(self._md, pos.ctypes.data, vel.ctypes.data, acc.ctypes.data,
                                            img.ctypes.data, ctypes.byref(ts), 0, _stream()), "azp_md_get_state")
        p.position = pos[:, :3].copy()
        p.velocity = vel[:, :3].copy()
        p.acceleration = acc
        p.image = img

    def _set_barrier(self, t0, steps):
        """Tabulate the barrier's locations for the timesteps whose forces a run of
        ``steps`` from ``t0`` evaluates (t0 .. t0 + steps), checked against the box
        as HarmonicBarrier::makeEvaluator checks them (src/HarmonicBarrier.h:121-130)."""
        loc = self._barrier.location
        if isinstance(loc, Constant):
            vals = np.array([loc.value])
        elif hasattr(loc, "values"):
            vals = np.asarray(loc.values(t0, steps + 1), dtype=np.float64)
        else:
            vals = np.array([float(loc(t)) for t in range(t0, t0 + steps + 1)], dtype=np.float64)
        for v in np.unique(vals):
            if not self._barrier._valid(float(v), self._box):
                raise RuntimeError("Barrier position is invalid")
        vals = np.ascontiguousarray(vals)
        _lib.check(self._L.azp_md_set_barrier_locations(self._md, int(t0), len(vals), vals.ctypes.data, _stream()),
                   "azp_md_set_barrier_locations")

    def _set_temperature(self, t0, steps):
        """Tabulate a varying kT for the timesteps a run of ``steps`` from ``t0``
        integrates (step two and the Brownian move of timestep t use kT(t))."""
        kT = self._kT
        if hasattr(kT, "values"):
            vals = np.asarray(kT.values(t0, steps + 1), dtype=np.float64)
        else:
            vals = np.array([float(kT(t)) for t in range(t0, t0 + steps + 1)], dtype=np.float64)
        vals = np.ascontiguousarray(vals)
        _lib.check(self._L.azp_md_set_temperatures(self._md, int(t0), len(vals), vals.ctypes.data, _stream()),
                   "azp_md_set_temperatures")

    def _chunks(self, steps):
        """Runs of at most BARRIER_ROWS - 1 steps when a moving barrier or a varying
        temperature is tabulated."""
        steps = int(steps)
        moving = self._barrier is not None and not isinstance(self._barrier.location, Constant)
        varying = not isinstance(self._kT, Constant)
        if not moving and not varying:
            if self._barrier is not None:
                self._set_barrier(self.timestep, steps)
            yield steps
            return
        while steps > 0:
            n = min(steps, BARRIER_ROWS - 1)
            if self._barrier is not None:
                self._set_barrier(self.timestep, n if moving else 0)
            if varying:
                self._set_temperature(self.timestep, n)
            yield n
            steps -= n

    def prepare_forces(self):
        """Before a forces-only evaluation (azp_md_forces / azp_md_thermo): the
        barrier location of the current timestep."""
        if self._barrier is not None:
            self._set_barrier(self.timestep, 0)

    def run(self, steps):
        """Advance with the overflow-safe entry (grows the list and replays)."""
        s = _stream()
        for n in self._chunks(steps):
            _lib.check(self._L.azp_md_run_checked(self._md, n, s), "azp_md_run_checked")
            self.timestep += n
        self.last_launches = int(self._L.azp_md_last_launches(self._md))
        err = ctypes.c_uint32(0)
        _lib.check(self._L.azp_md_error(self._md, ctypes.byref(err), s), "azp_md_error")
        if err.value & _lib.EBIT_NLIST_OVERFLOW:
            raise _lib.AzpError(-3, "azp_md_run")
        if err.value & _lib.EBIT_BOND:
            raise _lib.AzpError(-4, "azp_md_run")
        if err.value & _lib.EBIT_NONFINITE:
            raise _lib.AzpError(-7, "azp_md_run")

    def error_word(self):
        err = ctypes.c_uint32(0)
        _lib.check(self._L.azp_md_error(self._md, ctypes.byref(err), _stream()), "azp_md_error")
        return err.value

    def run_async(self, steps):
        """Enqueue ``steps`` timesteps without reading the error word back."""
        for n in self._chunks(steps):
            _lib.check(self._L.azp_md_run(self._md, n, _stream()), "azp_md_run")
            self.timestep += n
        self.last_launches = int(self._L.azp_md_last_launches(self._md))

    def forces(self):
        self.prepare_forces()
        f = np.empty((self.N, 4))
        w = np.empty((self.N, 6))
        _lib.check(self._L.azp_md_forces(self._md, f.ctypes.data, w.ctypes.data, 0, _stream()), "azp_md_forces")
        return f, w

    def thermo(self):
        out = np.zeros(9)
        # a barrier's forces are re-evaluated at the location of the current timestep
        self.prepare_forces()
        _lib.check(self._L.azp_md_thermo(self._md, out.ctypes.data, _stream()), "azp_md_thermo")
        return {
            "potential_energy": out[0],
            "kinetic_energy": out[1],
            "virial": out[2:8].copy(),
            "nlist_builds": int(out[8]),
        }

    def close(self):
        if getattr(self, "_md", None):
            self._L.azp_md_destroy(self._md)
            self._md = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
