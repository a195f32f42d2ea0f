"""Batched replicas: many independent systems advanced together (``azp_batch``).

Each replica has its own box, pair parameters and RNG seed and one particle
type; all replicas share the pair potential kind, dt, kT, gamma and the flow
field. One fused force + Langevin launch per timestep covers every replica,
replayed from a CUDA graph; the threads-per-particle of that launch is picked by
:meth:`ReplicaBatch.autotune` (timed with CUDA events on the launching stream).

A replica in the batch draws exactly the noise it draws when run alone with the
same seed (tags are per replica), so batched and separate runs agree to rounding.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class ReplicaBatch:
    """Args:
        snapshots: list of Snapshot (one particle type each; positions, velocities,
            masses, images; accelerations or zeros).
        pair_cls: a class of ``azplugins_gb300.pair``.
        params: list of parameter dicts, one per replica.
        r_cut: list of cutoffs, one per replica.
    """

    def __init__(self, snapshots, pair_cls, params, r_cut, seeds, dt, kT=1.0, gamma=1.0, r_buff=0.4, mode="none",
                 precision="fp32", flow=None, timestep=0):
        from .flow import ConstantFlow

        L = _lib.load()
        _lib.require_gpu()
        self._L = L
        self.S = len(snapshots)
        self.N = np.array([s.particles.N for s in snapshots], dtype=np.uint32)
        self.off = np.concatenate([[0], np.cumsum(self.N)]).astype(np.int64)
        box = np.array([s.configuration.box[:3] for s in snapshots], dtype=np.float64)
        pot = pair_cls(nlist=None, mode=mode)
        recs = np.zeros((self.S, _lib.record_doubles(_lib.RECORD_PAIR, pot.kind)))
        for r, d in enumerate(params):
            vals = np.ascontiguousarray([float(d[k]) for k in pot._keys], dtype=np.float64)
            _lib.check(L.azp_pair_params_from_values(pot.kind, vals.ctypes.data, recs[r].ctypes.data), "params")
        self._keep = [self.N, box, recs, np.ascontiguousarray(r_cut, dtype=np.float64),
                      np.ascontiguousarray(seeds, dtype=np.uint32)]
        c = _lib.BatchConfig()
        c.nsys = self.S
        c.N = self.N.ctypes.data
        c.L = box.ctypes.data
        c.precision = _lib.FP32 if precision == "fp32" else _lib.FP64
        c.pair_kind = pot.kind
        c.shift_mode = _lib.MODES[mode]
        c.pair_params = recs.ctypes.data
        c.r_cut = self._keep[3].ctypes.data
        c.r_buff = r_buff
        c.dt, c.kT, c.gamma = dt, kT, gamma
        c.seeds = self._keep[4].ctypes.data
        c.noiseless = 0
        c.flow = (flow or ConstantFlow((0.0, 0.0, 0.0)))._record()
        st = ctypes.c_int(0)
        self._b = L.azp_batch_create(ctypes.byref(c), ctypes.byref(st))
        _lib.check(st.value, "azp_batch_create")
        self.timestep = timestep
        self.set_state(snapshots)
        self.tpp = 1
        self.block = 256

    def set_state(self, snapshots):
        tot = int(self.off[-1])
        pos = np.zeros((tot, 4))
        vel = np.zeros((tot, 4))
        acc = np.zeros((tot, 3))
        img = np.zeros((tot, 3), dtype=np.int32)
        for r, s in enumerate(snapshots):
            a, b = self.off[r], self.off[r + 1]
            p = s.particles
            pos[a:b, :3] = p.position
            vel[a:b, :3] = p.velocity
            vel[a:b, 3] = p.mass
            if p.acceleration is not None:
                acc[a:b] = p.acceleration
            img[a:b] = p.image
        _lib.check(self._L.azp_batch_set_state(self._b, pos.ctypes.data, vel.ctypes.data, acc.ctypes.data,
                                               img.ctypes.data, int(self.timestep), _stream()), "azp_batch_set_state")

    def get_arrays(self):
        tot = int(self.off[-1])
        pos = np.zeros((tot, 4))
        vel = np.zeros((tot, 4))
        acc = np.zeros((tot, 3))
        img = np.zeros((tot, 3), dtype=np.int32)
        _lib.check(self._L.azp_batch_get_state(self._b, pos.ctypes.data, vel.ctypes.data, acc.ctypes.data,
                                               img.ctypes.data, _stream()), "azp_batch_get_state")
        return pos, vel, acc, img

    def replica(self, r, arrays=None):
        pos, vel, acc, img = arrays if arrays is not None else self.get_arrays()
        a, b = self.off[r], self.off[r + 1]
        return pos[a:b, :3], vel[a:b, :3], acc[a:b], img[a:b]

    def run(self, steps, check=True):
        _lib.check(self._L.azp_batch_run(self._b, int(steps), _stream()), "azp_batch_run")
        self.timestep += int(steps)
        if check:
            err = ctypes.c_uint32(0)
            nb = ctypes.c_uint32(0)
            _lib.check(self._L.azp_batch_error(self._b, ctypes.byref(err), ctypes.byref(nb), _stream()), "error")
            if err.value:
                raise _lib.AzpError(-3 if err.value & _lib.EBIT_NLIST_OVERFLOW else -7, "azp_batch_run")
            self.builds = nb.value

    @property
    def last_launches(self):
        return int(self._L.azp_batch_last_launches(self._b))

    def set_tpp(self, tpp):
        _lib.check(self._L.azp_batch_set_tpp(self._b, int(tpp)), "azp_batch_set_tpp")
        self.tpp = int(tpp)

    def set_block(self, block):
        _lib.check(self._L.azp_batch_set_block(self._b, int(block)), "azp_batch_set_block")
        self.block = int(block)

    def autotune(self, candidates=(1, 2, 4, 8), steps=20, repeats=2, blocks=(256,)):
        """Pick the threads-per-particle and the block size of the fused step by
        timing every pair (CUDA events on the launching stream).

        The state is restored afterwards; returns {tpp: ms per step} when one
        block size is tried, else {(tpp, block): ms per step}."""
        import torch

        saved = self.get_arrays()
        t0 = self.timestep
        res = {}
        for block in blocks:
            self.set_block(block)
            for tpp in candidates:
                self.set_tpp(tpp)
                self.run(2, check=False)  # graph capture + warm-up
                best = float("inf")
                for _ in range(repeats):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    self.run(steps, check=False)
                    e1.record()
                    torch.cuda.synchronize()
                    best = min(best, e0.elapsed_time(e1) / steps)
                res[(tpp, block)] = best
        tpp, block = min(res, key=res.get)
        self.set_block(block)
        self.set_tpp(tpp)
        if len(blocks) == 1:
            res = {k[0]: v for k, v in res.items()}
        self.timestep = t0
        pos, vel, acc, img = saved
        _lib.check(self._L.azp_batch_set_state(self._b, pos.ctypes.data, vel.ctypes.data, acc.ctypes.data,
                                               img.ctypes.data, int(t0), _stream()), "azp_batch_set_state")
        return res

    def close(self):
        if getattr(self, "_b", None):
            self._L.azp_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
