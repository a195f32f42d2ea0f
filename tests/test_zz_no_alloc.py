"""azp_pair_forces_static, the pair-force entry point that allocates nothing.

Some callers of this library cannot allocate device memory: a host simulation
code that reserves its whole device budget at start-up and lets plugins use only
the buffers it owns, or a caller that cannot accept cudaMalloc's implicit device
synchronisation. They cannot create the azp_nlist workspace that azp_pair_forces
keeps its scratch in, so azp_pair_forces_static keeps that scratch in one fixed
device array of the library instead. Here it is called through the C ABI and
checked against azp_pair_forces on the same inputs, for two calls in a row on
different systems (the second smaller, in the other precision, with more types),
so that nothing left in the shared array by the first call reaches the second.

Tolerances as for the pair driver: FP64 1e-12 and FP32 1e-5 relative (forces
norm-wise |dF_i| / max(|F_i|, F_rms), total energy, each virial component).
This file is named to be collected last.
"""

import ctypes

import numpy as np
import pytest

from helpers import force_error, random_fluid, rel

TOL = {"fp64": 1e-12, "fp32": 1e-5}


def _inputs(N, ntypes, seed, mode):
    """A fluid, its pair tables on the device and its neighbour list (azp_nlist)."""
    import torch

    import azplugins_gb300 as az
    from azplugins_gb300 import _compute, _lib

    snap = random_fluid(N, 0.7, seed, ntypes=ntypes)
    types = list(snap.particles.types)
    pot = az.pair.PerturbedLennardJones(nlist=az.nlist.Cell(buffer=0.4), default_r_cut=2.5, mode=mode,
                                        default_r_on=2.0)
    rng = np.random.Generator(np.random.PCG64(seed))
    for a in range(ntypes):
        for b in range(a, ntypes):
            pot.params[(types[a], types[b])] = dict(epsilon=float(rng.uniform(0.5, 1.5)),
                                                    sigma=float(rng.uniform(0.85, 1.1)),
                                                    attraction_scale_factor=float(rng.uniform(0.0, 1.0)))
            pot.r_cut[(types[a], types[b])] = float(rng.uniform(2.0, 3.0))
            pot.r_on[(types[a], types[b])] = 1.8
    rec, rc, ro = pot._tables(types)
    pos = _compute.device_positions(snap)
    sysd = _compute.make_system(snap, pos)
    nl = _compute.NeighborList(N, ntypes, rc, 0.4, tpp=4)
    nl.build(sysd)
    tables = [torch.from_numpy(np.ascontiguousarray(x).reshape(-1).copy()).cuda() for x in (rec, rc, ro)]
    return dict(snap=snap, pot=pot, pos=pos, sysd=sysd, nl=nl, tables=tables, kind=pot.kind,
                mode=_lib.MODES[mode])


def _out(N, precision):
    import torch

    from azplugins_gb300 import _lib

    dt = torch.float32 if precision == "fp32" else torch.float64
    force = torch.full((N, 4), float("nan"), dtype=dt, device="cuda")
    vir = torch.full((6, N), float("nan"), dtype=dt, device="cuda")
    out = _lib.Forces()
    out.force = force.data_ptr()
    out.virial = vir.data_ptr()
    out.virial_pitch = N
    out.precision = _lib.FP32 if precision == "fp32" else _lib.FP64
    return force, vir, out


def _both(inp, precision):
    """(existing entry point, static entry point) forces and virials as FP64 numpy."""
    import torch

    from azplugins_gb300 import _lib

    L = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    N = inp["snap"].particles.N
    p, rc, ro = (t.data_ptr() for t in inp["tables"])
    f_ref, w_ref, out_ref = _out(N, precision)
    _lib.check(L.azp_pair_forces(ctypes.byref(inp["sysd"]), inp["nl"].handle, inp["kind"], p, rc, ro, inp["mode"],
                                 ctypes.byref(out_ref), stream), "azp_pair_forces")
    counts, nbrs = ctypes.c_void_p(), ctypes.c_void_p()
    max_nn, nb = ctypes.c_uint32(), ctypes.c_uint32()
    _lib.check(L.azp_nlist_view(inp["nl"].handle, ctypes.byref(counts), ctypes.byref(nbrs), ctypes.byref(max_nn),
                                ctypes.byref(nb)), "azp_nlist_view")
    f_st, w_st, out_st = _out(N, precision)
    _lib.check(L.azp_pair_forces_static(ctypes.byref(inp["sysd"]), counts, nbrs, max_nn.value, inp["kind"], p, rc, ro,
                                        inp["mode"], ctypes.byref(out_st), stream), "azp_pair_forces_static")
    torch.cuda.synchronize()
    cvt = lambda t: t.double().cpu().numpy()  # noqa: E731
    return cvt(f_ref), cvt(w_ref).T, cvt(f_st), cvt(w_st).T


def _compare(f_ref, w_ref, f_st, w_st, tol):
    assert np.isfinite(f_st).all() and np.isfinite(w_st).all()
    # the same kernels with the same threads per particle on the same inputs:
    # bit-identical results (a stale byte of the shared array would show here)
    assert np.array_equal(f_st, f_ref)
    assert np.array_equal(w_st, w_ref)
    # and, as a diagnostic, within the tolerance the other GPU tests use
    assert force_error(f_st, f_ref) <= tol
    assert rel(f_st[:, 3].sum(), f_ref[:, 3].sum()) <= tol
    for c in range(6):
        ref = w_ref[:, c].sum()
        assert abs(w_st[:, c].sum() - ref) <= tol * max(abs(ref), np.abs(w_ref[:, c]).sum())


@pytest.mark.gpu
def test_static_entry_matches_pair_forces_two_calls():
    import azplugins_gb300 as az  # noqa: F401
    from azplugins_gb300 import _lib

    _lib.require_gpu()
    first = _inputs(24000, 1, seed=5, mode="shift")
    second = _inputs(9000, 3, seed=6, mode="xplor")
    try:
        for inp, precision in ((first, "fp32"), (second, "fp64")):
            f_ref, w_ref, f_st, w_st = _both(inp, precision)
            _compare(f_ref, w_ref, f_st, w_st, TOL[precision])
        # and once more on the first system, after the second call used the array
        f_ref, w_ref, f_st, w_st = _both(first, "fp32")
        _compare(f_ref, w_ref, f_st, w_st, TOL["fp32"])
    finally:
        first["nl"].close()
        second["nl"].close()


def test_static_entry_rejects_too_many_particles():
    """The size check comes before any device work, so this runs without a GPU."""
    from azplugins_gb300 import _lib

    L = _lib.load()
    limit = 262144
    s = _lib.System()
    s.N = limit + 1
    s.ntypes = 1
    s.pos = 1  # never dereferenced: the size check comes first
    for d in range(3):
        s.box.L[d] = 100.0
    out = _lib.Forces()
    out.force = 1
    out.precision = _lib.FP32
    one = np.zeros(16)
    st = L.azp_pair_forces_static(ctypes.byref(s), None, None, 0, 0, one.ctypes.data, one.ctypes.data, None, 0,
                                  ctypes.byref(out), None)
    assert st == -11
    assert b"262144" in L.azp_last_error()


def test_static_entry_rejects_too_many_types():
    """ntypes above the static table's 16 is refused before any device work."""
    from azplugins_gb300 import _lib

    L = _lib.load()
    s = _lib.System()
    s.N = 100
    s.ntypes = 17
    s.pos = 1  # never dereferenced: the type check comes first
    for d in range(3):
        s.box.L[d] = 100.0
    out = _lib.Forces()
    out.force = 1
    out.precision = _lib.FP64
    one = np.zeros(17 * 17 * 4)
    st = L.azp_pair_forces_static(ctypes.byref(s), None, None, 0, 0, one.ctypes.data, one.ctypes.data, None, 0,
                                  ctypes.byref(out), None)
    assert st == -1

