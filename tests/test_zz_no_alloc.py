"""qmin_energy_noalloc: the energy entry point for callers that cannot call
cudaMalloc (their device memory belongs to their own pool allocator, or is
fully committed).  It takes the caller's device arrays and writes the result
into a device array the caller owns, using only a static scratch array inside
the library.

This file sorts last so that a run stopping at the first failure has already
run every other test.  Each test calls the entry point through the C ABI and
checks its result against the allocating entry point qmin_energy on the same
state, within the FP64 energy tolerance the parity tests use (1e-12
relative): two calls in a row on different lattices, a lattice of exactly
QMIN_NOALLOC_MAX_SITES sites (the size the static scratch is laid out for),
and calls whose object table is shorter than a previous call's.  The file
passes alone in a fresh process and after the rest of the suite."""
import ctypes as C

import numpy as np
import pytest

from cases import gpu_lattice, load, oracle_system, parse_args

pytestmark = pytest.mark.gpu

TOL = 1e-12
MAX_SITES = 8388608          # QMIN_NOALLOC_MAX_SITES in include/qmin_gb300.h


def _fn(qmin):
    fn = qmin.lib().qmin_energy_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p,
                   C.c_void_p]
    fn.restype = C.c_int
    return fn


def _noalloc_energy(qmin, torch, s, stream, nobj=None):
    """Energy of oracle system `s` through qmin_energy_noalloc on torch-owned
    buffers; `nobj` (default: all of s's objects) is the object count passed."""
    nobj = s.nobj if nobj is None else nobj
    N = s.N
    Q_dev = torch.from_numpy(np.ascontiguousarray(s.Q.T)).to("cuda")          # SoA planes, stride N
    t_dev = torch.from_numpy(s.types.astype(np.int8)).to("cuda")
    out = torch.full((6,), 12345.0, dtype=torch.float64, device="cuda")
    p = s.p
    params = qmin.LdgParams()
    params.A, params.B, params.C = p.A, p.B, p.C
    params.L1, params.L2, params.L3, params.L4 = p.L1, p.L2, p.L3, p.L4
    params.multi_constant = p.multi_constant
    params.efield, params.hfield = p.efield, p.hfield
    for k in range(3):
        params.E[k], params.H[k] = p.E[k], p.H[k]
    params.eps, params.eps0, params.deps = p.eps, p.eps0, p.deps
    params.chi, params.mu0, params.dchi = p.chi, p.mu0, p.dchi
    objs = (qmin.Object * max(nobj, 1))()
    for k in range(nobj):
        objs[k].kind, objs[k].W, objs[k].S0 = s.objs[k].kind, s.objs[k].W, s.objs[k].S0
    desc = qmin.LatticeDesc(s.L[0], s.L[1], s.L[2], qmin.FP64, 0)
    rc = _fn(qmin)(C.byref(desc), C.byref(params), objs, nobj, C.c_void_p(Q_dev.data_ptr()), C.c_longlong(N),
                   C.c_void_p(t_dev.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == qmin.QMIN_OK, qmin.lib().qmin_last_error_string()
    stream.synchronize()
    return out.cpu().numpy()


def _allocating_energy(qmin, s):
    lat = gpu_lattice(qmin, s, qmin.FP64)
    e, comps = lat.energy()
    lat.close()
    return e, np.asarray(comps)


def _check(out, e, comps):
    assert abs(out[0] - e) <= TOL * abs(e), (out[0], e)
    np.testing.assert_allclose(out[1:], comps, rtol=TOL, atol=TOL * np.abs(comps).max())


def _golden_system(oracle, name):
    return oracle_system(oracle, parse_args(load(name)["args"]))


def test_energy_noalloc_matches_allocating_entry_point(qmin, oracle):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    # two calls in a row on different lattices: the shared scratch must not carry
    # anything from the first call into the second
    for name in ["l1234_planar_fields_fire", "edges_gaps_wrap"]:
        s = _golden_system(oracle, name)
        _check(_noalloc_energy(qmin, torch, s, stream), *_allocating_energy(qmin, s))


def test_energy_noalloc_at_maximum_size(qmin, oracle):
    """A lattice of exactly QMIN_NOALLOC_MAX_SITES sites (256 x 256 x 128: every
    partial-sum slot of the scratch in use) with walls, a sphere and L1-L3,
    called twice in a row with a small lattice in between."""
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    big = oracle.System((256, 256, 128), Ls=(2.32, 1.0, 0.5, 0.0))
    assert big.N == MAX_SITES
    big.random_nematic(5)
    big.add_wall(2, 0, 0, 5.3)
    big.add_sphere((128.0, 128.0, 64.0), 30.0, 0, 5.3)
    big.add_sphere((10.0, 250.0, 120.0), 12.0, 1, 2.0)     # wraps the periodic box, planar anchoring
    ref_big = _allocating_energy(qmin, big)
    small = _golden_system(oracle, "planar_sphere_fire")
    ref_small = _allocating_energy(qmin, small)
    _check(_noalloc_energy(qmin, torch, big, stream), *ref_big)
    _check(_noalloc_energy(qmin, torch, small, stream), *ref_small)
    _check(_noalloc_energy(qmin, torch, big, stream), *ref_big)


def test_energy_noalloc_object_table_is_not_carried_over(qmin, oracle):
    """A call with fewer objects than the previous one: the object slots the
    new call does not fill hold a NaN sentinel, so a lattice whose types name a
    missing object gets a NaN anchoring energy instead of the earlier call's
    object, and a lattice without objects is unaffected by what came before."""
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    s = _golden_system(oracle, "edges_gaps_wrap")
    assert s.nobj >= 2
    _check(_noalloc_energy(qmin, torch, s, stream), *_allocating_energy(qmin, s))
    short = _noalloc_energy(qmin, torch, s, stream, nobj=s.nobj - 1)      # last object missing
    assert np.isnan(short[0]) and np.isnan(short[3])
    assert np.isfinite(short[[1, 2, 4, 5]]).all()
    none = _noalloc_energy(qmin, torch, s, stream, nobj=0)
    assert np.isnan(none[0]) and np.isnan(none[3])
    bulk = _golden_system(oracle, "l1_bulk_fire")
    assert bulk.nobj == 0
    _check(_noalloc_energy(qmin, torch, bulk, stream, nobj=0), *_allocating_energy(qmin, bulk))


def test_energy_noalloc_rejects_oversized_lattice(qmin):
    torch = pytest.importorskip("torch")
    fn = _fn(qmin)
    params = qmin.LdgParams()
    # valid (small) device buffers: the call must refuse on the host before using them
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    ptr = C.c_void_p(buf.data_ptr())
    for dims in [(256, 256, 256), (256, 256, 129)]:      # 16.8M sites, and MAX_SITES + 65536
        desc = qmin.LatticeDesc(*dims, qmin.FP64, 0)
        n = dims[0] * dims[1] * dims[2]
        rc = fn(C.byref(desc), C.byref(params), None, 0, ptr, C.c_longlong(n), ptr, ptr, None)
        assert rc == qmin.QMIN_EINVAL
        assert b"static scratch covers at most 8388608 sites" in qmin.lib().qmin_last_error_string()
