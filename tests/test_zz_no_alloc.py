"""qmin_energy_noalloc: the energy entry point for callers that cannot call
cudaMalloc (their device memory belongs to their own pool allocator, or is
fully committed).  It takes the caller's device arrays and writes the result
into a device array the caller owns, using only a static scratch array inside
the library.

This file sorts last so that a run stopping at the first failure has already
run every other test.  The test calls the entry point through the C ABI twice
in a row, on two different lattices, and checks each result against the
allocating entry point qmin_energy on the same state, within the FP64 energy
tolerance the parity tests use (1e-12 relative).  It passes alone in a fresh
process and after the rest of the suite."""
import ctypes as C

import numpy as np
import pytest

from cases import gpu_lattice, load, oracle_system, parse_args

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc_energy(qmin, torch, s, stream):
    """Energy of oracle system `s` through qmin_energy_noalloc on torch-owned buffers."""
    N = s.N
    Q_dev = torch.from_numpy(np.ascontiguousarray(s.Q.T)).to("cuda")          # SoA planes, stride N
    t_dev = torch.from_numpy(s.types.astype(np.int8)).to("cuda")
    out = torch.full((6,), float("nan"), dtype=torch.float64, device="cuda")
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
    objs = (qmin.Object * max(s.nobj, 1))()
    for k in range(s.nobj):
        objs[k].kind, objs[k].W, objs[k].S0 = s.objs[k].kind, s.objs[k].W, s.objs[k].S0
    desc = qmin.LatticeDesc(s.L[0], s.L[1], s.L[2], qmin.FP64, 0)
    rc = qmin.lib().qmin_energy_noalloc(C.byref(desc), C.byref(params), objs, s.nobj,
                                        C.c_void_p(Q_dev.data_ptr()), C.c_longlong(N),
                                        C.c_void_p(t_dev.data_ptr()), C.c_void_p(out.data_ptr()),
                                        C.c_void_p(stream.cuda_stream))
    assert rc == qmin.QMIN_OK, qmin.lib().qmin_last_error_string()
    stream.synchronize()
    return out.cpu().numpy()


def test_energy_noalloc_matches_allocating_entry_point(qmin, oracle):
    torch = pytest.importorskip("torch")
    fn = qmin.lib().qmin_energy_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p,
                   C.c_void_p]
    fn.restype = C.c_int
    stream = torch.cuda.Stream()
    # two calls in a row on different lattices: the shared scratch must not carry
    # anything from the first call into the second
    for name in ["l1234_planar_fields_fire", "edges_gaps_wrap"]:
        cfg = parse_args(load(name)["args"])
        s = oracle_system(oracle, cfg)
        out = _noalloc_energy(qmin, torch, s, stream)
        lat = gpu_lattice(qmin, s, qmin.FP64)
        e, comps = lat.energy()
        lat.close()
        assert abs(out[0] - e) <= TOL * abs(e)
        np.testing.assert_allclose(out[1:], comps, rtol=TOL, atol=TOL * np.abs(comps).max())


def test_energy_noalloc_rejects_oversized_lattice(qmin):
    torch = pytest.importorskip("torch")
    fn = qmin.lib().qmin_energy_noalloc
    fn.restype = C.c_int
    desc = qmin.LatticeDesc(256, 256, 256, qmin.FP64, 0)   # 16.8M sites > QMIN_NOALLOC_MAX_SITES
    params = qmin.LdgParams()
    # valid (small) device buffers: the call must refuse on the host before using them
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    ptr = C.c_void_p(buf.data_ptr())
    rc = fn(C.byref(desc), C.byref(params), None, 0, ptr, C.c_longlong(256 ** 3), ptr, ptr, None)
    assert rc == qmin.QMIN_EINVAL
    assert b"static scratch covers at most 8388608 sites" in qmin.lib().qmin_last_error_string()
