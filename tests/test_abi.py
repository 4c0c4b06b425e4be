"""C-ABI library checks that need no GPU: it loads, exports every entry point
declared in include/qmin_gb300.h, rejects bad arguments with status codes,
and its host set-up helpers reproduce the reference's initial state."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from cases import GOLDEN_CASES, load, parse_args

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "qmin_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(qmin_\w+)\(", txt, re.M)))


def test_library_exports_every_declared_symbol(qmin):
    lib = qmin.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(qmin.EXPORTED_SYMBOLS) <= set(syms)


def test_status_codes_without_device(qmin):
    lib = qmin.lib()
    h = C.c_void_p()
    assert lib.qmin_create(None, C.byref(h)) == qmin.QMIN_EINVAL
    d = qmin.LatticeDesc(2, 8, 8, 0, 0)
    assert lib.qmin_create(C.byref(d), C.byref(h)) == qmin.QMIN_EINVAL
    assert b"lattice side" in lib.qmin_last_error_string()
    d = qmin.LatticeDesc(8, 8, 8, 7, 0)
    assert lib.qmin_create(C.byref(d), C.byref(h)) == qmin.QMIN_EINVAL
    assert lib.qmin_force(None, None) == qmin.QMIN_EINVAL
    assert lib.qmin_fire_run(None, 1, None) == qmin.QMIN_EINVAL
    # learned warm-start net: sides must be multiples of 8
    assert lib.qmin_warmnet_create(1, 12, 16, 16, 0, C.byref(h)) == qmin.QMIN_EINVAL
    assert b"multiple of 8" in lib.qmin_last_error_string()
    assert lib.qmin_warmnet_create(0, 16, 16, 16, 0, C.byref(h)) == qmin.QMIN_EINVAL
    assert lib.qmin_warmnet_forward(None) == qmin.QMIN_EINVAL
    assert lib.qmin_warm_start(None, None) == qmin.QMIN_EINVAL


def test_warmnet_parameter_layout(qmin):
    """The Python layer table matches the native parameter count."""
    sl = qmin.warmnet_param_slices()
    assert sl[-1][1].stop == 573760
    p = qmin.warmnet_init_params(0)
    assert p.dtype == np.float32 and p.size == 573760 and np.all(p[sl[0][1]] == 0)


def test_no_cpu_fallback(qmin):
    """On a machine without a GPU the compute path refuses loudly."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(qmin.QminError):
        qmin.Lattice((8, 8, 8))
    with pytest.raises(qmin.QminError):
        qmin.WarmNet(1, (16, 16, 16))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_host_setup_matches_reference(qmin, oracle, name):
    g = load(name)
    cfg = parse_args(g["args"])
    _, _, _, S0 = qmin.cli_phase_constants()
    Q = qmin.host_random_nematic(cfg["L"], cfg["seed"], S0)
    geo = qmin.Geometry(cfg["L"], Q)
    for xyz, plane, kind, W in cfg["walls"]:
        geo.add_wall(xyz, plane, kind, W, S0)
    for c, r, kind, W in cfg["spheres"]:
        geo.add_sphere(c, r, kind, W, S0)
    if "bfile" in cfg:
        geo.add_boundary_file(cfg["bfile"])
    if "loadstate" in cfg:
        from cases import load_state_text
        load_state_text(geo.Q, cfg["L"], cfg["loadstate"] + "_x0y0z0.txt")
    np.testing.assert_array_equal(geo.types, g["types"].astype(np.int32))
    m = np.isfinite(g["q0"])
    np.testing.assert_array_equal(geo.Q[m], g["q0"][m])


def test_host_setup_rejects_bad_arguments(qmin):
    lib = qmin.lib()
    Q = np.zeros((27, 5))
    t = np.zeros(27, dtype=np.int32)
    objs = (qmin.Object * 4)()
    n = C.c_int(0)
    dp = Q.ctypes.data_as(C.POINTER(C.c_double))
    ip = t.ctypes.data_as(C.POINTER(C.c_int))
    assert lib.qmin_host_add_wall(3, 3, 3, 5, 0, 0, 1.0, 0.5, dp, ip, objs, C.byref(n)) == qmin.QMIN_EINVAL
    assert lib.qmin_host_add_wall(3, 3, 3, 0, 0, 9, 1.0, 0.5, dp, ip, objs, C.byref(n)) == qmin.QMIN_EINVAL
    c = (C.c_double * 3)(1, 1, 1)
    assert lib.qmin_host_add_sphere(3, 3, 3, c, -1.0, 0, 1.0, 0.5, dp, ip, objs, C.byref(n)) == qmin.QMIN_EINVAL
    assert n.value == 0


def test_boundary_file_rejects_malformed_input(qmin, tmp_path):
    L = (6, 6, 6)
    geo = qmin.Geometry(L, np.zeros((216, 5)))
    with pytest.raises(qmin.QminError):
        geo.add_boundary_file(str(tmp_path / "missing.txt"))
    bad = tmp_path / "bad.txt"
    bad.write_text("1\n0 1.0 0.5 2\n1 1 1 0 0 0 0 0\n1 2 x 0 0 0 0 0\n")
    with pytest.raises(qmin.QminError):
        geo.add_boundary_file(str(bad))
