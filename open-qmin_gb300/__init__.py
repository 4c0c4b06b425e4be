"""qmin_gb300: GB300-native (sm_103a) Landau-de Gennes Q-tensor minimisation.

Python host layer over the C ABI in ``include/qmin_gb300.h``.  Two levels:

* ``Lattice``: a thin, 1:1 wrapper of the C handle (state resident in HBM);
* reference-shaped classes mirroring open-Qmin's model / force / updater /
  simulation interfaces (``qTensorLatticeModel``, ``landauDeGennesLC``,
  ``energyMinimizerFIRE``, ``energyMinimizerAdam``,
  ``energyMinimizerNesterovAG``, ``energyMinimizerLoLBFGS``,
  ``multirankSimulation``) so code written against the reference reads the
  same here.

All hot-path arithmetic runs in the CUDA library; there is no CPU fallback:
without the built library or a CUDA device every compute call raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqmin_gb300.so")

QMIN_OK, QMIN_EINVAL, QMIN_ECUDA, QMIN_ENOMEM, QMIN_ESTATE, QMIN_ENONFINITE, QMIN_ENODEVICE, QMIN_ETIMEOUT = range(8)
FP64, FP32 = 0, 1
METRIC_CPU, METRIC_SINGLE = 0, 1
LAYOUT_AOS, LAYOUT_SOA = 0, 1
HOMEOTROPIC, DEGENERATE_PLANAR = 0, 1

EXPORTED_SYMBOLS = [
    "qmin_create", "qmin_destroy", "qmin_set_stream", "qmin_last_error_string", "qmin_kernel_launches",
    "qmin_set_params", "qmin_set_objects", "qmin_set_state", "qmin_get_state", "qmin_n_active", "qmin_force",
    "qmin_energy", "qmin_fire_init", "qmin_fire_run", "qmin_adam_run", "qmin_nesterov_run", "qmin_lbfgs_run",
    "qmin_gd_run", "qmin_get_sides", "qmin_get_types", "qmin_set_positions", "qmin_defect_measures", "qmin_object_forces",
    "qmin_save_state", "qmin_load_state", "qmin_set_field_map", "qmin_load_field_map", "qmin_checkpoint_save", "qmin_checkpoint_load", "qmin_host_boundary_file",
    "qmin_host_random_nematic", "qmin_host_add_wall", "qmin_host_add_sphere", "qmin_set_fire_kernel",
    "qmin_set_fire_variant",
    "qmin_fire_profile", "qmin_fire_tuning", "qmin_energy_noalloc", "qmin_batch_create", "qmin_batch_destroy",
    "qmin_batch_set_params", "qmin_batch_set_solve", "qmin_batch_get_solve", "qmin_batch_fire_init",
    "qmin_batch_fire_run", "qmin_batch_kernel_launches", "qmin_warmnet_create", "qmin_warmnet_destroy",
    "qmin_warmnet_set_stream", "qmin_warmnet_param_count", "qmin_warmnet_shape", "qmin_warmnet_buffers",
    "qmin_warmnet_set_params", "qmin_warmnet_get_params", "qmin_warmnet_features", "qmin_warmnet_forward",
    "qmin_warmnet_backward", "qmin_warmnet_adam_step", "qmin_warmnet_write_state", "qmin_warmnet_sync",
    "qmin_warmnet_set_tensor_path", "qmin_set_wait_limit",
    "qmin_warmnet_kernel_launches", "qmin_warm_start",
]
FIRE_SEPARATE, FIRE_FUSED, FIRE_AUTO, FIRE_TILED, FIRE_SPLIT = 0, 1, 2, 3, 4


class QminError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"qmin error {code}: {msg}")
        self.code = code


class LatticeDesc(C.Structure):
    _fields_ = [("Lx", C.c_int), ("Ly", C.c_int), ("Lz", C.c_int), ("precision", C.c_int), ("metric_mode", C.c_int)]


class LdgParams(C.Structure):
    _fields_ = [("A", C.c_double), ("B", C.c_double), ("C", C.c_double),
                ("L1", C.c_double), ("L2", C.c_double), ("L3", C.c_double), ("L4", C.c_double),
                ("multi_constant", C.c_int), ("efield", C.c_int),
                ("E", C.c_double * 3), ("eps", C.c_double), ("eps0", C.c_double), ("deps", C.c_double),
                ("hfield", C.c_int),
                ("H", C.c_double * 3), ("chi", C.c_double), ("mu0", C.c_double), ("dchi", C.c_double),
                ("L6", C.c_double)]


class Object(C.Structure):
    _fields_ = [("kind", C.c_int), ("W", C.c_double), ("S0", C.c_double)]


class FireParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("alpha_start", C.c_double), ("dt_max", C.c_double), ("dt_inc", C.c_double),
                ("dt_dec", C.c_double), ("alpha_dec", C.c_double), ("alpha_min", C.c_double),
                ("force_cutoff", C.c_double), ("n_min", C.c_int)]


class FireResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("force_max", C.c_double), ("alpha", C.c_double), ("dt", C.c_double),
                ("power", C.c_double), ("n_since", C.c_int)]


class FireState(C.Structure):
    """qmin_fire_state: the FIRE updater's members that persist between minimize() calls."""
    _fields_ = [("iterations", C.c_int), ("force_max", C.c_double), ("alpha", C.c_double), ("dt", C.c_double),
                ("dt_min", C.c_double), ("power", C.c_double), ("n_since", C.c_int)]


_lib = None


def lib():
    """Load the native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"qmin_gb300 native library missing ({LIB_PATH}); run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        h, dp, ip, vp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
        sig = {
            "qmin_create": [C.POINTER(LatticeDesc), C.POINTER(C.c_void_p)],
            "qmin_destroy": [h], "qmin_set_stream": [h, vp],
            "qmin_kernel_launches": [h, C.POINTER(C.c_longlong)],
            "qmin_set_params": [h, C.POINTER(LdgParams)], "qmin_set_objects": [h, C.POINTER(Object), C.c_int],
            "qmin_set_state": [h, vp, vp, C.c_int], "qmin_get_state": [h, vp, vp, vp, C.c_int],
            "qmin_n_active": [h, C.POINTER(C.c_longlong)], "qmin_force": [h, vp],
            "qmin_energy": [h, dp, dp], "qmin_fire_init": [h, C.POINTER(FireParams)],
            "qmin_fire_run": [h, C.c_int, C.POINTER(FireResult)],
            "qmin_adam_run": [h, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, ip, dp],
            "qmin_nesterov_run": [h, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, ip, dp],
            "qmin_lbfgs_run": [h, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, ip, dp],
            "qmin_gd_run": [h, C.c_double, C.c_double, C.c_int, C.c_int, ip, dp],
            "qmin_get_sides": [h, ip, ip, ip], "qmin_get_types": [h, vp], "qmin_set_positions": [h, vp, C.c_int],
            "qmin_set_velocities": [h, vp, C.c_int], "qmin_fire_set_state": [h, C.POINTER(FireState)],
            "qmin_defect_measures": [h, C.c_int, vp], "qmin_object_forces": [h, vp, C.c_int, ip],
            "qmin_set_field_map": [h, vp, C.c_double, C.c_double, C.c_double],
            "qmin_load_field_map": [h, C.c_char_p, C.c_double, C.c_double, C.c_double],
            "qmin_save_state": [h, C.c_char_p, C.c_int, C.c_int], "qmin_load_state": [h, C.c_char_p],
            "qmin_checkpoint_save": [h, C.c_char_p], "qmin_checkpoint_load": [h, C.c_char_p],
            "qmin_host_boundary_file": [C.c_int, C.c_int, C.c_int, C.c_char_p, dp, ip, C.POINTER(Object), C.c_int,
                                        ip],
            "qmin_host_random_nematic": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, dp],
            "qmin_set_fire_kernel": [h, C.c_int],
            "qmin_set_fire_variant": [h, C.c_int],
            "qmin_batch_create": [C.c_int, ip, C.c_int, C.c_int, C.POINTER(C.c_void_p)],
            "qmin_batch_destroy": [h], "qmin_batch_set_params": [h, C.POINTER(LdgParams)],
            "qmin_batch_set_solve": [h, C.c_int, vp, vp, C.POINTER(Object), C.c_int],
            "qmin_batch_get_solve": [h, C.c_int, vp, vp],
            "qmin_batch_fire_init": [h, C.POINTER(FireParams)],
            "qmin_batch_fire_run": [h, C.c_int, ip, dp, ip],
            "qmin_batch_kernel_launches": [h, C.POINTER(C.c_longlong)],
            "qmin_batch_set_barrier_limit": [h, C.c_longlong],
            "qmin_batch_tuning": [h, ip, ip, dp],
            "qmin_batch_set_chunk_shape": [h, C.c_int],
            "qmin_fire_profile": [h, C.c_int, dp, ip],
            "qmin_fire_tuning": [h, ip, ip, ip, ip, ip, dp],
            "qmin_warmnet_create": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)],
            "qmin_warmnet_destroy": [h], "qmin_warmnet_set_stream": [h, vp],
            "qmin_warmnet_param_count": [h, C.POINTER(C.c_longlong)],
            "qmin_warmnet_shape": [h, ip, ip, ip, ip],
            "qmin_warmnet_buffers": [h, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)],
            "qmin_warmnet_set_params": [h, vp], "qmin_warmnet_get_params": [h, vp, vp],
            "qmin_warmnet_features": [h, C.c_int, vp, C.c_int, C.c_longlong, vp, C.POINTER(Object), C.c_int],
            "qmin_warmnet_forward": [h], "qmin_warmnet_backward": [h, vp, dp],
            "qmin_warmnet_adam_step": [h, C.c_double, C.c_double, C.c_double, C.c_double],
            "qmin_warmnet_write_state": [h, C.c_int, vp, C.c_int, C.c_longlong, vp],
            "qmin_warmnet_sync": [h], "qmin_warmnet_kernel_launches": [h, C.POINTER(C.c_longlong)],
            "qmin_warmnet_set_tensor_path": [h, C.c_int],
            "qmin_set_wait_limit": [C.c_longlong],
            "qmin_warm_start": [h, h],
            "qmin_host_add_wall": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, dp,
                                   ip, C.POINTER(Object), ip],
            "qmin_host_add_sphere": [C.c_int, C.c_int, C.c_int, dp, C.c_double, C.c_int, C.c_double, C.c_double, dp,
                                     ip, C.POINTER(Object), ip],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        L.qmin_tuning_cache_clear.argtypes = []
        L.qmin_tuning_cache_clear.restype = C.c_int
        L.qmin_last_error_string.restype = C.c_char_p
        L.qmin_last_error_string.argtypes = []
        _lib = L
    return _lib


def _check(code, iterations=None, force_max=None):
    """Raise QminError for a non-zero status; a minimiser's error carries the
    iterations it completed and the last forceMax (the C entry points write
    both before reporting a non-finite force norm)."""
    if code != QMIN_OK:
        err = QminError(code, lib().qmin_last_error_string().decode())
        err.iterations = iterations.value if iterations is not None else None
        err.forceMax = force_max.value if force_max is not None else None
        raise err


def set_wait_limit(polls=-1):
    """Polls of the library's TMA waits before a kernel gives up: the net's
    direct convolution (WarmNet.sync then raises QMIN_ETIMEOUT) and the
    TMA-staged deep-site FIRE kernel (fire_run raises QMIN_ETIMEOUT, the
    lattice's state is void).  0 gives up at once, a negative value restores
    the defaults.  Process-wide."""
    _check(lib().qmin_set_wait_limit(int(polls)))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def cli_phase_constants(A=-0.172, B=-2.12, Cc=1.73):
    """openQmin.cpp:173-175 rescaling and the S0 of openQmin.cpp:266."""
    a, b, c = -1.0, -B / A, -Cc / A
    S0 = (-b + np.sqrt(b * b - 24 * a * c)) / (6 * c)
    return a, b, c, float(S0)


# ---------------------------------------------------------------- host set-up
def host_random_nematic(L, seed, S0):
    """qTensorLatticeModel::setNematicQTensorRandomly with seed (host)."""
    N = L[0] * L[1] * L[2]
    Q = np.zeros((N, 5))
    _check(lib().qmin_host_random_nematic(L[0], L[1], L[2], int(seed), float(S0), _dp(Q)))
    return Q


class Geometry:
    """Q field, site types and object table under construction on the host."""

    def __init__(self, L, Q):
        self.L = tuple(int(x) for x in L)
        self.Q = np.ascontiguousarray(Q, dtype=np.float64)
        self.types = np.zeros(self.L[0] * self.L[1] * self.L[2], dtype=np.int32)
        self.objs = (Object * 127)()
        self.nobj = C.c_int(0)

    def add_wall(self, xyz, plane, kind, W, S0):
        _check(lib().qmin_host_add_wall(*self.L, int(xyz), int(plane), int(kind), float(W), float(S0), _dp(self.Q),
                                        _ip(self.types), self.objs, C.byref(self.nobj)))

    def add_sphere(self, center, radius, kind, W, S0):
        c = (C.c_double * 3)(*[float(x) for x in center])
        _check(lib().qmin_host_add_sphere(*self.L, c, float(radius), int(kind), float(W), float(S0), _dp(self.Q),
                                          _ip(self.types), self.objs, C.byref(self.nobj)))

    def add_boundary_file(self, path):
        """Objects from a boundary file in the reference's format (createBoundaryFromFile)."""
        _check(lib().qmin_host_boundary_file(*self.L, os.fsencode(path), _dp(self.Q), _ip(self.types), self.objs,
                                             127, C.byref(self.nobj)))

    def objects(self):
        return [(self.objs[k].kind, self.objs[k].W, self.objs[k].S0) for k in range(self.nobj.value)]


# -------------------------------------------------------------- C handle
class Lattice:
    """One lattice resident on the GPU (a qmin_handle)."""

    def __init__(self, L, precision=FP64, metric_mode=METRIC_CPU):
        self.L = tuple(int(x) for x in L)
        self.N = self.L[0] * self.L[1] * self.L[2]
        self.precision = precision
        d = LatticeDesc(self.L[0], self.L[1], self.L[2], precision, metric_mode)
        self._h = C.c_void_p()
        _check(lib().qmin_create(C.byref(d), C.byref(self._h)))

    def close(self):
        if self._h:
            lib().qmin_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, A, B, Cc, L1=0.0, L2=0.0, L3=0.0, L4=0.0, multi_constant=None, E=None, H=None, L6=0.0):
        p = LdgParams()
        p.A, p.B, p.C = A, B, Cc
        p.L1, p.L2, p.L3, p.L4, p.L6 = L1, L2, L3, L4, L6
        p.multi_constant = (int(any(x != 0 for x in (L2, L3, L4, L6))) if multi_constant is None
                            else int(multi_constant))
        if E is not None:
            p.efield = 1
            p.E[0], p.E[1], p.E[2], p.eps, p.eps0, p.deps = E
        if H is not None:
            p.hfield = 1
            p.H[0], p.H[1], p.H[2], p.chi, p.mu0, p.dchi = H
        _check(lib().qmin_set_params(self._h, C.byref(p)))

    def set_objects(self, objs):
        arr = (Object * max(len(objs), 1))()
        for k, (kind, W, S0) in enumerate(objs):
            arr[k].kind, arr[k].W, arr[k].S0 = kind, W, S0
        _check(lib().qmin_set_objects(self._h, arr, len(objs)))

    def set_state(self, Q, types, layout=LAYOUT_AOS):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        types = np.ascontiguousarray(types, dtype=np.int32)
        _check(lib().qmin_set_state(self._h, Q.ctypes.data, types.ctypes.data, layout))

    def set_state_ptr(self, q_ptr, t_ptr, layout=LAYOUT_AOS):
        _check(lib().qmin_set_state(self._h, q_ptr, t_ptr, layout))

    def get_state(self, Q=True, V=False, F=False, layout=LAYOUT_AOS):
        shape = (self.N, 5) if layout == LAYOUT_AOS else (5, self.N)
        out = [np.zeros(shape) if want else None for want in (Q, V, F)]
        ptrs = [o.ctypes.data if o is not None else None for o in out]
        _check(lib().qmin_get_state(self._h, *ptrs, layout))
        return out

    def get_state_ptr(self, q_ptr, v_ptr, f_ptr, layout=LAYOUT_AOS):
        _check(lib().qmin_get_state(self._h, q_ptr, v_ptr, f_ptr, layout))

    def n_active(self):
        n = C.c_longlong()
        _check(lib().qmin_n_active(self._h, C.byref(n)))
        return n.value

    def force(self, copy=True):
        F = np.zeros((self.N, 5)) if copy else None
        _check(lib().qmin_force(self._h, F.ctypes.data if copy else None))
        return F

    def energy(self):
        e = C.c_double()
        comps = np.zeros(5)
        _check(lib().qmin_energy(self._h, C.byref(e), _dp(comps)))
        return e.value, comps

    def fire_init(self, dt=5e-4, alpha_start=0.99, dt_max=None, dt_inc=1.1, dt_dec=0.95, alpha_dec=0.9,
                  n_min=4, force_cutoff=1e-12, alpha_min=0.0):
        """Defaults: the reference CLI's FIRE parameters (openQmin.cpp:256-258)."""
        p = FireParams(dt, alpha_start, 100 * dt if dt_max is None else dt_max, dt_inc, dt_dec, alpha_dec,
                       alpha_min, force_cutoff, n_min)
        _check(lib().qmin_fire_init(self._h, C.byref(p)))

    def fire_run(self, max_iterations):
        r = FireResult()
        _check(lib().qmin_fire_run(self._h, int(max_iterations), C.byref(r)))
        return dict(iterations=r.iterations, forceMax=r.force_max, alpha=r.alpha, dt=r.dt, power=r.power,
                    nsince=r.n_since)

    def set_velocities(self, V, layout=LAYOUT_AOS):
        V = np.ascontiguousarray(V, dtype=np.float64)
        _check(lib().qmin_set_velocities(self._h, V.ctypes.data, layout))

    def fire_set_state(self, iterations, force_max, alpha, dt, dt_min, power, n_since):
        """Restore the FIRE scalars an updater object keeps between minimize() calls."""
        st = FireState(int(iterations), force_max, alpha, dt, dt_min, power, int(n_since))
        _check(lib().qmin_fire_set_state(self._h, C.byref(st)))

    def adam_run(self, max_iterations, dt=1e-4, beta1=0.9, beta2=0.99, eps=1e-8, force_cutoff=1e-12, reset=True):
        it, fm = C.c_int(), C.c_double()
        _check(lib().qmin_adam_run(self._h, beta1, beta2, eps, dt, force_cutoff, int(max_iterations), int(reset),
                                   C.byref(it), C.byref(fm)), it, fm)
        return dict(iterations=it.value, forceMax=fm.value)

    def nesterov_run(self, max_iterations, dt=1e-4, mu=0.01, force_cutoff=1e-12, reset=True):
        it, fm = C.c_int(), C.c_double()
        _check(lib().qmin_nesterov_run(self._h, dt, mu, force_cutoff, int(max_iterations), int(reset), C.byref(it),
                                       C.byref(fm)), it, fm)
        return dict(iterations=it.value, forceMax=fm.value)

    def lbfgs_run(self, max_iterations, eta=1e-4, m=5, force_cutoff=1e-12, reset=True):
        it, fm = C.c_int(), C.c_double()
        _check(lib().qmin_lbfgs_run(self._h, int(m), eta, force_cutoff, int(max_iterations), int(reset), C.byref(it),
                                    C.byref(fm)), it, fm)
        return dict(iterations=it.value, forceMax=fm.value)

    def get_types(self):
        t = np.zeros(self.N, dtype=np.int32)
        _check(lib().qmin_get_types(self._h, t.ctypes.data))
        return t

    def set_positions(self, Q, layout=LAYOUT_AOS):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        _check(lib().qmin_set_positions(self._h, Q.ctypes.data, layout))

    def defect_measures(self, kind=0):
        """0 largest eigenvalue, 1 det Q, 2 (tr Q^2)^3 - 54 det(Q)^2 (object sites 0)."""
        out = np.zeros(self.N)
        _check(lib().qmin_defect_measures(self._h, int(kind), out.ctypes.data))
        return out

    def set_field_map(self, H, chi, mu0, dchi):
        """Per-site H field (N x 3; None switches it off); chi, mu0, dchi replace the H constants."""
        if H is None:
            _check(lib().qmin_set_field_map(self._h, None, chi, mu0, dchi))
            return
        H = np.ascontiguousarray(H, dtype=np.float64).reshape(self.N, 3)
        _check(lib().qmin_set_field_map(self._h, H.ctypes.data, chi, mu0, dchi))

    def load_field_map(self, prefix, chi, mu0, dchi):
        _check(lib().qmin_load_field_map(self._h, os.fsencode(prefix), chi, mu0, dchi))

    def object_forces(self):
        """Force on every object from the stress tensor (one-constant form): array [nobj, 3]."""
        out = np.zeros((127, 3))
        n = C.c_int()
        _check(lib().qmin_object_forces(self._h, out.ctypes.data, 127, C.byref(n)))
        return out[:n.value].copy()

    def save_state(self, prefix, lattice_skip=1, defect_kind=0):
        _check(lib().qmin_save_state(self._h, os.fsencode(prefix), int(lattice_skip), int(defect_kind)))

    def load_state(self, prefix):
        _check(lib().qmin_load_state(self._h, os.fsencode(prefix)))

    def checkpoint_save(self, path):
        _check(lib().qmin_checkpoint_save(self._h, os.fsencode(path)))

    def checkpoint_load(self, path):
        _check(lib().qmin_checkpoint_load(self._h, os.fsencode(path)))

    def gd_run(self, max_iterations, dt=0.01, force_cutoff=1e-7, reset=True):
        its, fm = C.c_int(), C.c_double()
        _check(lib().qmin_gd_run(self._h, dt, force_cutoff, int(max_iterations), int(bool(reset)), C.byref(its),
                                 C.byref(fm)), its, fm)
        return dict(iterations=its.value, forceMax=fm.value)

    def set_fire_kernel(self, mode):
        """FIRE_AUTO (default): autotuned; FIRE_FUSED: one tiled kernel per iteration; FIRE_SEPARATE;
        FIRE_TILED: separate predictor and derivatives, force + kick from shared-memory tiles (FP32);
        FIRE_SPLIT: deep bulk sites over Q on the 25-point stencil, the rest through derivative planes."""
        _check(lib().qmin_set_fire_kernel(self._h, int(mode)))

    def set_fire_variant(self, variant):
        """Pin one variant (index within the strategy set by set_fire_kernel), or -1 for the autotuner's choice."""
        _check(lib().qmin_set_fire_variant(self._h, int(variant)))

    def fire_profile(self, iterations=20):
        ms = (C.c_double * 4)()
        fused = C.c_int()
        _check(lib().qmin_fire_profile(self._h, int(iterations), ms, C.byref(fused)))
        return list(ms), bool(fused.value)

    def fire_tuning(self):
        path, var, tx, ty, zc = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        ms = (C.c_double * 29)()
        _check(lib().qmin_fire_tuning(self._h, C.byref(path), C.byref(var), C.byref(tx), C.byref(ty), C.byref(zc),
                                      ms))
        names = (["separate_1blk", "separate_2blk", "separate_3blk"]
                 + [f"fused_{a}x{b}_z{v}" for a, b in ((32, 8), (32, 16), (64, 8), (32, 4)) for v in (0, 1)]
                 + [f"tiled_{a}x{b}_z{v}" for a, b in ((32, 8), (32, 4), (16, 16)) for v in (0, 1)]
                 + ["split_1blk", "split_2blk", "split_smem_32x8", "split_smem_16x16", "split_pair_32x8_z8",
                    "split_pair_32x8_zfit", "split_pair_tma_32x8", "split_fused_32x8_z16", "split_fused_32x8_zfit",
                    "split_fused_32x4_z16", "split_fused_cp_32x8", "split_fused_cp_32x4"])
        return dict(path=["separate", "fused", "tiled", "split"][path.value], variant=var.value, tile=(tx.value, ty.value),
                    zc=zc.value, candidates_ms={n: m for n, m in zip(names, ms) if m >= 0})

    def launches(self):
        n = C.c_longlong()
        _check(lib().qmin_kernel_launches(self._h, C.byref(n)))
        return n.value

    def warm_start(self, net):
        """Replace Q on the sites the minimiser moves by the net's prediction
        from the current Q, types and objects (qmin_warm_start)."""
        _check(lib().qmin_warm_start(self._h, net._h))


class Batch:
    """Many independent lattices of uneven sizes minimised together (a qmin_batch)."""

    def __init__(self, dims, precision=FP64, metric_mode=METRIC_CPU):
        self.dims = [tuple(int(x) for x in d) for d in dims]
        arr = np.ascontiguousarray(np.array(self.dims, dtype=np.int32).ravel())
        self._h = C.c_void_p()
        _check(lib().qmin_batch_create(len(self.dims), _ip(arr), precision, metric_mode, C.byref(self._h)))

    def close(self):
        if self._h:
            lib().qmin_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, A, B, Cc, L1=0.0, L2=0.0, L3=0.0, L4=0.0, multi_constant=None, E=None, H=None, L6=0.0):
        p = LdgParams()
        p.A, p.B, p.C = A, B, Cc
        p.L1, p.L2, p.L3, p.L4, p.L6 = L1, L2, L3, L4, L6
        p.multi_constant = (int(any(x != 0 for x in (L2, L3, L4, L6))) if multi_constant is None
                            else int(multi_constant))
        if E is not None:
            p.efield = 1
            p.E[0], p.E[1], p.E[2], p.eps, p.eps0, p.deps = E
        if H is not None:
            p.hfield = 1
            p.H[0], p.H[1], p.H[2], p.chi, p.mu0, p.dchi = H
        _check(lib().qmin_batch_set_params(self._h, C.byref(p)))

    def set_solve(self, s, Q, types, objs):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        types = np.ascontiguousarray(types, dtype=np.int32)
        arr = (Object * max(len(objs), 1))()
        for k, (kind, W, S0) in enumerate(objs):
            arr[k].kind, arr[k].W, arr[k].S0 = kind, W, S0
        _check(lib().qmin_batch_set_solve(self._h, int(s), Q.ctypes.data, types.ctypes.data, arr, len(objs)))

    def get_solve(self, s, F=False):
        n = int(np.prod(self.dims[s]))
        Q = np.zeros((n, 5))
        Fo = np.zeros((n, 5)) if F else None
        _check(lib().qmin_batch_get_solve(self._h, int(s), Q.ctypes.data, Fo.ctypes.data if F else None))
        return (Q, Fo) if F else Q

    def fire_init(self, dt=5e-4, alpha_start=0.99, dt_max=None, dt_inc=1.1, dt_dec=0.95, alpha_dec=0.9, n_min=4,
                  force_cutoff=1e-12, alpha_min=0.0):
        p = FireParams(dt, alpha_start, 100 * dt if dt_max is None else dt_max, dt_inc, dt_dec, alpha_dec,
                       alpha_min, force_cutoff, n_min)
        _check(lib().qmin_batch_fire_init(self._h, C.byref(p)))

    def fire_run(self, max_iterations):
        n = len(self.dims)
        its = np.zeros(n, dtype=np.int32)
        fm = np.zeros(n)
        conv = C.c_int()
        _check(lib().qmin_batch_fire_run(self._h, int(max_iterations), _ip(its), _dp(fm), C.byref(conv)))
        return dict(iterations=its, forceMax=fm, converged=conv.value)

    def set_chunk_shape(self, shape):
        """0: 256 consecutive sites; 1-4: tiles of 32x8x1, 16x16x1, 16x4x4, 8x8x4; -1: tuned."""
        _check(lib().qmin_batch_set_chunk_shape(self._h, int(shape)))

    def set_barrier_limit(self, spins):
        _check(lib().qmin_batch_set_barrier_limit(self._h, int(spins)))

    def tuning(self):
        shape = C.c_int()
        tile = (C.c_int * 3)()
        ms = (C.c_double * 5)()
        _check(lib().qmin_batch_tuning(self._h, C.byref(shape), tile, ms))
        names = ["linear_256", "tile_32x8x1", "tile_16x16x1", "tile_16x4x4", "tile_8x8x4"]
        return dict(shape=shape.value, tile=tuple(tile), candidates_ms={n: m for n, m in zip(names, ms) if m >= 0})

    def launches(self):
        n = C.c_longlong()
        _check(lib().qmin_batch_kernel_launches(self._h, C.byref(n)))
        return n.value


# Learned warm-start net: (cin, cout, taps, stride, input level, relu) per
# layer, in the order of its flat parameter vector (weights [cout][tap][cin],
# then bias [cout]); the table the native library builds.
WARMNET_LAYERS = [(16, 32, 27, 1, 0, True), (32, 48, 27, 2, 0, True), (48, 64, 27, 2, 1, True),
                  (64, 128, 27, 2, 2, True), (128, 64, 1, 1, 3, False), (64, 64, 27, 1, 2, True),
                  (64, 48, 1, 1, 2, False), (48, 48, 27, 1, 1, True), (48, 32, 1, 1, 1, False),
                  (32, 32, 27, 1, 0, True), (32, 16, 1, 1, 0, False)]
WARMNET_IN, WARMNET_OUT = 16, 16


def warmnet_param_slices():
    """(weight slice, bias slice, layer spec) of every layer in the flat vector."""
    out, off = [], 0
    for spec in WARMNET_LAYERS:
        cin, cout, taps = spec[0], spec[1], spec[2]
        w = slice(off, off + cout * taps * cin)
        off += cout * taps * cin
        b = slice(off, off + cout)
        off += cout
        out.append((w, b, spec))
    return out


def warmnet_init_params(seed=0, head_scale=0.1):
    """He-normal weights, zero biases; the head starts small."""
    rng = np.random.default_rng(seed)
    sl = warmnet_param_slices()
    p = np.zeros(sl[-1][1].stop, dtype=np.float32)
    for i, (w, b, (cin, cout, taps, _s, _l, _r)) in enumerate(sl):
        fan_in = cin * taps
        if i == 0:
            fan_in = 10 * taps  # 10 of the 16 input channels carry features
        std = np.sqrt(2.0 / fan_in) * (head_scale if i == len(sl) - 1 else 1.0)
        p[w] = rng.normal(0.0, std, w.stop - w.start).astype(np.float32)
    return p


class _DevArray:
    """A device pointer with __cuda_array_interface__, for zero-copy torch views."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = dict(shape=tuple(shape), typestr=typestr, data=(int(ptr), False), version=2,
                                             strides=None)


class WarmNet:
    """The learned warm-start net (a qmin_warmnet): `batch` lattices of L sites."""

    def __init__(self, batch, L, train=False):
        self.batch, self.L = int(batch), tuple(int(x) for x in L)
        self._h = C.c_void_p()
        _check(lib().qmin_warmnet_create(self.batch, *self.L, int(bool(train)), C.byref(self._h)))
        n = C.c_longlong()
        _check(lib().qmin_warmnet_param_count(self._h, C.byref(n)))
        self.nparams = n.value
        self.sites = self.L[0] * self.L[1] * self.L[2]

    def close(self):
        if self._h:
            lib().qmin_warmnet_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tensor_path(self, path=1):
        """Convolutions on tcgen05.mma with tensor-memory accumulators: 1 (or True,
        the default) with the direct kernel's halo planes staged by TMA, 2 with
        them staged by the threads; 0 (or False) on mma.sync."""
        path = 1 if path is True else (0 if path is False else int(path))
        _check(lib().qmin_warmnet_set_tensor_path(self._h, path))

    def set_stream(self, stream_ptr):
        _check(lib().qmin_warmnet_set_stream(self._h, C.c_void_p(stream_ptr)))

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        _check(lib().qmin_warmnet_set_params(self._h, p.ctypes.data))

    def get_params(self, grads=False):
        p = np.zeros(self.nparams, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32) if grads else None
        _check(lib().qmin_warmnet_get_params(self._h, p.ctypes.data, g.ctypes.data if grads else None))
        return (p, g) if grads else p

    def buffers(self):
        """Device pointers of the input features, output and mask."""
        x, y, m = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(lib().qmin_warmnet_buffers(self._h, C.byref(x), C.byref(y), C.byref(m)))
        return x.value, y.value, m.value

    def torch_views(self):
        """Zero-copy torch views (x as bfloat16 [B, sites, 16], y float32
        [B, sites, 16], mask uint8 [B, sites]) of the net's device buffers."""
        import torch
        x, y, m = self.buffers()
        B, n = self.batch, self.sites
        xv = torch.as_tensor(_DevArray(x, (B, n, WARMNET_IN), "<i2"), device="cuda").view(torch.bfloat16)
        yv = torch.as_tensor(_DevArray(y, (B, n, WARMNET_OUT), "<f4"), device="cuda")
        mv = torch.as_tensor(_DevArray(m, (B, n), "|u1"), device="cuda")
        return xv, yv, mv

    def features(self, sample, q_ptr, precision, plane_stride, types_ptr, objs):
        arr = (Object * max(len(objs), 1))()
        for k, (kind, W, S0) in enumerate(objs):
            arr[k].kind, arr[k].W, arr[k].S0 = kind, W, S0
        _check(lib().qmin_warmnet_features(self._h, int(sample), C.c_void_p(q_ptr), int(precision),
                                           int(plane_stride), C.c_void_p(types_ptr), arr, len(objs)))

    def forward(self):
        _check(lib().qmin_warmnet_forward(self._h))

    def backward(self, target_ptr, want_loss=True):
        loss = C.c_double(float("nan"))
        _check(lib().qmin_warmnet_backward(self._h, C.c_void_p(target_ptr), C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        _check(lib().qmin_warmnet_adam_step(self._h, lr, beta1, beta2, eps))

    def write_state(self, sample, q_ptr, precision, plane_stride, types_ptr):
        _check(lib().qmin_warmnet_write_state(self._h, int(sample), C.c_void_p(q_ptr), int(precision),
                                              int(plane_stride), C.c_void_p(types_ptr)))

    def sync(self):
        _check(lib().qmin_warmnet_sync(self._h))

    def launches(self):
        n = C.c_longlong()
        _check(lib().qmin_warmnet_kernel_launches(self._h, C.byref(n)))
        return n.value


from .reference_api import (energyMinimizerAdam, energyMinimizerFIRE, energyMinimizerGradientDescent,  # noqa: E402,F401
                            energyMinimizerLoLBFGS,
                            energyMinimizerNesterovAG, landauDeGennesLC, multirankSimulation,
                            qTensorLatticeModel, boundaryObject, boundaryType)
