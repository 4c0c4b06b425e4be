"""ctypes binding of the C restatement oracle (oracle/qmin_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the test-suite, the smoke check and
bench.py's CPU-baseline leg, never by the product.  Arrays are numpy, AoS
(N, 5) float64 for Q/V/F and int32 for types, exactly as the reference stores
them.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqmin_oracle.so")


class Params(C.Structure):
    _fields_ = [("Lx", C.c_int), ("Ly", C.c_int), ("Lz", C.c_int),
                ("A", C.c_double), ("B", C.c_double), ("C", C.c_double),
                ("L1", C.c_double), ("L2", C.c_double), ("L3", C.c_double), ("L4", C.c_double),
                ("multi_constant", C.c_int), ("efield", C.c_int), ("hfield", C.c_int),
                ("E", C.c_double * 3), ("eps", C.c_double), ("eps0", C.c_double), ("deps", C.c_double),
                ("H", C.c_double * 3), ("chi", C.c_double), ("mu0", C.c_double), ("dchi", C.c_double),
                ("metric_mode", C.c_int), ("hvar", C.POINTER(C.c_double)), ("L6", C.c_double)]


class Object(C.Structure):
    _fields_ = [("kind", C.c_int), ("W", C.c_double), ("S0", C.c_double)]


class FireParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("alpha0", C.c_double), ("dtmax", C.c_double), ("dtinc", C.c_double),
                ("dtdec", C.c_double), ("alphadec", C.c_double), ("alphamin", C.c_double),
                ("fcut", C.c_double), ("nmin", C.c_int)]


class FireState(C.Structure):
    _fields_ = [("iterations", C.c_int), ("forceMax", C.c_double), ("alpha", C.c_double),
                ("dt", C.c_double), ("power", C.c_double), ("nsince", C.c_int)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.qo_random_nematic.argtypes = [C.c_int, C.c_uint, C.c_double, dp]
        L.qo_add_wall.argtypes = [ip, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, dp, ip, C.POINTER(Object), C.c_int]
        L.qo_add_sites.argtypes = [ip, C.c_int, ip, dp, C.c_int, C.c_double, C.c_double, dp, ip, C.POINTER(Object),
                                   C.c_int]
        L.qo_defects.argtypes = [C.POINTER(Params), dp, ip, C.c_int, dp]
        L.qo_object_forces.argtypes = [C.POINTER(Params), dp, ip, C.POINTER(Object), C.c_int, dp]
        L.qo_object_forces.restype = None
        L.qo_defects.restype = None
        L.qo_add_sphere.argtypes = [ip, dp, C.c_double, C.c_int, C.c_double, C.c_double, dp, ip, C.POINTER(Object), C.c_int]
        L.qo_count_active.argtypes = [C.c_int, ip]
        L.qo_force.argtypes = [C.POINTER(Params), dp, ip, C.POINTER(Object), dp]
        L.qo_energy.argtypes = [C.POINTER(Params), dp, ip, C.POINTER(Object), dp]
        L.qo_energy.restype = C.c_double
        L.qo_energy_densities.argtypes = [C.POINTER(Params), dp, ip, C.POINTER(Object), dp]
        L.qo_energy_densities.restype = None
        L.qo_fire_init.argtypes = [C.POINTER(FireParams), C.POINTER(FireState)]
        L.qo_fire.argtypes = [C.POINTER(Params), dp, dp, dp, ip, C.POINTER(Object), C.POINTER(FireParams), C.c_int,
                              C.POINTER(FireState), dp]
        L.qo_adam.argtypes = [C.POINTER(Params), dp, dp, ip, C.POINTER(Object), C.c_double, C.c_double, C.c_double,
                              C.c_double, C.c_double, C.c_int, dp, dp, dp]
        L.qo_nesterov.argtypes = [C.POINTER(Params), dp, dp, ip, C.POINTER(Object), C.c_double, C.c_double,
                                  C.c_double, C.c_int, dp, dp]
        L.qo_gd.argtypes = [C.POINTER(Params), dp, dp, ip, C.POINTER(Object), C.c_double, C.c_double, C.c_int, dp]
        L.qo_lbfgs.argtypes = [C.POINTER(Params), dp, dp, ip, C.POINTER(Object), C.c_int, C.c_double, C.c_double,
                               C.c_int, dp]
        L.qo_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def cli_phase(A=-0.172, B=-2.12, Cc=1.73):
    """openQmin.cpp:173-175: a = -1, b = -B/A, c = -C/A; S0 (openQmin.cpp:266)."""
    a, b, c = -1.0, -B / A, -Cc / A
    S0 = (-b + np.sqrt(b * b - 24 * a * c)) / (6 * c)
    return a, b, c, S0


class System:
    """A lattice, its Q field, site types and objects, plus force parameters."""

    def __init__(self, L, A=-0.172, B=-2.12, Cc=1.73, Ls=(2.32, 0, 0, 0), E=None, H=None, metric_mode=0):
        self.L = tuple(int(x) for x in L)
        self.N = self.L[0] * self.L[1] * self.L[2]
        a, b, c, self.S0 = cli_phase(A, B, Cc)
        p = Params()
        p.Lx, p.Ly, p.Lz = self.L
        p.A, p.B, p.C = a, b, c
        Ls = tuple(Ls) + (0,) * (5 - len(Ls))
        p.L1, p.L2, p.L3, p.L4, p.L6 = Ls[:5]
        p.multi_constant = int(any(x != 0 for x in Ls[1:]))
        if E is not None:
            p.efield = 1
            p.E[0], p.E[1], p.E[2], p.eps, p.eps0, p.deps = E
        if H is not None:
            p.hfield = 1
            p.H[0], p.H[1], p.H[2], p.chi, p.mu0, p.dchi = H
        p.metric_mode = metric_mode
        self.p = p
        self.Q = np.zeros((self.N, 5))
        self.types = np.zeros(self.N, dtype=np.int32)
        self.objs = (Object * 64)()
        self.nobj = 0

    def random_nematic(self, seed):
        lib().qo_random_nematic(self.N, seed, self.S0, _dp(self.Q))

    def add_wall(self, xyz, plane, kind, W):
        Lc = (C.c_int * 3)(*self.L)
        self.nobj = lib().qo_add_wall(Lc, xyz, plane, kind, W, self.S0, _dp(self.Q), _ip(self.types), self.objs,
                                      self.nobj)

    def add_sphere(self, center, radius, kind, W):
        Lc = (C.c_int * 3)(*self.L)
        cc = (C.c_double * 3)(*center)
        self.nobj = lib().qo_add_sphere(Lc, cc, radius, kind, W, self.S0, _dp(self.Q), _ip(self.types), self.objs,
                                        self.nobj)

    def set_field_map(self, H, chi, mu0, dchi):
        """landauDeGennesLC::setSpatiallyVaryingField: per-site H (N x 3); chi, mu0,
        dchi replace the uniform field's constants."""
        self._hvar = np.ascontiguousarray(H, dtype=np.float64).reshape(self.N, 3)
        self.p.hvar = _dp(self._hvar)
        self.p.chi, self.p.mu0, self.p.dchi = chi, mu0, dchi

    def add_sites(self, xyz, qs, kind, W, S0):
        """One object from explicit sites (wrapped into the box) and their Q."""
        Lc = (C.c_int * 3)(*self.L)
        xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        qs = np.ascontiguousarray(qs, dtype=np.float64).reshape(-1, 5)
        self.nobj = lib().qo_add_sites(Lc, len(xyz), _ip(xyz), _dp(qs), kind, W, S0, _dp(self.Q), _ip(self.types),
                                       self.objs, self.nobj)

    def add_boundary_file(self, path):
        """multirankSimulation::createBoundaryFromFile (multirankSimulationBoundaries.cpp:43-96):
        the object count, then per object "kind W S0 n" and n lines "x y z C1..C5"."""
        lines = open(path).read().split("\n")
        count = int(lines[0].split()[0])
        pos = 1
        for _ in range(count):
            kind, W, S0, n = lines[pos].split()[:4]
            pos += 1
            rows = [ln.split() for ln in lines[pos:pos + int(n)] if ln.strip()]
            pos += int(n)
            xyz = [[int(r[0]), int(r[1]), int(r[2])] for r in rows]
            qs = [[float(v) for v in r[3:8]] for r in rows]
            self.add_sites(xyz, qs, 0 if int(kind) == 0 else 1, float(W), float(S0))

    def defects(self, kind=0, Q=None):
        out = np.zeros(self.N)
        Q = self.Q if Q is None else np.ascontiguousarray(Q, dtype=np.float64)
        lib().qo_defects(C.byref(self.p), _dp(Q), _ip(self.types), int(kind), _dp(out))
        return out

    def object_forces(self, Q=None):
        """Force on every object from the one-constant stress tensor: [nobj, 3]."""
        out = np.zeros((max(self.nobj, 1), 3))
        Q = self.Q if Q is None else np.ascontiguousarray(Q, dtype=np.float64)
        lib().qo_object_forces(C.byref(self.p), _dp(Q), _ip(self.types), self.objs, self.nobj, _dp(out))
        return out[:self.nobj]

    def n_active(self):
        return lib().qo_count_active(self.N, _ip(self.types))

    def force(self, Q=None):
        Q = self.Q if Q is None else np.ascontiguousarray(Q, dtype=np.float64)
        F = np.zeros((self.N, 5))
        lib().qo_force(C.byref(self.p), _dp(Q), _ip(self.types), self.objs, _dp(F))
        return F

    def energy(self, Q=None):
        """Returns (E / NActive, components[5]) like multirankSimulation::computePotentialEnergy."""
        Q = self.Q if Q is None else np.ascontiguousarray(Q, dtype=np.float64)
        comps = np.zeros(5)
        e = lib().qo_energy(C.byref(self.p), _dp(Q), _ip(self.types), self.objs, _dp(comps))
        return e / self.n_active(), comps

    def energy_densities(self, Q=None):
        """Per-site energy densities (N, 5): phase, distortion, anchoring, E, H."""
        Q = self.Q if Q is None else np.ascontiguousarray(Q, dtype=np.float64)
        e = np.zeros((self.N, 5))
        lib().qo_energy_densities(C.byref(self.p), _dp(Q), _ip(self.types), self.objs, _dp(e))
        return e

    def energy_exact_sum(self, Q=None):
        """(E / NActive, components[5]) with every component summed exactly
        rounded (math.fsum) instead of the reference's sequential loop: the
        check for lattices whose sequential FP64 sum carries more rounding
        error than the 1e-12 parity tolerance (millions of sites)."""
        import math
        e = self.energy_densities(Q)
        comps = np.array([math.fsum(e[:, k]) for k in range(5)])
        return math.fsum(comps) / self.n_active(), comps

    def fire(self, iters, dt=5e-4, fcut=1e-12, trace=False, V=None):
        """CLI FIRE parameters (openQmin.cpp:256-258). Updates self.Q in place."""
        fp = FireParams(dt, 0.99, 100 * dt, 1.1, 0.95, 0.9, 0.0, fcut, 4)
        st = FireState()
        lib().qo_fire_init(C.byref(fp), C.byref(st))
        V = np.zeros((self.N, 5)) if V is None else V
        F = np.zeros((self.N, 5))
        tr = np.zeros((max(iters, 1), 5)) if trace else None
        n = lib().qo_fire(C.byref(self.p), _dp(self.Q), _dp(V), _dp(F), _ip(self.types), self.objs, C.byref(fp),
                          iters, C.byref(st), _dp(tr) if trace else None)
        return dict(iterations=st.iterations, forceMax=st.forceMax, alpha=st.alpha, dt=st.dt, power=st.power,
                    nsince=st.nsince, V=V, F=F, trace=tr[:n] if trace else None)

    def adam(self, iters, dt=1e-4, beta1=0.9, beta2=0.99, eps=1e-8, fcut=1e-12):
        M = np.zeros((self.N, 5))
        S = np.zeros((self.N, 5))
        F = np.zeros((self.N, 5))
        fm = C.c_double()
        n = lib().qo_adam(C.byref(self.p), _dp(self.Q), _dp(F), _ip(self.types), self.objs, beta1, beta2, eps, dt,
                          fcut, iters, _dp(M), _dp(S), C.byref(fm))
        return dict(iterations=n, forceMax=fm.value, F=F)

    def nesterov(self, iters, dt=1e-4, mu=0.01, fcut=1e-12):
        alt = self.Q.copy()
        F = np.zeros((self.N, 5))
        fm = C.c_double()
        n = lib().qo_nesterov(C.byref(self.p), _dp(self.Q), _dp(F), _ip(self.types), self.objs, dt, mu, fcut, iters,
                              _dp(alt), C.byref(fm))
        return dict(iterations=n, forceMax=fm.value, F=F)

    def gd(self, iters, dt=0.01, fcut=1e-7):
        """energyMinimizerGradientDescent defaults: dt 0.01, cutoff 1e-7."""
        F = np.zeros((self.N, 5))
        fm = C.c_double()
        n = lib().qo_gd(C.byref(self.p), _dp(self.Q), _dp(F), _ip(self.types), self.objs, dt, fcut, iters,
                        C.byref(fm))
        return dict(iterations=n, forceMax=fm.value, F=F)

    def lbfgs(self, iters, eta=1e-4, m=5, fcut=1e-12):
        F = np.zeros((self.N, 5))
        fm = C.c_double()
        n = lib().qo_lbfgs(C.byref(self.p), _dp(self.Q), _dp(F), _ip(self.types), self.objs, m, eta, fcut, iters,
                           C.byref(fm))
        return dict(iterations=n, forceMax=fm.value, F=F)


def set_threads(n):
    return lib().qo_set_threads(n)
