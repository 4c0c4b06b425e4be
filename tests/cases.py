"""Shared helpers: turn a golden case's dumper arguments into an oracle System
or a GPU Lattice set up the same way."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


_INPUT_DIR = None


def _input_dir():
    """A directory (removed at exit) holding the golden cases' input files."""
    global _INPUT_DIR
    if _INPUT_DIR is None:
        import atexit
        import shutil
        import tempfile
        _INPUT_DIR = tempfile.mkdtemp(prefix="qmin_golden_")
        atexit.register(shutil.rmtree, _INPUT_DIR, True)
    return _INPUT_DIR


def load(name):
    """A golden case; its input files (keys in_<file name with dots as _>) are
    written to a temporary directory that replaces "{d}" in its arguments."""
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    ins = [k for k in g if k.startswith("in_")]
    if ins:
        d = _input_dir()
        for k in ins:
            stem, _, ext = k[3:].rpartition("_")
            with open(os.path.join(d, stem + "." + ext), "w") as f:
                f.write(str(g[k]))
        g["args"] = np.array(str(g["args"]).replace("{d}", d))
    return g


def parse_args(args):
    if isinstance(args, np.ndarray):
        args = json.loads(str(args))
    cfg = {"walls": [], "spheres": [], "E": None, "H": None, "Ls": (2.32, 0, 0, 0, 0), "seed": 13371,
           "minimizer": "none", "iters": 0, "dt": 5e-4}
    for a in args:
        k, v = a.split("=", 1)
        if k == "L":
            cfg["L"] = tuple(int(x) for x in v.split(","))
        elif k == "Ls":
            cfg["Ls"] = tuple(float(x) for x in v.split(","))
        elif k == "seed":
            cfg["seed"] = int(v)
        elif k == "wall":
            w = v.split(",")
            cfg["walls"].append((int(w[0]), int(w[1]), 1 if w[2] == "p" else 0, float(w[3])))
        elif k == "sphere":
            s = v.split(",")
            cfg["spheres"].append(((float(s[0]), float(s[1]), float(s[2])), float(s[3]), 1 if s[4] == "p" else 0,
                                   float(s[5])))
        elif k in ("E", "H"):
            cfg[k] = tuple(float(x) for x in v.split(","))
        elif k == "minimizer":
            cfg["minimizer"] = v
        elif k == "iters":
            cfg["iters"] = int(v)
        elif k == "dt":
            cfg["dt"] = float(v)
        elif k in ("bfile", "loadstate"):
            cfg[k] = v
        elif k == "hfile":
            f = v.split(",")
            cfg["hfile"] = (f[0], float(f[1]), float(f[2]), float(f[3]))
    return cfg


def oracle_system(qo, cfg, metric_mode=0):
    s = qo.System(cfg["L"], Ls=cfg["Ls"][:5], E=cfg["E"], H=cfg["H"], metric_mode=metric_mode)
    s.random_nematic(cfg["seed"])
    for xyz, plane, kind, W in cfg["walls"]:
        s.add_wall(xyz, plane, kind, W)
    for c, r, kind, W in cfg["spheres"]:
        s.add_sphere(c, r, kind, W)
    if "bfile" in cfg:
        s.add_boundary_file(cfg["bfile"])
    if "loadstate" in cfg:
        load_state_text(s.Q, s.L, cfg["loadstate"] + "_x0y0z0.txt")
    if "hfile" in cfg:
        prefix, chi, mu0, dchi = cfg["hfile"]
        H = np.zeros((s.N, 3))
        vals = open(prefix + "_x0y0z0.txt").read().split()
        for r in range(len(vals) // 6):
            x, y, z = (int(float(v)) for v in vals[6 * r:6 * r + 3])
            H[x + s.L[0] * (y + s.L[1] * z)] = [float(v) for v in vals[6 * r + 3:6 * r + 6]]
        s.set_field_map(H, chi, mu0, dchi)
        s.hfile = cfg["hfile"]
    return s


def load_state_text(Q, L, path):
    """multirankSimulation::loadState (multirankSimulation.cpp:581-613): Q of every listed site."""
    vals = open(path).read().split()
    for r in range(len(vals) // 10):
        x, y, z = (int(v) for v in vals[10 * r:10 * r + 3])
        Q[x + L[0] * (y + L[1] * z)] = [float(v) for v in vals[10 * r + 3:10 * r + 8]]


def gpu_lattice(qmin, s, precision=0, metric_mode=0):
    """A GPU lattice with the oracle system's parameters, objects and state."""
    lat = qmin.Lattice(s.L, precision, metric_mode)
    p = s.p
    lat.set_params(p.A, p.B, p.C, p.L1, p.L2, p.L3, p.L4, multi_constant=p.multi_constant, L6=p.L6,
                   E=(p.E[0], p.E[1], p.E[2], p.eps, p.eps0, p.deps) if p.efield else None,
                   H=(p.H[0], p.H[1], p.H[2], p.chi, p.mu0, p.dchi) if p.hfield else None)
    lat.set_objects([(s.objs[k].kind, s.objs[k].W, s.objs[k].S0) for k in range(s.nobj)])
    lat.set_state(s.Q, s.types)
    if getattr(s, "hfile", None):
        lat.load_field_map(*s.hfile)  # the library's own reader of the field file
    return lat


def rel_err(a, b):
    """Normwise relative error max|a-b| / max|b| over finite entries of b."""
    m = np.isfinite(b)
    return float(np.abs(a[m] - b[m]).max() / max(np.abs(b[m]).max(), 1e-300))


GOLDEN_CASES = ["l1_bulk_fire", "l123_walls_sphere_fire", "planar_sphere_fire", "l1234_planar_fields_fire",
                "edges_gaps_wrap", "adam", "nesterov", "lbfgs", "gd", "boundary_file_defects", "load_state",
                "field_map", "l6_fire", "object_forces"]
