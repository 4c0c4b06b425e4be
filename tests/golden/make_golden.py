#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

Runs oracle/_ref/ref_dumper (the reference's own CPU objects, compiled from
the reference tree by oracle/ref/Makefile) on a set of small seeded cases and
stores its dumps as compressed .npz files.  Needs the reference tree, so it
runs only where that tree is mounted:

    make -C oracle/ref -j8 && python3 tests/golden/make_golden.py

Each case records: the arguments, the initial Q and site types, the force at
Q0 (CPU-path semantics), the energy at Q0 (E/NActive and its five
components), the per-iteration minimiser trace where available, and the final
Q, velocities, forces, forceMax and energy.
"""
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DUMPER = os.path.join(ROOT, "oracle", "_ref", "ref_dumper")

# name -> (dumper arguments, keep full arrays)
CASES = {
    # one-constant, all bulk (the 50^3 CLI configuration at a small size)
    "l1_bulk_fire": (["L=12,10,9", "seed=13371", "Ls=2.32,0,0,0,0", "minimizer=fire", "iters=40", "trace=1"], True),
    # multi-constant L1-L3, two homeotropic z-walls and a homeotropic sphere
    "l123_walls_sphere_fire": (["L=12,11,10", "seed=5", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3", "wall=2,9,h,5.3",
                                "sphere=6,5.5,4.5,2.6,h,5.3", "minimizer=fire", "iters=30", "trace=1"], True),
    # degenerate planar (Fournier-Galatola) sphere, one-constant
    "planar_sphere_fire": (["L=11,11,11", "seed=17", "Ls=2.32,0,0,0,0", "sphere=5.3,5.6,4.9,3.1,p,1.3",
                            "minimizer=fire", "iters=30", "trace=1"], True),
    # L1-L4, planar sphere + homeotropic x-wall, E and H fields
    "l1234_planar_fields_fire": (["L=10,9,11", "seed=23", "Ls=2.32,1.0,0.5,0.7,0", "wall=0,0,h,3.0",
                                  "sphere=5,4.5,5.5,2.3,p,2.0", "E=0.1,0.2,0.5,1,1,0.5", "H=0.3,0,0.2,1.2,0.9,0.4",
                                  "minimizer=fire", "iters=25", "trace=1"], True),
    # edge cases: sites squeezed between two objects along one axis (walls at z=0 and z=2),
    # a sphere wrapping through the periodic boundary, overlapping objects
    "edges_gaps_wrap": (["L=10,10,10", "seed=99", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3", "wall=2,2,p,1.0",
                         "sphere=0.5,0.5,6,2.4,h,4.0", "sphere=8.3,2.2,3.4,1.8,p,2.5", "minimizer=fire", "iters=20",
                         "trace=1"], True),
    # the other minimisers on a multi-constant lattice with objects
    "adam": (["L=10,9,8", "seed=3", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3", "sphere=5,4,4,2.1,p,1.5",
              "minimizer=adam", "iters=25", "dt=0.0005"], True),
    "nesterov": (["L=10,9,8", "seed=4", "Ls=2.32,1.0,0.5,0,0", "wall=1,0,h,5.3", "sphere=5,4,4,2.1,h,5.3",
                  "minimizer=nesterov", "iters=25", "dt=0.0005"], True),
    "lbfgs": (["L=10,9,8", "seed=6", "Ls=2.32,0,0,0,0", "wall=0,0,p,1.0", "sphere=5,4,4,2.1,h,5.3",
               "minimizer=lbfgs", "iters=25", "dt=0.0005"], True),
    # gradient descent (energyMinimizerGradientDescent, dt 0.01 is the class default)
    "gd": (["L=10,9,8", "seed=8", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3", "sphere=5,4,4.5,2.3,p,1.2",
            "minimizer=gd", "iters=30", "dt=0.01"], True),
    # objects read from a boundary file, FIRE, defect measures and saveState (skip 2, largest eigenvalue)
    "boundary_file_defects": (["L=12,10,9", "seed=31", "Ls=2.32,1.0,0.5,0,0", "bfile={d}/objects.txt",
                               "minimizer=fire", "iters=15", "trace=1", "defects=1", "savestate={d}/st,2,0"], True),
    # loadState of a state file (Q only; types are not loaded).  A FIRE updater is attached (with no
    # iterations) because finalizeObjects takes NActive, the energy's divisor, from the updaters
    "load_state": (["L=7,6,5", "seed=2", "Ls=2.32,0,0,0,0", "loadstate={d}/ld", "minimizer=fire", "iters=0"], True),
    # spatially varying H field read from a file, L1-L3, wall + planar sphere
    "field_map": (["L=9,8,7", "seed=41", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3", "sphere=4.5,4,4,2.2,p,1.7",
                   "hfile={d}/hf,1.3,0.8,0.6", "minimizer=fire", "iters=20", "trace=1"], True),
    # the cubic L6 term with L1-L3, homeotropic wall and sphere, planar sphere (bulk and boundary forms)
    "l6_fire": (["L=11,10,9", "seed=53", "Ls=2.32,1.0,0.5,0,0.8", "wall=2,0,h,5.3", "sphere=5,5,4.5,2.4,h,4.0",
                 "sphere=1.3,8.2,6.4,1.9,p,1.2", "minimizer=fire", "iters=20", "trace=1"], True),
    # forces on objects from the stress tensor (one-constant): a homeotropic sphere, a planar sphere
    # and a wall, after FIRE
    "object_forces": (["L=14,12,11", "seed=61", "Ls=2.32,0,0,0,0", "wall=2,0,h,5.3", "sphere=4.3,5.2,5.6,2.6,h,4.0",
                       "sphere=10.2,6.4,5.1,2.2,p,1.5", "minimizer=fire", "iters=25", "trace=1", "objforce=1"],
                      True),
    # the 50^3 one-constant CLI run (openQmin -i 100 -l 50 --L1 2.32): scalars only
    "c1_50cube_fire100": (["L=50,50,50", "seed=13371", "Ls=2.32,0,0,0,0", "minimizer=fire", "iters=100",
                           "trace=1"], False),
}


def boundary_file_text():
    """A boundary file in the reference's format (multirankSimulationBoundaries.cpp:7-41),
    written here: a homeotropic 3x3x2 block with a tilted preferred director, and a
    degenerate planar plate on z = 0 whose sites partly lie outside the box (x = -1
    and x = 12 wrap periodically)."""
    S0 = 0.53
    n = np.array([0.3, -0.5, 0.81])
    n = n / np.linalg.norm(n)
    qb = 1.5 * S0 * (np.outer(n, n) - np.eye(3) / 3.0)
    q5 = [qb[0, 0], qb[0, 1], qb[0, 2], qb[1, 1], qb[1, 2]]
    block = [(x, y, z) for z in (6, 7) for y in (3, 4, 5) for x in (2, 3, 4)]
    plate = [(x, y, 0) for y in range(0, 10, 3) for x in range(-1, 13)]
    lines = ["2", f"0 4.0 {S0} {len(block)}"]
    lines += [f"{x} {y} {z} " + " ".join(f"{v:.15g}" for v in q5) for (x, y, z) in block]
    lines += [f"1 1.5 {S0} {len(plate)}"]
    lines += [f"{x} {y} {z} 0 0 1 0 0" for (x, y, z) in plate]
    return "\n".join(lines) + "\n"


def state_file_text(L, seed):
    """A state file in saveState's layout (multirankSimulation.cpp:616-665) for every
    site of an L box, with seeded values, written here for the loadState case."""
    rng = np.random.default_rng(seed)
    rows = []
    for z in range(L[2]):
        for y in range(L[1]):
            for x in range(L[0]):
                q = rng.uniform(-0.3, 0.3, 5)
                rows.append(f"{x}\t{y}\t{z}\t" + "\t".join(f"{v:g}" for v in q) + "\t0\t0")
    return "\n".join(rows) + "\n"


def field_file_text(L):
    """A spatially varying H field file (landauDeGennesLC.cpp:81-123 layout: x y z Hx Hy Hz),
    written here: a smooth field on every site with x + y even (the others keep H = 0)."""
    rows = []
    for z in range(L[2]):
        for y in range(L[1]):
            for x in range(L[0]):
                if (x + y) % 2:
                    continue
                h = (0.4 * np.sin(2 * np.pi * x / L[0]), 0.15 + 0.05 * y, 0.3 * np.cos(2 * np.pi * z / L[2]))
                rows.append(f"{x} {y} {z} {h[0]:.12g} {h[1]:.12g} {h[2]:.12g}")
    return "\n".join(rows) + "\n"


# cases that need input files (written into the run directory; "{d}" in an
# argument is replaced by that directory) and collect output text files
FILES = {
    "boundary_file_defects": ({"objects.txt": boundary_file_text}, ["st_x0y0z0.txt"]),
    "load_state": ({"ld_x0y0z0.txt": lambda: state_file_text((7, 6, 5), 3)}, []),
    "field_map": ({"hf_x0y0z0.txt": lambda: field_file_text((9, 8, 7))}, []),
}


def run_case(name, args, full):
    with tempfile.TemporaryDirectory() as d:
        pre, post = FILES.get(name, ({}, []))
        for fn, make in pre.items():
            with open(os.path.join(d, fn), "w") as f:
                f.write(make())
        args = [a.replace("{d}", d) for a in args]
        subprocess.run([DUMPER, d] + args, check=True, capture_output=True)
        ld = lambda f, dt=np.float64: np.fromfile(os.path.join(d, f), dtype=dt)
        out = {"args": np.array(json.dumps(args))}
        e0 = np.array([float(x) for x in open(os.path.join(d, "energy0.txt")).read().split()])
        fin = np.array([float(x) for x in open(os.path.join(d, "final.txt")).read().split()])
        out["energy0"] = e0
        out["final"] = fin
        if os.path.exists(os.path.join(d, "trace.txt")):
            out["trace"] = np.loadtxt(os.path.join(d, "trace.txt"), ndmin=2)
        types = ld("types.i32", np.int32)
        out["types"] = types.astype(np.int8)
        if full:
            out["q0"] = ld("q0.f64").reshape(-1, 5)
            out["force0"] = ld("force0.f64").reshape(-1, 5)
            out["qfinal"] = ld("qfinal.f64").reshape(-1, 5)
            out["vfinal"] = ld("vfinal.f64").reshape(-1, 5)
            out["ffinal"] = ld("ffinal.f64").reshape(-1, 5)
        for fn, make in pre.items():
            out["in_" + fn.replace(".", "_")] = np.array(make())
        for fn in post:
            out["out_" + fn.replace(".", "_")] = np.array(open(os.path.join(d, fn)).read())
        if os.path.exists(os.path.join(d, "objforce.txt")):
            out["objforce"] = np.loadtxt(os.path.join(d, "objforce.txt"), ndmin=2)
        for k in range(3):
            if os.path.exists(os.path.join(d, f"defects{k}.f64")):
                out[f"defects{k}"] = ld(f"defects{k}.f64")
        out["args"] = np.array(json.dumps([a.replace(d, "{d}") for a in args]))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def main(names=None):
    """Regenerate every case, or only the named ones."""
    for name, (args, full) in CASES.items():
        if names and name not in names:
            continue
        run_case(name, args, full)
        print("wrote", name)


if __name__ == "__main__":
    import sys
    main(sys.argv[1:])
