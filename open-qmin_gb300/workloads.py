"""Synthetic workloads of the benchmark configurations, built with the
package's own host set-up (the reference's initial-condition and object
builders).  Geometry draws use Python's Mersenne Twister seeded with
1000003 + seed, separate from the Q initialisation stream (seed)."""
import math
import random

from . import DEGENERATE_PLANAR, HOMEOTROPIC, Geometry, cli_phase_constants, host_random_nematic


def c2_lattice(side=200, seed=13371):
    """200^3 box, homeotropic z-walls (planes 0 and side-1), centred homeotropic
    sphere r = 0.15 side (30 at 200^3), W = 5.3, random-director Q0."""
    a, b, c, S0 = cli_phase_constants()
    L = (side, side, side)
    g = Geometry(L, host_random_nematic(L, seed, S0))
    for plane in (0, side - 1):
        g.add_wall(2, plane, HOMEOTROPIC, 5.3, S0)
    g.add_sphere((side / 2.0, side / 2.0, side / 2.0), 0.15 * side, HOMEOTROPIC, 5.3, S0)
    return dict(L=L, consts=(a, b, c), S0=S0, Q=g.Q, types=g.types, objects=g.objects(), Ls=(2.32, 1.0, 0.5))


def c3_solve(seed, lo=16, hi=64):
    """One solve of the batched configuration: sides ~ U{lo..hi}, one degenerate
    planar (Fournier-Galatola) sphere, r ~ U[3, min(L)/4], centre ~ U(box),
    W = exp(U[ln 0.1, ln 10]), S0 of the bulk; random-director Q0 from `seed`."""
    a, b, c, S0 = cli_phase_constants()
    rng = random.Random(1000003 + seed)
    L = tuple(rng.randint(lo, hi) for _ in range(3))
    r = rng.uniform(3.0, min(L) / 4.0)
    centre = tuple(rng.uniform(0.0, L[k]) for k in range(3))
    W = math.exp(rng.uniform(math.log(0.1), math.log(10.0)))
    g = Geometry(L, host_random_nematic(L, seed, S0))
    g.add_sphere(centre, r, DEGENERATE_PLANAR, W, S0)
    return dict(L=L, consts=(a, b, c), S0=S0, Q=g.Q, types=g.types, objects=g.objects(), sphere=(centre, r, W))


def c4_solve(seed, side=64, wall_W=5.3, rfrac=(0.1, 0.2), Wrange=(1.0, 10.0), qseed=None):
    """One sample of the learned-warm-start set: the c2 generator scaled to
    side^3 (homeotropic z-walls on planes 0 and side-1 with W = 5.3, one
    homeotropic sphere) with the sphere's radius r ~ U[0.1, 0.2] side, centre
    x, y ~ U[0, side), z ~ U[r + 3, side - 4 - r] and strength
    W = exp(U[ln 1, ln 10]) drawn per sample; random-director Q0 from `seed`
    (or from `qseed`, to pair one geometry with several initial fields)."""
    a, b, c, S0 = cli_phase_constants()
    rng = random.Random(1000003 + seed)
    L = (side, side, side)
    r = rng.uniform(rfrac[0] * side, rfrac[1] * side)
    centre = (rng.uniform(0.0, side), rng.uniform(0.0, side), rng.uniform(r + 3.0, side - 4.0 - r))
    W = math.exp(rng.uniform(math.log(Wrange[0]), math.log(Wrange[1])))
    g = Geometry(L, host_random_nematic(L, seed if qseed is None else qseed, S0))
    for plane in (0, side - 1):
        g.add_wall(2, plane, HOMEOTROPIC, wall_W, S0)
    g.add_sphere(centre, r, HOMEOTROPIC, W, S0)
    return dict(L=L, consts=(a, b, c), S0=S0, Q=g.Q, types=g.types, objects=g.objects(), Ls=(2.32, 1.0, 0.5),
                sphere=(centre, r, W))


def c5_lattice(side=400, seed=13371, nspheres=8, rmin=10.0, rmax=25.0, gap=2.0):
    """400^3 box, `nspheres` non-overlapping random homeotropic spheres
    (r ~ U[rmin, rmax], centres ~ U(box), surfaces at least `gap` sites apart
    across the periodic box), W = 5.3, L1-L3 = 2.32/1.0/0.5, uniform E field
    along z (Ez = 0.5, eps = 1, eps0 = 1, deps = 0.5: the reference CLI's
    dielectric defaults)."""
    a, b, c, S0 = cli_phase_constants()
    L = (side, side, side)
    rng = random.Random(1000003 + seed)
    spheres = []
    while len(spheres) < nspheres:
        r = rng.uniform(rmin, rmax)
        ctr = tuple(rng.uniform(0.0, L[k]) for k in range(3))
        ok = True
        for (c2, r2) in spheres:
            d2 = 0.0
            for k in range(3):
                dk = abs(ctr[k] - c2[k])
                dk = min(dk, L[k] - dk)
                d2 += dk * dk
            if math.sqrt(d2) < r + r2 + gap:
                ok = False
                break
        if ok:
            spheres.append((ctr, r))
    g = Geometry(L, host_random_nematic(L, seed, S0))
    for ctr, r in spheres:
        g.add_sphere(ctr, r, HOMEOTROPIC, 5.3, S0)
    return dict(L=L, consts=(a, b, c), S0=S0, Q=g.Q, types=g.types, objects=g.objects(), Ls=(2.32, 1.0, 0.5),
                E=(0.0, 0.0, 0.5, 1.0, 1.0, 0.5), spheres=spheres)
