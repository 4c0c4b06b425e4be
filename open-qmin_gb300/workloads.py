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
