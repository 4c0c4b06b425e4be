"""Parity at the benchmark's own sizes, not only on small golden lattices.

* c2, the headline workload: 200^3 sites, homeotropic z-walls on planes 0 and
  199, a centred homeotropic sphere of radius 30, W = 5.3, L1-L3 =
  2.32/1.0/0.5, random-director Q0 from seed 13371 -- built by the package's
  own host set-up (the one bench.py times) and checked bit for bit against
  the oracle's set-up.  On it: one FP64 force evaluation (<= 1e-12 normwise),
  the energy and its components (<= 1e-12 of the oracle's per-site densities
  summed exactly rounded: the reference's own sequential loop over 8 M sites
  carries up to N eps ~ 1e-9 of rounding error, and at 200^3 it is 6e-11 off
  the exact sum, so it cannot referee a 1e-12 bound), and 10 FIRE iterations of the
  autotuned strategy (the split deep/listed kernels with the side stream
  inside the captured graph), every iteration's forceMax, alpha, dt, power and
  NSince against the oracle's minimize() trace (<= 1e-9), then the final Q
  and V (<= 1e-9); the FP32 form over the same 10 iterations (forceMax
  <= 1e-4, Q <= 1e-5 of the FP64 oracle).
* c5: 400^3 sites, 8 random homeotropic spheres and a uniform E field along
  z: one FP64 force evaluation and the energy against the oracle.
* c3: 16 solves of the batched generator (uneven sides 16..64, one planar
  sphere each), 50 FIRE iterations as one batch against each solve's oracle
  run (<= 1e-9).

The oracle (a C restatement of the reference's CPU path, pinned against the
reference's own dumps) runs on all host cores here."""
import importlib
import os

import numpy as np
import pytest

from cases import rel_err

pytestmark = pytest.mark.gpu

TOL_FORCE = 1e-12
TOL_TRAJ = 1e-9


@pytest.fixture(scope="module")
def qo(oracle):
    oracle.set_threads(os.cpu_count() or 1)
    return oracle


@pytest.fixture(scope="module")
def wl(qmin):
    return importlib.import_module("qmin_gb300.workloads")


def _lattice(qmin, d, prec):
    a, b, c = d["consts"]
    lat = qmin.Lattice(d["L"], prec)
    lat.set_params(a, b, c, *d["Ls"], E=d.get("E"))
    lat.set_objects(d["objects"])
    lat.set_state(d["Q"], d["types"])
    return lat


@pytest.fixture(scope="module")
def c2(qo, wl):
    d = wl.c2_lattice(200)
    s = qo.System(d["L"], Ls=(2.32, 1.0, 0.5, 0.0))
    s.random_nematic(13371)
    for plane in (0, 199):
        s.add_wall(2, plane, 0, 5.3)
    s.add_sphere((100.0, 100.0, 100.0), 30.0, 0, 5.3)
    return d, s


def test_c2_setup_matches_oracle(c2):
    d, s = c2
    assert np.array_equal(d["Q"], s.Q)
    assert np.array_equal(d["types"], s.types)
    objs = [(s.objs[k].kind, s.objs[k].W, s.objs[k].S0) for k in range(s.nobj)]
    assert objs == [tuple(o) for o in d["objects"]]


def test_c2_force_and_energy_fp64(qmin, c2):
    d, s = c2
    s.Q[:] = d["Q"]
    lat = _lattice(qmin, d, qmin.FP64)
    F = lat.force()
    Fo = s.force()
    assert rel_err(F, Fo) <= TOL_FORCE
    e, comps = lat.energy()
    eo, co = s.energy_exact_sum()
    lat.close()
    assert abs(e - eo) <= TOL_FORCE * abs(eo)
    np.testing.assert_allclose(comps, co, rtol=TOL_FORCE, atol=TOL_FORCE * np.abs(co).max())
    # the reference-ordered sequential sum agrees within its own rounding (N eps)
    es, _ = s.energy()
    assert abs(es - eo) <= s.N * 1.2e-16 * abs(eo)


def test_c2_fire_autotuned_fp64(qmin, c2):
    """10 FIRE iterations of the strategy the autotuner keeps (the split
    kernels), one minimize() call per iteration with a growing cap."""
    d, s = c2
    n = 10
    s.Q[:] = d["Q"]
    lat = _lattice(qmin, d, qmin.FP64)
    lat.fire_init(dt=5e-4)
    ro = s.fire(n, trace=True)
    tr = ro["trace"]
    assert len(tr) == n
    for k in range(1, n + 1):
        r = lat.fire_run(k)
        assert r["iterations"] == k
        # oracle trace rows: forceMax, alpha, dt, power, NSince
        np.testing.assert_allclose([r["forceMax"], r["alpha"], r["dt"], r["power"]], tr[k - 1, 0:4], rtol=TOL_TRAJ)
        assert r["nsince"] == int(tr[k - 1, 4])
    assert lat.fire_tuning()["path"] == "split"
    Q, V, _ = lat.get_state(Q=True, V=True)
    lat.close()
    assert rel_err(Q, s.Q) <= TOL_TRAJ
    assert rel_err(V, ro["V"]) <= 1e-7


def test_c2_fire_fp32_form(qmin, c2):
    """The FP32 form (FP32 state and stencils, FP64 reductions) over the same
    10 iterations, against the FP64 oracle."""
    d, s = c2
    n = 10
    s.Q[:] = d["Q"]
    ro = s.fire(n)
    lat = _lattice(qmin, d, qmin.FP32)
    lat.fire_init(dt=5e-4)
    r = lat.fire_run(n)
    assert r["iterations"] == n
    assert abs(r["forceMax"] - ro["forceMax"]) <= 1e-4 * ro["forceMax"]
    Q = lat.get_state()[0]
    lat.close()
    assert rel_err(Q, s.Q) <= 1e-5


def test_c5_force_and_energy_fp64(qmin, qo, wl):
    d = wl.c5_lattice(400)
    s = qo.System(d["L"], Ls=(2.32, 1.0, 0.5, 0.0), E=d["E"])
    s.random_nematic(13371)
    for ctr, r in d["spheres"]:
        s.add_sphere(ctr, r, 0, 5.3)
    assert np.array_equal(d["types"], s.types)
    assert np.array_equal(d["Q"], s.Q)
    lat = _lattice(qmin, d, qmin.FP64)
    F = lat.force()
    assert rel_err(F, s.force()) <= TOL_FORCE
    del F
    e, comps = lat.energy()
    lat.close()
    eo, co = s.energy_exact_sum()
    assert abs(e - eo) <= TOL_FORCE * abs(eo)
    np.testing.assert_allclose(comps, co, rtol=TOL_FORCE, atol=TOL_FORCE * np.abs(co).max())


def test_c3_batch_of_16_fp64(qmin, qo, wl):
    """16 solves of the batched configuration, 50 FIRE iterations in one batch."""
    n = 50
    solves = [wl.c3_solve(k) for k in range(16)]
    b = qmin.Batch([sv["L"] for sv in solves], qmin.FP64)
    a, bb, c = solves[0]["consts"]
    b.set_params(a, bb, c, 2.32)
    for k, sv in enumerate(solves):
        b.set_solve(k, sv["Q"], sv["types"], sv["objects"])
    b.fire_init()
    r = b.fire_run(n)
    for k, sv in enumerate(solves):
        s = qo.System(sv["L"], Ls=(2.32, 0.0, 0.0, 0.0))
        s.random_nematic(k)
        ctr, rad, W = sv["sphere"]
        s.add_sphere(ctr, rad, 1, W)
        assert np.array_equal(s.types, sv["types"])
        ro = s.fire(n)
        assert r["iterations"][k] == ro["iterations"] == n
        assert abs(r["forceMax"][k] - ro["forceMax"]) <= TOL_TRAJ * ro["forceMax"], k
        assert rel_err(b.get_solve(k), s.Q) <= TOL_TRAJ, k
    b.close()
