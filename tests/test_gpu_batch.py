"""Batched minimisation of uneven independent lattices against the oracle,
solve by solve.  Tolerances: FIRE trajectories 1e-9 relative (FP64),
FP32 batch within 1e-4 of the FP64 batch in forceMax, and (the fused FP32
one-constant iteration) within 1e-4 of the oracle's forceMax and 2e-5 of its
Q."""
import numpy as np
import pytest

from cases import oracle_system, parse_args, rel_err

pytestmark = pytest.mark.gpu


def _cfgs():
    return [
        ["L=9,10,11", "seed=1", "Ls=2.32,0,0,0,0", "sphere=4.3,5.1,5.7,2.2,p,0.7"],
        ["L=16,12,8", "seed=2", "Ls=2.32,0,0,0,0", "sphere=8.5,6.2,3.9,2.6,p,3.1"],
        ["L=20,7,13", "seed=3", "Ls=2.32,0,0,0,0"],
        ["L=5,19,6", "seed=4", "Ls=2.32,0,0,0,0", "sphere=2.5,9.5,3.1,1.7,h,5.3"],
        ["L=14,14,14", "seed=5", "Ls=2.32,0,0,0,0", "sphere=0.2,13.1,7.7,3.3,p,9.0"],
    ]


def _batch(qmin, systems, prec=0):
    b = qmin.Batch([s.L for s in systems], prec)
    p = systems[0].p
    b.set_params(p.A, p.B, p.C, p.L1, p.L2, p.L3, p.L4, multi_constant=p.multi_constant)
    for k, s in enumerate(systems):
        b.set_solve(k, s.Q, s.types, [(s.objs[j].kind, s.objs[j].W, s.objs[j].S0) for j in range(s.nobj)])
    return b


def test_batch_fire_matches_each_solve(qmin, oracle):
    systems = [oracle_system(oracle, parse_args(c)) for c in _cfgs()]
    b = _batch(qmin, systems)
    b.fire_init()
    r = b.fire_run(25)
    for k, s in enumerate(systems):
        ro = s.fire(25)
        assert r["iterations"][k] == ro["iterations"] == 25
        assert abs(r["forceMax"][k] - ro["forceMax"]) <= 1e-9 * ro["forceMax"]
        assert rel_err(b.get_solve(k), s.Q) <= 1e-9


def test_batch_multi_constant_with_walls(qmin, oracle):
    cfgs = [["L=12,11,10", "seed=5", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3", "wall=2,9,h,5.3",
             "sphere=6,5.5,4.5,2.6,h,5.3"],
            ["L=10,13,9", "seed=8", "Ls=2.32,1.0,0.5,0,0", "wall=0,0,p,1.0", "sphere=5.2,6.3,4.1,2.4,p,2.0"]]
    systems = [oracle_system(oracle, parse_args(c)) for c in cfgs]
    b = _batch(qmin, systems)
    b.fire_init()
    r = b.fire_run(20)
    for k, s in enumerate(systems):
        ro = s.fire(20)
        assert abs(r["forceMax"][k] - ro["forceMax"]) <= 1e-9 * ro["forceMax"]
        assert rel_err(b.get_solve(k), s.Q) <= 1e-9


def test_batch_retires_converged_solves(qmin, oracle):
    """Per-solve stopping: with a loose cutoff each solve stops at its own
    iteration, exactly where its own minimize() would."""
    systems = [oracle_system(oracle, parse_args(c)) for c in _cfgs()]
    fcut = 0.05
    b = _batch(qmin, systems)
    b.fire_init(force_cutoff=fcut)
    r = b.fire_run(400)
    its = []
    for k, s in enumerate(systems):
        ro = s.fire(400, fcut=fcut)
        its.append(ro["iterations"])
        assert r["iterations"][k] == ro["iterations"]
        assert abs(r["forceMax"][k] - ro["forceMax"]) <= 1e-9 * ro["forceMax"]
    assert len(set(its)) > 1, "the cases should stop at different iterations"
    assert r["converged"] == sum(1 for k in range(len(systems)) if r["forceMax"][k] <= fcut)


def test_batch_fp32_tracks_fp64(qmin, oracle):
    systems = [oracle_system(oracle, parse_args(c)) for c in _cfgs()]
    res = []
    for prec in (0, 1):
        b = _batch(qmin, systems, prec)
        b.fire_init()
        res.append(b.fire_run(40)["forceMax"])
    np.testing.assert_allclose(res[1], res[0], rtol=1e-4)


def test_batch_fp32_fused_retires_on_either_set(qmin, oracle):
    """The FP32 one-constant batch runs predictor, force and kick as one phase
    over two state sets: solves that stop after an odd and after an even
    number of iterations each come back (copied into the first set where their
    last iteration wrote the second) at their own oracle iteration, Q within
    FP32 accuracy of the FP64 oracle."""
    systems = [oracle_system(oracle, parse_args(c)) for c in _cfgs()]
    fcut = 0.05
    b = _batch(qmin, systems, qmin.FP32)
    b.fire_init(force_cutoff=fcut)
    r = b.fire_run(400)
    parities = set()
    for k, s in enumerate(systems):
        ro = s.fire(400, fcut=fcut)
        assert r["iterations"][k] == ro["iterations"], k
        parities.add(ro["iterations"] % 2)
        assert abs(r["forceMax"][k] - ro["forceMax"]) <= 1e-4 * ro["forceMax"], k
        assert rel_err(b.get_solve(k), s.Q) <= 2e-5, k
    assert parities == {0, 1}, "the cases should stop after odd and after even iteration counts"
    b.close()


def test_batch_fp32_fused_resumes(qmin, oracle):
    """Two FP32 runs of 7 and 6 iterations (the first ends in the second state
    set) follow one oracle run of 13."""
    systems = [oracle_system(oracle, parse_args(c)) for c in _cfgs()]
    b = _batch(qmin, systems, qmin.FP32)
    b.fire_init()
    b.fire_run(7)
    r = b.fire_run(13)
    for k, s in enumerate(systems):
        ro = s.fire(13)
        assert r["iterations"][k] == 13
        assert abs(r["forceMax"][k] - ro["forceMax"]) <= 1e-4 * ro["forceMax"], k
        assert rel_err(b.get_solve(k), s.Q) <= 2e-5, k
    b.close()


def test_c3_generator_and_batch_smoke(qmin):
    """The batched configuration's generator builds solves the batch accepts."""
    import importlib
    wl = importlib.import_module("qmin_gb300.workloads")
    solves = [wl.c3_solve(s) for s in range(6)]
    b = qmin.Batch([d["L"] for d in solves], qmin.FP32)
    a, bb, c = solves[0]["consts"]
    b.set_params(a, bb, c, 2.32)
    for k, d in enumerate(solves):
        b.set_solve(k, d["Q"], d["types"], d["objects"])
    b.fire_init()
    r = b.fire_run(50)
    assert (r["iterations"] == 50).all()
    assert np.isfinite(r["forceMax"]).all()


def test_batch_reproduces_reference_divergence(qmin, oracle):
    """Config-3 solve 51 (planar sphere W~8.8 wrapping the periodic corner)
    diverges under the reference's FIRE schedule (dt grows to its 0.05 cap):
    the oracle's forceMax turns non-finite at iteration 63, and so does the
    batched GPU solve; the other solves in the batch are unaffected."""
    import importlib
    wl = importlib.import_module("qmin_gb300.workloads")
    import ctypes as C
    ids = [50, 51, 52]
    solves = [wl.c3_solve(s) for s in ids]
    s51 = oracle.System(solves[1]["L"], Ls=(2.32, 0, 0, 0))
    s51.random_nematic(51)
    c, r, W = solves[1]["sphere"]
    s51.add_sphere(c, r, 1, W)
    tr = s51.fire(70, fcut=1e-6, trace=True)["trace"]
    first_bad = next(k for k in range(len(tr)) if not np.isfinite(tr[k, 0])) + 1
    b = qmin.Batch([d["L"] for d in solves], qmin.FP64)
    a, bb, cc = solves[0]["consts"]
    b.set_params(a, bb, cc, 2.32)
    for k, d in enumerate(solves):
        b.set_solve(k, d["Q"], d["types"], d["objects"])
    b.fire_init(force_cutoff=1e-6)
    its = np.zeros(3, dtype=np.int32)
    fm = np.zeros(3)
    conv = C.c_int()
    rc = qmin.lib().qmin_batch_fire_run(b._h, 200, qmin._ip(its), qmin._dp(fm), C.byref(conv))
    assert rc == qmin.QMIN_ENONFINITE
    assert not np.isfinite(fm[1]) and its[1] == first_bad
    assert np.isfinite(fm[0]) and np.isfinite(fm[2])


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4])
def test_batch_chunk_shapes_match_each_solve(qmin, oracle, shape):
    """Every chunk shape of the persistent batch loop (256 consecutive sites;
    tiles of 32x8x1, 16x16x1, 16x4x4, 8x8x4 sites cut where they overhang a
    solve's box) follows each solve's oracle run to 1e-9, one-constant and
    multi-constant (deep sites, walls, planar and homeotropic spheres)."""
    for cfgs in (_cfgs(), [["L=12,11,10", "seed=5", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3", "wall=2,9,h,5.3",
                            "sphere=6,5.5,4.5,2.6,h,5.3"],
                           ["L=10,13,9", "seed=8", "Ls=2.32,1.0,0.5,0,0", "wall=0,0,p,1.0",
                            "sphere=5.2,6.3,4.1,2.4,p,2.0"]]):
        systems = [oracle_system(oracle, parse_args(c)) for c in cfgs]
        b = _batch(qmin, systems)
        b.set_chunk_shape(shape)
        b.fire_init()
        r = b.fire_run(20)
        assert b.tuning()["shape"] == shape
        for k, s in enumerate(systems):
            ro = s.fire(20)
            assert abs(r["forceMax"][k] - ro["forceMax"]) <= 1e-9 * ro["forceMax"]
            assert rel_err(b.get_solve(k), s.Q) <= 1e-9
        b.close()


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4])
def test_batch_fp32_fused_every_chunk_shape(qmin, oracle, shape):
    """The FP32 one-constant batch (predictor, force and kick as one phase over
    two state sets) over every chunk shape, including tiles cut where they
    overhang a solve's box: 21 iterations (an odd count, so that every solve
    ends in the second set and is copied back) follow each solve's FP64
    oracle run within FP32 accuracy."""
    systems = [oracle_system(oracle, parse_args(c)) for c in _cfgs()]
    b = _batch(qmin, systems, qmin.FP32)
    b.set_chunk_shape(shape)
    b.fire_init()
    r = b.fire_run(21)
    assert b.tuning()["shape"] == shape
    for k, s in enumerate(systems):
        ro = s.fire(21)
        assert r["iterations"][k] == 21
        assert abs(r["forceMax"][k] - ro["forceMax"]) <= 1e-4 * ro["forceMax"], k
        assert rel_err(b.get_solve(k), s.Q) <= 2e-5, k
    b.close()


def test_batch_one_persistent_launch(qmin):
    """A run of many uneven solves is a handful of launches (the entry forces,
    the tuner's timings on the first run, one persistent launch, the final
    velocity mix), not launches per iteration."""
    import importlib
    wl = importlib.import_module("qmin_gb300.workloads")
    solves = [wl.c3_solve(s) for s in range(24)]
    b = qmin.Batch([d["L"] for d in solves], qmin.FP32)
    a, bb, c = solves[0]["consts"]
    b.set_params(a, bb, c, 2.32)
    for k, d in enumerate(solves):
        b.set_solve(k, d["Q"], d["types"], d["objects"])
    b.fire_init()
    b.fire_run(5)  # tunes the chunk shape
    t = b.tuning()
    assert 0 <= t["shape"] < 5 and len(t["candidates_ms"]) == 5
    l0 = b.launches()
    r = b.fire_run(400)
    assert (r["iterations"] >= 5).all() and r["iterations"].max() > 100
    assert b.launches() - l0 <= 5
    b.close()


def test_batch_barrier_timeout_then_normal_run(qmin, oracle):
    """With a grid barrier limit of one poll the persistent loop gives up at
    its first barrier: the run returns QMIN_ETIMEOUT and marks the solves;
    set again, the same batch with the default limit follows the oracle."""
    import ctypes as C
    systems = [oracle_system(oracle, parse_args(c)) for c in _cfgs()]
    b = _batch(qmin, systems)
    b.fire_init()
    b.set_barrier_limit(1)
    n = len(systems)
    its = np.zeros(n, dtype=np.int32)
    fm = np.zeros(n)
    conv = C.c_int()
    rc = qmin.lib().qmin_batch_fire_run(b._h, 30, qmin._ip(its), qmin._dp(fm), C.byref(conv))
    assert rc == qmin.QMIN_ETIMEOUT
    assert b"grid barrier" in qmin.lib().qmin_last_error_string()
    b.set_barrier_limit(0)
    for k, s in enumerate(systems):
        b.set_solve(k, s.Q, s.types, [(s.objs[j].kind, s.objs[j].W, s.objs[j].S0) for j in range(s.nobj)])
    b.fire_init()
    r = b.fire_run(25)
    for k, s in enumerate(systems):
        ro = s.fire(25)
        assert r["iterations"][k] == ro["iterations"] == 25
        assert abs(r["forceMax"][k] - ro["forceMax"]) <= 1e-9 * ro["forceMax"]
        assert rel_err(b.get_solve(k), s.Q) <= 1e-9
    b.close()
