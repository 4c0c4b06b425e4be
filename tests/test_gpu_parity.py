"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference's golden dumps.

Tolerances (written here, used below):
  FP64 single force evaluation / energy: <= 1e-12 normwise relative
  FP64 minimiser traces and final state after N iterations: <= 1e-9 relative
    (reduction order differs from the reference's sequential sums)
  FP32 form, single force evaluation: <= 2e-6 normwise relative to FP64
"""
import numpy as np
import pytest

from cases import GOLDEN_CASES, gpu_lattice, load, oracle_system, parse_args, rel_err

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-12
TOL_TRAJ = 1e-9
TOL_F32 = 2e-6


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("metric_mode", [0, 1])
def test_force_and_energy_fp64(qmin, oracle, name, metric_mode):
    g = load(name)
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg, metric_mode=metric_mode)
    lat = gpu_lattice(qmin, s, qmin.FP64, metric_mode)
    F = lat.force()
    assert rel_err(F, s.force()) <= TOL_F64
    if metric_mode == 0:
        assert rel_err(F, g["force0"]) <= TOL_F64
    e, comps = lat.energy()
    e_o, comps_o = s.energy()
    assert abs(e - e_o) <= TOL_F64 * abs(e_o)
    np.testing.assert_allclose(comps, comps_o, rtol=TOL_F64, atol=TOL_F64 * np.abs(comps_o).max())
    assert abs(e - g["energy0"][0]) <= TOL_F64 * abs(g["energy0"][0])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_force_fp32(qmin, oracle, name):
    g = load(name)
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    lat = gpu_lattice(qmin, s, qmin.FP32)
    F = lat.force()
    assert rel_err(F, g["force0"]) <= TOL_F32
    e, _ = lat.energy()
    assert abs(e - g["energy0"][0]) <= 1e-5 * abs(g["energy0"][0])


@pytest.mark.parametrize("name", ["l1_bulk_fire", "l123_walls_sphere_fire", "planar_sphere_fire",
                                  "l1234_planar_fields_fire", "edges_gaps_wrap", "field_map", "l6_fire"])
@pytest.mark.parametrize("mode", [0, 1, 4])
def test_fire_trajectory_fp64(qmin, oracle, name, mode):
    """The FIRE execution paths (separate kernels, fused tiled kernel, split
    deep/listed force + kick) against the reference."""
    g = load(name)
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    lat = gpu_lattice(qmin, s, qmin.FP64)
    lat.set_fire_kernel(mode)
    lat.fire_init(dt=cfg["dt"])
    n = cfg["iters"]
    r = lat.fire_run(n)
    tr = g["trace"]
    assert r["iterations"] == int(g["final"][0])
    assert abs(r["forceMax"] - tr[-1, 1]) <= TOL_TRAJ * tr[-1, 1]
    assert abs(r["alpha"] - tr[-1, 2]) <= TOL_TRAJ * tr[-1, 2]
    assert abs(r["dt"] - tr[-1, 3]) <= TOL_TRAJ * tr[-1, 3]
    assert r["nsince"] == int(tr[-1, 5])
    Q, V, F = lat.get_state(Q=True, V=True, F=True)
    assert rel_err(Q, g["qfinal"]) <= TOL_TRAJ
    assert rel_err(V, g["vfinal"]) <= 1e-7
    assert rel_err(F, g["ffinal"]) <= 1e-7
    e, _ = lat.energy()
    assert abs(e - g["final"][2]) <= TOL_TRAJ * abs(g["final"][2])


@pytest.mark.parametrize("mode", [0, 1])
def test_fire_per_iteration_trace(qmin, oracle, mode):
    """Run FIRE one iteration per call (as the reference's minimize() with a
    growing iteration cap) and compare every step's scalars."""
    g = load("l123_walls_sphere_fire")
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    lat = gpu_lattice(qmin, s, qmin.FP64)
    lat.set_fire_kernel(mode)
    lat.fire_init(dt=cfg["dt"])
    for k, row in enumerate(g["trace"], start=1):
        r = lat.fire_run(k)
        assert r["iterations"] == k
        np.testing.assert_allclose([r["forceMax"], r["alpha"], r["dt"], r["power"]], row[1:5], rtol=TOL_TRAJ)
        assert r["nsince"] == int(row[5])


@pytest.mark.parametrize("name", ["adam", "nesterov", "lbfgs", "gd"])
def test_other_minimisers_fp64(qmin, oracle, name):
    g = load(name)
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    lat = gpu_lattice(qmin, s, qmin.FP64)
    n, dt = cfg["iters"], cfg["dt"]
    if name == "adam":
        r = lat.adam_run(n, dt=dt)
    elif name == "nesterov":
        r = lat.nesterov_run(n, dt=dt)
    elif name == "gd":
        r = lat.gd_run(n, dt=dt)
        assert rel_err(lat.get_state(Q=False, F=True)[2], g["ffinal"]) <= TOL_TRAJ
    else:
        r = lat.lbfgs_run(n, eta=dt)
    assert r["iterations"] == int(g["final"][0])
    assert abs(r["forceMax"] - g["final"][1]) <= TOL_TRAJ * g["final"][1]
    Q = lat.get_state(Q=True)[0]
    assert rel_err(Q, g["qfinal"]) <= TOL_TRAJ


@pytest.mark.parametrize("name", ["l123_walls_sphere_fire", "l1234_planar_fields_fire"])
@pytest.mark.parametrize("m", [1, 2, 5])
def test_lbfgs_multi_constant(qmin, oracle, name, m):
    """L-BFGS through the multi-constant split force kernels and the fused
    two-loop passes: FP64 follows the oracle's L-BFGS to 1e-9 after 40
    iterations; 15 + 25 iterations (the second call resuming) give the
    40-iteration run bit for bit; the FP32 form stays within 1e-4 of the
    oracle in forceMax and Q."""
    g = load(name)
    cfg = parse_args(g["args"])
    eta, n = 5e-4, 40
    s = oracle_system(oracle, cfg)
    lat = gpu_lattice(qmin, s, qmin.FP64)
    lat32 = gpu_lattice(qmin, s, qmin.FP32)
    lat_resumed = gpu_lattice(qmin, s, qmin.FP64)
    ro = s.lbfgs(n, eta=eta, m=m)  # moves s.Q to the oracle's end state
    r = lat.lbfgs_run(n, eta=eta, m=m)
    assert r["iterations"] == ro["iterations"] == n
    assert abs(r["forceMax"] - ro["forceMax"]) <= TOL_TRAJ * ro["forceMax"]
    Q = lat.get_state(Q=True)[0]
    assert rel_err(Q, s.Q) <= TOL_TRAJ
    r1 = lat_resumed.lbfgs_run(15, eta=eta, m=m)
    assert r1["iterations"] == 15
    r2 = lat_resumed.lbfgs_run(n, eta=eta, m=m, reset=False)
    assert r2 == r
    np.testing.assert_array_equal(lat_resumed.get_state(Q=True)[0], Q)
    r32 = lat32.lbfgs_run(n, eta=eta, m=m)
    assert r32["iterations"] == n
    assert abs(r32["forceMax"] - ro["forceMax"]) <= 1e-4 * ro["forceMax"]
    assert rel_err(lat32.get_state(Q=True)[0], s.Q) <= 1e-4


def test_c1_50cube_fire100(qmin, oracle):
    """openQmin -i 100 -l 50 --L1 2.32 end state (reference pin)."""
    g = load("c1_50cube_fire100")
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    lat = gpu_lattice(qmin, s, qmin.FP64)
    lat.fire_init()
    r = lat.fire_run(100)
    assert r["iterations"] == 100
    assert abs(r["forceMax"] - g["final"][1]) <= TOL_TRAJ * g["final"][1]
    e, _ = lat.energy()
    assert abs(e - g["final"][2]) <= TOL_TRAJ * abs(g["final"][2])


def test_fp32_fire_tracks_fp64(qmin, oracle):
    """FP32 stencils with FP64 reductions: 100 FIRE steps of the 50^3 case stay
    within 1e-4 relative of the FP64 oracle in energy and forceMax."""
    g = load("c1_50cube_fire100")
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    lat = gpu_lattice(qmin, s, qmin.FP32)
    lat.fire_init()
    r = lat.fire_run(100)
    e, _ = lat.energy()
    assert abs(e - g["final"][2]) <= 1e-4 * abs(g["final"][2])
    assert abs(r["forceMax"] - g["final"][1]) <= 1e-3 * g["final"][1]


def test_reference_shaped_api(qmin, oracle):
    """The reference-shaped classes drive the same computation (openQmin.cpp flow)."""
    a, b, c, S0 = qmin.cli_phase_constants()
    model = qmin.qTensorLatticeModel(12, 11, 10)
    sim = qmin.multirankSimulation(0, 1, 1, 1, False, False)
    lc = qmin.landauDeGennesLC()
    sim.setConfiguration(model)
    lc.setPhaseConstants(a, b, c)
    lc.setElasticConstants(2.32, 1.0, 0.5)
    sim.addForce(lc)
    fire = qmin.energyMinimizerFIRE(model)
    fire.setMaximumIterations(30)
    fire.setFIREParameters(5e-4, .99, 100 * 5e-4, 1.1, 0.95, 0.9, 4, 1e-12, 0.0)
    sim.addUpdater(fire, model)
    model.setNematicQTensorRandomly(5, S0)
    hom = qmin.boundaryObject(qmin.boundaryType.homeotropic, 5.3, S0)
    sim.createWall(2, 0, hom)
    sim.createWall(2, 9, hom)
    sim.createSphericalColloid((6, 5.5, 4.5), 2.6, hom)
    sim.finalizeObjects()
    sim.performTimestep()
    g = load("l123_walls_sphere_fire")
    assert abs(fire.getMaxForce() - g["final"][1]) <= TOL_TRAJ * g["final"][1]
    assert abs(sim.computePotentialEnergy() - g["final"][2]) <= TOL_TRAJ * abs(g["final"][2])


def test_launches_counted(qmin, oracle):
    cfg = parse_args(["L=8,8,8", "seed=1", "Ls=2.32,0,0,0,0"])
    s = oracle_system(oracle, cfg)
    lat = gpu_lattice(qmin, s)
    before = lat.launches()
    lat.force(copy=False)
    assert lat.launches() > before


def test_cpp_host_example_reproduces_cli_pin(qmin):
    """The C++ host layer (open-qmin_gb300/host) runs the reference CLI's default
    50^3 / 100-iteration FIRE job and prints the reference's end state."""
    import os
    import subprocess
    exe = os.path.join(os.path.dirname(qmin.LIB_PATH), "example_fire")
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    fmax, e = float(out[2]), float(out[3].split("=")[1])
    g = load("c1_50cube_fire100")
    assert abs(fmax - g["final"][1]) <= TOL_TRAJ * g["final"][1]
    assert abs(e - g["final"][2]) <= TOL_TRAJ * abs(g["final"][2])


@pytest.mark.parametrize("L", [(16, 9, 7), (40, 33, 21), (65, 17, 30)])
@pytest.mark.parametrize("prec,other", [(0, 1), (1, 1), (1, 3), (0, 4), (1, 4)])
def test_fused_matches_separate_kernels(qmin, oracle, L, prec, other):
    """The fused tiled kernel (other = 1), the staged force + kick
    (other = 3, FP32 form) and the split force + kick (other = 4) on lattices that do not divide their tiles (partial
    tiles, lattices narrower than a tile, odd z extents) track the separate
    kernels: FP64 to 1e-12 after 7 iterations, FP32 to 1e-5."""
    cfg = parse_args([f"L={L[0]},{L[1]},{L[2]}", "seed=11", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3",
                      f"sphere={L[0] / 2},{L[1] / 2},{L[2] / 2},{min(L) / 4},p,2.0"])
    s = oracle_system(oracle, cfg)
    res = []
    for mode in (0, other):
        lat = gpu_lattice(qmin, s, prec)
        lat.set_fire_kernel(mode)
        lat.fire_init()
        r = lat.fire_run(7)
        res.append((r, lat.get_state(Q=True, V=True, F=True)))
    tol = 1e-12 if prec == 0 else 1e-5
    assert res[0][0]["iterations"] == res[1][0]["iterations"] == 7
    assert abs(res[0][0]["forceMax"] - res[1][0]["forceMax"]) <= tol * res[0][0]["forceMax"]
    for a, b in zip(res[0][1], res[1][1]):
        assert rel_err(b, a) <= tol


@pytest.mark.parametrize("L", [(16, 9, 7), (40, 33, 21), (65, 17, 30), (104, 30, 20)])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11])
def test_split_variants_match_separate(qmin, oracle, L, prec, variant):
    """Each pinned deep-site kernel of the split force + kick (0, 1: global
    memory at 1 or 2 blocks per SM; 2, 3: shared-memory tiles of 32 x 8 and
    16 x 16 sites, whose halos wrap across the periodic faces of lattices
    narrower than a tile; 4, 5, FP32 only: two x-adjacent sites per thread,
    the second past the edge of an odd Lx; 6, FP32 only: the same with the
    interior tiles' planes staged by TMA, which the 104 x 30 x 20 lattice has
    beside its periodic edge tiles; 7-11: the predictor fused into the
    deep-site kernel with ping-pong state sets and a one-site halo of raw
    planes, in registers (7, 8: 32 x 8 tiles with z chunks of 16 or about two
    waves; 9: 32 x 4) or copied into shared memory by 16-byte row chunks two
    planes ahead (10: 32 x 8; 11: 32 x 4; FP32 with Lx % 4 == 0), the listed
    sites forming their predicted Q on the fly; an odd
    iteration count leaves the state in the second set, which the run copies
    back) tracks the separate kernels, with an L4 term and an external field:
    FP64 to 1e-12 after 7 iterations, FP32 to 1e-5."""
    cfg = parse_args([f"L={L[0]},{L[1]},{L[2]}", "seed=13", "Ls=2.32,1.0,0.5,0.3,0", "wall=2,0,h,5.3",
                      f"sphere={L[0] / 2},{L[1] / 2},{L[2] / 2},{min(L) / 4},p,2.0", "H=0.1,0.2,0.3,0.5,1.0,0.2"])
    s = oracle_system(oracle, cfg)
    tma_ok = L[0] % 4 == 0 and L[0] >= 40 and L[1] >= 12
    if (4 <= variant <= 6 and prec == 0) or (variant == 6 and not tma_ok) or \
            (variant >= 10 and (prec == 0 or L[0] % 4 != 0)):
        lat = gpu_lattice(qmin, s, prec)
        lat.set_fire_kernel(4)
        with pytest.raises(qmin.QminError):
            lat.set_fire_variant(variant)
        return
    res = []
    for mode in (0, 4):
        lat = gpu_lattice(qmin, s, prec)
        lat.set_fire_kernel(mode)
        if mode == 4:
            lat.set_fire_variant(variant)
        lat.fire_init()
        r = lat.fire_run(7)
        res.append((r, lat.get_state(Q=True, V=True, F=True), lat.fire_tuning()))
    t = res[1][2]
    assert t["path"] == "split" and t["variant"] == variant
    assert list(t["candidates_ms"]) == [["split_1blk", "split_2blk", "split_smem_32x8", "split_smem_16x16",
                                         "split_pair_32x8_z8", "split_pair_32x8_zfit",
                                         "split_pair_tma_32x8", "split_fused_32x8_z16", "split_fused_32x8_zfit",
                                         "split_fused_32x4_z16", "split_fused_cp_32x8",
                                         "split_fused_cp_32x4"][variant]]
    tol = 1e-12 if prec == 0 else 1e-5
    assert res[0][0]["iterations"] == res[1][0]["iterations"] == 7
    assert abs(res[0][0]["forceMax"] - res[1][0]["forceMax"]) <= tol * res[0][0]["forceMax"]
    for a, b in zip(res[0][1], res[1][1]):
        assert rel_err(b, a) <= tol


def test_split_tma_wait_limit_reports_and_recovers(qmin, oracle):
    """The TMA-staged deep-site kernel's bounded waits made to run out: with a
    poll limit of zero every block gives up at its first wait for a plane,
    lets the boxes it issued land and raises the handle's device error word,
    and fire_run raises QMIN_ETIMEOUT.  With the default limit restored and
    the state set again, the same handle's run tracks a clean one."""
    L = (104, 30, 20)
    cfg = parse_args([f"L={L[0]},{L[1]},{L[2]}", "seed=13", "Ls=2.32,1.0,0.5,0.3,0", "wall=2,0,h,5.3",
                      f"sphere={L[0] / 2},{L[1] / 2},{L[2] / 2},{min(L) / 4},p,2.0", "H=0.1,0.2,0.3,0.5,1.0,0.2"])
    s = oracle_system(oracle, cfg)
    lats = []
    for _ in range(2):
        lat = gpu_lattice(qmin, s, qmin.FP32)
        lat.set_fire_kernel(4)
        lat.set_fire_variant(6)
        lat.fire_init()
        lats.append(lat)
    clean, lat = lats
    r0 = clean.fire_run(7)
    try:
        qmin.set_wait_limit(0)
        with pytest.raises(qmin.QminError) as err:
            lat.fire_run(7)
        assert err.value.code == qmin.QMIN_ETIMEOUT
        assert "gave up" in str(err.value)
    finally:
        qmin.set_wait_limit(-1)
    lat.set_state(s.Q, s.types)
    lat.fire_init()
    r1 = lat.fire_run(7)
    assert lat.fire_tuning()["variant"] == 6
    assert r1["iterations"] == r0["iterations"] == 7
    assert abs(r1["forceMax"] - r0["forceMax"]) <= 1e-6 * r0["forceMax"]
    for a, b in zip(clean.get_state(Q=True, V=True, F=True), lat.get_state(Q=True, V=True, F=True)):
        assert rel_err(b, a) <= 1e-6


def test_fire_variant_pin_errors(qmin, oracle):
    """A variant needs a pinned strategy and an index that strategy has; -1
    hands the choice back to the autotuner."""
    s = oracle_system(oracle, parse_args(["L=12,12,12", "seed=2", "Ls=2.32,1.0,0.5,0,0"]))
    lat = gpu_lattice(qmin, s, 0)
    with pytest.raises(qmin.QminError):
        lat.set_fire_variant(0)  # FIRE_AUTO
    lat.set_fire_kernel(4)
    with pytest.raises(qmin.QminError):
        lat.set_fire_variant(12)
    with pytest.raises(qmin.QminError):
        lat.set_fire_variant(5)  # FP32 only
    with pytest.raises(qmin.QminError):
        lat.set_fire_variant(-2)
    lat.set_fire_variant(3)
    lat.set_fire_variant(-1)
    lat.fire_init()
    lat.fire_run(2)
    assert len(lat.fire_tuning()["candidates_ms"]) == 7  # FP64: 4 split kernels + 3 fused


@pytest.mark.parametrize("Ls", ["2.32,0,0,0,0", "2.32,1.0,0.5,0,0"])
def test_staged_force_kick_matches_separate(qmin, oracle, Ls):
    """The staged force + kick (FP32 form) gives the separate kernels' forces
    to FP32 rounding (1e-6 normwise; the two compilations may contract
    different products into FMAs): one-constant and multi-constant, walls,
    spheres, periodic wrap across tile edges; FIRE scalars and state to 1e-5
    after 40 iterations."""
    cfg = parse_args(["L=37,29,23", "seed=5", f"Ls={Ls}", "wall=2,0,h,5.3", "wall=0,30,p,1.5",
                      "sphere=35.5,2.2,11.0,5.3,h,4.0", "sphere=12.0,20.0,20.5,4.1,p,0.8"])
    s = oracle_system(oracle, cfg)
    out = []
    for mode in (0, 3):
        lat = gpu_lattice(qmin, s, 1)
        lat.set_fire_kernel(mode)
        lat.fire_init()
        r = lat.fire_run(1)
        F1 = lat.get_state(Q=False, F=True)[2]
        r = lat.fire_run(40)
        out.append((F1, r, lat.get_state(Q=True, V=True, F=True), lat.fire_tuning()["path"]))
    assert out[0][3] == "separate" and out[1][3] == "tiled"
    assert rel_err(out[1][0], out[0][0]) <= 1e-6
    assert out[0][1]["iterations"] == out[1][1]["iterations"] == 40
    assert abs(out[0][1]["forceMax"] - out[1][1]["forceMax"]) <= 1e-5 * out[0][1]["forceMax"]
    for a, b in zip(out[0][2], out[1][2]):
        assert rel_err(b, a) <= 1e-5


def test_l6_batch_rejected(qmin):
    """The batched path has no L6 forms and says so."""
    b = qmin.Batch([(8, 8, 8)])
    with pytest.raises(qmin.QminError):
        b.set_params(-1.0, -12.3, 10.1, 2.32, 1.0, 0.5, L6=0.8)


def test_tuning_choice_kept_per_process(qmin, oracle):
    """A second handle on the same problem takes the autotuner's stored choice
    (the same per-candidate times, not re-measured); after
    qmin_tuning_cache_clear a new handle times the candidates afresh.  The
    trajectories agree whatever the choice."""
    cfg = parse_args(["L=24,20,18", "seed=3", "Ls=2.32,1.0,0.5,0,0", "wall=2,0,h,5.3", "sphere=12,10,9,3.5,h,5.3"])
    s = oracle_system(oracle, cfg)
    runs = []
    for clear in (False, False, True):
        if clear:
            assert qmin.lib().qmin_tuning_cache_clear() == qmin.QMIN_OK
        lat = gpu_lattice(qmin, s, 1)
        lat.fire_init()
        r = lat.fire_run(6)
        runs.append((lat.fire_tuning(), r))
        lat.close()
    assert runs[1][0] == runs[0][0]
    assert runs[2][0]["candidates_ms"] != runs[0][0]["candidates_ms"]
    for t, r in runs:
        assert abs(r["forceMax"] - runs[0][1]["forceMax"]) <= 1e-5 * runs[0][1]["forceMax"]
