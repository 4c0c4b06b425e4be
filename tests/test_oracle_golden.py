"""The C oracle against the reference's own dumps (tests/golden/).  CPU only.

Tolerances: initial Q and site types bit-exact; single force evaluation and
energy <= 1e-12 normwise relative; minimiser traces and final scalars
<= 1e-10 relative (sum order differs from the reference's only where noted)."""
import numpy as np
import pytest

from cases import GOLDEN_CASES, load, oracle_system, parse_args, rel_err


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_initial_state_and_force(oracle, name):
    g = load(name)
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    np.testing.assert_array_equal(s.types, g["types"].astype(np.int32))
    finite = np.isfinite(g["q0"])
    np.testing.assert_array_equal(s.Q[finite], g["q0"][finite])
    assert rel_err(s.force(), g["force0"]) <= 1e-12
    e, comps = s.energy()
    assert abs(e - g["energy0"][0]) <= 1e-12 * abs(g["energy0"][0])
    np.testing.assert_allclose(comps, g["energy0"][1:], rtol=1e-12, atol=1e-12 * np.abs(g["energy0"][1:]).max())


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_minimiser(oracle, name):
    g = load(name)
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    n = cfg["iters"]
    if cfg["minimizer"] == "none" or n == 0:
        np.testing.assert_array_equal(s.Q, g["qfinal"])
        return
    if cfg["minimizer"] == "fire":
        r = s.fire(n, dt=cfg["dt"], trace=True)
        tr = g["trace"]
        assert r["iterations"] == int(g["final"][0])
        np.testing.assert_allclose(r["trace"][:, :4], tr[:, 1:5], rtol=1e-10, atol=1e-14)
        np.testing.assert_array_equal(r["trace"][:, 4], tr[:, 5])
        assert rel_err(r["V"], g["vfinal"]) <= 1e-10
    elif cfg["minimizer"] == "adam":
        r = s.adam(n, dt=cfg["dt"])
    elif cfg["minimizer"] == "nesterov":
        r = s.nesterov(n, dt=cfg["dt"])
    elif cfg["minimizer"] == "gd":
        r = s.gd(n, dt=cfg["dt"])
        assert rel_err(r["F"], g["ffinal"]) <= 1e-10
    else:
        r = s.lbfgs(n, eta=cfg["dt"])
    assert r["iterations"] == int(g["final"][0])
    assert abs(r["forceMax"] - g["final"][1]) <= 1e-10 * g["final"][1]
    assert rel_err(s.Q, g["qfinal"]) <= 1e-10
    e, _ = s.energy()
    assert abs(e - g["final"][2]) <= 1e-10 * abs(g["final"][2])


def test_c1_50cube_pin(oracle):
    """openQmin -i 100 -l 50 --L1 2.32: final E/site and forceMax of the reference."""
    g = load("c1_50cube_fire100")
    cfg = parse_args(g["args"])
    s = oracle_system(oracle, cfg)
    e0, _ = s.energy()
    assert abs(e0 - g["energy0"][0]) <= 1e-12 * abs(g["energy0"][0])
    r = s.fire(100, trace=True)
    assert r["iterations"] == 100
    np.testing.assert_allclose(r["trace"][:, :4], g["trace"][:, 1:5], rtol=1e-10, atol=1e-14)
    e, _ = s.energy()
    assert abs(e - g["final"][2]) <= 1e-10 * abs(g["final"][2])
    assert abs(r["forceMax"] - g["final"][1]) <= 1e-10 * g["final"][1]


def test_metric_single_mode_is_one_correction(oracle):
    """SINGLE metric mode = M applied once on every site; on a boundary-free
    lattice it is M^-1 applied to the CPU-path force on bulk sites."""
    cfg = parse_args(["L=6,5,7", "seed=2", "Ls=2.32,0,0,0,0"])
    s_cpu = oracle_system(oracle, cfg, metric_mode=0)
    s_one = oracle_system(oracle, cfg, metric_mode=1)
    Fc, F1 = s_cpu.force(), s_one.force()
    # M on (F0, F3): (2/3)[[2,-1],[-1,2]]; apply M to F1 to get Fc
    m0 = (2.0 / 3.0) * (2 * F1[:, 0] - F1[:, 3])
    m3 = (2.0 / 3.0) * (2 * F1[:, 3] - F1[:, 0])
    np.testing.assert_allclose(m0, Fc[:, 0], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(m3, Fc[:, 3], rtol=1e-12, atol=1e-14)
    np.testing.assert_array_equal(F1[:, [1, 2, 4]], Fc[:, [1, 2, 4]])


def test_defect_measures(oracle):
    """computeDefectMeasures 0, 1, 2 on the reference's final state."""
    g = load("boundary_file_defects")
    s = oracle_system(oracle, parse_args(g["args"]))
    for k in range(3):
        d = s.defects(k, Q=g["qfinal"])
        scale = np.abs(g[f"defects{k}"]).max()
        np.testing.assert_allclose(d, g[f"defects{k}"], rtol=0, atol=1e-13 * scale)


def test_object_forces(oracle):
    """computeObjectForces of every object on the reference's final state."""
    g = load("object_forces")
    s = oracle_system(oracle, parse_args(g["args"]))
    f = s.object_forces(Q=g["qfinal"])
    np.testing.assert_allclose(f, g["objforce"], rtol=0, atol=1e-12 * np.abs(g["objforce"]).max())
