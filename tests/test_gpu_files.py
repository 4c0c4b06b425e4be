"""File formats and post-processing on the GPU path against the reference's
own outputs (tests/golden/): defect measures, saveState text, loadState,
and the binary exact-resume checkpoint.

Tolerances: defect measures 1e-12 of max(|result|, |Q|^degree) (FP64); the
saveState text has six significant digits, so every integer field must match
and every real field must agree to 2e-6 relative (1e-12 absolute for zeros),
and at least 99% of lines must match byte for byte; loadState exact;
checkpoint resume bit-exact."""
import numpy as np
import pytest

from cases import gpu_lattice, load, oracle_system, parse_args, rel_err

pytestmark = pytest.mark.gpu


def _reference_case(qmin, oracle, name, Q=None):
    g = load(name)
    s = oracle_system(oracle, parse_args(g["args"]))
    lat = gpu_lattice(qmin, s, qmin.FP64)
    if Q is not None:
        lat.set_positions(Q)
    return g, s, lat


def test_defect_measures_match_reference(qmin, oracle):
    g, s, lat = _reference_case(qmin, oracle, "boundary_file_defects", Q=None)
    lat.set_positions(g["qfinal"])
    qmax = np.abs(g["qfinal"][s.types <= 0]).max()
    for k in range(3):
        ref = g[f"defects{k}"]
        d = lat.defect_measures(k)
        # the measures are degree 1, 3 and 6 polynomials of Q whose terms cancel:
        # rounding scales with |Q|^degree, not with the (possibly small) result
        scale = max(np.abs(ref).max(), qmax ** (1, 3, 6)[k])
        assert np.abs(d - ref).max() <= 1e-12 * scale, k
        assert np.all(d[s.types > 0] == 0.0)


def _parse(text):
    rows = [ln.split("\t") for ln in text.strip("\n").split("\n")]
    return rows


def test_save_state_matches_reference_text(qmin, oracle, tmp_path):
    g, s, lat = _reference_case(qmin, oracle, "boundary_file_defects")
    lat.set_positions(g["qfinal"])
    lat.save_state(str(tmp_path / "st"), 2, 0)
    ours = (tmp_path / "st_x0y0z0.txt").read_text()
    ref = str(g["out_st_x0y0z0_txt"])
    a, b = _parse(ours), _parse(ref)
    assert len(a) == len(b) and len(a) == 6 * 5 * 5
    same = 0
    for ra, rb in zip(a, b):
        assert len(ra) == len(rb) == 10
        assert [int(x) for x in ra[:3]] == [int(x) for x in rb[:3]] and int(ra[8]) == int(rb[8])
        for fa, fb in zip(ra[3:8] + ra[9:], rb[3:8] + rb[9:]):
            va, vb = float(fa), float(fb)
            assert abs(va - vb) <= 2e-6 * abs(vb) + 1e-12, (ra, rb)
        same += ra == rb
    assert same >= 0.99 * len(a)


def test_load_state_matches_reference(qmin, oracle, tmp_path):
    g = load("load_state")
    cfg = parse_args(g["args"])
    s = oracle.System(cfg["L"], Ls=cfg["Ls"][:4])
    s.random_nematic(cfg["seed"])
    lat = gpu_lattice(qmin, s, qmin.FP64)
    lat.load_state(cfg["loadstate"])
    Q = lat.get_state()[0]
    np.testing.assert_array_equal(Q, g["q0"])
    np.testing.assert_array_equal(lat.get_types(), g["types"].astype(np.int32))


def test_save_then_load_round_trip(qmin, oracle, tmp_path):
    """Our own text, read back: Q to the six digits printed; types untouched."""
    g, s, lat = _reference_case(qmin, oracle, "boundary_file_defects")
    lat.fire_init()
    lat.fire_run(10)
    lat.save_state(str(tmp_path / "rt"), 1, 2)
    Q0 = lat.get_state()[0]
    lat2 = gpu_lattice(qmin, s, qmin.FP64)
    lat2.load_state(str(tmp_path / "rt"))
    Q1 = lat2.get_state()[0]
    assert np.abs(Q1 - Q0).max() <= 5e-6 * np.abs(Q0).max()
    np.testing.assert_array_equal(lat2.get_types(), s.types)


@pytest.mark.parametrize("prec", [0, 1])
def test_checkpoint_exact_resume(qmin, oracle, tmp_path, prec):
    g = load("l123_walls_sphere_fire")
    s = oracle_system(oracle, parse_args(g["args"]))
    lat = gpu_lattice(qmin, s, prec)
    lat.fire_init()
    lat.fire_run(12)
    lat.checkpoint_save(str(tmp_path / "ck.bin"))
    r_a = lat.fire_run(30)
    a = lat.get_state(Q=True, V=True, F=True)
    fresh = qmin.Lattice(s.L, prec)
    fresh.checkpoint_load(str(tmp_path / "ck.bin"))
    r_b = fresh.fire_run(30)
    b = fresh.get_state(Q=True, V=True, F=True)
    assert r_a == r_b
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert fresh.energy()[0] == lat.energy()[0]


@pytest.mark.parametrize("prec", [0, 1])
def test_checkpoint_exact_resume_lbfgs(qmin, oracle, tmp_path, prec):
    """A checkpoint taken between two L-BFGS calls carries the pair history,
    the kept pair products and the forces the next iteration starts from: the
    resumed run equals the uninterrupted one bit for bit."""
    g = load("l123_walls_sphere_fire")
    s = oracle_system(oracle, parse_args(g["args"]))
    lat = gpu_lattice(qmin, s, prec)
    lat.lbfgs_run(12, eta=5e-4)
    lat.checkpoint_save(str(tmp_path / "ck.bin"))
    r_a = lat.lbfgs_run(30, eta=5e-4, reset=False)
    a = lat.get_state(Q=True, F=True)
    fresh = qmin.Lattice(s.L, prec)
    fresh.checkpoint_load(str(tmp_path / "ck.bin"))
    r_b = fresh.lbfgs_run(30, eta=5e-4, reset=False)
    b = fresh.get_state(Q=True, F=True)
    assert r_a == r_b and r_a["iterations"] == 30
    for x, y in zip(a, b):
        if x is not None:
            np.testing.assert_array_equal(x, y)


def test_checkpoint_rejects_other_lattice(qmin, tmp_path):
    lat = qmin.Lattice((8, 8, 8))
    lat.set_params(-1.0, -12.3, 10.1, 2.32)
    lat.set_objects([])
    lat.set_state(np.zeros((512, 5)), np.zeros(512, dtype=np.int32))
    lat.checkpoint_save(str(tmp_path / "a.bin"))
    other = qmin.Lattice((8, 8, 9))
    with pytest.raises(qmin.QminError):
        other.checkpoint_load(str(tmp_path / "a.bin"))
    with pytest.raises(qmin.QminError):
        other.checkpoint_load(str(tmp_path / "missing.bin"))


def test_reference_shaped_file_calls(qmin, oracle, tmp_path):
    """createBoundaryFromFile / saveState / loadState / computeDefectMeasures
    through the reference-shaped classes."""
    g = load("boundary_file_defects")
    cfg = parse_args(g["args"])
    a, b, c, S0 = qmin.cli_phase_constants()
    model = qmin.qTensorLatticeModel(*cfg["L"])
    sim = qmin.multirankSimulation(0, 1, 1, 1, False, False)
    lc = qmin.landauDeGennesLC()
    sim.setConfiguration(model)
    lc.setPhaseConstants(a, b, c)
    lc.setElasticConstants(2.32, 1.0, 0.5)
    sim.addForce(lc)
    model.setNematicQTensorRandomly(cfg["seed"], S0)
    sim.createBoundaryFromFile(cfg["bfile"])
    sim.finalizeObjects()
    np.testing.assert_array_equal(model.returnTypes(), g["types"].astype(np.int32))
    assert rel_err(sim.computeForces(), g["force0"]) <= 1e-12
    sim.saveState(str(tmp_path / "x"), 1, 1)
    d = model.computeDefectMeasures(1)
    assert np.abs(d - oracle_system(oracle, cfg).defects(1)).max() <= 1e-13
    sim.loadState(str(tmp_path / "x"))


def test_object_forces_match_reference(qmin, oracle):
    """Force on each object from the one-constant stress tensor, on the
    reference's final state; the multi-constant form is refused."""
    g, s, lat = _reference_case(qmin, oracle, "object_forces")
    lat.set_positions(g["qfinal"])
    f = lat.object_forces()
    assert f.shape == g["objforce"].shape
    np.testing.assert_allclose(f, g["objforce"], rtol=0, atol=1e-12 * np.abs(g["objforce"]).max())
    g2, s2, lat2 = _reference_case(qmin, oracle, "l123_walls_sphere_fire")
    with pytest.raises(qmin.QminError):
        lat2.object_forces()
