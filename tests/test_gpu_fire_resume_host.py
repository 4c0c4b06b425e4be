"""The host round trip the C++ drop-in energyMinimizerFIRE_gb300 makes on
every performUpdate(): the reference keeps Q and the velocities in its model
and the FIRE scalars (iterations, forceMax, alpha, deltaT, deltaTMin, Power,
NSinceNegativePower) in its updater between minimize() calls, so each call
uploads them into the handle (qmin_set_state, qmin_fire_init,
qmin_fire_set_state, then qmin_set_velocities: qmin_fire_init starts FIRE from
rest) and reads them back after qmin_fire_run.
Two minimize() calls made that way, the second on a fresh handle, must give
what one handle continuing on the device gives, and what the oracle's two
uninterrupted minimize() to the same iteration gives (FIRE trajectories 1e-9
relative, as the parity tests; a call with a growing cap continues the same
trajectory, its entry force evaluation leaving the state unchanged)."""
import numpy as np
import pytest

from cases import gpu_lattice, load, oracle_system, parse_args, rel_err

pytestmark = pytest.mark.gpu

DT = 5e-4


@pytest.mark.parametrize("prec", [0, 1])
def test_two_minimize_calls_through_host_memory(qmin, oracle, prec):
    s = oracle_system(oracle, parse_args(load("l123_walls_sphere_fire")["args"]))
    Q0 = s.Q.copy()
    n1, n2 = 17, 45
    # one handle, the state staying on the device between the two calls
    a = gpu_lattice(qmin, s, prec)
    a.fire_init(dt=DT)
    a.fire_run(n1)
    ra = a.fire_run(n2)
    Qa, Va, _ = a.get_state(Q=True, V=True)
    a.close()
    # first call, then everything the reference keeps on the host
    b = gpu_lattice(qmin, s, prec)
    b.fire_init(dt=DT)
    r1 = b.fire_run(n1)
    Q1, V1, _ = b.get_state(Q=True, V=True)
    b.close()
    assert r1["iterations"] == n1
    # second call on a fresh handle from the host copies
    c = gpu_lattice(qmin, s, prec)
    c.set_state(Q1, s.types)
    c.fire_init(dt=DT)                 # starts FIRE from rest: the velocities come after it
    c.fire_set_state(r1["iterations"], r1["forceMax"], r1["alpha"], r1["dt"], DT * .01, r1["power"], r1["nsince"])
    c.set_velocities(V1)
    rc = c.fire_run(n2)
    Qc, Vc, _ = c.get_state(Q=True, V=True)
    c.close()
    tol = 1e-9 if prec == 0 else 1e-5
    assert rc["iterations"] == ra["iterations"] == n2
    for k in ("forceMax", "alpha", "dt", "power"):
        assert abs(rc[k] - ra[k]) <= tol * abs(ra[k]), k
    assert rc["nsince"] == ra["nsince"]
    assert rel_err(Qc, Qa) <= tol and rel_err(Vc, Va) <= 1e3 * tol
    if prec == 0:
        # and the oracle, uninterrupted to the same iteration
        s.Q[:] = Q0
        ro = s.fire(n2)
        assert abs(rc["forceMax"] - ro["forceMax"]) <= 1e-9 * ro["forceMax"]
        assert rel_err(Qc, s.Q) <= 1e-9


def test_fire_set_state_rejects_bad_input(qmin, oracle):
    s = oracle_system(oracle, parse_args(load("l1_bulk_fire")["args"]))
    lat = gpu_lattice(qmin, s, 0)
    with pytest.raises(qmin.QminError):
        lat.fire_set_state(0, 1.0, 0.99, DT, DT * .01, 0.0, 0)       # before qmin_fire_init
    lat.fire_init(dt=DT)
    with pytest.raises(qmin.QminError):
        lat.fire_set_state(-1, 1.0, 0.99, DT, DT * .01, 0.0, 0)
    with pytest.raises(qmin.QminError):
        lat.fire_set_state(0, 1.0, 0.99, 0.0, DT * .01, 0.0, 0)
    lat.close()
