"""The L-BFGS iteration as the CUDA path orders it (k_lb_pass / k_lb_step /
k_lb_post: 2m + 1 fused streaming passes, pair products s.y and y.y formed
once per pair and kept per slot, p entering each iteration as the forces),
restated here in numpy, against the oracle's L-BFGS in the reference's order
(energyMinimizerLoLBFGS.cpp:105-193) on the oracle's own forces.  CPU only;
the two differ only in dot-product summation order, so the end states agree
to 1e-9 relative after 40 iterations (the FP64 trajectory tolerance of the
GPU tests)."""
import numpy as np
import pytest

from cases import load, oracle_system, parse_args, rel_err


def lbfgs_fused(force, Q, m, eta, iters):
    n = Q.size
    s = np.zeros((m, n))
    y = np.zeros((m, n))
    sy = np.zeros(m)
    yy = np.zeros(m)
    alpha = np.zeros(m)
    F = force(Q).ravel()
    q = Q.ravel().copy()
    alpha0 = 0.0
    for it in range(iters):
        cur = it % m

        def slot(ii):
            return (cur - ii - 1 + m) % m

        def coef(num, t):
            return num / sy[t] if sy[t] != 0 else 0.0

        alpha[0] = alpha0
        p = F
        for ii in range(m - 1):  # step 2 with the next alpha's dot
            p = p + (-alpha[ii]) * y[slot(ii)]
            alpha[ii + 1] = coef(s[slot(ii + 1)] @ p, slot(ii + 1))
        p = p + (-alpha[m - 1]) * y[slot(m - 1)]  # last step-2 update, step 3
        t0 = slot(0)
        if yy[t0] != 0:
            p = p + (sy[t0] / yy[t0]) * y[t0]
        c = alpha[m - 1] - coef(y[slot(m - 1)] @ p, slot(m - 1))
        for ii in range(m - 1, 0, -1):  # step 4 with the next beta's dot
            if sy[slot(ii)] != 0:
                p = p + c * s[slot(ii)]
            c = alpha[ii - 1] - coef(y[slot(ii - 1)] @ p, slot(ii - 1))
        if sy[t0] != 0:  # last step-4 update and the step
            p = p + c * s[t0]
        s[cur] = eta * p
        y[cur] = F
        q = q + s[cur]
        F = force(q.reshape(Q.shape)).ravel()
        y[cur] = y[cur] + (-1.0) * F  # the pass after the force
        sy[cur] = s[cur] @ y[cur]
        yy[cur] = y[cur] @ y[cur]
        alpha0 = coef(s[cur] @ F, cur)
    return q.reshape(Q.shape), np.sqrt(F @ F) / Q.shape[0]


@pytest.mark.parametrize("m", [1, 2, 5])
def test_fused_passes_match_reference_order(oracle, m):
    g = load("l123_walls_sphere_fire")
    s = oracle_system(oracle, parse_args(g["args"]))
    Q0 = s.Q.copy()
    eta, n = 5e-4, 40
    q_fused, fm_fused = lbfgs_fused(lambda Q: s.force(Q), Q0, m, eta, n)
    s.Q[:] = Q0
    r = s.lbfgs(n, eta=eta, m=m)
    assert r["iterations"] == n
    assert rel_err(q_fused, s.Q) <= 1e-9
    assert abs(fm_fused - r["forceMax"]) <= 1e-9 * r["forceMax"]
