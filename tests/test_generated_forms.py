"""The generated 25-point bulk form is what its generator writes from the
in-tree distortion tables; the generator checks its shared-sum rewrite term
by term against the plain form before comparing."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_q25_header_up_to_date():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "ref", "gen_q25_form.py"), "--check"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "qmin_bulk_q25.h"
int main()
{
    std::mt19937 rng(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    double worst = 0.0;
    for (int trial = 0; trial < 200; ++trial) {
        static double q[5][5][5][5];
        for (auto &a : q) for (auto &b : a) for (auto &c : b) for (auto &d : c) d = u(rng);
        const double Lt[4] = {u(rng), u(rng), 0.0, 1.0 + u(rng)};  // L2, L3, L4 = 0, L1
        double cq[5 * QMIN_Q25_W], cqs[5 * QMIN_Q25_W];
        for (int k = 0; k < 5; ++k)
            for (int n = 0; n < QMIN_Q25_W; ++n) {
                double c = 0, cs = 0;
                for (int t = 0; t < 4; ++t) {
                    c += Lt[t] * qmin_q25_k[t][k][n] * 0.125;
                    cs += Lt[t] * qmin_q25c_k[t][k][n] * 0.125;
                }
                cq[k * QMIN_Q25_W + n] = c;
                cqs[k * QMIN_Q25_W + n] = cs;
            }
#define QQ(dx, dy, dz, c) q[(dx) + 2][(dy) + 2][(dz) + 2][c]
        double full[5], plain[5], shared[5];
        { QMIN_BULK_Q25(cq, full); }
        { QMIN_BULK_Q25_NO_L4_PLAIN(cq, plain); }
        { QMIN_BULK_Q25_NO_L4(cqs, shared); }
#undef QQ
        double scale = 0;
        for (int k = 0; k < 5; ++k) scale = std::fmax(scale, std::fabs(full[k]));
        for (int k = 0; k < 5; ++k) {
            worst = std::fmax(worst, std::fabs(plain[k] - full[k]) / scale);
            worst = std::fmax(worst, std::fabs(shared[k] - full[k]) / scale);
        }
    }
    std::printf("%.3e\n", worst);
    return 0;
}
"""


def test_q25_forms_agree_numerically(tmp_path):
    """The three generated 25-point macros (with L4 at L4 = 0, the plain and
    the shared-sum L4-free forms) give the same sums to FP64 rounding on
    random stencil values and elastic constants."""
    import shutil
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "q25.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "q25"
    subprocess.run([gxx, "-std=c++17", "-O1", "-ffp-contract=off", "-I",
                    os.path.join(ROOT, "open-qmin_gb300", "csrc"), str(src), "-o", str(exe)], check=True)
    worst = float(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    assert worst <= 1e-14
