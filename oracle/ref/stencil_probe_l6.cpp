// Black-box probe of the reference's L6 distortion stencils (lcForces.h:
// bulkL6Force, boundaryL6Force).  Each is a homogeneous quadratic form in its
// 125 inputs (q, six neighbours, six neighbour derivative vectors):
// f_c(x) = sum_{i<=j} B_c[i][j] x_i x_j.  f(e_i) gives B_ii and
// f(e_i + e_j) - f(e_i) - f(e_j) gives B_ij.  The probe also checks the form
// is homogeneous quadratic (f(2 e_i) = 4 f(e_i), f(0) = 0) and reproduces the
// function on random inputs, reporting the largest deviation on stderr.
// The output is a test fixture and a table source; it is never compiled into
// the product.  Written for this project.
//
// Output lines: "L6 <case> <component> <input i> <input j> <coefficient>"
//   case -1 = bulk form, 0..63 = boundary case index; inputs numbered as in stencil_probe.cpp
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "std_include.h"
#include "lcForces.h"

static void eval(int bcase, const double *in, double *out)
{
    dVec q, n[6];
    cubicLatticeDerivativeVector d[6];
    for (int c = 0; c < 5; ++c) q[c] = in[c];
    for (int k = 0; k < 6; ++k)
        for (int c = 0; c < 5; ++c) n[k][c] = in[5 + 5 * k + c];
    for (int k = 0; k < 6; ++k)
        for (int c = 0; c < 15; ++c) d[k][c] = in[35 + 15 * k + c];
    dVec st(0.0);
    const double L = 2.0;  // the functions scale by 0.5*L
    if (bcase < 0)
        lcForce::bulkL6Force(L, q, n[0], n[1], n[2], n[3], n[4], n[5], d[0], d[1], d[2], d[3], d[4], d[5], st);
    else
        lcForce::boundaryL6Force(L, bcase, q, n[0], n[1], n[2], n[3], n[4], n[5], d[0], d[1], d[2], d[3], d[4], d[5],
                                 st);
    for (int c = 0; c < 5; ++c) out[c] = st[c];
}

int main()
{
    const int NI = 125;
    std::vector<double> in(NI, 0.0), diag(5 * NI);
    double out[5], o2[5];
    double worst_h = 0.0, worst_r = 0.0;
    srand(12345);
    for (int bcase = -1; bcase < 64; ++bcase) {
        if (bcase >= 0) {
            int xx = bcase & 3, yy = (bcase >> 2) & 3, zz = (bcase >> 4) & 3;
            if (xx == 3 || yy == 3 || zz == 3) continue;
        }
        std::vector<double> B(5 * NI * NI, 0.0);
        eval(bcase, in.data(), out);
        for (int c = 0; c < 5; ++c) worst_h = std::fmax(worst_h, std::fabs(out[c]));
        for (int i = 0; i < NI; ++i) {
            in[i] = 1.0;
            eval(bcase, in.data(), out);
            in[i] = 2.0;
            eval(bcase, in.data(), o2);
            in[i] = 0.0;
            for (int c = 0; c < 5; ++c) {
                diag[c * NI + i] = out[c];
                worst_h = std::fmax(worst_h, std::fabs(o2[c] - 4.0 * out[c]));
                B[(c * NI + i) * NI + i] = out[c];
            }
        }
        for (int i = 0; i < NI; ++i)
            for (int j = i + 1; j < NI; ++j) {
                in[i] = 1.0;
                in[j] = 1.0;
                eval(bcase, in.data(), out);
                in[i] = 0.0;
                in[j] = 0.0;
                for (int c = 0; c < 5; ++c) B[(c * NI + i) * NI + j] = out[c] - diag[c * NI + i] - diag[c * NI + j];
            }
        for (int c = 0; c < 5; ++c)
            for (int i = 0; i < NI; ++i)
                for (int j = i; j < NI; ++j) {
                    const double v = B[(c * NI + i) * NI + j];
                    if (v != 0.0) printf("L6 %d %d %d %d %.17g\n", bcase, c, i, j, v);
                }
        // reproduce the function on random inputs
        for (int trial = 0; trial < 4; ++trial) {
            for (int i = 0; i < NI; ++i) in[i] = (double)rand() / RAND_MAX - 0.5;
            eval(bcase, in.data(), out);
            for (int c = 0; c < 5; ++c) {
                double s = 0.0, mag = 0.0;
                for (int i = 0; i < NI; ++i)
                    for (int j = i; j < NI; ++j) {
                        s += B[(c * NI + i) * NI + j] * in[i] * in[j];
                        mag += std::fabs(B[(c * NI + i) * NI + j] * in[i] * in[j]);
                    }
                worst_r = std::fmax(worst_r, std::fabs(s - out[c]) / (mag > 0 ? mag : 1.0));
            }
            for (int i = 0; i < NI; ++i) in[i] = 0.0;
        }
    }
    fprintf(stderr, "homogeneity deviation %.3g, random-input relative deviation %.3g\n", worst_h, worst_r);
    return 0;
}
