// Black-box probe of the reference's multi-constant distortion stencils
// (lcForces.h: bulkL2Force/boundaryL2Force, bulkL3Force/boundaryL3Force,
// bulkL4Force/boundaryL4Force).  Each of those functions is linear in its 125
// inputs (q, six neighbours, six neighbour derivative vectors), so feeding unit
// vectors recovers its coefficients.  The output is a test fixture used to
// check this project's own derivation of the stencils; it is never compiled
// into the product.  Written for this project.
//
// Output lines: "<term> <case> <component> <input> <coefficient>"
//   term in {L2, L3, L4}; case -1 = bulk form, 0..63 = boundary case index
//   input 0..4 q, 5..34 neighbours (xd,xu,yd,yu,zd,zu)x5, 35..124 derivatives (xd..zu)x15
#include "std_include.h"
#include "lcForces.h"

typedef void (*bulk_fn)(const scalar, const dVec &, const dVec &, const dVec &, const dVec &, const dVec &,
                        const dVec &, const dVec &, const cubicLatticeDerivativeVector &,
                        const cubicLatticeDerivativeVector &, const cubicLatticeDerivativeVector &,
                        const cubicLatticeDerivativeVector &, const cubicLatticeDerivativeVector &,
                        const cubicLatticeDerivativeVector &, dVec &);
typedef void (*bnd_fn)(const scalar, int, const dVec &, const dVec &, const dVec &, const dVec &, const dVec &,
                       const dVec &, const dVec &, const cubicLatticeDerivativeVector &,
                       const cubicLatticeDerivativeVector &, const cubicLatticeDerivativeVector &,
                       const cubicLatticeDerivativeVector &, const cubicLatticeDerivativeVector &,
                       const cubicLatticeDerivativeVector &, dVec &);

static void eval(int which, int bcase, const double *in, double *out)
{
    dVec q, n[6];
    cubicLatticeDerivativeVector d[6];
    for (int c = 0; c < 5; ++c) q[c] = in[c];
    for (int k = 0; k < 6; ++k)
        for (int c = 0; c < 5; ++c) n[k][c] = in[5 + 5 * k + c];
    for (int k = 0; k < 6; ++k)
        for (int c = 0; c < 15; ++c) d[k][c] = in[35 + 15 * k + c];
    dVec st(0.0);
    const double L = 2.0; // the functions scale by 0.5*L
    if (bcase < 0) {
        if (which == 2) lcForce::bulkL2Force(L, q, n[0], n[1], n[2], n[3], n[4], n[5], d[0], d[1], d[2], d[3], d[4], d[5], st);
        if (which == 3) lcForce::bulkL3Force(L, q, n[0], n[1], n[2], n[3], n[4], n[5], d[0], d[1], d[2], d[3], d[4], d[5], st);
        if (which == 4) lcForce::bulkL4Force(L, q, n[0], n[1], n[2], n[3], n[4], n[5], d[0], d[1], d[2], d[3], d[4], d[5], st);
    } else {
        if (which == 2) lcForce::boundaryL2Force(L, bcase, q, n[0], n[1], n[2], n[3], n[4], n[5], d[0], d[1], d[2], d[3], d[4], d[5], st);
        if (which == 3) lcForce::boundaryL3Force(L, bcase, q, n[0], n[1], n[2], n[3], n[4], n[5], d[0], d[1], d[2], d[3], d[4], d[5], st);
        if (which == 4) lcForce::boundaryL4Force(L, bcase, q, n[0], n[1], n[2], n[3], n[4], n[5], d[0], d[1], d[2], d[3], d[4], d[5], st);
    }
    for (int c = 0; c < 5; ++c) out[c] = st[c];
}

int main()
{
    double in[125], out0[5], out[5];
    for (int which = 2; which <= 4; ++which) {
        for (int bcase = -1; bcase < 64; ++bcase) {
            if (bcase >= 0) {
                int xx = bcase & 3, yy = (bcase >> 2) & 3, zz = (bcase >> 4) & 3;
                if (xx == 3 || yy == 3 || zz == 3) continue;
            }
            for (int i = 0; i < 125; ++i) in[i] = 0.0;
            eval(which, bcase, in, out0);
            for (int i = 0; i < 125; ++i) {
                in[i] = 1.0;
                eval(which, bcase, in, out);
                in[i] = 0.0;
                for (int c = 0; c < 5; ++c) {
                    double v = out[c] - out0[c];
                    if (v != 0.0) printf("L%d %d %d %d %.17g\n", which, bcase, c, i, v);
                }
            }
        }
    }
    return 0;
}
