/* qmin oracle: CPU restatement of the reference's single-rank CPU path.
 * TEST INFRASTRUCTURE ONLY (see qmin_oracle.h): never part of the product.
 *
 * Each function names the reference code it restates (paths relative to the
 * open-Qmin source tree).  Per-site loops may run under OpenMP; every sum is
 * taken sequentially in site order, as the reference does, so results do not
 * depend on the thread count. */
#include "qmin_oracle.h"
#include "distortion_coeffs.h"
#include "distortion_coeffs_l6.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define QO_PI 3.14159265358979323846 /* inc/std_include.h:37 */

int qo_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------------------ RNG --
 * std::mt19937 (Matsumoto & Nishimura 1998) and libstdc++'s
 * uniform_real_distribution<double>(0,1), i.e. generate_canonical<double,53>
 * with two 32-bit draws ([rand.util.canonical]); the reference draws through
 * noiseSource::getRealUniform (src/utilities/noiseSource.cpp:16-25). */
typedef struct { uint32_t mt[624]; int idx; } qo_mt;

static void mt_seed(qo_mt *g, uint32_t s)
{
    g->mt[0] = s;
    for (int i = 1; i < 624; ++i) g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->idx = 624;
}

static uint32_t mt_next(qo_mt *g)
{
    if (g->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
            g->mt[i] = g->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        g->idx = 0;
    }
    uint32_t y = g->mt[g->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

static double mt_uniform(qo_mt *g)
{
    double sum = (double)mt_next(g);
    sum += (double)mt_next(g) * 4294967296.0;
    double r = sum / 18446744073709551616.0;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    return r;
}

/* qTensorFromDirector (inc/qTensorFunctions.h:34-51) */
static void q_from_director(double nx, double ny, double nz, double S0, double *q)
{
    double scale = sqrt(nx * nx + ny * ny + nz * nz);
    if (scale == 0) {
        q[0] = -0.5 * S0;
        q[3] = -0.5 * S0;
    } else if (scale != 1) {
        nx /= scale;
        ny /= scale;
        nz /= scale;
    }
    q[0] = 1.5 * S0 * (nx * nx - 1.0 / 3.0);
    q[1] = 1.5 * S0 * nx * ny;
    q[2] = 1.5 * S0 * nx * nz;
    q[3] = 1.5 * S0 * (ny * ny - 1.0 / 3.0);
    q[4] = 1.5 * S0 * ny * nz;
}

/* qTensorLatticeModel::setNematicQTensorRandomly (src/model/qTensorLatticeModel.cpp:134-162):
 * two global draws, then two draws per site for every site, in index order. */
void qo_random_nematic(int N, unsigned seed, double S0, double *Q)
{
    qo_mt g;
    mt_seed(&g, seed);
    (void)mt_uniform(&g); /* globalTheta */
    (void)mt_uniform(&g); /* globalPhi */
    for (int i = 0; i < N; ++i) {
        double theta = acos(2.0 * mt_uniform(&g) - 1);
        double phi = 2.0 * QO_PI * mt_uniform(&g);
        q_from_director(cos(phi) * sin(theta), sin(phi) * sin(theta), cos(theta), S0, Q + 5 * (size_t)i);
    }
}

/* ------------------------------------------------------------- geometry -- */
static int wrapi(int x, int m) /* inc/functions.h:299-307 */
{
    int a = x;
    if (x >= m) a = x % m;
    while (a < 0) a += m;
    return a;
}

static size_t site_index(const int L[3], int x, int y, int z)
{
    return (size_t)x + (size_t)L[0] * ((size_t)y + (size_t)L[1] * (size_t)z);
}

/* cubicLattice::createBoundaryObject (src/model/cubicLattice.cpp:267-294) after
 * multirankSimulation::createMultirankBoundaryObject (multirankSimulationBoundaries.cpp:512-543):
 * positions are wrapped into the box, the object's sites take type nobj+1 and
 * their six neighbours with type < 1 become -1. */
static int add_object(const int L[3], int nsites, const int *xyz, const double *qs, int kind, double W, double S0,
                      double *Q, int *types, qo_object *objs, int nobj)
{
    int j = nobj + 1;
    size_t *idx = (size_t *)malloc(sizeof(size_t) * (size_t)(nsites > 0 ? nsites : 1));
    for (int s = 0; s < nsites; ++s) {
        int x = wrapi(xyz[3 * s], L[0]), y = wrapi(xyz[3 * s + 1], L[1]), z = wrapi(xyz[3 * s + 2], L[2]);
        idx[s] = site_index(L, x, y, z);
        memcpy(Q + 5 * idx[s], qs + 5 * (size_t)s, 5 * sizeof(double));
    }
    for (int s = 0; s < nsites; ++s) types[idx[s]] = j;
    for (int s = 0; s < nsites; ++s) {
        size_t i = idx[s];
        int x = (int)(i % (size_t)L[0]), y = (int)((i / (size_t)L[0]) % (size_t)L[1]), z = (int)(i / ((size_t)L[0] * L[1]));
        size_t nb[6] = {site_index(L, wrapi(x - 1, L[0]), y, z), site_index(L, wrapi(x + 1, L[0]), y, z),
                        site_index(L, x, wrapi(y - 1, L[1]), z), site_index(L, x, wrapi(y + 1, L[1]), z),
                        site_index(L, x, y, wrapi(z - 1, L[2])), site_index(L, x, y, wrapi(z + 1, L[2]))};
        for (int k = 0; k < 6; ++k)
            if (types[nb[k]] < 1) types[nb[k]] = -1;
    }
    free(idx);
    objs[nobj].kind = kind;
    objs[nobj].W = W;
    objs[nobj].S0 = S0;
    return nobj + 1;
}

/* one object from an explicit site list (the core of
 * multirankSimulation::createBoundaryFromFile, multirankSimulationBoundaries.cpp:43-96) */
int qo_add_sites(const int L[3], int nsites, const int *xyz, const double *qs, int kind, double W, double S0,
                 double *Q, int *types, qo_object *objs, int nobj)
{
    return add_object(L, nsites, xyz, qs, kind, W, S0, Q, types, objs, nobj);
}

/* multirankSimulation::createWall (multirankSimulationBoundaries.cpp:101-167) */
int qo_add_wall(const int L[3], int xyz, int plane, int kind, double W, double S0,
                double *Q, int *types, qo_object *objs, int nobj)
{
    double q[5] = {0, 0, 0, 0, 0};
    if (kind == 0) {
        if (xyz == 0) { q[0] = S0; q[3] = -0.5 * S0; }
        else if (xyz == 1) { q[0] = -0.5 * S0; q[3] = S0; }
        else { q[0] = -0.5 * S0; q[3] = -0.5 * S0; }
    } else {
        q[xyz] = 1.0;
    }
    int s1 = xyz == 0 ? L[1] : L[0];
    int s2 = xyz == 2 ? L[1] : L[2];
    int n = s1 * s2;
    int *pos = (int *)malloc(sizeof(int) * 3 * (size_t)n);
    double *qs = (double *)malloc(sizeof(double) * 5 * (size_t)n);
    int s = 0;
    for (int a = 0; a < s1; ++a)
        for (int b = 0; b < s2; ++b, ++s) {
            if (xyz == 0) { pos[3 * s] = plane; pos[3 * s + 1] = a; pos[3 * s + 2] = b; }
            else if (xyz == 1) { pos[3 * s] = a; pos[3 * s + 1] = plane; pos[3 * s + 2] = b; }
            else { pos[3 * s] = a; pos[3 * s + 1] = b; pos[3 * s + 2] = plane; }
            memcpy(qs + 5 * (size_t)s, q, sizeof q);
        }
    int r = add_object(L, n, pos, qs, kind, W, S0, Q, types, objs, nobj);
    free(pos);
    free(qs);
    return r;
}

/* multirankSimulation::createSphericalColloid (multirankSimulationBoundaries.cpp:169-215):
 * integer sites in [ceil(c-r), floor(c+r)) per axis with |x-c|^2 < r^2. */
int qo_add_sphere(const int L[3], const double c[3], double r, int kind, double W, double S0,
                  double *Q, int *types, qo_object *objs, int nobj)
{
    int x0 = (int)ceil(c[0] - r), y0 = (int)ceil(c[1] - r), z0 = (int)ceil(c[2] - r);
    int cap = 0;
    for (int x = x0; x < floor(c[0] + r); ++x)
        for (int y = y0; y < floor(c[1] + r); ++y)
            for (int z = z0; z < floor(c[2] + r); ++z) ++cap;
    int *pos = (int *)malloc(sizeof(int) * 3 * (size_t)(cap + 1));
    double *qs = (double *)malloc(sizeof(double) * 5 * (size_t)(cap + 1));
    double q[5] = {0, 0, 0, 0, 0};
    int n = 0;
    for (int x = x0; x < floor(c[0] + r); ++x)
        for (int y = y0; y < floor(c[1] + r); ++y)
            for (int z = z0; z < floor(c[2] + r); ++z) {
                double dx = x - c[0], dy = y - c[1], dz = z - c[2];
                if (dx * dx + dy * dy + dz * dz < r * r) {
                    pos[3 * n] = x; pos[3 * n + 1] = y; pos[3 * n + 2] = z;
                    if (kind == 0) {
                        q_from_director(dx, dy, dz, S0, q);
                    } else {
                        double nrm = sqrt(dx * dx + dy * dy + dz * dz);
                        q[0] = dx / nrm; q[1] = dy / nrm; q[2] = dz / nrm;
                    }
                    memcpy(qs + 5 * (size_t)n, q, sizeof q);
                    ++n;
                }
            }
    int rr = add_object(L, n, pos, qs, kind, W, S0, Q, types, objs, nobj);
    free(pos);
    free(qs);
    return rr;
}

/* updater::getNTotal (src/updaters/baseUpdater.cpp:10-28) */
int qo_count_active(int N, const int *types)
{
    int n = N;
    for (int i = 0; i < N; ++i)
        if (types[i] > 0) n -= 1;
    return n;
}

/* ---------------------------------------------------- Q-tensor algebra --
 * inc/qTensorFunctions.h:54-107 */
static double tr_q2(const double *q)
{
    return 2.0 * (q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + q[4] * q[4] + q[0] * q[3]);
}
static double tr_q3(const double *q)
{
    return -3.0 * ((-(q[1] * q[1]) + q[3] * q[3] + q[4] * q[4]) * q[0] + q[0] * q[0] * q[3] - q[1] * q[1] * q[3] +
                   q[2] * q[2] * q[3] - 2 * q[1] * q[2] * q[4]);
}
static void d_tr_q2(const double *q, double *d)
{
    d[0] = 2. * (2 * q[0] + q[3]);
    d[1] = 4. * q[1];
    d[2] = 4. * q[2];
    d[3] = 2. * (q[0] + 2 * q[3]);
    d[4] = 4. * q[4];
}
static void d_tr_q3(const double *q, double *d)
{
    d[0] = -3.0 * (-q[1] * q[1] + q[3] * q[3] + q[4] * q[4] + 2 * q[0] * q[3]);
    d[1] = 6 * (q[0] * q[1] + q[1] * q[3] + q[2] * q[4]);
    d[2] = -6 * q[2] * q[3] + 6 * q[1] * q[4];
    d[3] = -3 * (q[0] * q[0] - q[1] * q[1] + q[2] * q[2] + 2 * q[0] * q[3]);
    d[4] = 6 * q[1] * q[2] - 6 * q[0] * q[4];
}
static void d_tr_q2_sq(const double *q, double *d)
{
    double s = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + q[4] * q[4] + q[0] * q[3];
    d[0] = 8.0 * (2.0 * q[0] + q[3]) * s;
    d[1] = 16 * q[1] * s;
    d[2] = 16 * q[2] * s;
    d[3] = 8.0 * (q[0] + 2.0 * q[3]) * s;
    d[4] = 16 * q[4] * s;
}

/* bulk phase force: force -= a dTrQ2 + b dTrQ3 + c d(TrQ2)^2 with a = A/2, b = B/3, c = C/4
 * (landauDeGennesLCDistortionTerms.cpp:23-38) */
static void phase_force(const qo_params *p, const double *q, double *f)
{
    double a = 0.5 * p->A, b = p->B / 3.0, c = 0.25 * p->C;
    double d2[5], d3[5], d4[5];
    d_tr_q2(q, d2);
    d_tr_q3(q, d3);
    d_tr_q2_sq(q, d4);
    for (int k = 0; k < 5; ++k) f[k] = 0.0 - a * d2[k];
    for (int k = 0; k < 5; ++k) f[k] -= b * d3[k];
    for (int k = 0; k < 5; ++k) f[k] -= c * d4[k];
}

/* ----------------------------------------------------------- lattice --- */
typedef struct { size_t nb[6]; } qo_nbrs; /* x-, x+, y-, y+, z-, z+ (cubicLattice.cpp:179-244) */

static void neighbours(const int L[3], size_t i, qo_nbrs *n)
{
    int x = (int)(i % (size_t)L[0]), y = (int)((i / (size_t)L[0]) % (size_t)L[1]), z = (int)(i / ((size_t)L[0] * L[1]));
    n->nb[0] = site_index(L, x == 0 ? L[0] - 1 : x - 1, y, z);
    n->nb[1] = site_index(L, x == L[0] - 1 ? 0 : x + 1, y, z);
    n->nb[2] = site_index(L, x, y == 0 ? L[1] - 1 : y - 1, z);
    n->nb[3] = site_index(L, x, y == L[1] - 1 ? 0 : y + 1, z);
    n->nb[4] = site_index(L, x, y, z == 0 ? L[2] - 1 : z - 1);
    n->nb[5] = site_index(L, x, y, z == L[2] - 1 ? 0 : z + 1);
}

/* landauDeGennesLC::computeFirstDerivatives (landauDeGennesLCOtherForces.cpp:15-145):
 * central differences, one-sided at type < 0 sites; when both neighbours along
 * an axis are objects the "up is an object" branch wins.  Object sites keep a
 * zero vector (the reference never writes them; its buffer starts zeroed). */
static void first_derivatives(const int L[3], const double *Q, const int *types, double *D)
{
    size_t N = (size_t)L[0] * L[1] * L[2];
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)N; ++ii) {
        size_t i = (size_t)ii;
        double *d = D + 15 * i;
        memset(d, 0, 15 * sizeof(double));
        if (types[i] > 0) continue;
        qo_nbrs n;
        neighbours(L, i, &n);
        const double *q = Q + 5 * i;
        for (int ax = 0; ax < 3; ++ax) {
            size_t dn = n.nb[2 * ax], up = n.nb[2 * ax + 1];
            const double *qd = Q + 5 * dn, *qu = Q + 5 * up;
            for (int k = 0; k < 5; ++k) {
                double v;
                if (types[i] == 0 || (types[dn] <= 0 && types[up] <= 0)) v = 0.5 * (qu[k] - qd[k]);
                else if (types[up] > 0) v = q[k] - qd[k];
                else v = qu[k] - q[k];
                d[5 * ax + k] = v;
            }
        }
    }
}

/* lcForce::getBoundaryCase (lcForces.h:13-25) */
static int boundary_case(const int *t6)
{
    int xx = 0, yy = 0, zz = 0;
    if (t6[1] > 0) xx = 1;
    if (t6[0] > 0) xx = 2;
    if (t6[3] > 0) yy = 1;
    if (t6[2] > 0) yy = 2;
    if (t6[5] > 0) zz = 1;
    if (t6[4] > 0) zz = 2;
    return xx + 4 * yy + 16 * zz;
}

/* lcForce::bulkL1Force / boundaryL1Force (lcForces.h:26-63) */
static void l1_term(double L1, const double *q, const double *const nq[6], const int *t6, int boundary, double *s)
{
    if (!boundary) {
        for (int k = 0; k < 5; ++k)
            s[k] = L1 * (6.0 * q[k] - nq[0][k] - nq[1][k] - nq[2][k] - nq[3][k] - nq[4][k] - nq[5][k]);
    } else {
        for (int k = 0; k < 5; ++k) s[k] = 0.0;
        for (int ax = 0; ax < 3; ++ax) {
            if (t6[2 * ax] > 0)
                for (int k = 0; k < 5; ++k) s[k] -= (nq[2 * ax + 1][k] - q[k]);
            if (t6[2 * ax + 1] > 0)
                for (int k = 0; k < 5; ++k) s[k] -= (nq[2 * ax][k] - q[k]);
        }
        for (int k = 0; k < 5; ++k) s[k] = s[k] * L1;
    }
    double cross = s[0] + s[3];
    s[0] += cross;
    s[1] *= 2.0;
    s[2] *= 2.0;
    s[3] += cross;
    s[4] *= 2.0;
}

/* multi-constant forms: (0.5 L) * (sum_i k_i x_i / 2), the coefficients k_i of
 * lcForces.h's bulk/boundary L2, L3, L4 forms (tables in distortion_coeffs.h) */
typedef struct { int n; short in[32]; short k[32]; } qo_form;
static qo_form qo_forms[3][64][5];
static int qo_forms_ready;

static void build_forms(void)
{
    if (qo_forms_ready) return;
#pragma omp critical(qo_forms_init)
    {
        if (!qo_forms_ready) {
            memset(qo_forms, 0, sizeof qo_forms);
            for (int e = 0; e < QO_DISTORTION_NENTRIES; ++e) {
                const short *r = qo_distortion_entries[e];
                qo_form *f = &qo_forms[r[0]][r[1]][r[2]];
                f->in[f->n] = r[3];
                f->k[f->n] = r[4];
                f->n++;
            }
            qo_forms_ready = 1;
        }
    }
}

static void multi_term(int term, double Lc, int bcase, const double *x125, double *s)
{
    for (int k = 0; k < 5; ++k) {
        const qo_form *f = &qo_forms[term][bcase][k];
        double acc = 0.0;
        for (int j = 0; j < f->n; ++j) acc += (double)f->k[j] * x125[f->in[j]];
        s[k] = (0.5 * Lc) * (acc / 2.);
    }
}

/* L6 forms: (0.5 L6) * sum_{i<=j} (k/2) x_i x_j, the quadratic forms of
 * lcForces.h's bulkL6Force / boundaryL6Force (tables in distortion_coeffs_l6.h;
 * the bulk form equals boundary case 0).  qo_l6_start[(case + 1) * 5 + c] is
 * the first entry of (case, component c); the entries are grouped that way. */
static int qo_l6_start[65 * 5 + 1];
static int qo_l6_ready;

static void build_l6(void)
{
    if (qo_l6_ready) return;
#pragma omp critical(qo_l6_init)
    {
        if (!qo_l6_ready) {
            int count[65 * 5];
            memset(count, 0, sizeof count);
            for (int e = 0; e < QO_L6_N; ++e) count[(qo_l6_entries[e][0] + 1) * 5 + qo_l6_entries[e][1]]++;
            qo_l6_start[0] = 0;
            for (int slot = 0; slot < 65 * 5; ++slot) qo_l6_start[slot + 1] = qo_l6_start[slot] + count[slot];
            qo_l6_ready = 1;
        }
    }
}

static void l6_term(double L6, int bcase, const double *x125, double *s)
{
    for (int k = 0; k < 5; ++k) {
        const int slot = (bcase + 1) * 5 + k;
        double acc = 0.0;
        for (int e = qo_l6_start[slot]; e < qo_l6_start[slot + 1]; ++e) {
            const short *r = qo_l6_entries[e];
            acc += (double)r[4] / 2.0 * x125[r[2]] * x125[r[3]];
        }
        s[k] = (0.5 * L6) * acc;
    }
}

/* boundary anchoring force on an LC site from one object neighbour
 * (landauDeGennesLCBoundary.h:26-74).
 * Homeotropic (Rapini-Papoular): E = W tr((q-qB)^2), F = -dE/dq.
 * Degenerate planar (Fournier-Galatola, W1 = W2 = W): with Qt = Q + S0/2 I,
 * P = I - nu nu, D = Qt - P Qt P:  E = W tr(D^2) + W (tr Qt^2 - (3 S0/2)^2)^2
 * and dE/dQt = 2 W D + 4 W (tr Qt^2 - 9 S0^2/4) Qt; F = -dE/dq through
 * Q = Q(q0..q4) with Qzz = -q0-q3. */
static void tensor3(const double *q, double Qm[3][3])
{
    Qm[0][0] = q[0]; Qm[0][1] = q[1]; Qm[0][2] = q[2];
    Qm[1][0] = q[1]; Qm[1][1] = q[3]; Qm[1][2] = q[4];
    Qm[2][0] = q[2]; Qm[2][1] = q[4]; Qm[2][2] = -q[0] - q[3];
}

static void planar_D(const double *q, const double *nu, double S0, double D[3][3])
{
    double Qt[3][3];
    tensor3(q, Qt);
    for (int a = 0; a < 3; ++a) Qt[a][a] += 0.5 * S0;
    double w[3];
    for (int a = 0; a < 3; ++a) w[a] = Qt[a][0] * nu[0] + Qt[a][1] * nu[1] + Qt[a][2] * nu[2];
    double s = nu[0] * w[0] + nu[1] * w[1] + nu[2] * w[2];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) D[a][b] = nu[a] * w[b] + w[a] * nu[b] - s * nu[a] * nu[b];
}

static void anchoring_force(const double *q, const double *qb, const qo_object *o, double *f)
{
    if (o->kind == 0) {
        double d[5];
        for (int k = 0; k < 5; ++k) d[k] = 2.0 * (q[k] - qb[k]);
        double ans[5];
        for (int k = 0; k < 5; ++k) ans[k] = 2.0 * d[k];
        ans[0] += d[3];
        ans[3] += d[0];
        for (int k = 0; k < 5; ++k) f[k] = -o->W * ans[k];
    } else {
        double D[3][3];
        planar_D(q, qb, o->S0, D);
        double g[5]; /* dE1/dq */
        g[0] = 2.0 * o->W * (D[0][0] - D[2][2]);
        g[1] = 4.0 * o->W * D[0][1];
        g[2] = 4.0 * o->W * D[0][2];
        g[3] = 2.0 * o->W * (D[1][1] - D[2][2]);
        g[4] = 4.0 * o->W * D[1][2];
        double sq = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + q[4] * q[4] + q[0] * q[3];
        double c2 = 3.0 * (o->S0 * o->S0) - 4.0 * sq;
        f[0] = 2 * o->W * (2 * q[0] + q[3]) * c2 - g[0];
        f[1] = 4 * o->W * q[1] * c2 - g[1];
        f[2] = 4 * o->W * q[2] * c2 - g[2];
        f[3] = 2 * o->W * (q[0] + 2 * q[3]) * c2 - g[3];
        f[4] = 4 * o->W * q[4] * c2 - g[4];
    }
}

/* computeBoundaryEnergy (landauDeGennesLCBoundary.h:77-124) */
static double anchoring_energy(const double *q, const double *qb, const qo_object *o)
{
    if (o->kind == 0) {
        double d[5];
        for (int k = 0; k < 5; ++k) d[k] = q[k] - qb[k];
        return o->W * tr_q2(d);
    }
    double D[3][3];
    planar_D(q, qb, o->S0, D);
    double e1 = 0.0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) e1 += D[a][b] * D[a][b];
    double e2 = 3. * (o->S0 * o->S0) - 4. * (q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[0] * q[3] + q[3] * q[3] + q[4] * q[4]);
    return o->W * e1 + 0.25 * o->W * e2 * e2;
}

/* uniform E or H field force (landauDeGennesLCOtherForces.cpp:285-312) */
static void field_force(const double *fld, double aniso, double perm, double *ff)
{
    double pr = aniso * perm;
    ff[0] = -0.5 * pr * (fld[0] * fld[0] - fld[2] * fld[2]);
    ff[1] = -pr * fld[0] * fld[1];
    ff[2] = -pr * fld[0] * fld[2];
    ff[3] = -0.5 * pr * (fld[1] * fld[1] - fld[2] * fld[2]);
    ff[4] = -pr * fld[1] * fld[2];
}

/* correctForceFromMetric (landauDeGennesLC.cpp:137-160) */
static void metric(double *f)
{
    double f0 = f[0], f3 = f[3];
    f[0] = (2. / 3.) * (2. * f0 - f3);
    f[3] = (2. / 3.) * (2. * f3 - f0);
}

/* ------------------------------------------------------------- force --
 * multirankSimulation::computeForces CPU branch (multirankSimulation.cpp:462-466):
 * pass 0 (type == 0 sites) then the metric correction, pass 1 (type < 0 sites,
 * anchoring, fields on all type <= 0 sites) then the metric correction again
 * (landauDeGennesLC.cpp:125-202).  metric_mode 1 reproduces the reference GPU
 * branch (landauDeGennesLC.cpp:357-398): one pass, one correction. */
void qo_force(const qo_params *p, const double *Q, const int *types, const qo_object *objs, double *F)
{
    const int L[3] = {p->Lx, p->Ly, p->Lz};
    size_t N = (size_t)L[0] * L[1] * L[2];
    double *D = NULL;
    if (p->multi_constant) {
        build_forms();
        build_l6();
        D = (double *)malloc(sizeof(double) * 15 * N);
        first_derivatives(L, Q, types, D);
    }
    double fE[5] = {0}, fH[5] = {0};
    if (p->efield) field_force(p->E, p->deps, p->eps0, fE);
    if (p->hfield) field_force(p->H, p->dchi, p->mu0, fH);

#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)N; ++ii) {
        size_t i = (size_t)ii;
        double *f = F + 5 * i;
        int t = types[i];
        for (int k = 0; k < 5; ++k) f[k] = 0.0;
        if (t > 0) continue;
        const double *q = Q + 5 * i;
        qo_nbrs n;
        neighbours(L, i, &n);
        const double *nq[6];
        int t6[6];
        for (int k = 0; k < 6; ++k) {
            nq[k] = Q + 5 * n.nb[k];
            t6[k] = types[n.nb[k]];
        }
        int boundary_form = (t == -1); /* type -2 uses the bulk forms (DT:241-279) */
        double force[5], s[5], ind[5];
        phase_force(p, q, force);
        if (!p->multi_constant) {
            l1_term(p->L1, q, nq, t6, boundary_form, s);
        } else {
            for (int k = 0; k < 5; ++k) s[k] = 0.0;
            if (p->L1 != 0) {
                l1_term(p->L1, q, nq, t6, boundary_form, ind);
                for (int k = 0; k < 5; ++k) s[k] += ind[k];
            }
            double x[125];
            memcpy(x, q, 5 * sizeof(double));
            for (int k = 0; k < 6; ++k) memcpy(x + 5 + 5 * k, nq[k], 5 * sizeof(double));
            for (int k = 0; k < 6; ++k) memcpy(x + 35 + 15 * k, D + 15 * n.nb[k], 15 * sizeof(double));
            int bcase = boundary_form ? boundary_case(t6) : 0;
            const double Lc[3] = {p->L2, p->L3, p->L4};
            for (int term = 0; term < 3; ++term) {
                if (Lc[term] == 0) continue;
                multi_term(term, Lc[term], bcase, x, ind);
                for (int k = 0; k < 5; ++k) s[k] += ind[k];
            }
            if (p->L6 != 0) {
                /* DT:183-187, 273-277, 315-319: bulk form on type 0 and -2, case form on -1 */
                l6_term(p->L6, boundary_form ? bcase : -1, x, ind);
                for (int k = 0; k < 5; ++k) s[k] += ind[k];
            }
        }
        for (int k = 0; k < 5; ++k) force[k] -= s[k];

        if (p->metric_mode == 0 && t == 0) {
            /* pass 0 result, corrected; pass 1 adds the field force; corrected again */
            for (int k = 0; k < 5; ++k) f[k] = force[k];
            metric(f);
        } else {
            for (int k = 0; k < 5; ++k) f[k] = force[k];
        }
        if (t < 0) {
            for (int k = 0; k < 6; ++k) {
                if (t6[k] > 0) {
                    double af[5];
                    anchoring_force(q, nq[k], &objs[t6[k] - 1], af);
                    for (int c = 0; c < 5; ++c) f[c] += af[c];
                }
            }
        }
        if (p->efield)
            for (int k = 0; k < 5; ++k) f[k] -= fE[k];
        if (p->hfield)
            for (int k = 0; k < 5; ++k) f[k] -= fH[k];
        if (p->hvar) {
            /* landauDeGennesLC::computeSpatiallyVaryingFieldCPU (landauDeGennesLCOtherForces.cpp:254-283) */
            double g[5];
            field_force(p->hvar + 3 * i, p->dchi, p->mu0, g);
            for (int k = 0; k < 5; ++k) f[k] -= g[k];
        }
        metric(f);
    }
    free(D);
}

/* ------------------------------------------------------------ energy --
 * landauDeGennesLC::computeEnergyCPU (landauDeGennesLC.cpp:204-353).  The
 * distortion densities are written from the functionals they discretise:
 *   L1/2 dk Qij dk Qij,  L2/2 (dj Qij)^2,  L3/2 dk Qij dj Qik,
 *   L4/2 eps_lik Qlj dk Qij (chiral),
 * with central differences, one-sided next to objects (up-object wins). */
static void grad_tensor(const double *dx, const double *dy, const double *dz, double G[3][3][3])
{
    tensor3(dx, G[0]);
    tensor3(dy, G[1]);
    tensor3(dz, G[2]);
}

/* per-site energy densities e[5 i + k] (phase, distortion, anchoring, E, H) */
static void site_energies(const qo_params *p, const double *Q, const int *types, const qo_object *objs, double *e)
{
    const int L[3] = {p->Lx, p->Ly, p->Lz};
    size_t N = (size_t)L[0] * L[1] * L[2];
    double a = 0.5 * p->A, b = p->B / 3.0, c = 0.25 * p->C;
#pragma omp parallel for schedule(static)
    for (long long ii = 0; ii < (long long)N; ++ii) {
        size_t i = (size_t)ii;
        double *ei = e + 5 * i;
        for (int k = 0; k < 5; ++k) ei[k] = 0.0;
        int t = types[i];
        if (t > 0) continue;
        const double *q = Q + 5 * i;
        double t2 = tr_q2(q);
        ei[0] = a * t2 + b * tr_q3(q) + c * (t2 * t2);
        if (p->efield) {
            const double *E = p->E;
            ei[3] = p->eps0 * (-0.5 * E[0] * E[0] * (p->eps + p->deps * q[0]) - p->deps * E[0] * E[1] * q[1] -
                               p->deps * E[0] * E[2] * q[2] -
                               0.5 * E[2] * E[2] * (p->eps - p->deps * q[0] - p->deps * q[3]) -
                               0.5 * E[1] * E[1] * (p->eps + p->deps * q[3]) - p->deps * E[1] * E[2] * q[4]);
        }
        if (p->hfield) {
            const double *H = p->H;
            ei[4] = p->mu0 * (-0.5 * H[0] * H[0] * (p->chi + p->dchi * q[0]) - p->dchi * H[0] * H[1] * q[1] -
                              p->dchi * H[0] * H[2] * q[2] -
                              0.5 * H[2] * H[2] * (p->chi - p->dchi * q[0] - p->dchi * q[3]) -
                              0.5 * H[1] * H[1] * (p->chi + p->dchi * q[3]) - p->dchi * H[1] * H[2] * q[4]);
        }
        if (p->hvar) {
            /* landauDeGennesLC.cpp:256-265: same density as the uniform H field, per-site H */
            const double *H = p->hvar + 3 * i;
            ei[4] += p->mu0 * (-0.5 * H[0] * H[0] * (p->chi + p->dchi * q[0]) - p->dchi * H[0] * H[1] * q[1] -
                               p->dchi * H[0] * H[2] * q[2] -
                               0.5 * H[2] * H[2] * (p->chi - p->dchi * q[0] - p->dchi * q[3]) -
                               0.5 * H[1] * H[1] * (p->chi + p->dchi * q[3]) - p->dchi * H[1] * H[2] * q[4]);
        }
        qo_nbrs n;
        neighbours(L, i, &n);
        double d[3][5];
        for (int ax = 0; ax < 3; ++ax) {
            const double *qd = Q + 5 * n.nb[2 * ax], *qu = Q + 5 * n.nb[2 * ax + 1];
            for (int k = 0; k < 5; ++k) d[ax][k] = 0.5 * (qu[k] - qd[k]);
        }
        if (t < 0) {
            for (int ax = 0; ax < 3; ++ax) {
                size_t dn = n.nb[2 * ax], up = n.nb[2 * ax + 1];
                const double *qd = Q + 5 * dn, *qu = Q + 5 * up;
                if (types[dn] > 0) {
                    ei[2] += anchoring_energy(q, qd, &objs[types[dn] - 1]);
                    for (int k = 0; k < 5; ++k) d[ax][k] = qu[k] - q[k];
                }
                if (types[up] > 0) {
                    ei[2] += anchoring_energy(q, qu, &objs[types[up] - 1]);
                    for (int k = 0; k < 5; ++k) d[ax][k] = q[k] - qd[k];
                }
            }
        }
        double G[3][3][3];
        grad_tensor(d[0], d[1], d[2], G);
        double dist = 0.0;
        if (p->L1 != 0) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int x = 0; x < 3; ++x)
                    for (int y = 0; y < 3; ++y) s += G[k][x][y] * G[k][x][y];
            dist += 0.5 * p->L1 * s;
        }
        if (p->L2 != 0) {
            double s = 0.0;
            for (int x = 0; x < 3; ++x) {
                double div = G[0][x][0] + G[1][x][1] + G[2][x][2];
                s += div * div;
            }
            dist += 0.5 * p->L2 * s;
        }
        if (p->L3 != 0) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int x = 0; x < 3; ++x)
                    for (int y = 0; y < 3; ++y) s += G[k][x][y] * G[y][x][k];
            dist += 0.5 * p->L3 * s;
        }
        if (p->L4 != 0) {
            /* chiral term L4/2 eps_lik Q_lj dk Q_ij */
            static const int lc[6][4] = {{0, 1, 2, 1}, {1, 2, 0, 1}, {2, 0, 1, 1}, {0, 2, 1, -1}, {2, 1, 0, -1}, {1, 0, 2, -1}};
            double Qm[3][3];
            tensor3(q, Qm);
            double s = 0.0;
            for (int e6 = 0; e6 < 6; ++e6) {
                int l = lc[e6][0], x = lc[e6][1], k = lc[e6][2];
                for (int y = 0; y < 3; ++y) s += lc[e6][3] * Qm[l][y] * G[k][x][y];
            }
            dist += 0.5 * p->L4 * s;
        }
        if (p->L6 != 0) {
            /* cubic term L6/2 Q_ab da Q_ij db Q_ij */
            double Qm[3][3];
            tensor3(q, Qm);
            double s = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double g = 0.0;
                    for (int x = 0; x < 3; ++x)
                        for (int y = 0; y < 3; ++y) g += G[a][x][y] * G[b][x][y];
                    s += Qm[a][b] * g;
                }
            dist += 0.5 * p->L6 * s;
        }
        ei[1] = dist;
    }
}

/* The per-site energy densities that qo_energy sums (5 per site: phase,
 * distortion, anchoring, E field, H field; zero on object sites), for checks
 * that sum them in another order than the reference's sequential loop. */
void qo_energy_densities(const qo_params *p, const double *Q, const int *types, const qo_object *objs, double *e)
{
    site_energies(p, Q, types, objs, e);
}

double qo_energy(const qo_params *p, const double *Q, const int *types, const qo_object *objs, double comps[5])
{
    size_t N = (size_t)p->Lx * p->Ly * p->Lz;
    double *e = (double *)malloc(sizeof(double) * 5 * N);
    site_energies(p, Q, types, objs, e);
    double cs[5] = {0, 0, 0, 0, 0};
    for (size_t i = 0; i < N; ++i)
        for (int k = 0; k < 5; ++k) cs[k] += e[5 * i + k];
    free(e);
    if (comps)
        for (int k = 0; k < 5; ++k) comps[k] = cs[k];
    return cs[0] + cs[1] + cs[2] + cs[3] + cs[4];
}

/* landauDeGennesLC::computeObjectForces / computeStressTensors, one-constant
 * (landauDeGennesLCOtherForces.cpp:147-251): for object j, the sum over its
 * surface sites (LC sites with an object-j neighbour) of sigma . a with
 * sigma_ab = e delta_ab - L1 B(d_a q, d_b q), B(u, v) = 2 (u0 v0 + u3 v3) +
 * u0 v3 + u3 v0 + 4 (u1 v1 + u2 v2 + u4 v4), e the site's total energy density,
 * d_a q the first derivatives, a the +-1 direction to object neighbours (up wins). */
void qo_object_forces(const qo_params *p, const double *Q, const int *types, const qo_object *objs, int nobj,
                      double *out)
{
    const int L[3] = {p->Lx, p->Ly, p->Lz};
    size_t N = (size_t)L[0] * L[1] * L[2];
    double *e = (double *)malloc(sizeof(double) * 5 * N);
    double *D = (double *)malloc(sizeof(double) * 15 * N);
    site_energies(p, Q, types, objs, e);
    first_derivatives(L, Q, types, D);
    for (int j = 0; j < 3 * nobj; ++j) out[j] = 0.0;
    for (size_t i = 0; i < N; ++i) {
        if (types[i] > 0) continue;
        qo_nbrs n;
        neighbours(L, i, &n);
        int tn[6];
        for (int s = 0; s < 6; ++s) tn[s] = types[n.nb[s]];
        const double *ei = e + 5 * i;
        double et = ei[0] + ei[3] + ei[4] + ei[2] + ei[1];
        double a[3];
        for (int ax = 0; ax < 3; ++ax) {
            a[ax] = 0.0;
            if (tn[2 * ax] > 0) a[ax] = -1.0;
            if (tn[2 * ax + 1] > 0) a[ax] = 1.0;
        }
        double f[3];
        for (int r = 0; r < 3; ++r) {
            f[r] = 0.0;
            for (int cc = 0; cc < 3; ++cc) {
                const double *u = D + 15 * i + 5 * r, *v = D + 15 * i + 5 * cc;
                double B = 2.0 * (u[0] * v[0] + u[3] * v[3]) + u[0] * v[3] + u[3] * v[0] +
                           4.0 * (u[1] * v[1] + u[2] * v[2] + u[4] * v[4]);
                f[r] += (-p->L1 * B + (r == cc ? et : 0.0)) * a[cc];
            }
        }
        for (int obj = 1; obj <= nobj; ++obj) {
            int next = 0;
            for (int s = 0; s < 6; ++s) next |= tn[s] == obj;
            if (next)
                for (int r = 0; r < 3; ++r) out[3 * (obj - 1) + r] += f[r];
        }
    }
    free(e);
    free(D);
}

/* ------------------------------------------------------------- FIRE ---- */
static double dot_qt(const double *x, const double *y) /* dotVec, inc/functions.h:140-147 */
{
    double s = 0.0;
    for (int k = 0; k < 5; ++k) s += x[k] * y[k];
    s += x[0] * y[3];
    return s;
}
static double dot_plain(const double *x, const double *y) /* dot, inc/functions.h:131-138 */
{
    double s = 0.0;
    for (int k = 0; k < 5; ++k) s += x[k] * y[k];
    return s;
}

/* energyMinimizerFIRE::initializeParameters / setFIREParameters (energyMinimizerFIRE.cpp:24-43, 172-183) */
void qo_fire_init(const qo_fire_params *fp, qo_fire_state *st)
{
    st->iterations = 0;
    st->forceMax = 100.;
    st->alpha = fp->alpha0;
    st->dt = fp->dt;
    st->power = 0.0;
    st->nsince = 0;
}

/* energyMinimizerFIRE::minimize (energyMinimizerFIRE.cpp:151-170) with
 * velocityVerlet::integrateEOMCPU (velocityVerlet.cpp:8-40) and
 * fireStepCPU (energyMinimizerFIRE.cpp:77-145).  F must hold the force at Q
 * on entry; minimize() recomputes it, as the reference does.  trace (if not
 * NULL) receives per iteration: forceMax, alpha, dt, power, nsince. */
int qo_fire(const qo_params *p, double *Q, double *V, double *F, const int *types, const qo_object *objs,
            const qo_fire_params *fp, int max_iters, qo_fire_state *st, double *trace)
{
    size_t N = (size_t)p->Lx * p->Ly * p->Lz;
    int nTotal = qo_count_active((int)N, types);
    double dtmin = fp->dt * .01;
    double *tmp = (double *)malloc(sizeof(double) * 3 * N);
    qo_force(p, Q, types, objs, F);
    int start = st->iterations, done = 0;
    while ((st->iterations < max_iters && st->forceMax > fp->fcut) || st->iterations == start) {
        st->iterations += 1;
        double dt = st->dt;
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)(5 * N); ++ii) {
            size_t j = (size_t)ii;
            double disp = dt * V[j] + (0.5 * dt * dt) * F[j];
            V[j] += (0.5) * dt * F[j];
            Q[j] += disp;
        }
        qo_force(p, Q, types, objs, F);
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)(5 * N); ++ii) V[ii] += (0.5) * dt * F[ii];

        /* fireStepCPU */
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)N; ++ii) {
            size_t i = (size_t)ii;
            tmp[3 * i] = dot_qt(F + 5 * i, F + 5 * i);
            tmp[3 * i + 1] = dot_qt(V + 5 * i, V + 5 * i);
            tmp[3 * i + 2] = dot_qt(F + 5 * i, V + 5 * i);
        }
        double fn = 0.0, vn = 0.0, pw = 0.0;
        for (size_t i = 0; i < N; ++i) {
            fn += tmp[3 * i];
            vn += tmp[3 * i + 1];
            pw += tmp[3 * i + 2];
        }
        st->power = pw;
        st->forceMax = sqrt(fn) / ((double)nTotal);
        double scaling = 0.0;
        if (fn > 0.) scaling = sqrt(vn / fn);
        double alpha = st->alpha;
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)(5 * N); ++ii)
            V[ii] = (1.0 - alpha) * V[ii] + alpha * scaling * F[ii];
        if (pw > 0 && st->iterations % 500 != 0) {
            if (st->nsince > fp->nmin) {
                st->dt = fmin(st->dt * fp->dtinc, fp->dtmax);
                st->alpha = st->alpha * fp->alphadec;
                st->alpha = fmax(st->alpha, fp->alphamin);
            }
            st->nsince += 1;
        } else {
            st->nsince = 0;
            st->dt = st->dt * fp->dtdec;
            st->dt = fmax(st->dt, dtmin);
            st->alpha = fp->alpha0;
            memset(V, 0, sizeof(double) * 5 * N);
        }
        if (trace) {
            double *t = trace + 5 * (size_t)done;
            t[0] = st->forceMax;
            t[1] = st->alpha;
            t[2] = st->dt;
            t[3] = st->power;
            t[4] = st->nsince;
        }
        ++done;
    }
    free(tmp);
    return done;
}

/* energyMinimizerAdam::minimize / adamStepCPU (energyMinimizerAdam.cpp:25-76);
 * M, S are the biased moment estimates (zero on the first call). */
int qo_adam(const qo_params *p, double *Q, double *F, const int *types, const qo_object *objs,
            double beta1, double beta2, double eps, double dt, double fcut, int max_iters,
            double *M, double *S, double *forcemax_out)
{
    size_t N = (size_t)p->Lx * p->Ly * p->Lz;
    double b1t = beta1, b2t = beta2, forceMax = 110.0;
    double *tmp = (double *)malloc(sizeof(double) * N);
    int it = 0;
    while (it < max_iters && forceMax > fcut) {
        it += 1;
        qo_force(p, Q, types, objs, F);
        double c1 = 1.0 / (1.0 - b1t), c2 = 1.0 / (1.0 - b2t);
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)N; ++ii) {
            size_t i = (size_t)ii;
            tmp[i] = dot_plain(F + 5 * i, F + 5 * i);
            for (int k = 0; k < 5; ++k) {
                size_t j = 5 * i + k;
                M[j] = beta1 * M[j] + (beta1 - 1) * F[j];
                S[j] = beta2 * S[j] + (1 - beta2) * (F[j] * F[j]);
                double mc = M[j] * c1, vc = S[j] * c2;
                double root = sqrt(vc);
                if (root == 0) root = eps;
                Q[j] += -dt * mc / (root);
            }
        }
        double fn = 0.0;
        for (size_t i = 0; i < N; ++i) fn += tmp[i];
        forceMax = sqrt(fn) / N;
        b1t *= beta1;
        b2t *= beta2;
    }
    free(tmp);
    if (forcemax_out) *forcemax_out = forceMax;
    return it;
}

/* energyMinimizerNesterovAG::minimize / nesterovStepCPU (energyMinimizerNesterovAG.cpp:75-120),
 * fixed momentum mu; alt is the alternate sequence (initially a copy of Q). */
int qo_nesterov(const qo_params *p, double *Q, double *F, const int *types, const qo_object *objs,
                double dt, double mu, double fcut, int max_iters, double *alt, double *forcemax_out)
{
    size_t N = (size_t)p->Lx * p->Ly * p->Lz;
    double forceMax = 110.0;
    double *tmp = (double *)malloc(sizeof(double) * N);
    int it = 0;
    while (it < max_iters && forceMax > fcut) {
        it += 1;
        qo_force(p, Q, types, objs, F);
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)N; ++ii) {
            size_t i = (size_t)ii;
            tmp[i] = dot_plain(F + 5 * i, F + 5 * i);
            for (int k = 0; k < 5; ++k) {
                size_t j = 5 * i + k;
                double old = alt[j];
                alt[j] = Q[j] + dt * F[j];
                Q[j] = alt[j] + mu * (alt[j] - old);
            }
        }
        double fn = 0.0;
        for (size_t i = 0; i < N; ++i) fn += tmp[i];
        forceMax = sqrt(fn) / N;
    }
    free(tmp);
    if (forcemax_out) *forcemax_out = forceMax;
    return it;
}

/* determinantOfQ (qTensorFunctions.h:136-140) */
static double det_q(const double *q)
{
    return q[3] * (q[1] * q[1] - q[0] * q[0] - q[2] * q[2]) + 2 * q[1] * q[2] * q[4] +
           q[0] * (q[1] * q[1] - q[3] * q[3] - q[4] * q[4]);
}

/* qTensorLatticeModel::computeDefectMeasures (qTensorLatticeModel.cpp:95-133) with
 * eigenvaluesOfQ (qTensorFunctions.h:215-241); object sites get 0 */
void qo_defects(const qo_params *p, const double *Q, const int *types, int kind, double *out)
{
    const double pi = 3.14159265358979323846;
    size_t N = (size_t)p->Lx * p->Ly * p->Lz;
    for (size_t i = 0; i < N; ++i) {
        const double *q = Q + 5 * i;
        double v = 0.0;
        if (types[i] <= 0) {
            if (kind == 0) {
                double a, b, c;
                double p1 = q[1] * q[1] + q[2] * q[2] + q[4] * q[4];
                if (p1 == 0) {
                    a = q[0]; b = q[3]; c = -q[0] - q[3];
                } else {
                    double p2 = 2 * (q[0] * q[0] + q[3] * q[3] + q[0] * q[3]) + 2 * p1;
                    double pp = sqrt(p2 / 6.0), ip = 1.0 / pp;
                    double B[5] = {ip * q[0], ip * q[1], ip * q[2], ip * q[3], ip * q[4]};
                    double r = 0.5 * det_q(B);
                    double phi = r <= -1 ? pi / 3.0 : (r >= 1 ? 0.0 : acos(r) / 3.0);
                    a = 2.0 * pp * cos(phi);
                    c = 2.0 * pp * cos(phi + 2.0 * pi / 3.0);
                    b = -a - c;
                }
                v = fmax(fmax(a, b), c);
            } else if (kind == 1) {
                v = det_q(q);
            } else {
                double t2 = 2.0 * (q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + q[4] * q[4] + q[0] * q[3]);
                double d = det_q(q);
                v = t2 * t2 * t2 - 54.0 * d * d;
            }
        }
        out[i] = v;
    }
}

/* energyMinimizerGradientDescent::minimize / gradientDescentCPU
 * (energyMinimizerGradientDescent.cpp:64-106): forces at Q on entry, then per
 * iteration Q += dt F (qTensorLatticeModel::moveParticles), forces at the new Q,
 * forceMax = sqrt(sum_i F_i.F_i) / nTotal with the plain dot product and
 * nTotal = non-object sites; at least one iteration. */
int qo_gd(const qo_params *p, double *Q, double *F, const int *types, const qo_object *objs, double dt, double fcut,
          int max_iters, double *forcemax_out)
{
    size_t N = (size_t)p->Lx * p->Ly * p->Lz;
    long long nTotal = 0;
    for (size_t i = 0; i < N; ++i) nTotal += types[i] <= 0;
    double *tmp = (double *)malloc(sizeof(double) * N);
    double forceMax = 0.0;
    int it = 0;
    qo_force(p, Q, types, objs, F);
    do {
        it += 1;
#pragma omp parallel for schedule(static)
        for (long long j = 0; j < (long long)(5 * N); ++j) Q[j] += dt * F[j];
        qo_force(p, Q, types, objs, F);
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)N; ++ii) tmp[ii] = dot_plain(F + 5 * ii, F + 5 * ii);
        double fn = 0.0;
        for (size_t i = 0; i < N; ++i) fn += tmp[i];
        forceMax = sqrt(fn) / (double)nTotal;
    } while (it < max_iters && forceMax > fcut);
    free(tmp);
    if (forcemax_out) *forcemax_out = forceMax;
    return it;
}

/* host_dVec_dot_products (src/utilities/utilities.cpp:4-11): site-major sequential sum */
static double vdot(const double *x, const double *y, size_t n5)
{
    double s = 0.0;
    for (size_t j = 0; j < n5; ++j) s += x[j] * y[j];
    return s;
}
static void vaxpy(double *y, const double *x, double a, size_t n5) /* host_dVec_plusEqual_dVec */
{
#pragma omp parallel for schedule(static)
    for (long long j = 0; j < (long long)n5; ++j) y[j] = y[j] + a * x[j];
}

/* energyMinimizerLoLBFGS::minimize / LoLBFGSStepCPU (energyMinimizerLoLBFGS.cpp:105-226):
 * two-loop recursion over m (s, y) pairs on the force direction, fixed gain eta,
 * no line search (the call at :177 is commented out in the reference). */
int qo_lbfgs(const qo_params *p, double *Q, double *F, const int *types, const qo_object *objs,
             int m, double eta, double fcut, int max_iters, double *forcemax_out)
{
    size_t N = (size_t)p->Lx * p->Ly * p->Lz, n5 = 5 * N;
    double *pv = (double *)calloc(n5, sizeof(double));
    double *s = (double *)calloc(n5 * (size_t)m, sizeof(double));
    double *y = (double *)calloc(n5 * (size_t)m, sizeof(double));
    double *sy = (double *)calloc((size_t)m, sizeof(double));
    double *al = (double *)calloc((size_t)m, sizeof(double));
    double forceMax = 100.;
    int it = 0, cur = 0, start = 0;
    while ((it < max_iters && forceMax > fcut) || it == start) {
        int lastM = (cur - 1 + m) % m;
        if (it == 0) {
            qo_force(p, Q, types, objs, F);
            memcpy(pv, F, sizeof(double) * n5);
        }
        for (int ii = 0; ii < m; ++ii) {
            int t = (cur - ii - 1 + m) % m;
            sy[ii] = vdot(s + n5 * t, y + n5 * t, n5);
            al[ii] = 0;
            if (sy[ii] != 0) al[ii] = vdot(s + n5 * t, pv, n5) / sy[ii];
            vaxpy(pv, y + n5 * t, -al[ii], n5);
        }
        {
            double v1 = sy[0], v2 = vdot(y + n5 * lastM, y + n5 * lastM, n5);
            if (v2 != 0) vaxpy(pv, y + n5 * lastM, v1 / v2, n5);
        }
        for (int ii = m - 1; ii >= 0; --ii) {
            int t = (cur - ii - 1 + m) % m;
            if (sy[ii] != 0) {
                double beta = vdot(y + n5 * t, pv, n5) / sy[ii];
                vaxpy(pv, s + n5 * t, al[ii] - beta, n5);
            }
        }
        double *sc = s + n5 * cur, *yc = y + n5 * cur;
        for (size_t j = 0; j < n5; ++j) sc[j] = eta * pv[j];
        memcpy(yc, F, sizeof(double) * n5);
        for (size_t j = 0; j < n5; ++j) Q[j] += sc[j];
        qo_force(p, Q, types, objs, F);
        memcpy(pv, F, sizeof(double) * n5);
        vaxpy(yc, pv, -1.0, n5);
        forceMax = sqrt(vdot(pv, pv, n5)) / N;
        it += 1;
        cur = (cur + 1) % m;
    }
    free(pv); free(s); free(y); free(sy); free(al);
    if (forcemax_out) *forcemax_out = forceMax;
    return it;
}
