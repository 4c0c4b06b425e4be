/* qmin oracle: a CPU restatement, in plain C, of the reference's (open-Qmin)
 * single-rank CPU minimisation path.  TEST INFRASTRUCTURE ONLY: the test
 * suite, the smoke check and bench.py's CPU-baseline leg use it as the
 * checker; the product never links, loads or calls it.
 *
 * Pinned against the reference itself: tests/golden/ holds dumps made by the
 * reference's own CPU objects (oracle/ref/ref_dumper.cpp, built from the
 * reference tree by oracle/ref/Makefile), and tests/test_oracle_golden.py
 * checks this restatement against every one of them.
 *
 * Conventions follow the reference: AoS Q[5*i + k], k = (Qxx, Qxy, Qxz, Qyy,
 * Qyz) (inc/qTensorFunctions.h:8-12); site index i = x + Lx*(y + Ly*z)
 * (inc/indexer.h:71-131); types: 0 bulk LC, -1 LC next to an object, -2 LC at
 * a rank face (treated as bulk-formula/boundary-pass), j > 0 object j-1
 * (src/model/multirankQTensorLatticeModel.h:9-15). */
#ifndef QMIN_ORACLE_H
#define QMIN_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int Lx, Ly, Lz;
    double A, B, C;          /* phase constants as landauDeGennesLC stores them (openQmin.cpp:173-175) */
    double L1, L2, L3, L4;   /* elastic constants (landauDeGennesLC.h:35) */
    int multi_constant;      /* 0: one-constant path, 1: first derivatives + multi-constant forms */
    int efield, hfield;
    double E[3], eps, eps0, deps;  /* setEField (landauDeGennesLC.h:76-83) */
    double H[3], chi, mu0, dchi;   /* setHField (landauDeGennesLC.h:84-91) */
    int metric_mode;         /* 0: CPU path (M^2 on type 0, M on type < 0), 1: M once everywhere */
    const double *hvar;      /* spatially varying H field, N x 3 per site, or NULL
                                (landauDeGennesLC::setSpatiallyVaryingField, landauDeGennesLC.cpp:81-123) */
    double L6;               /* cubic elastic constant (landauDeGennesLC.h:35, lcForces.h:801-1047) */
} qo_params;

typedef struct { int kind; double W, S0; } qo_object; /* kind 0 homeotropic, 1 degenerate planar */

typedef struct {
    double dt, alpha0, dtmax, dtinc, dtdec, alphadec, alphamin, fcut;
    int nmin;
} qo_fire_params;

typedef struct {
    int iterations;          /* updater::iterations after the run */
    double forceMax, alpha, dt, power;
    int nsince;
} qo_fire_state;

/* host initialisation and geometry */
void qo_random_nematic(int N, unsigned seed, double S0, double *Q);
int qo_add_wall(const int L[3], int xyz, int plane, int kind, double W, double S0,
                double *Q, int *types, qo_object *objs, int nobj);
int qo_add_sites(const int L[3], int nsites, const int *xyz, const double *qs, int kind, double W, double S0,
                 double *Q, int *types, qo_object *objs, int nobj);
void qo_defects(const qo_params *p, const double *Q, const int *types, int kind, double *out);
void qo_object_forces(const qo_params *p, const double *Q, const int *types, const qo_object *objs, int nobj,
                      double *out);
int qo_add_sphere(const int L[3], const double center[3], double radius, int kind, double W, double S0,
                  double *Q, int *types, qo_object *objs, int nobj);
int qo_count_active(int N, const int *types);

/* force and energy */
void qo_force(const qo_params *p, const double *Q, const int *types, const qo_object *objs, double *F);
void qo_energy_densities(const qo_params *p, const double *Q, const int *types, const qo_object *objs, double *e);
double qo_energy(const qo_params *p, const double *Q, const int *types, const qo_object *objs, double comps[5]);

/* minimisers; each returns the number of iterations it performed */
void qo_fire_init(const qo_fire_params *fp, qo_fire_state *st);
int qo_fire(const qo_params *p, double *Q, double *V, double *F, const int *types, const qo_object *objs,
            const qo_fire_params *fp, int max_iters, qo_fire_state *st, double *trace);
int qo_adam(const qo_params *p, double *Q, double *F, const int *types, const qo_object *objs,
            double beta1, double beta2, double eps, double dt, double fcut, int max_iters,
            double *M, double *S, double *forcemax_out);
int qo_gd(const qo_params *p, double *Q, double *F, const int *types, const qo_object *objs, double dt, double fcut,
          int max_iters, double *forcemax_out);
int qo_nesterov(const qo_params *p, double *Q, double *F, const int *types, const qo_object *objs,
                double dt, double mu, double fcut, int max_iters, double *alt, double *forcemax_out);
int qo_lbfgs(const qo_params *p, double *Q, double *F, const int *types, const qo_object *objs,
             int m, double eta, double fcut, int max_iters, double *forcemax_out);

/* threads used by the per-site loops (OpenMP builds only); returns the count in effect */
int qo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
