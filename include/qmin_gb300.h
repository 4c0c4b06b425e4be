/* qmin_gb300: GB300-native (sm_103a) Landau-de Gennes Q-tensor minimisation
 * engine with the capabilities of open-Qmin's minimisation hot path.
 *
 * C ABI: plain pointers and sizes, int status codes (QMIN_OK = 0), no
 * exceptions across the boundary.  A handle owns all device memory for one
 * lattice; callers own every host buffer they pass.  A handle is used from one
 * host thread at a time.  All work is issued on the handle's CUDA stream
 * (qmin_set_stream; default: a stream the handle creates).  A process drives
 * one GPU: handles and nets use the current CUDA device, which stays the same
 * for the life of the process (the kernels' shared-memory limits are set
 * once per process).
 *
 * Host arrays use the reference's layout unless a layout argument says
 * otherwise: Q/V/F as AoS double[N][5] with components (Qxx, Qxy, Qxz, Qyy,
 * Qyz) (open-Qmin inc/qTensorFunctions.h:8-12), site index
 * i = x + Lx*(y + Ly*z) (inc/indexer.h:71-131), site types int32 with
 * 0 = bulk LC, -1 = LC next to an object, -2 = LC on a rank face, j > 0 =
 * site of object j-1 (src/model/multirankQTensorLatticeModel.h:9-15).
 *
 * Each entry point names the reference interface it replaces. */
#ifndef QMIN_GB300_H
#define QMIN_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define QMIN_OK 0
#define QMIN_EINVAL 1      /* bad argument (null pointer, size, enum) */
#define QMIN_ECUDA 2       /* CUDA runtime error (message in qmin_last_error_string) */
#define QMIN_ENOMEM 3      /* device allocation failed */
#define QMIN_ESTATE 4      /* call out of order (e.g. force before set_state) */
#define QMIN_ENONFINITE 5  /* a reduction produced NaN/Inf (state left as computed) */
#define QMIN_ENODEVICE 6   /* no CUDA device / extension not usable */
#define QMIN_ETIMEOUT 7    /* a bounded device-side wait gave up (the run stopped; see the entry point) */

/* precision of the resident state and stencil arithmetic */
#define QMIN_FP64 0        /* every operation in FP64 (oracle-parity form) */
#define QMIN_FP32 1        /* FP32 state and stencils, FP64 reductions */

/* metric correction semantics (landauDeGennesLC::correctForceFromMetric) */
#define QMIN_METRIC_CPU 0    /* reference CPU path: M^2 on bulk sites, M on boundary sites */
#define QMIN_METRIC_SINGLE 1 /* reference GPU path: M once on every site */

/* host array layouts */
#define QMIN_LAYOUT_AOS 0  /* double[N][5] */
#define QMIN_LAYOUT_SOA 1  /* double[5][N] */

/* object (boundary) kinds, open-Qmin src/model/latticeBoundaries.h:8 */
#define QMIN_HOMEOTROPIC 0
#define QMIN_DEGENERATE_PLANAR 1

typedef struct qmin_ctx *qmin_handle;

typedef struct {
    int Lx, Ly, Lz;
    int precision;   /* QMIN_FP64 or QMIN_FP32 */
    int metric_mode; /* QMIN_METRIC_CPU or QMIN_METRIC_SINGLE */
} qmin_lattice_desc;

/* landauDeGennesLC parameters (landauDeGennesLC.h:34-36, 76-91).  A, B, C are
 * the phase constants exactly as the force class stores them (the CLI passes
 * a = -1, b = -B/A, c = -C/A, openQmin.cpp:173-175). */
typedef struct {
    double A, B, C;
    double L1, L2, L3, L4;
    int multi_constant;  /* 0: one-constant (L1 only) path; 1: multi-constant forms */
    int efield;          /* uniform E field on */
    double E[3], eps, eps0, deps;
    int hfield;          /* uniform H field on */
    double H[3], chi, mu0, dchi;
    double L6;           /* cubic elastic constant (setElasticConstants' l6); needs multi_constant;
                            single-lattice handles only (a batch rejects it) */
} qmin_ldg_params;

/* boundaryObject{boundary, P1 = W, P2 = S0} (latticeBoundaries.h:20-39) */
typedef struct {
    int kind;
    double W;
    double S0;
} qmin_object;

/* energyMinimizerFIRE::setFIREParameters (energyMinimizerFIRE.h:33) */
typedef struct {
    double dt, alpha_start, dt_max, dt_inc, dt_dec, alpha_dec, alpha_min, force_cutoff;
    int n_min;
} qmin_fire_params;

typedef struct {
    int iterations;   /* updater::iterations (cumulative across runs) */
    double force_max; /* sqrt(sum F._QT F) / nTotal (energyMinimizerFIRE.cpp:110) */
    double alpha, dt, power;
    int n_since;
} qmin_fire_result;

/* ---- lifetime (replaces constructing multirankQTensorLatticeModel +
 *      landauDeGennesLC + GPUArray storage, openQmin.cpp:194-197) ---- */
int qmin_create(const qmin_lattice_desc *desc, qmin_handle *out);
int qmin_destroy(qmin_handle h);
/* cudaStream_t passed as void* so the header needs no CUDA includes */
int qmin_set_stream(qmin_handle h, void *stream);
const char *qmin_last_error_string(void);
/* count of this library's kernel launches issued through the handle */
int qmin_kernel_launches(qmin_handle h, long long *count);

/* ---- configuration ---- */
/* landauDeGennesLC::setPhaseConstants / setElasticConstants / setEField / setHField */
int qmin_set_params(qmin_handle h, const qmin_ldg_params *p);
/* cubicLattice::boundaries (the GPUArray<boundaryObject> that createBoundaryObject grows) */
int qmin_set_objects(qmin_handle h, const qmin_object *objs, int n);
/* model positions + types (simpleModel::returnPositions/returnTypes, simpleModel.h:65-77);
 * velocities are zeroed (simpleModel::initializeSimpleModel, simpleModel.cpp:39) */
int qmin_set_state(qmin_handle h, const double *Q, const int32_t *types, int layout);
/* read back positions/velocities/forces; any pointer may be NULL */
int qmin_get_state(qmin_handle h, double *Q, double *V, double *F, int layout);
/* number of non-object sites (updater::getNTotal, baseUpdater.cpp:10-28) */
int qmin_n_active(qmin_handle h, long long *n);
/* lattice sides of the handle (cubicLattice::latticeSites) */
int qmin_get_sides(qmin_handle h, int *Lx, int *Ly, int *Lz);
/* site types as int32 (simpleModel::returnTypes) */
int qmin_get_types(qmin_handle h, int32_t *types);
/* overwrite Q only, keeping types, velocities and minimiser state (writing
 * through simpleModel::returnPositions, as multirankSimulation::loadState does) */
int qmin_set_positions(qmin_handle h, const double *Q, int layout);
/* overwrite the velocities (writing through simpleModel::returnVelocities,
 * simpleModel.h:67): a caller whose own model holds the velocities between
 * minimize() calls (the reference keeps them in the model) restores them
 * after qmin_set_state and qmin_fire_init, which both zero them */
int qmin_set_velocities(qmin_handle h, const double *V, int layout);
/* qTensorLatticeModel::computeDefectMeasures (qTensorLatticeModel.cpp:95-133):
 * kind 0 largest eigenvalue of Q, 1 det Q, 2 (tr Q^2)^3 - 54 (det Q)^2, on
 * sites with type <= 0; object sites get 0.  out: host, N doubles. */
int qmin_defect_measures(qmin_handle h, int kind, double *out);

/* landauDeGennesLC::computeObjectForces (landauDeGennesLCOtherForces.cpp:147-251):
 * the force on every object from the stress tensor of the LC sites next to it,
 * forces[3*j .. 3*j+2] for object j (host; capacity = number of objects it
 * holds; *nobj_out, may be NULL, receives the object count).  One-constant
 * form only, as in the reference (QMIN_EINVAL otherwise).  Each call returns
 * the force of the current state; the reference instead adds it to a running
 * per-object total (cubicLattice::boundaryForce) on every call. */
int qmin_object_forces(qmin_handle h, double *forces, int capacity, int *nobj_out);

/* landauDeGennesLC::setSpatiallyVaryingField (landauDeGennesLC.cpp:81-123) with
 * the field given directly: H is host AoS double[N][3] (NULL switches the
 * field off); chi, mu0, dchi replace the H-field constants of qmin_set_params,
 * as the reference's setter does.  Its force (landauDeGennesLCOtherForces.cpp:254-283)
 * and energy (landauDeGennesLC.cpp:256-265) are the uniform H field's with
 * each site's own H, on sites with type <= 0.  Call after qmin_set_params. */
int qmin_set_field_map(qmin_handle h, const double *H, double chi, double mu0, double dchi);

/* ---- files ---- */
/* the same field read from <prefix>_x0y0z0.txt, lines "x y z Hx Hy Hz"
 * (sites not listed get H = 0) */
int qmin_load_field_map(qmin_handle h, const char *prefix, double chi, double mu0, double dchi);
/* multirankSimulation::saveState (multirankSimulation.cpp:616-665), single
 * rank: writes <prefix>_x0y0z0.txt, one line per site whose x, y and z are
 * multiples of lattice_skip: "x y z Qxx Qxy Qxz Qyy Qyz type defect"
 * (tab-separated, numbers as C++ streams print them), defect =
 * qmin_defect_measures(defect_kind). */
int qmin_save_state(qmin_handle h, const char *prefix, int lattice_skip, int defect_kind);
/* multirankSimulation::loadState (multirankSimulation.cpp:566-614), single
 * rank: reads <prefix>_x0y0z0.txt and sets Q of every listed site; types and
 * velocities are kept.  QMIN_EINVAL if the file cannot be opened or a listed
 * site lies outside the lattice. */
int qmin_load_state(qmin_handle h, const char *prefix);
/* Binary exact-resume checkpoint (no reference counterpart): resident state,
 * parameters, objects, FIRE / minimiser scalars and buffers, FIRE strategy.
 * Loading needs a handle of the same sides, precision and metric mode; a run
 * resumed from it repeats the saved run's iterations bit for bit. */
int qmin_checkpoint_save(qmin_handle h, const char *path);
int qmin_checkpoint_load(qmin_handle h, const char *path);

/* ---- force and energy ---- */
/* multirankSimulation::computeForces -> landauDeGennesLC::computeForces
 * (multirankSimulation.cpp:452-473, landauDeGennesLC.cpp:125-202).  The
 * forces stay resident; F_out (host, AoS) may be NULL. */
int qmin_force(qmin_handle h, double *F_out);
/* multirankSimulation::computePotentialEnergy (multirankSimulation.cpp:475-490):
 * e_per_active = E / NActive; comps = phase, distortion, anchoring, E-field,
 * H-field totals (landauDeGennesLC::energyComponents). */
int qmin_energy(qmin_handle h, double *e_per_active, double comps[5]);

/* ---- minimisers (updater::Update -> performUpdate -> minimize) ---- */
/* energyMinimizerFIRE constructor + setFIREParameters: resets alpha, dt,
 * counters (energyMinimizerFIRE.cpp:24-43) */
int qmin_fire_init(qmin_handle h, const qmin_fire_params *p);
/* energyMinimizerFIRE::minimize (energyMinimizerFIRE.cpp:151-170) with
 * setMaximumIterations(max_iterations); velocity Verlet + FIRE on the GPU,
 * graph-captured, no host synchronisation inside a chunk of iterations.
 * QMIN_ETIMEOUT when a wait of the TMA-staged deep-site kernel (split variant
 * 6) gave up (qmin_set_wait_limit): the lattice's state is then void. */
int qmin_fire_run(qmin_handle h, int max_iterations, qmin_fire_result *res);
/* The FIRE updater's state that persists between minimize() calls in the
 * reference: updater::iterations and energyMinimizerFIRE's forceMax, alpha,
 * deltaT, deltaTMin, Power and NSinceNegativePower (energyMinimizerFIRE.h:66-94). */
typedef struct {
    int iterations;
    double force_max, alpha, dt, dt_min, power;
    int n_since;
} qmin_fire_state;
/* A caller that keeps those members in its own updater object (a subclass of
 * energyMinimizerFIRE) restores them after qmin_fire_init; the next
 * qmin_fire_run continues from them as minimize() does.  Requires
 * qmin_fire_init first. */
int qmin_fire_set_state(qmin_handle h, const qmin_fire_state *st);
/* energyMinimizerAdam::setAdamParameters + minimize (energyMinimizerAdam.h:20-31,
 * energyMinimizerAdam.cpp:56-76); moments reset when reset != 0 */
int qmin_adam_run(qmin_handle h, double beta1, double beta2, double eps, double dt, double force_cutoff,
                  int max_iterations, int reset, int *iterations, double *force_max);
/* energyMinimizerNesterovAG::setNesterovAGParameters + minimize
 * (energyMinimizerNesterovAG.h:24-29, .cpp:94-120); the alternate sequence is
 * re-seeded from Q when reset != 0 */
int qmin_nesterov_run(qmin_handle h, double dt, double mu, double force_cutoff, int max_iterations, int reset,
                      int *iterations, double *force_max);
/* energyMinimizerLoLBFGS::setLoLBFGSParameters + minimize
 * (energyMinimizerLoLBFGS.h:29-44, .cpp:195-226); history reset when reset != 0.
 * Each iteration starts its two-loop recursion from the resident forces (the
 * reference's unscaledStep, which equals them after every iteration), so a
 * call with reset = 0 after the state or forces were changed by another call
 * continues from the forces now resident.  *iterations and *force_max are
 * written before QMIN_ENONFINITE is returned. */
int qmin_lbfgs_run(qmin_handle h, int m, double eta, double force_cutoff, int max_iterations, int reset,
                   int *iterations, double *force_max);

/* energyMinimizerGradientDescent::setGradientDescentParameters + minimize
 * (energyMinimizerGradientDescent.cpp:64-115): Q += dt F, forces at the new Q,
 * forceMax = sqrt(sum F.F) / nTotal; at least one iteration; the iteration
 * count restarts from 0 when reset != 0 (class defaults: dt 0.01, cutoff 1e-7) */
int qmin_gd_run(qmin_handle h, double dt, double force_cutoff, int max_iterations, int reset, int *iterations,
                double *force_max);

/* ---- FIRE iteration strategy and diagnostics ---- */
#define QMIN_FIRE_SEPARATE 0 /* predictor, derivative planes, force+kick, control as separate kernels */
#define QMIN_FIRE_FUSED 1    /* one shared-memory tiled kernel per iteration */
#define QMIN_FIRE_AUTO 2     /* the autotuner picks the fastest (default): of the split and separate
                                strategies where the split path applies, of all the others elsewhere */
#define QMIN_FIRE_TILED 3    /* separate predictor and derivative planes, force + kick from shared-memory
                                tiles (FP32 form only) */
#define QMIN_FIRE_SPLIT 4    /* deep bulk sites' force + kick over Q on the 25-point stencil (no derivative
                                planes), the sites near objects through the plane forms (multi-constant
                                form without L6; otherwise the separate kernels run) */
/* Choose how qmin_fire_run executes an iteration; all strategies give the
 * same results to rounding.  No reference counterpart (execution strategy). */
int qmin_set_fire_kernel(qmin_handle h, int mode);
/* Run `iterations` FIRE iterations with direct (non-graph) launches and CUDA
 * events around every kernel; kernel_ms receives the average device time per
 * launch of [0] predictor, [1] first-derivative planes, [2] force + half kick
 * + reductions (for the fused kernel: the whole fused iteration), [3] FIRE
 * scalar control; *fused (may be NULL) tells which path ran.  The FIRE state
 * advances exactly as in qmin_fire_run.  No reference counterpart (profiling). */
int qmin_fire_profile(qmin_handle h, int iterations, double kernel_ms[4], int *fused);
/* (kernel_ms[2] is the staged force + kick when path 2 runs; *fused is 1 only for path 1) */
/* Pin one variant of the strategy chosen with qmin_set_fire_kernel (its index
 * among that strategy's candidates in qmin_fire_tuning's ms[]: 0-2 separate,
 * 0-3 fused, 0-2 staged, 0-11 split with 4-6 and 10-11 FP32 only), or -1 to let the autotuner pick (the
 * default; qmin_set_fire_kernel resets it).  QMIN_EINVAL for an index the
 * strategy does not have or when no strategy is pinned.  No reference
 * counterpart (execution strategy). */
int qmin_set_fire_variant(qmin_handle h, int variant);
/* The FIRE strategy the autotuner chose on the first run (path 0 separate
 * kernels sized for `variant` + 1 blocks per SM; path 1 fused kernel and
 * path 2 staged force + kick, each with tile shape `variant` = tile_x x tile_y
 * and `zc` z planes per block; path 3 split force + kick with deep-site
 * kernel `variant`, as in ms[17 + v] below) and the measured ms per
 * iteration of every candidate: ms[0..2] separate (1, 2, 3 blocks per SM),
 * ms[3 + 2*cfg + v] fused (4 shapes, v = 0/1 for the two z extents tried),
 * ms[11 + 2*cfg + v] staged (3 shapes), ms[17 + v] split (v = 0, 1: deep
 * sites from global memory at 1 or 2 blocks per SM; v = 2, 3: deep sites
 * from shared-memory tiles of 32 x 8 or 16 x 16 sites; v = 4, 5, FP32
 * only: two x-adjacent sites per thread on 32 x 8 tiles, z chunks of 8
 * planes or long enough that the grid is about two waves; v = 6, FP32 only:
 * as 5 with the interior tiles' planes staged by TMA, offered when the x
 * extent is a multiple of 4 and at least 40; v = 7 .. 11: the predictor
 * fused into the deep-site kernel, which reads one of two state buffer sets
 * and writes the other, staging raw Q, V, F of each plane with a one-site
 * halo: raw planes prefetched into registers one plane ahead on 32 x 8 tiles
 * with z chunks of 16 planes (7) or about two waves (8), on 32 x 4 tiles
 * (9), or copied into shared memory cooperatively by 16-byte row chunks two
 * planes ahead on 32 x 8 (10) or 32 x 4 (11) tiles, FP32 with an x extent
 * that is a multiple of 4; the listed sites form their predicted Q on the
 * fly); -1 = not run.
 * No reference counterpart (the reference's kernelTuner scans block sizes,
 * src/utilities/kernelTuner.cpp:5-125). */
#define QMIN_TUNE_CANDIDATES 29
/* The autotuner's choices are kept for the life of the process: a handle whose
 * problem the process has already tuned (same sides, precision, metric, force
 * form, field terms, strategy request and site-class counts) takes the stored
 * choice on its first run instead of timing the candidates again.  This call
 * forgets every stored choice (the next first run of each problem tunes
 * afresh).  No reference counterpart (execution strategy). */
int qmin_tuning_cache_clear(void);
int qmin_fire_tuning(qmin_handle h, int *path, int *variant, int *tile_x, int *tile_y, int *zc,
                     double ms[QMIN_TUNE_CANDIDATES]);

/* ---- energy without allocation ---- */
/* Largest lattice (in sites) qmin_energy_noalloc accepts: the size of its
 * static reduction scratch (one block of 256 sites per partial sum). */
#define QMIN_NOALLOC_MAX_SITES 8388608

/* Energy of a Q field held in the caller's own device memory, for callers
 * that cannot call cudaMalloc (their device memory is owned by a pool
 * allocator of their own, or is fully committed).  Allocates nothing: its
 * scratch is a static device array of about 1.6 MB inside this library.  FP64 only.
 *   Q_dev:       device, SoA double planes Q_dev[k * plane_stride + i], k = 0..4
 *   types_dev:   device, int8 site types (same meaning as qmin_set_state's);
 *                an object type j must satisfy j <= nobj: a site next to an
 *                object past nobj makes the anchoring energy and E NaN
 *   out_dev:     device, 6 doubles: E / NActive, then the phase, distortion,
 *                anchoring, E-field and H-field totals (as qmin_energy)
 *   objs:        host array of nobj objects; stream: cudaStream_t or NULL
 * Results match qmin_energy on the same state.  Returns QMIN_EINVAL for a
 * lattice larger than QMIN_NOALLOC_MAX_SITES sites.
 * CUDA loads this library's device code and the scratch array lazily by
 * default, so the first call on a device is what places them there (they stay
 * until the process exits): a caller that later commits all of its device
 * memory makes one call on each device before doing so (any small lattice),
 * or runs with CUDA_MODULE_LOADING=EAGER.  That first call also looks up the
 * scratch address; make it before any stream capture.
 * All calls share the scratch: calls that overlap on the GPU race, so
 * serialise them.  The result is ready when the stream reaches it.
 * No counterpart in the reference (an addition for allocation-free callers). */
int qmin_energy_noalloc(const qmin_lattice_desc *desc, const qmin_ldg_params *p, const qmin_object *objs, int nobj,
                        const double *Q_dev, long long plane_stride, const int8_t *types_dev, double *out_dev,
                        void *stream);

/* ---- batched solves (many independent lattices of uneven sizes) ---- */
/* A batch packs nsolves (at most 16384) independent lattices (dims[3*s ..
 * 3*s+2] = Lx, Ly, Lz) into one device state and minimises them together:
 * each solve follows energyMinimizerFIRE::minimize on its own lattice (its own
 * FIRE scalars, stopping rule and iteration count), converged solves retire.
 * qmin_batch_fire_run runs all iterations of all solves in one persistent
 * cooperative launch (grid barriers between the phases of an iteration; FP32
 * one-constant batches run the predictor, force and kick as one phase over two
 * state sets, and the device memory for the second set is allocated on their
 * first run).  All
 * solves share the force parameters; each has up to 16 objects.  No reference
 * counterpart for the batching itself (the reference minimises one lattice per
 * process). */
typedef struct qmin_batch_ctx *qmin_batch;
int qmin_batch_create(int nsolves, const int32_t *dims, int precision, int metric_mode, qmin_batch *out);
int qmin_batch_destroy(qmin_batch b);
int qmin_batch_set_params(qmin_batch b, const qmin_ldg_params *p);
/* state of solve s: AoS Q, int32 types (objects numbered 1..nobj within the solve) */
int qmin_batch_set_solve(qmin_batch b, int s, const double *Q, const int32_t *types, const qmin_object *objs,
                         int nobj);
/* read back solve s's Q and/or forces (AoS, either pointer may be NULL) */
int qmin_batch_get_solve(qmin_batch b, int s, double *Q, double *F);
/* FIRE parameters for every solve (energyMinimizerFIRE::setFIREParameters) */
int qmin_batch_fire_init(qmin_batch b, const qmin_fire_params *p);
/* minimise every solve; per-solve iteration counts and forceMax (arrays of
 * nsolves, may be NULL) and the number of solves with forceMax <= cutoff.
 * QMIN_ETIMEOUT when a grid barrier of the persistent loop waited longer than
 * its limit (qmin_batch_set_barrier_limit): every solve still running then
 * has QMIN_ETIMEOUT in its status and stops, with the state of an unfinished
 * iteration; set those solves again before the next run. */
int qmin_batch_fire_run(qmin_batch b, int max_iterations, int *iterations, double *force_max, int *converged);
/* polls a block makes at one grid barrier before the run gives up (0: the
 * default, about a second).  No reference counterpart. */
int qmin_batch_set_barrier_limit(qmin_batch b, long long spins);
/* the chunk shape the tuner chose (-1 before the first run; 0: 256
 * consecutive sites, 1-4: tiles of 32x8x1, 16x16x1, 16x4x4, 8x8x4 sites, as
 * tile[3]) and the force + kick time of each shape in ms (-1: not timed).
 * No reference counterpart (execution strategy). */
int qmin_batch_tuning(qmin_batch b, int *shape, int tile[3], double ms[5]);
/* pin the chunk shape (0-4 as in qmin_batch_tuning) or hand it back to the
 * tuner (-1, the default); takes effect at the next run.  Every shape gives
 * the same results to rounding.  No reference counterpart. */
int qmin_batch_set_chunk_shape(qmin_batch b, int shape);
int qmin_batch_kernel_launches(qmin_batch b, long long *count);

/* ---- learned warm start ----
 * A 3-D U-Net (4 levels, 32-128 channels, about 0.57M parameters; BF16
 * weights and activations, FP32 accumulation on the tensor cores) that maps a
 * lattice's initial Q, object/boundary masks and anchoring kind/strength to a
 * near-minimal Q, which a minimiser then finishes.  One net object serves
 * `batch` lattices of Lx x Ly x Lz sites (each side a multiple of 8).  Input
 * features: [batch][sites][16] BF16; output: [batch][sites][16] FP32 whose
 * channels 0..4 are the predicted Q (AoS per site).  No reference
 * counterpart: the reference has no learned component. */
typedef struct qmin_warmnet_ctx *qmin_warmnet;
/* train = 0 allocates only what inference needs */
int qmin_warmnet_create(int batch, int Lx, int Ly, int Lz, int train, qmin_warmnet *out);
int qmin_warmnet_destroy(qmin_warmnet n);
/* run on a caller's cudaStream_t (NULL = legacy default stream) */
int qmin_warmnet_set_stream(qmin_warmnet n, void *stream);
int qmin_warmnet_param_count(qmin_warmnet n, long long *count);
int qmin_warmnet_shape(qmin_warmnet n, int *batch, int *Lx, int *Ly, int *Lz);
/* the net's device buffers: input features, output, training mask */
int qmin_warmnet_buffers(qmin_warmnet n, void **x, float **y, uint8_t **mask);
/* FP32 parameters (host, param_count floats); resets the Adam moments */
int qmin_warmnet_set_params(qmin_warmnet n, const float *host);
/* FP32 parameters and/or the last backward's gradients (host, may be NULL) */
int qmin_warmnet_get_params(qmin_warmnet n, float *params, float *grads);
/* build sample `sample`'s input features from a lattice's device state:
 * Q_dev SoA planes (QMIN_FP64 or QMIN_FP32, stride plane_stride), int8 types
 * (qmin_set_state's meaning), host objects (at most 64) */
int qmin_warmnet_features(qmin_warmnet n, int sample, const void *Q_dev, int precision, long long plane_stride,
                          const int8_t *types_dev, const qmin_object *objs, int nobj);
int qmin_warmnet_forward(qmin_warmnet n);
/* masked mean-squared error of output channels 0..4 against target_dev
 * ([batch][sites][5] FP32, device) over the sites with type <= 0, and the
 * gradient of every parameter (overwritten, not accumulated); *loss (host,
 * may be NULL) waits for the result */
int qmin_warmnet_backward(qmin_warmnet n, const float *target_dev, double *loss);
/* one Adam step on the FP32 master parameters (bias-corrected) */
int qmin_warmnet_adam_step(qmin_warmnet n, double lr, double beta1, double beta2, double eps);
/* write sample `sample`'s predicted Q into SoA planes on the sites with
 * type <= 0 (object sites keep their imposed Q) */
int qmin_warmnet_write_state(qmin_warmnet n, int sample, void *Q_dev, int precision, long long plane_stride,
                             const int8_t *types_dev);
int qmin_warmnet_sync(qmin_warmnet n);
/* Tensor-core instruction family of the convolutions: 1 (default) the
 * 5th-generation tcgen05.mma with tensor-memory accumulators, the direct 3^3
 * kernel's halo planes staged by TMA (cp.async.bulk.tensor) where the grid
 * holds a 10 x 18 box; 2 the same with the halo planes staged by the threads;
 * 0 the mma.sync kernels.  All compute BF16 x BF16 -> FP32; paths 1 and 2 give
 * identical bits.  QMIN_EINVAL for another value.  No reference counterpart. */
int qmin_warmnet_set_tensor_path(qmin_warmnet n, int path);
/* Polls of the library's TMA waits before a kernel gives up: the TMA direct
 * convolution's waits for its copies and MMAs (the pass's outputs are then
 * void and qmin_warmnet_sync returns QMIN_ETIMEOUT) and the TMA-staged
 * deep-site FIRE kernel's waits for its next planes (qmin_fire_run returns
 * QMIN_ETIMEOUT and the lattice's state is void).  0 makes every such wait
 * give up at once (a pass then fails at its first wait: the reporting path,
 * for tests), a negative value restores the defaults (about a second).
 * Process-wide: it applies to every net and handle.  The waits that let the
 * copies and MMAs in flight land before a CTA that gave up exits always use
 * the default.  No reference counterpart. */
int qmin_set_wait_limit(long long polls);
int qmin_warmnet_kernel_launches(qmin_warmnet n, long long *count);
/* Warm-start a lattice in place: features from its current Q, types and
 * objects, one forward pass, the prediction written into its Q on the sites
 * the minimiser moves.  The net must have batch 1 and the lattice's sides.
 * Call qmin_fire_init (or another minimiser) afterwards. */
int qmin_warm_start(qmin_handle h, qmin_warmnet n);

/* ---- host-side set-up helpers (the reference runs these on the host even
 *      in GPU runs, openQmin.cpp:261-268) ---- */
/* qTensorLatticeModel::setNematicQTensorRandomly (qTensorLatticeModel.cpp:134-162)
 * with noiseSource::setReproducibleSeed(seed): Q is AoS double[N][5] */
int qmin_host_random_nematic(int Lx, int Ly, int Lz, int seed, double S0, double *Q);
/* multirankSimulation::createWall (multirankSimulationBoundaries.cpp:101-167);
 * *nobj is the number of objects so far and is incremented; objs has room
 * for at least *nobj + 1 entries */
int qmin_host_add_wall(int Lx, int Ly, int Lz, int xyz, int plane, int kind, double W, double S0, double *Q,
                       int32_t *types, qmin_object *objs, int *nobj);
/* multirankSimulation::createSphericalColloid (multirankSimulationBoundaries.cpp:169-215) */
int qmin_host_add_sphere(int Lx, int Ly, int Lz, const double center[3], double radius, int kind, double W,
                         double S0, double *Q, int32_t *types, qmin_object *objs, int *nobj);

/* multirankSimulation::createBoundaryFromFile (multirankSimulationBoundaries.cpp:7-96),
 * single rank: reads a boundary file (first line the object count; per object
 * a line "kind W S0 n" with kind 0 oriented / 1 degenerate planar, then n
 * lines "x y z C1 C2 C3 C4 C5") and adds each object as qmin_host_add_wall
 * does (sites wrapped periodically, their Q set to C1..C5, neighbours marked
 * -1).  objs has room for max_objs entries; *nobj is updated.  QMIN_EINVAL on
 * a missing file or a malformed line. */
int qmin_host_boundary_file(int Lx, int Ly, int Lz, const char *path, double *Q, int32_t *types, qmin_object *objs,
                            int max_objs, int *nobj);

#ifdef __cplusplus
}
#endif
#endif
