// Internal declarations shared by the qmin_gb300 translation units.
#pragma once
#include <cuda.h>  // CUtensorMap (the type only; the encoder is fetched from the driver at run time)
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/qmin_gb300.h"
#include "qmin_bulk_forms.h"
#include "qmin_bulk_q25.h"
#include "qmin_boundary_forms.h"

namespace qmin {

// Object table entry on the device (boundaryObject, latticeBoundaries.h:20-39).
template <class T> struct ObjDev {
    int kind;
    T W, S0;
};

// split force + kick (multi-constant, no L6): site classes (0 deep bulk, 1 other
// LC site, 2 object), the class-1 sites, and the sites whose derivative planes
// the class-1 forms read
struct SplitLists {
    const uint8_t *cls;
    const int *sites;
    int n_sites;
    const int *derivs;
    int n_derivs;
    const CUtensorMap *tmap_q;  // host copy of the FP32 Q planes' tensor map (interior tiles by TMA), or null
    int *err;                   // device word set when a TMA wait gives up
};

// Everything a lattice kernel needs, passed by value.  Planes are SoA:
// component k of site i lives at X[k * P + i]; P = N rounded up to 32.
template <class T> struct Lat {
    int Lx, Ly, Lz, N;
    long long P;
    T *Q, *V, *F;
    const int8_t *types;
    T *D;  // 15 derivative planes (multi-constant only)
    const ObjDev<T> *objs;
    T a, b, c;          // A/2, B/3, C/4
    T L1, L2, L3, L4, L6;
    T fE[5], fH[5];     // uniform-field force vectors (subtracted, as the reference does)
    const T *Hv;        // spatially varying H field, 3 planes of stride P, or null
    T hvp;              // its dchi * mu0
    int metric_mode, multi, efield, hfield;
    T cb[5 * QMIN_BULK_W];  // combined bulk multi-constant coefficients
    T cq[5 * QMIN_Q25_W];   // the same form over Q on the 25-point stencil (deep bulk sites;
                            // without L4 over shared sums of stencil values)
    T cqp[sizeof(T) == 4 ? 5 * QMIN_Q25_W : 1];  // FP32: the 25-point form term by term
    const T *cbd;           // merged boundary L2-L4 coefficients [27][5][QMIN_BND_W] in device memory, or null
    SplitLists split;       // deep / listed site classes and lists (all null when not built)
};

// force parameters shared by every kernel (qmin_capi.cu)
template <class T> void fill_lat_params(Lat<T> &L, const qmin_ldg_params &p, int metric_mode);
// the merged boundary coefficients for one parameter set, [27][5][QMIN_BND_W] (qmin_capi.cu)
template <class T> void fill_boundary_coeffs(const qmin_ldg_params &p, T *out);

// FIRE state resident on the device.  The velocity mix that ends one
// iteration is deferred into the next iteration's first kernel.
struct FireDev {
    double alpha, dt, alpha0, dtmax, dtmin, dtinc, dtdec, alphadec, alphamin, fcut;
    double power, forceMax, scaling, mixA, mixS;
    int nmin, nsince, iterations, max_iters, active, pending, reset, status;
    long long nTotal;
};

// Scalar state for Adam / Nesterov / L-BFGS loops resident on the device.
struct IterDev {
    double forceMax, fcut, b1t, b2t;
    int iterations, max_iters, active, status;
    long long ndof;
    double lb[64];  // L-BFGS scalars: sy[0..m), alpha[0..m), scratch
};

constexpr int kBlock = 256;

// message behind the last non-zero status returned on this host thread
extern thread_local std::string g_last_error;

// launchers (qmin_kernels.cu); each returns the number of kernels launched
template <class T> int launch_derivs(const Lat<T> &L, cudaStream_t s);
// forces at Q: the split kernels (deep sites over Q, listed sites through the
// plane forms) where L.split is built and the form is multi-constant without
// L6, else the derivative planes and the full-lattice force kernel
template <class T> int launch_force(const Lat<T> &L, int grid, cudaStream_t s);
template <class T> int launch_split_force(const Lat<T> &L, int grid, cudaStream_t s);
template <class T> int launch_fire_pred(const Lat<T> &L, FireDev *fd, cudaStream_t s);
template <class T>
int launch_force_kick(const Lat<T> &L, FireDev *fd, double *partials, int grid, cudaStream_t s, int cap);
template <class T>
int launch_force_kick_only(const Lat<T> &L, FireDev *fd, double *partials, int grid, cudaStream_t s, int cap);
int launch_fire_control(FireDev *fd, const double *partials, int nparts, cudaStream_t s);
template <class T> int launch_fire_finish(const Lat<T> &L, FireDev *fd, cudaStream_t s);
template <class T>
int launch_energy_full(const Lat<T> &L, double *partials, int grid, double *out5, const double *E, double eps,
                       double eps0, double deps, const double *H, double chi, double mu0, double dchi, cudaStream_t s);
template <class T> int launch_aos_to_soa(const double *aos, T *soa, int N, long long P, int layout, cudaStream_t s);
template <class T> int launch_soa_to_aos(const T *soa, double *aos, int N, long long P, int layout, cudaStream_t s);
int launch_types_to_i8(const int32_t *t32, int8_t *t8, int N, cudaStream_t s);
template <class T> int launch_fill(T *x, T v, long long n, cudaStream_t s);

// Adam / Nesterov / L-BFGS
template <class T>
int launch_adam_step(const Lat<T> &L, T *M, T *S, IterDev *it, double beta1, double beta2, double eps, double dt,
                     double *partials, int grid, cudaStream_t s);
template <class T>
int launch_nesterov_step(const Lat<T> &L, T *alt, IterDev *it, double dt, double mu, double *partials, int grid,
                         cudaStream_t s);
template <class T> int launch_defects(const Lat<T> &L, int kind, double *out, cudaStream_t s);
template <class T>
int launch_object_forces(const Lat<T> &L, int nobj, const double *E, double eps, double eps0, double deps,
                         const double *H, double chi, double mu0, double dchi, double *partials, int grid,
                         double *out, cudaStream_t s);
template <class T> int launch_gd_move(const Lat<T> &L, IterDev *it, double dt, cudaStream_t s);
template <class T> int launch_ff_dot(const Lat<T> &L, IterDev *it, double *partials, int grid, cudaStream_t s);
int launch_norm_control(IterDev *it, const double *partials, int nparts, int adam, double beta1, double beta2,
                        cudaStream_t s);
// one L-BFGS iteration; p enters as L.F (the forces at Q), so the forces
// must be current when the first iteration starts
template <class T>
int launch_lbfgs_iteration(const Lat<T> &L, T *p, T *sbase, T *ybase, IterDev *it, int m, double eta,
                           double *partials, int grid, cudaStream_t s);

int reduction_grid(int N);

// fused tiled FIRE iteration (qmin_fused.cu): tile configuration cfg in
// [0, kFusedConfigs), z planes per block zc; returns launches or -1
constexpr int kFusedConfigs = 4;
constexpr int kMaxFusedBlocks = 16384;
template <class T>
int launch_fire_fused(int cfg, const Lat<T> &L, T *Qn, T *Vn, T *Fn, FireDev *fd, double *partials, int zc,
                      cudaStream_t s, int *nblocks);
int fused_tile_shape(int cfg, int *tx, int *ty);
// force + second half kick from shared-memory tiles (FP32 form): tile shape
// cfg in [0, kTiledConfigs), zc z planes per block, *nblocks partial sums;
// returns launches or -1 (FP64, or the shape could not be configured)
constexpr int kTiledConfigs = 3;
template <class T>
int launch_force_kick_tiled(int cfg, const Lat<T> &L, FireDev *fd, double *partials, int zc, cudaStream_t s,
                            int *nblocks);
int tiled_tile_shape(int cfg, int *tx, int *ty);

template <class T> int launch_split_derivs(const Lat<T> &L, const SplitLists &sl, FireDev *fd, cudaStream_t s);
// partials: the deep kernel's grid blocks, then the list kernel's; *nparts their total
template <class T>
int launch_split_force_kick(const Lat<T> &L, const SplitLists &sl, FireDev *fd, double *partials, int grid, int cap,
                            cudaStream_t s, int *nparts);
// the two halves separately: the deep-site kernel `cap` (returns its block
// count, partials[0 .. 3 count)) and the listed sites (returns its block count,
// 0 without listed sites); they touch disjoint sites and may run concurrently
template <class T>
int launch_split_deep(const Lat<T> &L, const SplitLists &sl, FireDev *fd, double *partials, int grid, int cap,
                      cudaStream_t s);
// fused split iteration (predictor inside): the deep sites from the input set
// Lin into the output set (Qo, Vo, Fo; returns the block count, -1 for an
// unknown variant), and the listed sites (derivative planes of the predicted
// Q, force + kick into Vo, Fo; returns the launch count, *nblocks its partials)
// site types on the device (qmin_geometry.cu): min, max, count of types <= 0 and
// count of sites that differ from old8 (when given) into out_host[0..3] (the
// call synchronises the stream; part: 4 * 608 ints, out_dev: 4 ints)
template <class TT>
int scan_types(const TT *t, const int8_t *old8, int N, int *part, int *out_dev, int *out_host, cudaStream_t s);
// the split path's classes and lists from the device types (qmin_geometry.cu):
// cls (N bytes) written, *sites / *derivs grown as needed, host_totals: 29 ints;
// scratch of split_scratch_bytes(N).  Returns the launch count, < 0 on failure.
size_t split_scratch_bytes(int N);
int build_split_lists_dev(const int8_t *t8, int Lx, int Ly, int Lz, uint8_t *cls, void *scratch, int *host_totals,
                          int **sites, int *sites_cap, int *n_sites, int **derivs, int *derivs_cap, int *n_derivs,
                          cudaStream_t s);
template <class T>
int launch_split_fused_deep(const Lat<T> &Lin, T *Qo, T *Vo, T *Fo, const SplitLists &sl, FireDev *fd,
                            double *partials, int variant, cudaStream_t s);
template <class T>
int launch_split_fused_list(const Lat<T> &Lin, T *Vo, T *Fo, const SplitLists &sl, FireDev *fd, double *partials,
                            cudaStream_t s, int *nblocks);
template <class T>
int launch_split_list(const Lat<T> &L, const SplitLists &sl, FireDev *fd, double *partials, cudaStream_t s);
// polls of the TMA deep-site kernel's waits for its next planes before a block
// gives up (the waits that let boxes in flight land always use the default)
constexpr int kSplitWaitPolls = 1 << 22;
cudaError_t split_set_wait_limit(int polls);

}  // namespace qmin
