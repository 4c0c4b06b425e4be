// qmin_gb300 C ABI: handle lifetime, state transfer, force/energy and the
// minimiser drivers.  Minimiser loops run as captured CUDA graphs of a fixed
// chunk of iterations; the loop condition lives on the device (every kernel of
// an iteration returns at once when the minimiser is no longer active), and
// the host reads it back once per chunk.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "../../include/qmin_gb300.h"
#include "qmin_bulk_forms.h"
#include "qmin_internal.h"

using namespace qmin;

namespace qmin {
thread_local std::string g_last_error;
}

static int fail(int code, const std::string &msg)
{
    qmin::g_last_error = msg;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(QMIN_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

static const int kSepVariants = 3;  // separate-kernel force + kick with 1, 2, 3 blocks per SM
// deep-site kernel: 1 or 2 blocks per SM, shared-memory 32x8 or 16x16, and
// (FP32 only) two sites per thread on 32x8 tiles, z chunks of 8 planes or about
// two waves of columns, the latter also with TMA staging of interior tiles
static const int kSplitVariants = 12;
static const int kSplitTma = 6;
static const int kSplitFp32First = 4;
// variants 7-11: the predictor fused into the deep-site kernel (ping-pong state
// sets, the listed sites' predicted Q formed on the fly), both precisions
static const int kSplitFusedFirst = 7;
static bool split_fused(int cap) { return cap >= kSplitFusedFirst; }
static const int kTuneCandidates = kSepVariants + 2 * kFusedConfigs + 2 * kTiledConfigs + kSplitVariants;
static_assert(kTuneCandidates == QMIN_TUNE_CANDIDATES, "tuning candidate count");

struct qmin_ctx {
    int Lx = 0, Ly = 0, Lz = 0, N = 0;
    long long P = 0;
    int prec = QMIN_FP64, metric_mode = QMIN_METRIC_CPU;
    size_t esz = 8;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // FP32 Q planes as a TMA tensor map (interior tiles of the split path), built on first use
    CUtensorMap tmap_q;
    bool tmap_tried = false, tmap_ok = false;
    int *dev_err = nullptr;  // set by a kernel whose bounded TMA wait gave up
    // side stream (highest priority) and fork/join events for the listed sites of the split path
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    void *Q = nullptr, *V = nullptr, *F = nullptr, *D = nullptr;
    void *cbd = nullptr;  // merged boundary coefficients (multi-constant)
    int8_t *types = nullptr;
    void *objs = nullptr;
    int nobj = 0;
    std::vector<qmin_object> objs_host;
    // site-type scan and split-list building on the device (qmin_geometry.cu)
    void *geo_scratch = nullptr;
    size_t geo_scratch_bytes = 0;
    int *scan_part = nullptr, *scan_out = nullptr;
    double *partials = nullptr;
    int grid = 1;
    double *stage = nullptr;
    int32_t *stage_t = nullptr;
    FireDev *fire = nullptr;
    FireDev *fire_h = nullptr;  // pinned mirror
    IterDev *iter = nullptr;
    IterDev *iter_h = nullptr;  // pinned mirror
    double *out5 = nullptr;
    double *out5_h = nullptr;
    void *M = nullptr, *S = nullptr, *alt = nullptr, *lbp = nullptr, *lbs = nullptr, *lby = nullptr;
    int lb_m = 0;
    qmin_ldg_params params{};
    bool have_params = false, have_state = false, fire_ready = false;
    int max_type = 0;
    long long nTotal = 0;
    long long launches = 0;
    // cached chunk graphs: 0 FIRE, 1 Adam, 2 Nesterov, 3 L-BFGS, 4 gradient descent
    cudaGraphExec_t graph[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int graph_per_iter[5] = {0, 0, 0, 0, 0};
    int graph_key[5] = {0, 0, 0, 0, 0};
    double graph_args[5][4] = {};  // scalar kernel arguments baked into each graph
    int version = 1;  // bumped whenever kernel arguments change
    // fused tiled FIRE path: second state buffer set (ping-pong) and the tile
    // configuration chosen by the autotuner for the current parameters
    void *Q2 = nullptr, *V2 = nullptr, *F2 = nullptr;
    void *hvar = nullptr;  // spatially varying H field (3 planes), active when hvar_on
    bool hvar_on = false;
    int fire_mode = QMIN_FIRE_AUTO;  // strategy requested by the caller
    int fire_variant = -1;           // variant of that strategy the caller pinned (-1: the tuner picks)
    int tuned_variant = -1;
    // strategy chosen by the autotuner for the current parameters
    int path = -1;  // 0 separate kernels, 1 fused tiled kernel, 2 separate with the staged force + kick
    int sep_cap = 0, fused_cfg = -1, fused_zc = 0, fused_nblocks = 0, tuned_version = 0, tuned_mode = -1;
    int tiled_cfg = -1, tiled_zc = 0, tiled_nblocks = 0;
    int split_cap = 0;  // path 3: register cap of the deep-site kernel
    // split path: site classes (0 deep bulk, 1 other LC, 2 object), the class-1
    // sites and the sites whose derivative planes they read
    uint8_t *split_cls = nullptr;
    int *split_sites = nullptr, *split_derivs = nullptr;
    int n_split_sites = 0, n_split_derivs = 0, split_sites_cap = 0, split_derivs_cap = 0;
    // separate (register caps), fused (cfg, z extent), staged force + kick (cfg, z extent)
    double tune_ms[kTuneCandidates] = {};
};

// whether this handle can run split variant cap: 4-6 FP32 only (6 also needs the
// tensor map), 7-11 need 32-bit component offsets (5 P < 2^31), 10-11 FP32 with
// an x extent that is a multiple of 4
static bool split_variant_ok(const qmin_ctx *h, int cap)
{
    if (cap >= kSplitFp32First && !split_fused(cap) && h->prec != QMIN_FP32) return false;
    if (split_fused(cap) && 5LL * h->P >= (1LL << 31)) return false;
    if (cap >= kSplitFusedFirst + 3 && (h->prec != QMIN_FP32 || h->Lx % 4 != 0)) return false;
    return true;
}

static const int kChunk = 32;  // iterations per captured graph

namespace qmin {
// Force parameters shared by every kernel: phase constants as the force uses
// them, elastic constants, field force vectors and the combined bulk linear
// form's coefficients.
template <class T> void fill_lat_params(Lat<T> &L, const qmin_ldg_params &p, int metric_mode)
{
    L.a = T(0.5 * p.A);
    L.b = T(p.B / 3.0);
    L.c = T(0.25 * p.C);
    L.L1 = T(p.L1);
    L.L2 = T(p.L2);
    L.L3 = T(p.L3);
    L.L4 = T(p.L4);
    L.L6 = T(p.L6);
    // uniform-field force vectors (landauDeGennesLCOtherForces.cpp:297-303)
    auto field = [](const double *fld, double aniso, double perm, T *out) {
        double pr = aniso * perm;
        out[0] = T(-0.5 * pr * (fld[0] * fld[0] - fld[2] * fld[2]));
        out[1] = T(-pr * fld[0] * fld[1]);
        out[2] = T(-pr * fld[0] * fld[2]);
        out[3] = T(-0.5 * pr * (fld[1] * fld[1] - fld[2] * fld[2]));
        out[4] = T(-pr * fld[1] * fld[2]);
    };
    if (p.efield) field(p.E, p.deps, p.eps0, L.fE);
    if (p.hfield) field(p.H, p.dchi, p.mu0, L.fH);
    L.metric_mode = metric_mode;
    L.multi = p.multi_constant;
    L.efield = p.efield;
    L.hfield = p.hfield;
    const double Lt[4] = {p.L2, p.L3, p.L4, p.L1};
    for (int k = 0; k < 5; ++k)
        for (int n = 0; n < QMIN_BULK_W; ++n) {
            double c = 0.0;
            if (n < qmin_bulk_n[k]) {
                // k L / 4 per input; halved for derivative inputs (index >= 35), which
                // the accessors deliver as twice the derivative
                const double unit = qmin_bulk_in[k][n] >= 35 ? 0.125 : 0.25;
                for (int t = 0; t < 4; ++t) c += Lt[t] * (double)qmin_bulk_k[t][k][n] * unit;
            }
            L.cb[k * QMIN_BULK_W + n] = T(c);
        }
    // the kernels take the shared-sum form (its own coefficient layout) when L4
    // is zero in the site precision; FP32 keeps the term-by-term form beside it
    const auto &q25k = L.L4 == T(0) ? qmin_q25c_k : qmin_q25_k;
    for (int k = 0; k < 5; ++k)
        for (int n = 0; n < QMIN_Q25_W; ++n) {
            double c = 0.0, cp = 0.0;  // k L / 8 per stencil value or shared sum
            for (int t = 0; t < 4; ++t) {
                c += Lt[t] * (double)q25k[t][k][n] * 0.125;
                cp += Lt[t] * (double)qmin_q25_k[t][k][n] * 0.125;
            }
            L.cq[k * QMIN_Q25_W + n] = T(c);
            if constexpr (sizeof(T) == 4) L.cqp[k * QMIN_Q25_W + n] = T(cp);
        }
}
template void fill_lat_params<double>(Lat<double> &, const qmin_ldg_params &, int);
template void fill_lat_params<float>(Lat<float> &, const qmin_ldg_params &, int);

// k L / 4 per input of the merged boundary forms; halved for derivative inputs
template <class T> void fill_boundary_coeffs(const qmin_ldg_params &p, T *out)
{
    const double Lt[3] = {p.L2, p.L3, p.L4};
    for (int n = 0; n < QMIN_BND_CASES; ++n)
        for (int k = 0; k < 5; ++k)
            for (int m = 0; m < QMIN_BND_W; ++m) {
                double c = 0.0;
                for (int t = 0; t < 3; ++t) c += Lt[t] * (double)qmin_bnd_k[n][k][m][t];
                out[(n * 5 + k) * QMIN_BND_W + m] = T(c * (qmin_bnd_dn[n][k][m] ? 0.125 : 0.25));
            }
}
template void fill_boundary_coeffs<double>(const qmin_ldg_params &, double *);
template void fill_boundary_coeffs<float>(const qmin_ldg_params &, float *);
}  // namespace qmin

// The FP32 Q planes as a 4-D tensor map (x, y, z, component) for the TMA-staged
// deep kernel: boxes of 40 x 12 x 1 x 5 floats.  Needs x extent % 4 == 0 (the
// row pitch must be a multiple of 16 bytes) and a lattice that has interior
// tiles; the encoder comes from the driver (no link-time dependency).
static bool ensure_tmap(qmin_ctx *h)
{
    if (h->tmap_tried) return h->tmap_ok;
    h->tmap_tried = true;
    h->tmap_ok = false;
    if (h->prec != QMIN_FP32 || h->Lx % 4 != 0 || h->Lx < 40 || h->Ly < 12) return false;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return false;
    }
    if (!h->dev_err) {
        if (cudaMalloc(&h->dev_err, sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            h->dev_err = nullptr;
            return false;
        }
        cudaMemset(h->dev_err, 0, sizeof(int));
    }
    auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    const cuuint64_t dims[4] = {(cuuint64_t)h->Lx, (cuuint64_t)h->Ly, (cuuint64_t)h->Lz, 5};
    const cuuint64_t strides[3] = {(cuuint64_t)h->Lx * 4, (cuuint64_t)h->Lx * h->Ly * 4, (cuuint64_t)h->P * 4};
    const cuuint32_t box[4] = {40, 12, 1, 5};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = encode(&h->tmap_q, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->Q, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    h->tmap_ok = r == CUDA_SUCCESS;
    return h->tmap_ok;
}

template <class T> static Lat<T> make_lat(qmin_ctx *h)
{
    Lat<T> L;
    memset(&L, 0, sizeof L);
    L.Lx = h->Lx;
    L.Ly = h->Ly;
    L.Lz = h->Lz;
    L.N = h->N;
    L.P = h->P;
    L.Q = (T *)h->Q;
    L.V = (T *)h->V;
    L.F = (T *)h->F;
    L.types = h->types;
    L.D = (T *)h->D;
    L.objs = (const ObjDev<T> *)h->objs;
    fill_lat_params(L, h->params, h->metric_mode);
    L.Hv = h->hvar_on ? (const T *)h->hvar : nullptr;
    L.hvp = T(h->params.dchi * h->params.mu0);
    L.cbd = (const T *)h->cbd;
    if (h->prec == QMIN_FP32) ensure_tmap(h);
    L.split = SplitLists{h->split_cls, h->split_sites, h->n_split_sites, h->split_derivs, h->n_split_derivs,
                         h->tmap_ok ? &h->tmap_q : nullptr, h->dev_err};
    return L;
}

static void free_ctx(qmin_ctx *h)
{
    for (int g = 0; g < 5; ++g)
        if (h->graph[g]) cudaGraphExecDestroy(h->graph[g]);
    void *bufs[] = {h->Q, h->V, h->F, h->D, h->types, h->objs, h->partials, h->stage, h->stage_t, h->fire, h->iter,
                    h->out5, h->M, h->S, h->alt, h->lbp, h->lbs, h->lby, h->Q2, h->V2, h->F2, h->hvar,
                    h->split_cls, h->split_sites, h->split_derivs, h->cbd, h->dev_err, h->geo_scratch,
                    h->scan_part, h->scan_out};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (h->fire_h) cudaFreeHost(h->fire_h);
    if (h->iter_h) cudaFreeHost(h->iter_h);
    if (h->out5_h) cudaFreeHost(h->out5_h);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    if (h->aux) cudaStreamDestroy(h->aux);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    delete h;
}

static void invalidate_graphs(qmin_ctx *h)
{
    h->version++;
    for (int g = 0; g < 5; ++g)
        if (h->graph[g]) {
            cudaGraphExecDestroy(h->graph[g]);
            h->graph[g] = nullptr;
        }
}

// The API functions below take C linkage from their declarations in
// qmin_gb300.h (included above).

const char *qmin_last_error_string(void) { return qmin::g_last_error.c_str(); }

int qmin_create(const qmin_lattice_desc *desc, qmin_handle *out)
{
    if (!desc || !out) return fail(QMIN_EINVAL, "qmin_create: null argument");
    *out = nullptr;
    if (desc->Lx < 3 || desc->Ly < 3 || desc->Lz < 3)
        return fail(QMIN_EINVAL, "qmin_create: every lattice side must be >= 3");
    long long N = (long long)desc->Lx * desc->Ly * desc->Lz;
    if (N > 1500000000LL) return fail(QMIN_EINVAL, "qmin_create: lattice too large (N > 1.5e9 sites)");
    if (desc->precision != QMIN_FP64 && desc->precision != QMIN_FP32)
        return fail(QMIN_EINVAL, "qmin_create: precision must be QMIN_FP64 or QMIN_FP32");
    if (desc->metric_mode != QMIN_METRIC_CPU && desc->metric_mode != QMIN_METRIC_SINGLE)
        return fail(QMIN_EINVAL, "qmin_create: bad metric_mode");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(QMIN_ENODEVICE, "qmin_create: no CUDA device available");
    }
    qmin_ctx *h = new qmin_ctx();
    h->Lx = desc->Lx;
    h->Ly = desc->Ly;
    h->Lz = desc->Lz;
    h->N = (int)N;
    h->P = (N + 31) / 32 * 32;
    h->prec = desc->precision;
    h->metric_mode = desc->metric_mode;
    h->esz = h->prec == QMIN_FP64 ? 8 : 4;
    h->grid = reduction_grid(h->N);
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete h;
        return fail(QMIN_ECUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    h->own_stream = true;
    size_t plane = (size_t)h->P * h->esz;
    bool ok = cudaMalloc(&h->Q, 5 * plane) == cudaSuccess && cudaMalloc(&h->V, 5 * plane) == cudaSuccess &&
              cudaMalloc(&h->F, 5 * plane) == cudaSuccess && cudaMalloc(&h->types, (size_t)h->P) == cudaSuccess &&
              cudaMalloc(&h->partials, sizeof(double) * std::max(8 * (size_t)h->grid, (size_t)3 * kMaxFusedBlocks)) == cudaSuccess &&
              cudaMalloc(&h->fire, sizeof(FireDev)) == cudaSuccess &&
              cudaMalloc(&h->iter, sizeof(IterDev)) == cudaSuccess &&
              cudaMalloc(&h->out5, sizeof(double) * 8) == cudaSuccess &&
              cudaMallocHost(&h->fire_h, sizeof(FireDev)) == cudaSuccess &&
              cudaMallocHost(&h->iter_h, sizeof(IterDev)) == cudaSuccess &&
              cudaMallocHost(&h->out5_h, sizeof(double) * 8) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        free_ctx(h);
        return fail(QMIN_ENOMEM, "qmin_create: device allocation failed");
    }
    cudaMemsetAsync(h->Q, 0, 5 * plane, h->stream);
    cudaMemsetAsync(h->V, 0, 5 * plane, h->stream);
    cudaMemsetAsync(h->F, 0, 5 * plane, h->stream);
    cudaMemsetAsync(h->types, 0, (size_t)h->P, h->stream);
    memset(h->fire_h, 0, sizeof(FireDev));
    memset(h->iter_h, 0, sizeof(IterDev));
    *out = h;
    return QMIN_OK;
}

int qmin_destroy(qmin_handle h)
{
    if (!h) return fail(QMIN_EINVAL, "qmin_destroy: null handle");
    cudaStreamSynchronize(h->stream);
    free_ctx(h);
    return QMIN_OK;
}

int qmin_set_stream(qmin_handle h, void *stream)
{
    if (!h) return fail(QMIN_EINVAL, "qmin_set_stream: null handle");
    CK(cudaStreamSynchronize(h->stream));
    if (h->own_stream) cudaStreamDestroy(h->stream);
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
    invalidate_graphs(h);
    return QMIN_OK;
}

int qmin_kernel_launches(qmin_handle h, long long *count)
{
    if (!h || !count) return fail(QMIN_EINVAL, "qmin_kernel_launches: null argument");
    *count = h->launches;
    return QMIN_OK;
}

int qmin_set_params(qmin_handle h, const qmin_ldg_params *p)
{
    if (!h || !p) return fail(QMIN_EINVAL, "qmin_set_params: null argument");
    h->params = *p;
    if (p->multi_constant && !h->D) {
        if (cudaMalloc(&h->D, 15 * (size_t)h->P * h->esz) != cudaSuccess) {
            cudaGetLastError();
            return fail(QMIN_ENOMEM, "qmin_set_params: derivative planes allocation failed");
        }
        CK(cudaMemsetAsync(h->D, 0, 15 * (size_t)h->P * h->esz, h->stream));
    }
    if (p->multi_constant) {
        const size_t n = (size_t)QMIN_BND_CASES * 5 * QMIN_BND_W;
        if (!h->cbd && cudaMalloc(&h->cbd, n * h->esz) != cudaSuccess) {
            cudaGetLastError();
            return fail(QMIN_ENOMEM, "qmin_set_params: boundary coefficient allocation failed");
        }
        if (h->prec == QMIN_FP64) {
            std::vector<double> c(n);
            fill_boundary_coeffs(*p, c.data());
            CK(cudaMemcpyAsync(h->cbd, c.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        } else {
            std::vector<float> c(n);
            fill_boundary_coeffs(*p, c.data());
            CK(cudaMemcpyAsync(h->cbd, c.data(), n * sizeof(float), cudaMemcpyHostToDevice, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        }
    }
    h->have_params = true;
    invalidate_graphs(h);
    return QMIN_OK;
}

int qmin_set_objects(qmin_handle h, const qmin_object *objs, int n)
{
    if (!h || (n > 0 && !objs) || n < 0) return fail(QMIN_EINVAL, "qmin_set_objects: bad argument");
    if (n > 127) return fail(QMIN_EINVAL, "qmin_set_objects: at most 127 objects (int8 site types)");
    for (int k = 0; k < n; ++k)
        if (objs[k].kind != QMIN_HOMEOTROPIC && objs[k].kind != QMIN_DEGENERATE_PLANAR)
            return fail(QMIN_EINVAL, "qmin_set_objects: unknown object kind");
    h->objs_host.assign(objs, objs + n);
    h->nobj = n;
    if (h->objs) cudaFree(h->objs);
    h->objs = nullptr;
    size_t bytes = (size_t)std::max(n, 1) * (h->prec == QMIN_FP64 ? sizeof(ObjDev<double>) : sizeof(ObjDev<float>));
    CK(cudaMalloc(&h->objs, bytes));
    if (h->prec == QMIN_FP64) {
        std::vector<ObjDev<double>> o(std::max(n, 1));
        for (int k = 0; k < n; ++k) o[k] = {objs[k].kind, objs[k].W, objs[k].S0};
        CK(cudaMemcpy(h->objs, o.data(), bytes, cudaMemcpyHostToDevice));
    } else {
        std::vector<ObjDev<float>> o(std::max(n, 1));
        for (int k = 0; k < n; ++k) o[k] = {objs[k].kind, (float)objs[k].W, (float)objs[k].S0};
        CK(cudaMemcpy(h->objs, o.data(), bytes, cudaMemcpyHostToDevice));
    }
    invalidate_graphs(h);
    return QMIN_OK;
}

static int ensure_stage(qmin_ctx *h)
{
    if (!h->stage) {
        if (cudaMalloc(&h->stage, sizeof(double) * 5 * (size_t)h->N) != cudaSuccess ||
            cudaMalloc(&h->stage_t, sizeof(int32_t) * (size_t)h->N) != cudaSuccess) {
            cudaGetLastError();
            return fail(QMIN_ENOMEM, "staging buffer allocation failed");
        }
    }
    return QMIN_OK;
}

// classes and index lists of the split force + kick, built on the device from
// the device site types (h->types)
static int build_split_lists(qmin_ctx *h)
{
    const size_t need = split_scratch_bytes(h->N);
    if (!h->split_cls && cudaMalloc(&h->split_cls, (size_t)h->N) != cudaSuccess) {
        cudaGetLastError();
        return fail(QMIN_ENOMEM, "split site classes: allocation failed");
    }
    if (h->geo_scratch_bytes < need) {
        if (h->geo_scratch) cudaFree(h->geo_scratch);
        h->geo_scratch = nullptr;
        h->geo_scratch_bytes = 0;
        if (cudaMalloc(&h->geo_scratch, need) != cudaSuccess) {
            cudaGetLastError();
            return fail(QMIN_ENOMEM, "split site lists: scratch allocation failed");
        }
        h->geo_scratch_bytes = need;
    }
    int totals[32];
    const int n = build_split_lists_dev(h->types, h->Lx, h->Ly, h->Lz, h->split_cls, h->geo_scratch, totals,
                                        &h->split_sites, &h->split_sites_cap, &h->n_split_sites, &h->split_derivs,
                                        &h->split_derivs_cap, &h->n_split_derivs, h->stream);
    if (n == -2) {
        cudaGetLastError();
        return fail(QMIN_ENOMEM, "split site lists: allocation failed");
    }
    if (n < 0) return fail(QMIN_ECUDA, std::string("split site lists: ") + cudaGetErrorString(cudaGetLastError()));
    h->launches += n;
    // the derivative planes of object sites are read as zero and no longer
    // written (object sites are not in the derivative list): clear planes a
    // previous geometry left behind
    if (h->D) CK(cudaMemsetAsync(h->D, 0, 15 * (size_t)h->P * h->esz, h->stream));
    return QMIN_OK;
}

// min / max type, count of types <= 0 and sites changed from the device types
// (when `compare`), of int32 (t32) or int8 (t8) types on the device
static int scan_device_types(qmin_ctx *h, const int32_t *t32, const int8_t *t8, bool compare, int out[4])
{
    if (!h->scan_part && (cudaMalloc(&h->scan_part, sizeof(int) * 4 * 152 * 4) != cudaSuccess ||
                          cudaMalloc(&h->scan_out, sizeof(int) * 4) != cudaSuccess)) {
        cudaGetLastError();
        return fail(QMIN_ENOMEM, "site-type scan: allocation failed");
    }
    const int r = t32 ? scan_types<int32_t>(t32, compare ? h->types : nullptr, h->N, h->scan_part, h->scan_out, out,
                                            h->stream)
                      : scan_types<int8_t>(t8, nullptr, h->N, h->scan_part, h->scan_out, out, h->stream);
    if (r < 0) return fail(QMIN_ECUDA, std::string("site-type scan: ") + cudaGetErrorString(cudaGetLastError()));
    h->launches += r;
    return QMIN_OK;
}

static SplitLists split_lists(const qmin_ctx *h)
{
    return SplitLists{h->split_cls, h->split_sites, h->n_split_sites, h->split_derivs, h->n_split_derivs,
                      h->tmap_ok ? &h->tmap_q : nullptr, h->dev_err};
}

int qmin_set_state(qmin_handle h, const double *Q, const int32_t *types, int layout)
{
    if (!h || !Q || !types) return fail(QMIN_EINVAL, "qmin_set_state: null argument");
    if (layout != QMIN_LAYOUT_AOS && layout != QMIN_LAYOUT_SOA) return fail(QMIN_EINVAL, "qmin_set_state: bad layout");
    int r = ensure_stage(h);
    if (r) return r;
    CK(cudaMemcpyAsync(h->stage, Q, sizeof(double) * 5 * (size_t)h->N, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->stage_t, types, sizeof(int32_t) * (size_t)h->N, cudaMemcpyHostToDevice, h->stream));
    // the types are checked on the device before any resident state changes
    int sc[4];
    if ((r = scan_device_types(h, h->stage_t, nullptr, h->have_state, sc))) return r;
    if (sc[0] < -2 || sc[1] > 127) return fail(QMIN_EINVAL, "qmin_set_state: site type out of range [-2, 127]");
    h->nTotal = sc[2];
    h->max_type = std::max(0, sc[1]);
    const bool same_geometry = h->have_state && sc[3] == 0;
    if (h->prec == QMIN_FP64)
        h->launches += launch_aos_to_soa<double>(h->stage, (double *)h->Q, h->N, h->P, layout, h->stream);
    else
        h->launches += launch_aos_to_soa<float>(h->stage, (float *)h->Q, h->N, h->P, layout, h->stream);
    h->launches += launch_types_to_i8(h->stage_t, h->types, h->N, h->stream);
    CK(cudaMemsetAsync(h->V, 0, 5 * (size_t)h->P * h->esz, h->stream));
    CK(cudaMemsetAsync(h->F, 0, 5 * (size_t)h->P * h->esz, h->stream));
    CK(cudaGetLastError());
    if (same_geometry) {
        // the split lists, the tuned strategy and the captured graphs (which
        // hold buffer pointers, not contents) stay valid
        CK(cudaStreamSynchronize(h->stream));
        return QMIN_OK;
    }
    if ((r = build_split_lists(h))) return r;
    CK(cudaStreamSynchronize(h->stream));
    invalidate_graphs(h);
    h->have_state = true;
    return QMIN_OK;
}

int qmin_get_state(qmin_handle h, double *Q, double *V, double *F, int layout)
{
    if (!h) return fail(QMIN_EINVAL, "qmin_get_state: null handle");
    if (layout != QMIN_LAYOUT_AOS && layout != QMIN_LAYOUT_SOA) return fail(QMIN_EINVAL, "qmin_get_state: bad layout");
    int r = ensure_stage(h);
    if (r) return r;
    void *src[3] = {h->Q, h->V, h->F};
    double *dst[3] = {Q, V, F};
    for (int a = 0; a < 3; ++a) {
        if (!dst[a]) continue;
        if (h->prec == QMIN_FP64)
            h->launches += launch_soa_to_aos<double>((const double *)src[a], h->stage, h->N, h->P, layout, h->stream);
        else
            h->launches += launch_soa_to_aos<float>((const float *)src[a], h->stage, h->N, h->P, layout, h->stream);
        CK(cudaMemcpyAsync(dst[a], h->stage, sizeof(double) * 5 * (size_t)h->N, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return QMIN_OK;
}

int qmin_set_field_map(qmin_handle h, const double *H, double chi, double mu0, double dchi)
{
    if (!h) return fail(QMIN_EINVAL, "qmin_set_field_map: null handle");
    if (!h->have_params) return fail(QMIN_ESTATE, "qmin_set_field_map: qmin_set_params has not been called");
    h->params.chi = chi;  // setSpatiallyVaryingField replaces the field constants (landauDeGennesLC.cpp:83-85)
    h->params.mu0 = mu0;
    h->params.dchi = dchi;
    invalidate_graphs(h);
    if (!H) {
        h->hvar_on = false;
        return QMIN_OK;
    }
    if (!h->hvar && cudaMalloc(&h->hvar, 3 * (size_t)h->P * h->esz) != cudaSuccess) {
        cudaGetLastError();
        return fail(QMIN_ENOMEM, "qmin_set_field_map: allocation failed");
    }
    // AoS N x 3 -> 3 planes in the state precision
    const size_t N = (size_t)h->N, P = (size_t)h->P;
    if (h->prec == QMIN_FP64) {
        std::vector<double> planes(3 * P, 0.0);
        for (size_t i = 0; i < N; ++i)
            for (int c = 0; c < 3; ++c) planes[c * P + i] = H[3 * i + c];
        CK(cudaMemcpy(h->hvar, planes.data(), 3 * P * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> planes(3 * P, 0.0f);
        for (size_t i = 0; i < N; ++i)
            for (int c = 0; c < 3; ++c) planes[c * P + i] = (float)H[3 * i + c];
        CK(cudaMemcpy(h->hvar, planes.data(), 3 * P * sizeof(float), cudaMemcpyHostToDevice));
    }
    h->hvar_on = true;
    return QMIN_OK;
}

int qmin_get_sides(qmin_handle h, int *Lx, int *Ly, int *Lz)
{
    if (!h) return fail(QMIN_EINVAL, "qmin_get_sides: null handle");
    if (Lx) *Lx = h->Lx;
    if (Ly) *Ly = h->Ly;
    if (Lz) *Lz = h->Lz;
    return QMIN_OK;
}

int qmin_get_types(qmin_handle h, int32_t *types)
{
    if (!h || !types) return fail(QMIN_EINVAL, "qmin_get_types: null argument");
    if (!h->have_state) return fail(QMIN_ESTATE, "qmin_get_types: no state set");
    std::vector<int8_t> t8((size_t)h->N);
    CK(cudaMemcpyAsync(t8.data(), h->types, (size_t)h->N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < h->N; ++i) types[i] = t8[i];
    return QMIN_OK;
}

int qmin_set_positions(qmin_handle h, const double *Q, int layout)
{
    if (!h || !Q) return fail(QMIN_EINVAL, "qmin_set_positions: null argument");
    if (layout != QMIN_LAYOUT_AOS && layout != QMIN_LAYOUT_SOA) return fail(QMIN_EINVAL, "qmin_set_positions: bad layout");
    if (!h->have_state) return fail(QMIN_ESTATE, "qmin_set_positions: qmin_set_state has not been called");
    int r = ensure_stage(h);
    if (r) return r;
    CK(cudaMemcpyAsync(h->stage, Q, sizeof(double) * 5 * (size_t)h->N, cudaMemcpyHostToDevice, h->stream));
    if (h->prec == QMIN_FP64)
        h->launches += launch_aos_to_soa<double>(h->stage, (double *)h->Q, h->N, h->P, layout, h->stream);
    else
        h->launches += launch_aos_to_soa<float>(h->stage, (float *)h->Q, h->N, h->P, layout, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    return QMIN_OK;
}

int qmin_set_velocities(qmin_handle h, const double *V, int layout)
{
    if (!h || !V) return fail(QMIN_EINVAL, "qmin_set_velocities: null argument");
    if (layout != QMIN_LAYOUT_AOS && layout != QMIN_LAYOUT_SOA)
        return fail(QMIN_EINVAL, "qmin_set_velocities: bad layout");
    if (!h->have_state) return fail(QMIN_ESTATE, "qmin_set_velocities: qmin_set_state has not been called");
    int r = ensure_stage(h);
    if (r) return r;
    CK(cudaMemcpyAsync(h->stage, V, sizeof(double) * 5 * (size_t)h->N, cudaMemcpyHostToDevice, h->stream));
    if (h->prec == QMIN_FP64)
        h->launches += launch_aos_to_soa<double>(h->stage, (double *)h->V, h->N, h->P, layout, h->stream);
    else
        h->launches += launch_aos_to_soa<float>(h->stage, (float *)h->V, h->N, h->P, layout, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    return QMIN_OK;
}

int qmin_defect_measures(qmin_handle h, int kind, double *out)
{
    if (!h || !out) return fail(QMIN_EINVAL, "qmin_defect_measures: null argument");
    if (kind < 0 || kind > 2) return fail(QMIN_EINVAL, "qmin_defect_measures: kind must be 0, 1 or 2");
    if (!h->have_state) return fail(QMIN_ESTATE, "qmin_defect_measures: no state set");
    int r = ensure_stage(h);
    if (r) return r;
    if (h->prec == QMIN_FP64) h->launches += launch_defects<double>(make_lat<double>(h), kind, h->stage, h->stream);
    else h->launches += launch_defects<float>(make_lat<float>(h), kind, h->stage, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, h->stage, sizeof(double) * (size_t)h->N, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return QMIN_OK;
}

int qmin_n_active(qmin_handle h, long long *n)
{
    if (!h || !n) return fail(QMIN_EINVAL, "qmin_n_active: null argument");
    if (!h->have_state) return fail(QMIN_ESTATE, "qmin_n_active: no state set");
    *n = h->nTotal;
    return QMIN_OK;
}

static int ready(qmin_ctx *h, const char *who)
{
    if (!h) return fail(QMIN_EINVAL, std::string(who) + ": null handle");
    if (!h->have_state) return fail(QMIN_ESTATE, std::string(who) + ": qmin_set_state has not been called");
    if (!h->have_params) return fail(QMIN_ESTATE, std::string(who) + ": qmin_set_params has not been called");
    if (h->max_type > h->nobj)
        return fail(QMIN_ESTATE, std::string(who) + ": a site type names an object that qmin_set_objects did not define");
    if (h->nobj > 0 && !h->objs) return fail(QMIN_ESTATE, std::string(who) + ": objects missing");
    if (!h->objs) {
        // a one-entry dummy table keeps the kernel argument valid
        if (cudaMalloc(&h->objs, sizeof(ObjDev<double>)) != cudaSuccess) return fail(QMIN_ENOMEM, "object table");
    }
    return QMIN_OK;
}

template <class T> static int force_impl(qmin_ctx *h)
{
    Lat<T> L = make_lat<T>(h);
    h->launches += launch_force<T>(L, h->grid, h->stream);
    CK(cudaGetLastError());
    return QMIN_OK;
}

int qmin_force(qmin_handle h, double *F_out)
{
    int r = ready(h, "qmin_force");
    if (r) return r;
    r = h->prec == QMIN_FP64 ? force_impl<double>(h) : force_impl<float>(h);
    if (r) return r;
    if (F_out) return qmin_get_state(h, nullptr, nullptr, F_out, QMIN_LAYOUT_AOS);
    CK(cudaStreamSynchronize(h->stream));
    return QMIN_OK;
}

int qmin_energy(qmin_handle h, double *e_per_active, double comps[5])
{
    int r = ready(h, "qmin_energy");
    if (r) return r;
    const qmin_ldg_params &p = h->params;
    double E0[3] = {0, 0, 0}, H0[3] = {0, 0, 0};
    const double *E = p.efield ? p.E : E0, *H = p.hfield ? p.H : H0;
    if (h->prec == QMIN_FP64)
        h->launches += launch_energy_full<double>(make_lat<double>(h), h->partials, h->grid, h->out5, E, p.eps, p.eps0,
                                                  p.deps, H, p.chi, p.mu0, p.dchi, h->stream);
    else
        h->launches += launch_energy_full<float>(make_lat<float>(h), h->partials, h->grid, h->out5, E, p.eps, p.eps0,
                                                 p.deps, H, p.chi, p.mu0, p.dchi, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->out5_h, h->out5, sizeof(double) * 5, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    const double *c = h->out5_h;
    double total = c[0] + c[1] + c[2] + c[3] + c[4];
    if (comps)
        for (int k = 0; k < 5; ++k) comps[k] = c[k];
    if (e_per_active) *e_per_active = h->nTotal != 0 ? total / (1.0 * (double)h->nTotal) : total;
    if (!std::isfinite(total)) return fail(QMIN_ENONFINITE, "qmin_energy: non-finite energy");
    return QMIN_OK;
}

// ------------------------------------------------------------- graphs
// Record `per_iter` launches of one iteration kChunk times into a graph.
template <class F> static int capture_chunk(qmin_ctx *h, int slot, const double (&args)[4], F &&one_iteration)
{
    if (h->graph[slot] && h->graph_key[slot] == h->version &&
        memcmp(h->graph_args[slot], args, sizeof(args)) == 0)
        return QMIN_OK;
    if (h->graph[slot]) {
        cudaGraphExecDestroy(h->graph[slot]);
        h->graph[slot] = nullptr;
    }
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int per = 0;
    for (int k = 0; k < kChunk; ++k) per = one_iteration();
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (e != cudaSuccess) return fail(QMIN_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    // per-node priorities: the side stream's list kernels carry the greatest one
    e = cudaGraphInstantiate(&h->graph[slot], g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(QMIN_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    h->graph_per_iter[slot] = per;
    h->graph_key[slot] = h->version;
    memcpy(h->graph_args[slot], args, sizeof(args));
    return QMIN_OK;
}

// Launch chunks until the device-side `active` flag (at byte offset `flag_off`
// of the pinned mirror) drops; returns after the final state has been copied.
template <class S> static int run_chunks(qmin_ctx *h, int slot, S *dev, S *host, int max_chunks)
{
    for (int c = 0; c < max_chunks; ++c) {
        CK(cudaGraphLaunch(h->graph[slot], h->stream));
        h->launches += (long long)kChunk * h->graph_per_iter[slot];
        CK(cudaMemcpyAsync(host, dev, sizeof(S), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (!host->active) break;
    }
    return QMIN_OK;
}

int qmin_fire_init(qmin_handle h, const qmin_fire_params *p)
{
    if (!h || !p) return fail(QMIN_EINVAL, "qmin_fire_init: null argument");
    if (!(p->dt > 0)) return fail(QMIN_EINVAL, "qmin_fire_init: dt must be > 0");
    FireDev *f = h->fire_h;
    memset(f, 0, sizeof(FireDev));
    // energyMinimizerFIRE::initializeParameters + setFIREParameters (energyMinimizerFIRE.cpp:24-43, 172-183)
    f->dt = p->dt;
    f->dtmin = p->dt * .01;
    f->alpha = p->alpha_start;
    f->alpha0 = p->alpha_start;
    f->dtmax = p->dt_max;
    f->dtinc = p->dt_inc;
    f->dtdec = p->dt_dec;
    f->alphadec = p->alpha_dec;
    f->alphamin = p->alpha_min;
    f->fcut = p->force_cutoff;
    f->nmin = p->n_min;
    f->forceMax = 100.;
    CK(cudaMemcpyAsync(h->fire, f, sizeof(FireDev), cudaMemcpyHostToDevice, h->stream));
    if (h->have_state) CK(cudaMemsetAsync(h->V, 0, 5 * (size_t)h->P * h->esz, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->fire_ready = true;
    return QMIN_OK;
}

int qmin_fire_set_state(qmin_handle h, const qmin_fire_state *st)
{
    if (!h || !st) return fail(QMIN_EINVAL, "qmin_fire_set_state: null argument");
    if (!h->fire_ready) return fail(QMIN_ESTATE, "qmin_fire_set_state: qmin_fire_init has not been called");
    if (st->iterations < 0 || st->n_since < 0 || !(st->dt > 0) || !(st->dt_min >= 0))
        return fail(QMIN_EINVAL, "qmin_fire_set_state: negative counter, dt <= 0 or dt_min < 0");
    FireDev *f = h->fire_h;
    CK(cudaMemcpyAsync(f, h->fire, sizeof(FireDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    // the updater's persistent members between minimize() calls
    // (energyMinimizerFIRE.h:66-94): no velocity mix is pending between calls
    f->iterations = st->iterations;
    f->forceMax = st->force_max;
    f->alpha = st->alpha;
    f->dt = st->dt;
    f->dtmin = st->dt_min;
    f->power = st->power;
    f->nsince = st->n_since;
    f->pending = 0;
    f->reset = 0;
    CK(cudaMemcpyAsync(h->fire, f, sizeof(FireDev), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return QMIN_OK;
}

static int ensure_aux(qmin_ctx *h)
{
    if (h->aux) return QMIN_OK;
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&h->aux, cudaStreamNonBlocking, greatest));
    CK(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
    return QMIN_OK;
}

static int ensure_pingpong(qmin_ctx *h)
{
    if (h->Q2) return QMIN_OK;
    const size_t bytes = 5 * (size_t)h->P * h->esz;
    if (cudaMalloc(&h->Q2, bytes) != cudaSuccess || cudaMalloc(&h->V2, bytes) != cudaSuccess ||
        cudaMalloc(&h->F2, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(QMIN_ENOMEM, "fused FIRE: second state buffer allocation failed");
    }
    CK(cudaMemsetAsync(h->Q2, 0, bytes, h->stream));
    CK(cudaMemsetAsync(h->V2, 0, bytes, h->stream));
    CK(cudaMemsetAsync(h->F2, 0, bytes, h->stream));
    return QMIN_OK;
}

// after an odd number of fused iterations the newest state sits in the second
// buffer set: copy it back so the resident state is always the first set
static int settle_pingpong(qmin_ctx *h, int executed)
{
    if (!(executed & 1)) return QMIN_OK;
    const size_t bytes = 5 * (size_t)h->P * h->esz;
    CK(cudaMemcpyAsync(h->Q, h->Q2, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->V, h->V2, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->F, h->F2, bytes, cudaMemcpyDeviceToDevice, h->stream));
    return QMIN_OK;
}

// The autotuner's choices, kept for the life of the process: a handle that
// meets a problem the process has already tuned (same sides, precision,
// metric, force form, strategy request and site-class counts) takes the
// stored choice instead of timing every candidate again.
struct TuneKey {
    int Lx, Ly, Lz, prec, metric, multi, l6, l4, fields, mode, variant, tmap;
    long long nTotal, n_sites, n_derivs;
    bool operator==(const TuneKey &o) const { return memcmp(this, &o, sizeof(TuneKey)) == 0; }
};
struct TuneChoice {
    int path, sep_cap, fused_cfg, fused_zc, fused_nblocks, tiled_cfg, tiled_zc, tiled_nblocks, split_cap;
    double ms[kTuneCandidates];
};
static std::mutex g_tune_mutex;
static std::vector<std::pair<TuneKey, TuneChoice>> g_tune_cache;

static TuneKey tune_key(const qmin_ctx *h)
{
    TuneKey k;
    memset(&k, 0, sizeof k);  // padding included: the key is compared bytewise
    k.Lx = h->Lx;
    k.Ly = h->Ly;
    k.Lz = h->Lz;
    k.prec = h->prec;
    k.metric = h->metric_mode;
    k.multi = h->params.multi_constant;
    k.l6 = h->params.L6 != 0;
    k.l4 = h->params.L4 != 0;
    k.fields = (h->params.efield ? 1 : 0) | (h->params.hfield ? 2 : 0) | (h->hvar_on ? 4 : 0);
    k.mode = h->fire_mode;
    k.variant = h->fire_variant;
    k.tmap = h->tmap_ok;
    k.nTotal = h->nTotal;
    k.n_sites = h->n_split_sites;
    k.n_derivs = h->n_split_derivs;
    return k;
}

// Autotuner for the FIRE iteration: times the candidate strategies on the live
// lattice with CUDA events and keeps the fastest.  Candidates: the split force
// + kick (deep-site kernel variants), the separate kernels (predictor,
// derivative planes, force + kick) with and without a register cap, the staged
// FP32 force + kick and the fused tiled kernel for each tile shape and two z
// extents; a candidate whose first launch takes more than twice the best time
// so far is not timed further.  The timing launches leave the state as it was:
// the fused kernel writes only the second buffer set and the partials, the
// predictor is timed on the second buffer set, and the velocities are restored
// after the force + kick timings (whose forces equal the ones already resident).
template <class T> static int tune_fire(qmin_ctx *h, const Lat<T> &L)
{
    // a strategy restored from a checkpoint that this handle cannot launch is tuned afresh
    if (h->path == 3 && h->split_cap == kSplitTma && !h->tmap_ok) h->path = -1;
    if (h->path >= 0 && h->tuned_version == h->version && h->tuned_mode == h->fire_mode &&
        h->tuned_variant == h->fire_variant)
        return QMIN_OK;
    // a pinned variant restricts every loop below to that index
    auto pinned_out = [&](int v) { return h->fire_variant >= 0 && v != h->fire_variant; };
    int r = ensure_pingpong(h);
    if (r) return r;
    const TuneKey key = tune_key(h);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        for (const auto &e : g_tune_cache)
            if (e.first == key) {
                const TuneChoice &c = e.second;
                h->path = c.path;
                h->sep_cap = c.sep_cap;
                h->fused_cfg = c.fused_cfg;
                h->fused_zc = c.fused_zc;
                h->fused_nblocks = c.fused_nblocks;
                h->tiled_cfg = c.tiled_cfg;
                h->tiled_zc = c.tiled_zc;
                h->tiled_nblocks = c.tiled_nblocks;
                h->split_cap = c.split_cap;
                memcpy(h->tune_ms, c.ms, sizeof c.ms);
                h->tuned_version = h->version;
                h->tuned_mode = h->fire_mode;
                h->tuned_variant = h->fire_variant;
                return QMIN_OK;
            }
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    auto elapsed = [&](auto &&body) -> float {
        cudaEventRecord(e0, h->stream);
        body();
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms;
    };
    // mean of three launches after a warm-up (which also sets kernel
    // attributes), one launch when the warm-up took over 2 ms; a candidate
    // whose warm-up already exceeds `budget` ms cannot win and keeps that
    // time.  `launch` returns its kernel count.
    auto timed = [&](auto &&launch, float budget) -> float {
        const float warm = elapsed([&]() { h->launches += launch(); });
        if (warm > budget) return warm;
        const int reps = warm > 2.f ? 1 : 3;
        return elapsed([&]() {
                   for (int k = 0; k < reps; ++k) h->launches += launch();
               }) / reps;
    };
    const float kNoBudget = 1e30f;
    const int H = L.multi ? 2 : 1;
    float best = kNoBudget;
    auto budget_for = [&](float fixed) { return best < kNoBudget ? 1.25f * best - fixed : kNoBudget; };
    for (int k = 0; k < kTuneCandidates; ++k) h->tune_ms[k] = -1;
    Lat<T> LB = L;
    LB.Q = (T *)h->Q2;
    LB.V = (T *)h->V2;
    LB.F = (T *)h->F2;
    // the L6 forms are compiled into the uncapped separate kernels only
    const bool l6 = L.multi && L.L6 != T(0);
    const bool auto_mode = h->fire_mode == QMIN_FIRE_AUTO;
    const bool split_ok = L.multi && !l6 && h->split_cls;
    // automatic choice: the split path and the separate kernels where the split
    // path exists (the fused and staged paths are measured slower there on
    // GB300 and stay available when pinned), every strategy elsewhere
    const bool try_split = split_ok && (auto_mode || h->fire_mode == QMIN_FIRE_SPLIT);
    const bool try_sep = l6 || auto_mode || h->fire_mode == QMIN_FIRE_SEPARATE ||
                         (h->fire_mode == QMIN_FIRE_SPLIT && !split_ok);
    const bool try_tiled = !l6 && sizeof(T) == 4 && ((auto_mode && !split_ok) || h->fire_mode == QMIN_FIRE_TILED);
    const bool try_fused = !l6 && ((auto_mode && !split_ok) || h->fire_mode == QMIN_FIRE_FUSED);
    if (try_sep || try_tiled || try_split) {
        const float t_pred = timed([&]() { return launch_fire_pred<T>(LB, h->fire, h->stream); }, kNoBudget);
        const size_t bytes = 5 * (size_t)h->P * h->esz;
        // the force + kick candidates kick V; it is restored afterwards (their forces equal the resident ones)
        CK(cudaMemcpyAsync(h->V2, h->V, bytes, cudaMemcpyDeviceToDevice, h->stream));
        if (try_split) {
            const SplitLists sl = split_lists(h);
            const float t_dl = timed([&]() { return launch_split_derivs<T>(L, sl, h->fire, h->stream); }, kNoBudget);
            for (int cap = 0; cap < kSplitFusedFirst; ++cap) {
                if (pinned_out(cap) || (sizeof(T) == 8 && cap >= kSplitFp32First)) continue;
                if (cap == kSplitTma && !h->tmap_ok) continue;
                int np = 0;
                const float t_fk = timed(
                    [&]() {
                        return launch_split_force_kick<T>(L, sl, h->fire, h->partials, h->grid, cap, h->stream, &np);
                    },
                    budget_for(t_pred + t_dl));
                const float ms = t_pred + t_dl + t_fk;
                h->tune_ms[kSepVariants + 2 * kFusedConfigs + 2 * kTiledConfigs + cap] = ms;
                if (ms < best) {
                    best = ms;
                    h->path = 3;
                    h->split_cap = cap;
                }
            }
        }
        const float t_der = (try_sep || try_tiled) && L.multi
                                ? timed([&]() { return launch_derivs<T>(L, h->stream); }, kNoBudget)
                                : 0.f;
        for (int cap = 0; try_sep && cap < kSepVariants; ++cap) {
            if (pinned_out(cap)) continue;
            const float t_fk = timed(
                [&]() { return launch_force_kick_only<T>(L, h->fire, h->partials, h->grid, h->stream, cap); },
                budget_for(t_pred + t_der));
            const float ms = t_pred + t_der + t_fk;
            h->tune_ms[cap] = ms;
            if (ms < best) {
                best = ms;
                h->path = 0;
                h->sep_cap = cap;
            }
        }
        for (int cfg = 0; try_tiled && cfg < kTiledConfigs; ++cfg) {
            if (pinned_out(cfg)) continue;
            int tx, ty;
            tiled_tile_shape(cfg, &tx, &ty);
            const int ntiles = ((h->Lx + tx - 1) / tx) * ((h->Ly + ty - 1) / ty);
            // short z chunks: many blocks per SM over the launch keep the last wave small
            int zc0 = 4;
            while ((long long)ntiles * ((h->Lz + zc0 - 1) / zc0) > kMaxFusedBlocks) ++zc0;
            for (int v = 0; v < 2; ++v) {
                const int zc = std::min(h->Lz, zc0 << v);
                int nb = 0, ok = 1;
                const float t_fk = timed(
                    [&]() {
                        const int n = launch_force_kick_tiled<T>(cfg, L, h->fire, h->partials, zc, h->stream, &nb);
                        if (n < 0) ok = 0;
                        return n < 0 ? 0 : n;
                    },
                    budget_for(t_pred + t_der));
                if (!ok || cudaGetLastError() != cudaSuccess) break;
                const float ms = t_pred + t_der + t_fk;
                h->tune_ms[kSepVariants + 2 * kFusedConfigs + 2 * cfg + v] = ms;
                if (ms < best) {
                    best = ms;
                    h->path = 2;
                    h->tiled_cfg = cfg;
                    h->tiled_zc = zc;
                    h->tiled_nblocks = nb;
                }
                if (zc >= h->Lz) break;
            }
        }
        CK(cudaMemcpyAsync(h->V, h->V2, bytes, cudaMemcpyDeviceToDevice, h->stream));
    }
    // the fused split variants: the whole iteration but the control, writing only
    // the second buffer set, the derivative planes and the partials (timed after
    // the velocities above are restored from the second set)
    for (int cap = kSplitFusedFirst; try_split && cap < kSplitVariants; ++cap) {
        if (pinned_out(cap) || !split_variant_ok(h, cap)) continue;
        const SplitLists sl = split_lists(h);
        const float ms = timed(
            [&]() {
                const int nd = launch_split_fused_deep<T>(L, (T *)h->Q2, (T *)h->V2, (T *)h->F2, sl, h->fire,
                                                          h->partials, cap - kSplitFusedFirst, h->stream);
                int nl = 0;
                return 1 + launch_split_fused_list<T>(L, (T *)h->V2, (T *)h->F2, sl, h->fire,
                                                      h->partials + 3 * std::max(nd, 0), h->stream, &nl);
            },
            budget_for(0.f));
        if (cudaGetLastError() != cudaSuccess) continue;
        h->tune_ms[kSepVariants + 2 * kFusedConfigs + 2 * kTiledConfigs + cap] = ms;
        if (ms < best) {
            best = ms;
            h->path = 3;
            h->split_cap = cap;
        }
    }
    // the fused kernel writes only the second buffer set and the partials
    for (int cfg = 0; try_fused && cfg < kFusedConfigs; ++cfg) {
        if (pinned_out(cfg)) continue;
        int tx, ty;
        fused_tile_shape(cfg, &tx, &ty);
        const int ntiles = ((h->Lx + tx - 1) / tx) * ((h->Ly + ty - 1) / ty);
        int zc0 = (int)std::ceil((double)h->Lz * ntiles / (152.0 * 4.0));
        zc0 = std::max(zc0, 2 * H + 2);
        for (int v = 0; v < 2; ++v) {
            const int zc = std::min(h->Lz, zc0 << v);
            const int nz = (h->Lz + zc - 1) / zc;
            if ((long long)ntiles * nz > kMaxFusedBlocks) continue;
            int nb = 0, ok = 1;
            const float ms = timed(
                [&]() {
                    const int n = launch_fire_fused<T>(cfg, L, (T *)h->Q2, (T *)h->V2, (T *)h->F2, h->fire,
                                                       h->partials, zc, h->stream, &nb);
                    if (n < 0) ok = 0;
                    return n < 0 ? 0 : n;
                },
                budget_for(0.f));
            if (!ok || cudaGetLastError() != cudaSuccess) continue;
            h->tune_ms[kSepVariants + 2 * cfg + v] = ms;
            if (ms < best) {
                best = ms;
                h->path = 1;
                h->fused_cfg = cfg;
                h->fused_zc = zc;
                h->fused_nblocks = nb;
            }
            if (zc >= h->Lz) break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(cudaGetLastError());
    if (h->path < 0) return fail(QMIN_ECUDA, "FIRE autotuner: no strategy could be launched");
    {
        TuneChoice c{h->path, h->sep_cap, h->fused_cfg, h->fused_zc, h->fused_nblocks, h->tiled_cfg, h->tiled_zc,
                     h->tiled_nblocks, h->split_cap, {}};
        memcpy(c.ms, h->tune_ms, sizeof c.ms);
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache.emplace_back(key, c);
    }
    h->tuned_version = h->version;
    h->tuned_mode = h->fire_mode;
    h->tuned_variant = h->fire_variant;
    return QMIN_OK;
}

template <class T> static int fire_impl(qmin_ctx *h, int max_iterations)
{
    Lat<T> L = make_lat<T>(h);
    const int it0 = h->fire_h->iterations;
    // minimize(): forces at the current Q first (energyMinimizerFIRE.cpp:157)
    h->launches += launch_force<T>(L, h->grid, h->stream);
    int r = tune_fire<T>(h, L);
    if (r) return r;
    if (h->path == 3 && (r = ensure_aux(h))) return r;
    Lat<T> LB = L;  // the second buffer set as input
    LB.Q = (T *)h->Q2;
    LB.V = (T *)h->V2;
    LB.F = (T *)h->F2;
    int parity = 0;
    const int variant = h->path == 0 ? h->sep_cap
                        : h->path == 1 ? h->fused_cfg
                        : h->path == 2 ? h->tiled_cfg
                                       : h->split_cap;
    const double args[4] = {(double)h->path, (double)variant, (double)(h->path == 2 ? h->tiled_zc : h->fused_zc), 0};
    r = capture_chunk(h, 0, args, [&]() {
        int n;
        if (h->path == 0) {
            n = launch_fire_pred<T>(L, h->fire, h->stream);
            n += launch_force_kick<T>(L, h->fire, h->partials, h->grid, h->stream, h->sep_cap);
            n += launch_fire_control(h->fire, h->partials, h->grid, h->stream);
        } else if (h->path == 3 && split_fused(h->split_cap)) {
            // predictor fused into the deep-site kernel: one buffer set in, the
            // other out; the listed sites on the side stream form their predicted
            // Q from the input set
            const SplitLists sl = split_lists(h);
            const Lat<T> &Lin = parity == 0 ? L : LB;
            T *Qo = (T *)(parity == 0 ? h->Q2 : h->Q), *Vo = (T *)(parity == 0 ? h->V2 : h->V),
              *Fo = (T *)(parity == 0 ? h->F2 : h->F);
            parity ^= 1;
            cudaEventRecord(h->ev_fork, h->stream);
            cudaStreamWaitEvent(h->aux, h->ev_fork, 0);
            const int nd = launch_split_fused_deep<T>(Lin, Qo, Vo, Fo, sl, h->fire, h->partials,
                                                      h->split_cap - kSplitFusedFirst, h->stream);
            n = 1;
            int nl = 0;
            n += launch_split_fused_list<T>(Lin, Vo, Fo, sl, h->fire, h->partials + 3 * nd, h->aux, &nl);
            cudaEventRecord(h->ev_join, h->aux);
            cudaStreamWaitEvent(h->stream, h->ev_join, 0);
            n += launch_fire_control(h->fire, h->partials, nd + nl, h->stream);
        } else if (h->path == 3) {
            // the listed sites (derivative planes, then force + kick) on the
            // high-priority side stream, beside the deep-site kernel
            const SplitLists sl = split_lists(h);
            n = launch_fire_pred<T>(L, h->fire, h->stream);
            cudaEventRecord(h->ev_fork, h->stream);
            cudaStreamWaitEvent(h->aux, h->ev_fork, 0);
            const int nd = launch_split_deep<T>(L, sl, h->fire, h->partials, h->grid, h->split_cap, h->stream);
            n += 1;
            n += launch_split_derivs<T>(L, sl, h->fire, h->aux);
            const int nl = launch_split_list<T>(L, sl, h->fire, h->partials + 3 * nd, h->aux);
            n += nl > 0 ? 1 : 0;
            cudaEventRecord(h->ev_join, h->aux);
            cudaStreamWaitEvent(h->stream, h->ev_join, 0);
            n += launch_fire_control(h->fire, h->partials, nd + nl, h->stream);
        } else if (h->path == 2) {
            int nb = 0;
            n = launch_fire_pred<T>(L, h->fire, h->stream);
            if (L.multi) n += launch_derivs<T>(L, h->stream);
            n += launch_force_kick_tiled<T>(h->tiled_cfg, L, h->fire, h->partials, h->tiled_zc, h->stream, &nb);
            n += launch_fire_control(h->fire, h->partials, nb, h->stream);
        } else {
            int nb = 0;
            if (parity == 0)
                n = launch_fire_fused<T>(h->fused_cfg, L, (T *)h->Q2, (T *)h->V2, (T *)h->F2, h->fire, h->partials,
                                         h->fused_zc, h->stream, &nb);
            else
                n = launch_fire_fused<T>(h->fused_cfg, LB, (T *)h->Q, (T *)h->V, (T *)h->F, h->fire, h->partials,
                                         h->fused_zc, h->stream, &nb);
            parity ^= 1;
            n += launch_fire_control(h->fire, h->partials, nb, h->stream);
        }
        return n;
    });
    if (r) return r;
    int remaining = std::max(max_iterations - it0, 1);
    r = run_chunks(h, 0, h->fire, h->fire_h, (remaining + kChunk - 1) / kChunk + 1);
    if (r) return r;
    if ((h->path == 1 || (h->path == 3 && split_fused(h->split_cap))) &&
        (r = settle_pingpong(h, h->fire_h->iterations - it0)))
        return r;
    if (h->path == 3 && h->split_cap == kSplitTma && h->dev_err) {
        int e = 0;
        CK(cudaMemcpyAsync(&e, h->dev_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (e) {
            cudaMemsetAsync(h->dev_err, 0, sizeof(int), h->stream);
            return fail(QMIN_ETIMEOUT, "qmin_fire_run: a TMA wait in the deep-site kernel gave up "
                                       "(the lattice's state is void)");
        }
    }
    h->launches += launch_fire_finish<T>(L, h->fire, h->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->fire_h, h->fire, sizeof(FireDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return QMIN_OK;
}

int qmin_fire_run(qmin_handle h, int max_iterations, qmin_fire_result *res)
{
    int r = ready(h, "qmin_fire_run");
    if (r) return r;
    if (!h->fire_ready) return fail(QMIN_ESTATE, "qmin_fire_run: qmin_fire_init has not been called");
    FireDev *f = h->fire_h;
    CK(cudaMemcpyAsync(f, h->fire, sizeof(FireDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    f->max_iters = max_iterations;
    f->active = 1;  // minimize() always iterates at least once (energyMinimizerFIRE.cpp:158-160)
    f->status = 0;
    f->nTotal = h->nTotal;
    CK(cudaMemcpyAsync(h->fire, f, sizeof(FireDev), cudaMemcpyHostToDevice, h->stream));
    r = h->prec == QMIN_FP64 ? fire_impl<double>(h, max_iterations) : fire_impl<float>(h, max_iterations);
    if (r) return r;
    if (res) {
        res->iterations = f->iterations;
        res->force_max = f->forceMax;
        res->alpha = f->alpha;
        res->dt = f->dt;
        res->power = f->power;
        res->n_since = f->nsince;
    }
    if (f->status) return fail(QMIN_ENONFINITE, "qmin_fire_run: non-finite force norm");
    return QMIN_OK;
}

// ---------------------------------------------------- Adam / Nesterov
static int alloc_planes(qmin_ctx *h, void **p, int count)
{
    if (*p) return QMIN_OK;
    if (cudaMalloc(p, (size_t)count * 5 * (size_t)h->P * h->esz) != cudaSuccess) {
        cudaGetLastError();
        return fail(QMIN_ENOMEM, "minimiser state allocation failed");
    }
    return QMIN_OK;
}

static int iter_begin(qmin_ctx *h, int reset, double fm0, double fcut, int max_iterations, bool at_least_once)
{
    IterDev *it = h->iter_h;
    CK(cudaMemcpyAsync(it, h->iter, sizeof(IterDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (reset) {
        memset(it, 0, sizeof(IterDev));
        it->forceMax = fm0;
    }
    if (fm0 > 0 && !at_least_once) it->forceMax = fm0;
    it->fcut = fcut;
    it->max_iters = max_iterations;
    it->ndof = h->N;
    it->status = 0;
    it->active = at_least_once ? 1 : ((it->iterations < max_iterations && it->forceMax > fcut) ? 1 : 0);
    CK(cudaMemcpyAsync(h->iter, it, sizeof(IterDev), cudaMemcpyHostToDevice, h->stream));
    return QMIN_OK;
}

template <class T>
static int adam_impl(qmin_ctx *h, double b1, double b2, double eps, double dt, int max_iterations)
{
    Lat<T> L = make_lat<T>(h);
    const double args[4] = {b1, b2, eps, dt};
    int r = capture_chunk(h, 1, args, [&]() {
        int n = launch_force<T>(L, h->grid, h->stream);
        n += launch_adam_step<T>(L, (T *)h->M, (T *)h->S, h->iter, b1, b2, eps, dt, h->partials, h->grid, h->stream);
        n += launch_norm_control(h->iter, h->partials, h->grid, 1, b1, b2, h->stream);
        return n;
    });
    if (r) return r;
    return run_chunks(h, 1, h->iter, h->iter_h, max_iterations / kChunk + 2);
}

int qmin_adam_run(qmin_handle h, double beta1, double beta2, double eps, double dt, double force_cutoff,
                  int max_iterations, int reset, int *iterations, double *force_max)
{
    int r = ready(h, "qmin_adam_run");
    if (r) return r;
    if ((r = alloc_planes(h, &h->M, 1)) || (r = alloc_planes(h, &h->S, 1))) return r;
    if (reset) {
        CK(cudaMemsetAsync(h->M, 0, 5 * (size_t)h->P * h->esz, h->stream));
        CK(cudaMemsetAsync(h->S, 0, 5 * (size_t)h->P * h->esz, h->stream));
        invalidate_graphs(h);
    }
    // minimize() resets forceMax to 110 (energyMinimizerAdam.cpp:60)
    r = iter_begin(h, reset, 110.0, force_cutoff, max_iterations, false);
    if (r) return r;
    if (reset) {
        h->iter_h->b1t = beta1;  // setAdamParameters (energyMinimizerAdam.h:20-29)
        h->iter_h->b2t = beta2;
        CK(cudaMemcpyAsync(h->iter, h->iter_h, sizeof(IterDev), cudaMemcpyHostToDevice, h->stream));
    }
    if (h->iter_h->active) {
        r = h->prec == QMIN_FP64 ? adam_impl<double>(h, beta1, beta2, eps, dt, max_iterations)
                                 : adam_impl<float>(h, beta1, beta2, eps, dt, max_iterations);
        if (r) return r;
    }
    CK(cudaMemcpyAsync(h->iter_h, h->iter, sizeof(IterDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (iterations) *iterations = h->iter_h->iterations;
    if (force_max) *force_max = h->iter_h->forceMax;
    if (h->iter_h->status) return fail(QMIN_ENONFINITE, "qmin_adam_run: non-finite force norm");
    return QMIN_OK;
}

template <class T> static int nesterov_impl(qmin_ctx *h, double dt, double mu, int max_iterations)
{
    Lat<T> L = make_lat<T>(h);
    const double args[4] = {dt, mu, 0, 0};
    int r = capture_chunk(h, 2, args, [&]() {
        int n = launch_force<T>(L, h->grid, h->stream);
        n += launch_nesterov_step<T>(L, (T *)h->alt, h->iter, dt, mu, h->partials, h->grid, h->stream);
        n += launch_norm_control(h->iter, h->partials, h->grid, 0, 0.0, 0.0, h->stream);
        return n;
    });
    if (r) return r;
    return run_chunks(h, 2, h->iter, h->iter_h, max_iterations / kChunk + 2);
}

int qmin_nesterov_run(qmin_handle h, double dt, double mu, double force_cutoff, int max_iterations, int reset,
                      int *iterations, double *force_max)
{
    int r = ready(h, "qmin_nesterov_run");
    if (r) return r;
    if ((r = alloc_planes(h, &h->alt, 1))) return r;
    if (reset) {
        // energyMinimizerNesterovAG::initializeFromModel: alternateSequence = positions
        CK(cudaMemcpyAsync(h->alt, h->Q, 5 * (size_t)h->P * h->esz, cudaMemcpyDeviceToDevice, h->stream));
        invalidate_graphs(h);
    }
    r = iter_begin(h, reset, 110.0, force_cutoff, max_iterations, false);
    if (r) return r;
    if (h->iter_h->active) {
        r = h->prec == QMIN_FP64 ? nesterov_impl<double>(h, dt, mu, max_iterations)
                                 : nesterov_impl<float>(h, dt, mu, max_iterations);
        if (r) return r;
    }
    CK(cudaMemcpyAsync(h->iter_h, h->iter, sizeof(IterDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (iterations) *iterations = h->iter_h->iterations;
    if (force_max) *force_max = h->iter_h->forceMax;
    if (h->iter_h->status) return fail(QMIN_ENONFINITE, "qmin_nesterov_run: non-finite force norm");
    return QMIN_OK;
}

template <class T> static int gd_impl(qmin_ctx *h, double dt, int max_iterations)
{
    Lat<T> L = make_lat<T>(h);
    const double args[4] = {dt, 0, 0, 0};
    int r = capture_chunk(h, 4, args, [&]() {
        int n = launch_gd_move<T>(L, h->iter, dt, h->stream);
        n += launch_force<T>(L, h->grid, h->stream);
        n += launch_ff_dot<T>(L, h->iter, h->partials, h->grid, h->stream);
        n += launch_norm_control(h->iter, h->partials, h->grid, 0, 0.0, 0.0, h->stream);
        return n;
    });
    if (r) return r;
    return run_chunks(h, 4, h->iter, h->iter_h, max_iterations / kChunk + 2);
}

int qmin_gd_run(qmin_handle h, double dt, double force_cutoff, int max_iterations, int reset, int *iterations,
                double *force_max)
{
    int r = ready(h, "qmin_gd_run");
    if (r) return r;
    // minimize(): forces at the current Q first, at least one iteration
    // (energyMinimizerGradientDescent.cpp:91-98)
    h->launches += h->prec == QMIN_FP64 ? launch_force<double>(make_lat<double>(h), h->grid, h->stream)
                                        : launch_force<float>(make_lat<float>(h), h->grid, h->stream);
    r = iter_begin(h, reset, 0.0, force_cutoff, max_iterations, true);
    if (r) return r;
    h->iter_h->ndof = h->nTotal;  // forceMax divides by nTotal (energyMinimizerGradientDescent.cpp:82)
    CK(cudaMemcpyAsync(h->iter, h->iter_h, sizeof(IterDev), cudaMemcpyHostToDevice, h->stream));
    r = h->prec == QMIN_FP64 ? gd_impl<double>(h, dt, max_iterations) : gd_impl<float>(h, dt, max_iterations);
    if (r) return r;
    CK(cudaMemcpyAsync(h->iter_h, h->iter, sizeof(IterDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (iterations) *iterations = h->iter_h->iterations;
    if (force_max) *force_max = h->iter_h->forceMax;
    if (h->iter_h->status) return fail(QMIN_ENONFINITE, "qmin_gd_run: non-finite force norm");
    return QMIN_OK;
}

template <class T> static int lbfgs_impl(qmin_ctx *h, int m, double eta, int max_iterations)
{
    Lat<T> L = make_lat<T>(h);
    if (h->iter_h->iterations == 0) {
        // LoLBFGSStepCPU step 1 (energyMinimizerLoLBFGS.cpp:110-116): p = forces at Q,
        // which the iteration's first pass reads from F
        h->launches += launch_force<T>(L, h->grid, h->stream);
    }
    const double args[4] = {(double)m, eta, 0, 0};
    int r = capture_chunk(h, 3, args, [&]() {
        return launch_lbfgs_iteration<T>(L, (T *)h->lbp, (T *)h->lbs, (T *)h->lby, h->iter, m, eta, h->partials,
                                         h->grid, h->stream);
    });
    if (r) return r;
    return run_chunks(h, 3, h->iter, h->iter_h, max_iterations / kChunk + 2);
}

int qmin_lbfgs_run(qmin_handle h, int m, double eta, double force_cutoff, int max_iterations, int reset,
                   int *iterations, double *force_max)
{
    int r = ready(h, "qmin_lbfgs_run");
    if (r) return r;
    if (m < 1 || m > 16) return fail(QMIN_EINVAL, "qmin_lbfgs_run: m must be in [1, 16]");
    if (h->lb_m != m) {
        if (h->lbs) cudaFree(h->lbs);
        if (h->lby) cudaFree(h->lby);
        h->lbs = h->lby = nullptr;
        h->lb_m = m;
        reset = 1;
    }
    if ((r = alloc_planes(h, &h->lbp, 1)) || (r = alloc_planes(h, &h->lbs, m)) || (r = alloc_planes(h, &h->lby, m)))
        return r;
    if (reset) {
        CK(cudaMemsetAsync(h->lbs, 0, (size_t)m * 5 * (size_t)h->P * h->esz, h->stream));
        CK(cudaMemsetAsync(h->lby, 0, (size_t)m * 5 * (size_t)h->P * h->esz, h->stream));
        CK(cudaMemsetAsync(h->lbp, 0, 5 * (size_t)h->P * h->esz, h->stream));
        invalidate_graphs(h);
    }
    // forceMax starts at 100 (energyMinimizerLoLBFGS.cpp:27); always one iteration (:203)
    r = iter_begin(h, reset, reset ? 100.0 : -1.0, force_cutoff, max_iterations, true);
    if (r) return r;
    r = h->prec == QMIN_FP64 ? lbfgs_impl<double>(h, m, eta, max_iterations)
                             : lbfgs_impl<float>(h, m, eta, max_iterations);
    if (r) return r;
    CK(cudaMemcpyAsync(h->iter_h, h->iter, sizeof(IterDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (iterations) *iterations = h->iter_h->iterations;
    if (force_max) *force_max = h->iter_h->forceMax;
    if (h->iter_h->status) return fail(QMIN_ENONFINITE, "qmin_lbfgs_run: non-finite force norm");
    return QMIN_OK;
}


// ------------------------------------------------------------ diagnostics
template <class T> static int fire_profile_impl(qmin_ctx *h, int iterations, double *ms)
{
    Lat<T> L = make_lat<T>(h);
    int r = tune_fire<T>(h, L);
    if (r) return r;
    cudaEvent_t ev[5];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    double acc[4] = {0, 0, 0, 0};
    const bool sfused = h->path == 3 && split_fused(h->split_cap);
    const bool fused = h->path == 1, tiled = h->path == 2, split = h->path == 3 && !sfused;
    const SplitLists sl = split_lists(h);
    Lat<T> LB = L;
    LB.Q = (T *)h->Q2;
    LB.V = (T *)h->V2;
    LB.F = (T *)h->F2;
    for (int it = 0; it < iterations; ++it) {
        CK(cudaEventRecord(ev[0], h->stream));
        if (!fused && !sfused) h->launches += launch_fire_pred<T>(L, h->fire, h->stream);
        CK(cudaEventRecord(ev[1], h->stream));
        if (split) h->launches += launch_split_derivs<T>(L, sl, h->fire, h->stream);
        else if (!fused && !sfused && L.multi) h->launches += launch_derivs<T>(L, h->stream);
        CK(cudaEventRecord(ev[2], h->stream));
        int nparts = h->grid;
        if (sfused) {
            // deep sites and listed sites in sequence (the graph runs the latter beside the former)
            const Lat<T> &Lin = (it & 1) == 0 ? L : LB;
            T *Qo = (T *)((it & 1) == 0 ? h->Q2 : h->Q), *Vo = (T *)((it & 1) == 0 ? h->V2 : h->V),
              *Fo = (T *)((it & 1) == 0 ? h->F2 : h->F);
            const int nd = launch_split_fused_deep<T>(Lin, Qo, Vo, Fo, sl, h->fire, h->partials,
                                                      h->split_cap - kSplitFusedFirst, h->stream);
            int nl = 0;
            h->launches += 1 + launch_split_fused_list<T>(Lin, Vo, Fo, sl, h->fire, h->partials + 3 * nd, h->stream,
                                                          &nl);
            nparts = nd + nl;
        } else if (split) {
            h->launches += launch_split_force_kick<T>(L, sl, h->fire, h->partials, h->grid, h->split_cap, h->stream,
                                                      &nparts);
        } else if (tiled) {
            h->launches += launch_force_kick_tiled<T>(h->tiled_cfg, L, h->fire, h->partials, h->tiled_zc, h->stream,
                                                      &nparts);
        } else if (!fused) {
            h->launches += launch_force_kick_only<T>(L, h->fire, h->partials, h->grid, h->stream, h->sep_cap);
        } else if ((it & 1) == 0) {
            h->launches += launch_fire_fused<T>(h->fused_cfg, L, (T *)h->Q2, (T *)h->V2, (T *)h->F2, h->fire,
                                                h->partials, h->fused_zc, h->stream, &nparts);
        } else {
            h->launches += launch_fire_fused<T>(h->fused_cfg, LB, (T *)h->Q, (T *)h->V, (T *)h->F, h->fire,
                                                h->partials, h->fused_zc, h->stream, &nparts);
        }
        CK(cudaEventRecord(ev[3], h->stream));
        h->launches += launch_fire_control(h->fire, h->partials, nparts, h->stream);
        CK(cudaEventRecord(ev[4], h->stream));
        CK(cudaEventSynchronize(ev[4]));
        for (int k = 0; k < 4; ++k) {
            float t = 0;
            CK(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            acc[k] += t;
        }
    }
    for (int k = 0; k < 4; ++k) ms[k] = iterations > 0 ? acc[k] / iterations : 0.0;
    if ((fused || sfused) && (r = settle_pingpong(h, iterations))) return r;
    h->launches += launch_fire_finish<T>(L, h->fire, h->stream);
    for (auto &e : ev) cudaEventDestroy(e);
    CK(cudaMemcpyAsync(h->fire_h, h->fire, sizeof(FireDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return QMIN_OK;
}

int qmin_fire_profile(qmin_handle h, int iterations, double kernel_ms[4], int *fused)
{
    int r = ready(h, "qmin_fire_profile");
    if (r) return r;
    if (!h->fire_ready) return fail(QMIN_ESTATE, "qmin_fire_profile: qmin_fire_init has not been called");
    if (!kernel_ms || iterations < 1) return fail(QMIN_EINVAL, "qmin_fire_profile: bad argument");
    FireDev *f = h->fire_h;
    CK(cudaMemcpyAsync(f, h->fire, sizeof(FireDev), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    f->max_iters = f->iterations + iterations;
    f->active = 1;
    f->status = 0;
    f->nTotal = h->nTotal;
    CK(cudaMemcpyAsync(h->fire, f, sizeof(FireDev), cudaMemcpyHostToDevice, h->stream));
    r = h->prec == QMIN_FP64 ? fire_profile_impl<double>(h, iterations, kernel_ms)
                             : fire_profile_impl<float>(h, iterations, kernel_ms);
    if (fused) *fused = h->path == 1;
    return r;
}

int qmin_set_fire_kernel(qmin_handle h, int mode)
{
    if (!h) return fail(QMIN_EINVAL, "qmin_set_fire_kernel: null handle");
    if (mode != QMIN_FIRE_SEPARATE && mode != QMIN_FIRE_FUSED && mode != QMIN_FIRE_AUTO && mode != QMIN_FIRE_TILED &&
        mode != QMIN_FIRE_SPLIT)
        return fail(QMIN_EINVAL,
                    "qmin_set_fire_kernel: mode must be QMIN_FIRE_SEPARATE, _FUSED, _TILED, _SPLIT or _AUTO");
    if (mode == QMIN_FIRE_TILED && h->prec != QMIN_FP32)
        return fail(QMIN_EINVAL, "qmin_set_fire_kernel: the staged force + kick is built for the FP32 form only");
    if (h->fire_mode != mode) invalidate_graphs(h);
    h->fire_mode = mode;
    h->fire_variant = -1;
    return QMIN_OK;
}

int qmin_set_fire_variant(qmin_handle h, int variant)
{
    if (!h) return fail(QMIN_EINVAL, "qmin_set_fire_variant: null handle");
    if (variant < -1) return fail(QMIN_EINVAL, "qmin_set_fire_variant: variant must be -1 or an index");
    if (variant >= 0) {
        const int n = h->fire_mode == QMIN_FIRE_SEPARATE ? kSepVariants
                      : h->fire_mode == QMIN_FIRE_FUSED  ? kFusedConfigs
                      : h->fire_mode == QMIN_FIRE_TILED  ? kTiledConfigs
                      : h->fire_mode == QMIN_FIRE_SPLIT  ? kSplitVariants
                                                         : 0;
        if (n == 0) return fail(QMIN_EINVAL, "qmin_set_fire_variant: pin a strategy with qmin_set_fire_kernel first");
        if (variant >= n) return fail(QMIN_EINVAL, "qmin_set_fire_variant: no such variant of this strategy");
        if (h->fire_mode == QMIN_FIRE_SPLIT && !split_variant_ok(h, variant))
            return fail(QMIN_EINVAL, "qmin_set_fire_variant: this split variant needs the FP32 form (4-6, 10-11), "
                                     "an x extent that is a multiple of 4 (10-11) and at most 2^31 / 5 sites "
                                     "per plane set (7-11)");
        if (h->fire_mode == QMIN_FIRE_SPLIT && variant == kSplitTma && !ensure_tmap(h))
            return fail(QMIN_EINVAL, "qmin_set_fire_variant: TMA staging needs an x extent that is a multiple of 4 "
                                     "and at least 40 (and a driver that encodes tensor maps)");
    }
    if (h->fire_variant != variant) invalidate_graphs(h);
    h->fire_variant = variant;
    return QMIN_OK;
}

int qmin_tuning_cache_clear(void)
{
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache.clear();
    return QMIN_OK;
}

int qmin_fire_tuning(qmin_handle h, int *path, int *variant, int *tile_x, int *tile_y, int *zc, double *ms)
{
    if (!h) return fail(QMIN_EINVAL, "qmin_fire_tuning: null handle");
    if (h->path < 0) return fail(QMIN_ESTATE, "qmin_fire_tuning: no FIRE run has been tuned yet");
    if (path) *path = h->path;
    if (variant)
        *variant = h->path == 0 ? h->sep_cap : (h->path == 1 ? h->fused_cfg : (h->path == 2 ? h->tiled_cfg : h->split_cap));
    int tx = 0, ty = 0;
    if (h->path == 1) fused_tile_shape(h->fused_cfg, &tx, &ty);
    if (h->path == 2) tiled_tile_shape(h->tiled_cfg, &tx, &ty);
    if (h->path == 3 && h->split_cap >= 2) tx = h->split_cap == 3 ? 16 : 32, ty = h->split_cap == 3 ? 16 : 8;
    if (tile_x) *tile_x = tx;
    if (tile_y) *tile_y = ty;
    if (zc) *zc = h->path == 1 ? h->fused_zc : (h->path == 2 ? h->tiled_zc : 0);
    if (ms)
        for (int k = 0; k < kTuneCandidates; ++k) ms[k] = h->tune_ms[k];
    return QMIN_OK;
}

int qmin_warm_start(qmin_handle h, qmin_warmnet n)
{
    int rc = ready(h, "qmin_warm_start");
    if (rc) return rc;
    int b = 0, x = 0, y = 0, z = 0;
    rc = qmin_warmnet_shape(n, &b, &x, &y, &z);
    if (rc) return rc;
    if (b != 1 || x != h->Lx || y != h->Ly || z != h->Lz)
        return fail(QMIN_EINVAL, "qmin_warm_start: the net needs batch 1 and the lattice's sides");
    CK(cudaStreamSynchronize(h->stream));
    rc = qmin_warmnet_features(n, 0, h->Q, h->prec, h->P, h->types, h->objs_host.data(), (int)h->objs_host.size());
    if (!rc) rc = qmin_warmnet_forward(n);
    if (!rc) rc = qmin_warmnet_write_state(n, 0, h->Q, h->prec, h->P, h->types);
    if (!rc) rc = qmin_warmnet_sync(n);
    h->fire_ready = false;
    return rc;
}

// ------------------------------------------------------------ checkpoint
// Binary exact-resume checkpoint: the resident state in the device layout,
// the force parameters and objects, the FIRE / minimiser scalars and optional
// minimiser buffers, and the FIRE strategy in use (so a resumed run takes the
// same reduction order).  Little-endian host format, version 1.
namespace {
struct CkpHeader {
    char magic[8];
    int32_t version, Lx, Ly, Lz, prec, metric_mode, nobj, have_params, fire_ready, lb_m, flags;
    int32_t path, sep_cap, fused_cfg, fused_zc, fused_nblocks, tiled_cfg, tiled_zc, tiled_nblocks, fire_mode;
    int32_t split_cap, fire_variant1;  // pinned variant + 1 (0: none)
    int64_t N, P;
};
enum { kCkpM = 1, kCkpS = 2, kCkpAlt = 4, kCkpLb = 8 };
const char kCkpMagic[8] = {'Q', 'M', 'I', 'N', 'C', 'K', 'P', '1'};
}  // namespace

int qmin_checkpoint_save(qmin_handle h, const char *path)
{
    int r = ready(h, "qmin_checkpoint_save");
    if (r) return r;
    if (!path) return fail(QMIN_EINVAL, "qmin_checkpoint_save: null path");
    CkpHeader hd;
    memset(&hd, 0, sizeof hd);
    memcpy(hd.magic, kCkpMagic, 8);
    hd.version = 1;
    hd.Lx = h->Lx; hd.Ly = h->Ly; hd.Lz = h->Lz;
    hd.prec = h->prec; hd.metric_mode = h->metric_mode;
    hd.nobj = (int32_t)h->objs_host.size();
    hd.have_params = h->have_params; hd.fire_ready = h->fire_ready; hd.lb_m = h->lb_m;
    hd.flags = (h->M ? kCkpM : 0) | (h->S ? kCkpS : 0) | (h->alt ? kCkpAlt : 0) | (h->lbp ? kCkpLb : 0);
    hd.path = h->path; hd.sep_cap = h->sep_cap; hd.fused_cfg = h->fused_cfg; hd.fused_zc = h->fused_zc;
    hd.fused_nblocks = h->fused_nblocks; hd.tiled_cfg = h->tiled_cfg; hd.tiled_zc = h->tiled_zc;
    hd.tiled_nblocks = h->tiled_nblocks; hd.fire_mode = h->fire_mode; hd.split_cap = h->split_cap;
    hd.fire_variant1 = h->fire_variant + 1;
    hd.N = h->N; hd.P = h->P;
    const size_t plane = 5 * (size_t)h->P * h->esz;
    std::vector<char> buf(plane);
    FILE *f = fopen(path, "wb");
    if (!f) return fail(QMIN_EINVAL, std::string("qmin_checkpoint_save: cannot open ") + path);
    bool ok = fwrite(&hd, sizeof hd, 1, f) == 1 && fwrite(&h->params, sizeof h->params, 1, f) == 1;
    if (ok && hd.nobj) ok = fwrite(h->objs_host.data(), sizeof(qmin_object), hd.nobj, f) == (size_t)hd.nobj;
    auto put = [&](const void *dev, size_t bytes) {
        if (!ok) return;
        if (buf.size() < bytes) buf.resize(bytes);
        ok = cudaMemcpy(buf.data(), dev, bytes, cudaMemcpyDeviceToHost) == cudaSuccess &&
             fwrite(buf.data(), 1, bytes, f) == bytes;
    };
    CK(cudaStreamSynchronize(h->stream));
    put(h->Q, plane);
    put(h->V, plane);
    put(h->F, plane);
    put(h->types, (size_t)h->N);
    put(h->fire, sizeof(FireDev));
    put(h->iter, sizeof(IterDev));
    if (h->M) put(h->M, plane);
    if (h->S) put(h->S, plane);
    if (h->alt) put(h->alt, plane);
    if (h->lbp) {
        put(h->lbp, plane);
        put(h->lbs, plane * h->lb_m);
        put(h->lby, plane * h->lb_m);
    }
    ok = fclose(f) == 0 && ok;
    if (!ok) return fail(QMIN_ECUDA, "qmin_checkpoint_save: write failed");
    return QMIN_OK;
}

int qmin_checkpoint_load(qmin_handle h, const char *path)
{
    if (!h || !path) return fail(QMIN_EINVAL, "qmin_checkpoint_load: null argument");
    FILE *f = fopen(path, "rb");
    if (!f) return fail(QMIN_EINVAL, std::string("qmin_checkpoint_load: cannot open ") + path);
    CkpHeader hd;
    if (fread(&hd, sizeof hd, 1, f) != 1 || memcmp(hd.magic, kCkpMagic, 8) != 0 || hd.version != 1) {
        fclose(f);
        return fail(QMIN_EINVAL, "qmin_checkpoint_load: not a version-1 qmin checkpoint");
    }
    if (hd.Lx != h->Lx || hd.Ly != h->Ly || hd.Lz != h->Lz || hd.prec != h->prec || hd.metric_mode != h->metric_mode ||
        hd.P != h->P) {
        fclose(f);
        return fail(QMIN_EINVAL, "qmin_checkpoint_load: lattice, precision or metric mode differ from the handle's");
    }
    qmin_ldg_params p;
    std::vector<qmin_object> objs((size_t)std::max(hd.nobj, 0));
    bool ok = fread(&p, sizeof p, 1, f) == 1 && hd.nobj >= 0 && hd.nobj <= 127;
    if (ok && hd.nobj) ok = fread(objs.data(), sizeof(qmin_object), hd.nobj, f) == (size_t)hd.nobj;
    if (ok && hd.have_params) ok = qmin_set_params(h, &p) == QMIN_OK;
    if (ok) ok = qmin_set_objects(h, objs.data(), hd.nobj) == QMIN_OK;
    const size_t plane = 5 * (size_t)h->P * h->esz;
    std::vector<char> buf(plane);
    auto get = [&](void *dev, size_t bytes) {
        if (!ok) return;
        if (buf.size() < bytes) buf.resize(bytes);
        ok = fread(buf.data(), 1, bytes, f) == bytes &&
             cudaMemcpy(dev, buf.data(), bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    CK(cudaStreamSynchronize(h->stream));
    get(h->Q, plane);
    get(h->V, plane);
    get(h->F, plane);
    get(h->types, (size_t)h->N);
    get(h->fire, sizeof(FireDev));
    get(h->iter, sizeof(IterDev));
    if (ok && (hd.flags & kCkpM) && !alloc_planes(h, &h->M, 1)) get(h->M, plane);
    if (ok && (hd.flags & kCkpS) && !alloc_planes(h, &h->S, 1)) get(h->S, plane);
    if (ok && (hd.flags & kCkpAlt) && !alloc_planes(h, &h->alt, 1)) get(h->alt, plane);
    if (ok && (hd.flags & kCkpLb)) {
        if (h->lb_m != hd.lb_m) {
            if (h->lbs) cudaFree(h->lbs);
            if (h->lby) cudaFree(h->lby);
            h->lbs = h->lby = nullptr;
            h->lb_m = hd.lb_m;
        }
        ok = !alloc_planes(h, &h->lbp, 1) && !alloc_planes(h, &h->lbs, hd.lb_m) && !alloc_planes(h, &h->lby, hd.lb_m);
        get(h->lbp, plane);
        get(h->lbs, plane * hd.lb_m);
        get(h->lby, plane * hd.lb_m);
    }
    fclose(f);
    if (!ok) return fail(QMIN_EINVAL, "qmin_checkpoint_load: truncated or unreadable checkpoint");
    // site counts and split lists from the restored types
    int sc[4];
    if (int rr = scan_device_types(h, nullptr, h->types, false, sc)) return rr;
    h->nTotal = sc[2];
    h->max_type = std::max(0, sc[1]);
    if (int rr = build_split_lists(h)) return rr;
    CK(cudaStreamSynchronize(h->stream));
    h->have_state = true;
    h->fire_ready = hd.fire_ready != 0;
    CK(cudaMemcpy(h->fire_h, h->fire, sizeof(FireDev), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(h->iter_h, h->iter, sizeof(IterDev), cudaMemcpyDeviceToHost));
    invalidate_graphs(h);
    // the FIRE strategy of the saved run, so the resumed run reduces in the same order
    h->fire_mode = hd.fire_mode;
    h->fire_variant = hd.fire_variant1 - 1;
    if (hd.path >= 0) {
        int r = ensure_pingpong(h);
        if (r) return r;
        h->path = hd.path;
        h->sep_cap = hd.sep_cap;
        h->fused_cfg = hd.fused_cfg;
        h->fused_zc = hd.fused_zc;
        h->fused_nblocks = hd.fused_nblocks;
        h->tiled_cfg = hd.tiled_cfg;
        h->tiled_zc = hd.tiled_zc;
        h->tiled_nblocks = hd.tiled_nblocks;
        h->split_cap = hd.split_cap;
        h->tuned_version = h->version;
        h->tuned_mode = h->fire_mode;
        h->tuned_variant = h->fire_variant;
    }
    return QMIN_OK;
}

int qmin_object_forces(qmin_handle h, double *forces, int capacity, int *nobj_out)
{
    int r = ready(h, "qmin_object_forces");
    if (r) return r;
    if (h->params.multi_constant)
        return fail(QMIN_EINVAL, "qmin_object_forces: the stress tensor is defined for the one-constant form only");
    const int nobj = (int)h->objs_host.size();
    if (nobj_out) *nobj_out = nobj;
    if (nobj == 0) return QMIN_OK;
    if (!forces || capacity < nobj)
        return fail(QMIN_EINVAL, "qmin_object_forces: forces must hold 3 doubles for every object");
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * 3 * nobj) != cudaSuccess) {
        cudaGetLastError();
        return fail(QMIN_ENOMEM, "qmin_object_forces: allocation failed");
    }
    const qmin_ldg_params &p = h->params;
    double E0[3] = {0, 0, 0}, H0[3] = {0, 0, 0};
    const double *E = p.efield ? p.E : E0, *H = p.hfield ? p.H : H0;
    if (h->prec == QMIN_FP64)
        h->launches += launch_object_forces<double>(make_lat<double>(h), nobj, E, p.eps, p.eps0, p.deps, H, p.chi,
                                                    p.mu0, p.dchi, h->partials, h->grid, out, h->stream);
    else
        h->launches += launch_object_forces<float>(make_lat<float>(h), nobj, E, p.eps, p.eps0, p.deps, H, p.chi,
                                                   p.mu0, p.dchi, h->partials, h->grid, out, h->stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(forces, out, sizeof(double) * 3 * nobj, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(out);
    if (e != cudaSuccess) return fail(QMIN_ECUDA, std::string("qmin_object_forces: ") + cudaGetErrorString(e));
    return QMIN_OK;
}
