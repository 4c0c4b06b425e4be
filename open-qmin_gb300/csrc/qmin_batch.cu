// Batched minimisation: many independent lattices of uneven sizes minimised
// together.  Every solve is an independent energyMinimizerFIRE::minimize
// (energyMinimizerFIRE.cpp:151-170) on its own lattice; the batch packs all of
// them into one set of SoA planes and runs each FIRE iteration for all active
// solves in one launch per kernel, over a work list of 256-site chunks that
// never straddle two solves.  Per-solve FIRE scalars live on the device; a
// solve that converged or ran out of iterations retires (its chunks return at
// once) while the others continue.  The step loop is a captured CUDA graph of
// a fixed number of iterations; the host reads one "any solve still active"
// word per graph replay.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "qmin_force_core.cuh"

namespace qmin {

struct SolveDesc {
    int Lx, Ly, Lz;
    int off;      // first packed site of this solve
    int chunk0;   // first chunk of this solve
    int nchunks;  // chunks of this solve
    int obj_base; // first object-table entry of this solve
    int pad;
};

struct ChunkDesc {
    int solve;
    int start;  // solve-local site index of the chunk's first site
};

template <class T> struct BatchArgs {
    Lat<T> L;  // packed planes (L.N = total sites, L.P = plane stride) and shared force parameters
    const SolveDesc *solves;
    const ChunkDesc *chunks;
    int nchunks;
    // multi-constant: site classes (0 deep bulk, 1 other LC site, 2 object) and
    // the sites whose derivative planes the class-1 forms read
    const uint8_t *cls, *needd;
};

// accessor for a site of a packed solve: neighbours wrap inside that solve's box
template <class T> struct BatchAcc {
    const T *Q;
    const T *D;
    const int8_t *types;
    const ObjDev<T> *objs;
    long long P;
    int i;
    int nb[6];
    __device__ __forceinline__ BatchAcc(const Lat<T> &L, const SolveDesc &sd, int li)
        : Q(L.Q), D(L.D), types(L.types), objs(L.objs + sd.obj_base), P(L.P), i(sd.off + li)
    {
        const int x = li % sd.Lx, r = li / sd.Lx, y = r % sd.Ly, z = r / sd.Ly;
        const int sx = sd.Lx, sy = sd.Lx * sd.Ly;
        nb[0] = i + (x == 0 ? sd.Lx - 1 : -1);
        nb[1] = i + (x == sd.Lx - 1 ? -(sd.Lx - 1) : 1);
        nb[2] = i + (y == 0 ? (sd.Ly - 1) * sx : -sx);
        nb[3] = i + (y == sd.Ly - 1 ? -(sd.Ly - 1) * sx : sx);
        nb[4] = i + (z == 0 ? (sd.Lz - 1) * sy : -sy);
        nb[5] = i + (z == sd.Lz - 1 ? -(sd.Lz - 1) * sy : sy);
    }
    __device__ __forceinline__ int tn(int s) const { return types[nb[s]]; }
    __device__ __forceinline__ T q(int k) const { return ld(Q + (long long)k * P + i); }
    __device__ __forceinline__ T nq(int s, int k) const { return ld(Q + (long long)k * P + nb[s]); }
    __device__ __forceinline__ T dn(int s, int d) const { return ld(D + (long long)d * P + nb[s]); }
    __device__ __forceinline__ ObjDev<T> obj(int t) const { return objs[t - 1]; }
};

// ---------------------------------------------------------------- kernels
template <class T> __global__ void __launch_bounds__(kBlock) k_b_pred(BatchArgs<T> B, const FireDev *fds)
{
    for (int c = blockIdx.x; c < B.nchunks; c += gridDim.x) {
        const ChunkDesc ch = B.chunks[c];
        const FireDev &fd = fds[ch.solve];
        if (!fd.active) continue;  // uniform per block
        // the deferred mix folded into the Verlet coefficients, as k_fire_pred does:
        // v' = cvv v + cvf f, q' = q + dt v'; formed in FP64 by one lane per warp
        double cf[3] = {0.0, 0.0, 0.0};
        if ((threadIdx.x & 31) == 0) {
            const double dt = fd.dt, hdt = 0.5 * dt;
            double mv = 1.0, mf = 0.0;
            if (fd.pending) {
                mv = fd.reset ? 0.0 : 1.0 - fd.mixA;
                mf = fd.reset ? 0.0 : fd.mixA * fd.mixS;
            }
            cf[0] = mv;
            cf[1] = mf + hdt;
            cf[2] = dt;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) cf[k] = __shfl_sync(0xffffffffu, cf[k], 0);
        const T cvv = T(cf[0]), cvf = T(cf[1]), tdt = T(cf[2]);
        const SolveDesc sd = B.solves[ch.solve];
        const int li = ch.start + threadIdx.x;
        if (li >= sd.Lx * sd.Ly * sd.Lz) continue;
        const int i = sd.off + li;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const long long j = (long long)k * B.L.P + i;
            const T vn = cvv * B.L.V[j] + cvf * B.L.F[j];
            B.L.V[j] = vn;
            B.L.Q[j] += tdt * vn;
        }
    }
}

// twice the first derivatives of every LC site (see qmin_force_core.cuh)
template <class T> __global__ void __launch_bounds__(kBlock) k_b_derivs(BatchArgs<T> B, const FireDev *fds)
{
    for (int c = blockIdx.x; c < B.nchunks; c += gridDim.x) {
        const ChunkDesc ch = B.chunks[c];
        if (fds && !fds[ch.solve].active) continue;
        const SolveDesc sd = B.solves[ch.solve];
        const int li = ch.start + threadIdx.x;
        if (li >= sd.Lx * sd.Ly * sd.Lz) continue;
        if (B.needd && !B.needd[sd.off + li]) continue;
        BatchAcc<T> a(B.L, sd, li);
        const int t = B.L.types[a.i];
        const long long P = B.L.P;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int dn = a.nb[2 * ax], up = a.nb[2 * ax + 1];
            const int td = t < 0 ? B.L.types[dn] : 0, tu = t < 0 ? B.L.types[up] : 0;
#pragma unroll
            for (int k = 0; k < 5; ++k)
                B.L.D[(5 * ax + k) * P + a.i] =
                    deriv2_rule(t, td, tu, ld(B.L.Q + k * P + dn), ld(B.L.Q + k * P + a.i), ld(B.L.Q + k * P + up));
        }
    }
}

// force (KICK = 0) or force + half kick + per-chunk FIRE reductions (KICK = 1);
// ONE_CONST: the one-constant form only (a batch whose parameters are one-constant)
template <class T, int KICK, int CAP, bool ONE_CONST = false>
__global__ void __launch_bounds__(kBlock, CAP + 1) k_b_force(BatchArgs<T> B, const FireDev *fds, double *partials)
{
    for (int c = blockIdx.x; c < B.nchunks; c += gridDim.x) {
        const ChunkDesc ch = B.chunks[c];
        if (KICK && !fds[ch.solve].active) continue;  // uniform per block
        const SolveDesc sd = B.solves[ch.solve];
        const int li = ch.start + threadIdx.x;
        // the site's three dot products in the site precision (FP32 warp sums for
        // the FP32 form, FP64 across warps and chunks)
        T acc[3] = {T(0), T(0), T(0)};
        if (li < sd.Lx * sd.Ly * sd.Lz) {
            const int gi = sd.off + li;
            T f[5];
            if (!ONE_CONST && B.cls && B.cls[gi] == 0) {
                // deep bulk site: the 25-point form over Q, no derivative planes
                deep_force_box(B.L, sd.off, sd.Lx, sd.Ly, sd.Lz, li, (long long)gi, f);
            } else {
                BatchAcc<T> a(B.L, sd, li);
                site_force_core<T, BatchAcc<T>, false, !ONE_CONST, ONE_CONST>(B.L, a, B.L.types[gi], f);
            }
            const long long P = B.L.P;
            if (KICK) {
                const T hdt = T(0.5) * T(fds[ch.solve].dt);
                T v[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    v[k] = B.L.V[k * P + gi] + hdt * f[k];
                    B.L.V[k * P + gi] = v[k];
                }
                acc[0] = dot_qt(f, f);
                acc[1] = dot_qt(v, v);
                acc[2] = dot_qt(f, v);
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) B.L.F[k * P + gi] = f[k];
        }
        if (KICK) {
            double sum[3];
            if constexpr (sizeof(T) == 4) {
                block_sum_f32<3>(acc, sum);
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) sum[k] = acc[k];
                block_sum_smem<3>(sum);
            }
            if (threadIdx.x == 0) {
                partials[3 * c + 0] = sum[0];
                partials[3 * c + 1] = sum[1];
                partials[3 * c + 2] = sum[2];
            }
        }
    }
}

// one warp per solve: deterministic sum of its chunks' partials, then the
// fireStepCPU scalar logic (energyMinimizerFIRE.cpp:104-144) and the loop
// condition of minimize(); raises *any when the solve stays active
__global__ void k_b_control(FireDev *fds, const SolveDesc *solves, int nsolves, const double *partials, int *any)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nsolves) return;
    FireDev *fd = fds + w;
    if (!fd->active) return;  // uniform per warp
    const SolveDesc sd = solves[w];
    double v[3] = {0.0, 0.0, 0.0};
    for (int c = lane; c < sd.nchunks; c += 32)
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k] += partials[3 * (sd.chunk0 + c) + k];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane != 0) return;
    const double fn = v[0], vn = v[1], pw = v[2];
    const int it = fd->iterations + 1;
    fd->power = pw;
    fd->forceMax = sqrt(fn) / ((double)fd->nTotal);
    double scaling = 0.0;
    if (fn > 0.) scaling = sqrt(vn / fn);
    fd->scaling = scaling;
    fd->mixA = fd->alpha;
    fd->mixS = scaling;
    fd->pending = 1;
    fd->reset = 0;
    if (pw > 0 && it % 500 != 0) {
        if (fd->nsince > fd->nmin) {
            fd->dt = fmin(fd->dt * fd->dtinc, fd->dtmax);
            fd->alpha = fmax(fd->alpha * fd->alphadec, fd->alphamin);
        }
        fd->nsince += 1;
    } else {
        fd->nsince = 0;
        fd->dt = fmax(fd->dt * fd->dtdec, fd->dtmin);
        fd->alpha = fd->alpha0;
        fd->reset = 1;
    }
    fd->iterations = it;
    if (!isfinite(fn) || !isfinite(vn) || !isfinite(pw)) {
        fd->status = 1;
        fd->active = 0;
        return;
    }
    fd->active = (it < fd->max_iters && fd->forceMax > fd->fcut) ? 1 : 0;
    if (fd->active) atomicOr(any, 1);
}

// apply each solve's last deferred velocity mix
template <class T> __global__ void __launch_bounds__(kBlock) k_b_finish(BatchArgs<T> B, FireDev *fds)
{
    for (int c = blockIdx.x; c < B.nchunks; c += gridDim.x) {
        const ChunkDesc ch = B.chunks[c];
        const FireDev &fd = fds[ch.solve];
        if (!fd.pending) continue;
        const SolveDesc sd = B.solves[ch.solve];
        const int li = ch.start + threadIdx.x;
        if (li >= sd.Lx * sd.Ly * sd.Lz) continue;
        const T ma = T(1.0 - fd.mixA), mb = T(fd.mixA * fd.mixS);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const long long j = (long long)k * B.L.P + sd.off + li;
            B.L.V[j] = fd.reset ? T(0) : ma * B.L.V[j] + mb * B.L.F[j];
        }
    }
}

__global__ void k_b_clear_pending(FireDev *fds, int n)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) fds[s].pending = 0;
}

}  // namespace qmin

using namespace qmin;

namespace {

int bfail(int code, const std::string &m)
{
    qmin::g_last_error = m;
    return code;
}

#define BCK(call)                                                                              \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return bfail(QMIN_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

constexpr int kObjPerSolve = 16;
constexpr int kBatchChunk = 32;  // iterations per captured graph

}  // namespace

struct qmin_batch_ctx {
    int nsolves = 0, prec = QMIN_FP64, metric_mode = QMIN_METRIC_CPU;
    size_t esz = 8;
    int N = 0;  // total packed sites
    long long P = 0;
    int nchunks = 0, maxN = 0;
    std::vector<SolveDesc> solves_h;
    std::vector<ChunkDesc> chunks_h;
    std::vector<long long> ntotal_h;
    SolveDesc *solves = nullptr;
    ChunkDesc *chunks = nullptr;
    void *Q = nullptr, *V = nullptr, *F = nullptr, *D = nullptr, *objs = nullptr;
    int8_t *types = nullptr;
    uint8_t *cls = nullptr, *needd = nullptr;  // per packed site (multi-constant split of the force)
    void *cbd = nullptr;                       // merged boundary coefficients (multi-constant)
    double *partials = nullptr, *stage = nullptr;
    int32_t *stage_t = nullptr;
    FireDev *fds = nullptr;
    std::vector<FireDev> fds_h;
    int *any = nullptr, *any_h = nullptr;
    cudaStream_t stream = nullptr;
    qmin_ldg_params params{};
    bool have_params = false, fire_ready = false;
    int cap = -1;  // force + kick register cap chosen by the tuner
    cudaGraphExec_t graph = nullptr;
    int graph_cap = -1;
    long long launches = 0;
};

template <class T> static BatchArgs<T> batch_args(qmin_batch_ctx *b)
{
    BatchArgs<T> B;
    memset(&B, 0, sizeof B);
    B.L.N = b->N;
    B.L.P = b->P;
    B.L.Q = (T *)b->Q;
    B.L.V = (T *)b->V;
    B.L.F = (T *)b->F;
    B.L.D = (T *)b->D;
    B.L.types = b->types;
    B.L.objs = (const ObjDev<T> *)b->objs;
    fill_lat_params(B.L, b->params, b->metric_mode);
    B.L.cbd = (const T *)b->cbd;
    B.cls = b->params.multi_constant ? b->cls : nullptr;
    B.needd = b->params.multi_constant ? b->needd : nullptr;
    B.solves = b->solves;
    B.chunks = b->chunks;
    B.nchunks = b->nchunks;
    return B;
}

static int grid_for(int nchunks) { return std::min(nchunks, 152 * 8); }

template <class T> static int launch_b_force(const BatchArgs<T> &B, const FireDev *fds, double *partials, int kick,
                                             int cap, cudaStream_t s)
{
    const int g = grid_for(B.nchunks);
    int n = 0;
    if (B.L.multi) {
        k_b_derivs<T><<<g, kBlock, 0, s>>>(B, kick ? fds : nullptr);
        ++n;
    }
    if (!B.L.multi) {
        if (!kick) k_b_force<T, 0, 0, true><<<g, kBlock, 0, s>>>(B, fds, partials);
        else if (cap == 2) k_b_force<T, 1, 2, true><<<g, kBlock, 0, s>>>(B, fds, partials);
        else if (cap == 1) k_b_force<T, 1, 1, true><<<g, kBlock, 0, s>>>(B, fds, partials);
        else k_b_force<T, 1, 0, true><<<g, kBlock, 0, s>>>(B, fds, partials);
        return n + 1;
    }
    if (!kick) k_b_force<T, 0, 0><<<g, kBlock, 0, s>>>(B, fds, partials);
    else if (cap == 2) k_b_force<T, 1, 2><<<g, kBlock, 0, s>>>(B, fds, partials);
    else if (cap == 1) k_b_force<T, 1, 1><<<g, kBlock, 0, s>>>(B, fds, partials);
    else k_b_force<T, 1, 0><<<g, kBlock, 0, s>>>(B, fds, partials);
    return n + 1;
}

template <class T> static int launch_b_iteration(qmin_batch_ctx *b, const BatchArgs<T> &B, int cap)
{
    cudaMemsetAsync(b->any, 0, sizeof(int), b->stream);
    k_b_pred<T><<<grid_for(B.nchunks), kBlock, 0, b->stream>>>(B, b->fds);
    int n = 1 + launch_b_force<T>(B, b->fds, b->partials, 1, cap, b->stream);
    k_b_control<<<(b->nsolves * 32 + 255) / 256, 256, 0, b->stream>>>(b->fds, b->solves, b->nsolves, b->partials,
                                                                        b->any);
    return n + 1;
}

// The API functions below take C linkage from their declarations in qmin_gb300.h.

int qmin_batch_create(int nsolves, const int32_t *dims, int precision, int metric_mode, qmin_batch *out)
{
    if (!out || !dims || nsolves < 1) return bfail(QMIN_EINVAL, "qmin_batch_create: bad argument");
    if (precision != QMIN_FP64 && precision != QMIN_FP32) return bfail(QMIN_EINVAL, "qmin_batch_create: precision");
    if (metric_mode != QMIN_METRIC_CPU && metric_mode != QMIN_METRIC_SINGLE)
        return bfail(QMIN_EINVAL, "qmin_batch_create: metric_mode");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return bfail(QMIN_ENODEVICE, "qmin_batch_create: no CUDA device available");
    }
    auto *b = new qmin_batch_ctx();
    b->nsolves = nsolves;
    b->prec = precision;
    b->metric_mode = metric_mode;
    b->esz = precision == QMIN_FP64 ? 8 : 4;
    long long off = 0;
    for (int s = 0; s < nsolves; ++s) {
        const int Lx = dims[3 * s], Ly = dims[3 * s + 1], Lz = dims[3 * s + 2];
        if (Lx < 3 || Ly < 3 || Lz < 3) {
            delete b;
            return bfail(QMIN_EINVAL, "qmin_batch_create: every lattice side must be >= 3");
        }
        const int n = Lx * Ly * Lz;
        SolveDesc sd{Lx, Ly, Lz, (int)off, (int)b->chunks_h.size(), (n + kBlock - 1) / kBlock, s * kObjPerSolve, 0};
        for (int c = 0; c < sd.nchunks; ++c) b->chunks_h.push_back({s, c * kBlock});
        b->solves_h.push_back(sd);
        b->maxN = std::max(b->maxN, n);
        off += n;
        if (off > 1500000000LL) {
            delete b;
            return bfail(QMIN_EINVAL, "qmin_batch_create: more than 1.5e9 sites in the batch");
        }
    }
    b->N = (int)off;
    b->P = (off + 31) / 32 * 32;
    b->nchunks = (int)b->chunks_h.size();
    b->ntotal_h.assign(nsolves, 0);
    const size_t plane = (size_t)b->P * b->esz;
    bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&b->Q, 5 * plane) == cudaSuccess && cudaMalloc(&b->V, 5 * plane) == cudaSuccess &&
              cudaMalloc(&b->F, 5 * plane) == cudaSuccess && cudaMalloc(&b->types, (size_t)b->P) == cudaSuccess &&
              cudaMalloc(&b->objs, sizeof(ObjDev<double>) * kObjPerSolve * nsolves) == cudaSuccess &&
              cudaMalloc(&b->solves, sizeof(SolveDesc) * nsolves) == cudaSuccess &&
              cudaMalloc(&b->chunks, sizeof(ChunkDesc) * b->nchunks) == cudaSuccess &&
              cudaMalloc(&b->partials, sizeof(double) * 3 * b->nchunks) == cudaSuccess &&
              cudaMalloc(&b->stage, sizeof(double) * 5 * (size_t)b->maxN) == cudaSuccess &&
              cudaMalloc(&b->stage_t, sizeof(int32_t) * (size_t)b->maxN) == cudaSuccess &&
              cudaMalloc(&b->fds, sizeof(FireDev) * nsolves) == cudaSuccess &&
              cudaMalloc(&b->any, sizeof(int)) == cudaSuccess && cudaMallocHost(&b->any_h, sizeof(int)) == cudaSuccess &&
              cudaMalloc(&b->cls, (size_t)b->P) == cudaSuccess && cudaMalloc(&b->needd, (size_t)b->P) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        qmin_batch_destroy(b);
        return bfail(QMIN_ENOMEM, "qmin_batch_create: device allocation failed");
    }
    cudaMemsetAsync(b->Q, 0, 5 * plane, b->stream);
    cudaMemsetAsync(b->V, 0, 5 * plane, b->stream);
    cudaMemsetAsync(b->F, 0, 5 * plane, b->stream);
    cudaMemsetAsync(b->types, 0, (size_t)b->P, b->stream);
    cudaMemsetAsync(b->cls, 2, (size_t)b->P, b->stream);    // nothing deep until a solve is set
    cudaMemsetAsync(b->needd, 1, (size_t)b->P, b->stream);  // every derivative until then
    cudaMemsetAsync(b->objs, 0, sizeof(ObjDev<double>) * kObjPerSolve * nsolves, b->stream);
    cudaMemcpyAsync(b->solves, b->solves_h.data(), sizeof(SolveDesc) * nsolves, cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(b->chunks, b->chunks_h.data(), sizeof(ChunkDesc) * b->nchunks, cudaMemcpyHostToDevice, b->stream);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) {
        qmin_batch_destroy(b);
        return bfail(QMIN_ECUDA, "qmin_batch_create: initialisation failed");
    }
    *out = b;
    return QMIN_OK;
}

int qmin_batch_destroy(qmin_batch b)
{
    if (!b) return bfail(QMIN_EINVAL, "qmin_batch_destroy: null handle");
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    void *bufs[] = {b->Q, b->V, b->F, b->D, b->objs, b->types, b->partials, b->stage, b->stage_t, b->fds, b->any,
                    b->solves, b->chunks, b->cls, b->needd, b->cbd};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (b->any_h) cudaFreeHost(b->any_h);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return QMIN_OK;
}

int qmin_batch_set_params(qmin_batch b, const qmin_ldg_params *p)
{
    if (!b || !p) return bfail(QMIN_EINVAL, "qmin_batch_set_params: null argument");
    if (p->multi_constant && p->L6 != 0.0)
        return bfail(QMIN_EINVAL, "qmin_batch_set_params: the L6 term is supported by single-lattice handles only");
    b->params = *p;
    if (p->multi_constant && !b->D) {
        if (cudaMalloc(&b->D, 15 * (size_t)b->P * b->esz) != cudaSuccess) {
            cudaGetLastError();
            return bfail(QMIN_ENOMEM, "qmin_batch_set_params: derivative planes allocation failed");
        }
        BCK(cudaMemsetAsync(b->D, 0, 15 * (size_t)b->P * b->esz, b->stream));
    }
    if (p->multi_constant) {
        // the merged boundary coefficients of the straight-line boundary forms
        const size_t n = (size_t)QMIN_BND_CASES * 5 * QMIN_BND_W;
        if (!b->cbd && cudaMalloc(&b->cbd, n * b->esz) != cudaSuccess) {
            cudaGetLastError();
            b->cbd = nullptr;
            return bfail(QMIN_ENOMEM, "qmin_batch_set_params: boundary coefficient allocation failed");
        }
        if (b->prec == QMIN_FP64) {
            std::vector<double> c(n);
            fill_boundary_coeffs(*p, c.data());
            BCK(cudaMemcpyAsync(b->cbd, c.data(), n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
            BCK(cudaStreamSynchronize(b->stream));
        } else {
            std::vector<float> c(n);
            fill_boundary_coeffs(*p, c.data());
            BCK(cudaMemcpyAsync(b->cbd, c.data(), n * sizeof(float), cudaMemcpyHostToDevice, b->stream));
            BCK(cudaStreamSynchronize(b->stream));
        }
    }
    b->have_params = true;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->cap = -1;
    return QMIN_OK;
}

int qmin_batch_set_solve(qmin_batch b, int s, const double *Q, const int32_t *types, const qmin_object *objs,
                         int nobj)
{
    if (!b || !Q || !types || s < 0 || s >= b->nsolves || nobj < 0 || (nobj > 0 && !objs))
        return bfail(QMIN_EINVAL, "qmin_batch_set_solve: bad argument");
    if (nobj > kObjPerSolve) return bfail(QMIN_EINVAL, "qmin_batch_set_solve: at most 16 objects per solve");
    const SolveDesc &sd = b->solves_h[s];
    const int n = sd.Lx * sd.Ly * sd.Lz;
    long long nT = 0;
    for (int i = 0; i < n; ++i) {
        if (types[i] < -2 || types[i] > nobj)
            return bfail(QMIN_EINVAL, "qmin_batch_set_solve: site type out of range for this solve's objects");
        if (types[i] <= 0) ++nT;
    }
    b->ntotal_h[s] = nT;
    {
        // site classes of the split force (deep bulk: type 0 with six type-0
        // neighbours; 1: other LC sites; 2: objects) and the sites whose
        // derivative planes the class-1 forms read, with this solve's periodic wrap
        std::vector<uint8_t> cls((size_t)n), need((size_t)n, 0);
        auto nb = [&](int i, int k) {
            const int x = i % sd.Lx, r = i / sd.Lx, y = r % sd.Ly, z = r / sd.Ly;
            switch (k) {
            case 0: return (x == 0 ? sd.Lx - 1 : x - 1) + sd.Lx * (y + sd.Ly * z);
            case 1: return (x == sd.Lx - 1 ? 0 : x + 1) + sd.Lx * (y + sd.Ly * z);
            case 2: return x + sd.Lx * ((y == 0 ? sd.Ly - 1 : y - 1) + sd.Ly * z);
            case 3: return x + sd.Lx * ((y == sd.Ly - 1 ? 0 : y + 1) + sd.Ly * z);
            case 4: return x + sd.Lx * (y + sd.Ly * (z == 0 ? sd.Lz - 1 : z - 1));
            default: return x + sd.Lx * (y + sd.Ly * (z == sd.Lz - 1 ? 0 : z + 1));
            }
        };
        for (int i = 0; i < n; ++i) {
            if (types[i] > 0) {
                cls[i] = 2;
                continue;
            }
            bool deep = types[i] == 0;
            for (int k = 0; k < 6 && deep; ++k) deep = types[nb(i, k)] == 0;
            cls[i] = deep ? 0 : 1;
            if (!deep)
                for (int k = 0; k < 6; ++k) need[nb(i, k)] = 1;
        }
        BCK(cudaMemcpyAsync(b->cls + sd.off, cls.data(), (size_t)n, cudaMemcpyHostToDevice, b->stream));
        BCK(cudaMemcpyAsync(b->needd + sd.off, need.data(), (size_t)n, cudaMemcpyHostToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
    }
    BCK(cudaMemcpyAsync(b->stage, Q, sizeof(double) * 5 * (size_t)n, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->stage_t, types, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, b->stream));
    if (b->prec == QMIN_FP64)
        b->launches += launch_aos_to_soa<double>(b->stage, (double *)b->Q + sd.off, n, b->P, QMIN_LAYOUT_AOS, b->stream);
    else
        b->launches += launch_aos_to_soa<float>(b->stage, (float *)b->Q + sd.off, n, b->P, QMIN_LAYOUT_AOS, b->stream);
    b->launches += launch_types_to_i8(b->stage_t, b->types + sd.off, n, b->stream);
    for (int k = 0; k < 5; ++k) {
        BCK(cudaMemsetAsync((char *)b->V + ((size_t)k * b->P + sd.off) * b->esz, 0, (size_t)n * b->esz, b->stream));
        BCK(cudaMemsetAsync((char *)b->F + ((size_t)k * b->P + sd.off) * b->esz, 0, (size_t)n * b->esz, b->stream));
    }
    if (nobj > 0) {
        if (b->prec == QMIN_FP64) {
            std::vector<ObjDev<double>> o(nobj);
            for (int k = 0; k < nobj; ++k) o[k] = {objs[k].kind, objs[k].W, objs[k].S0};
            BCK(cudaMemcpyAsync((ObjDev<double> *)b->objs + sd.obj_base, o.data(), sizeof(ObjDev<double>) * nobj,
                                cudaMemcpyHostToDevice, b->stream));
        } else {
            std::vector<ObjDev<float>> o(nobj);
            for (int k = 0; k < nobj; ++k) o[k] = {objs[k].kind, (float)objs[k].W, (float)objs[k].S0};
            BCK(cudaMemcpyAsync((ObjDev<float> *)b->objs + sd.obj_base, o.data(), sizeof(ObjDev<float>) * nobj,
                                cudaMemcpyHostToDevice, b->stream));
        }
    }
    BCK(cudaStreamSynchronize(b->stream));
    return QMIN_OK;
}

int qmin_batch_get_solve(qmin_batch b, int s, double *Q, double *F)
{
    if (!b || s < 0 || s >= b->nsolves) return bfail(QMIN_EINVAL, "qmin_batch_get_solve: bad argument");
    const SolveDesc &sd = b->solves_h[s];
    const int n = sd.Lx * sd.Ly * sd.Lz;
    double *dst[2] = {Q, F};
    void *src[2] = {b->Q, b->F};
    for (int a = 0; a < 2; ++a) {
        if (!dst[a]) continue;
        if (b->prec == QMIN_FP64)
            b->launches += launch_soa_to_aos<double>((const double *)src[a] + sd.off, b->stage, n, b->P,
                                                     QMIN_LAYOUT_AOS, b->stream);
        else
            b->launches += launch_soa_to_aos<float>((const float *)src[a] + sd.off, b->stage, n, b->P,
                                                    QMIN_LAYOUT_AOS, b->stream);
        BCK(cudaMemcpyAsync(dst[a], b->stage, sizeof(double) * 5 * (size_t)n, cudaMemcpyDeviceToHost, b->stream));
    }
    BCK(cudaStreamSynchronize(b->stream));
    return QMIN_OK;
}

int qmin_batch_fire_init(qmin_batch b, const qmin_fire_params *p)
{
    if (!b || !p || !(p->dt > 0)) return bfail(QMIN_EINVAL, "qmin_batch_fire_init: bad argument");
    FireDev f;
    memset(&f, 0, sizeof f);
    f.dt = p->dt;
    f.dtmin = p->dt * .01;
    f.alpha = f.alpha0 = p->alpha_start;
    f.dtmax = p->dt_max;
    f.dtinc = p->dt_inc;
    f.dtdec = p->dt_dec;
    f.alphadec = p->alpha_dec;
    f.alphamin = p->alpha_min;
    f.fcut = p->force_cutoff;
    f.nmin = p->n_min;
    f.forceMax = 100.;
    b->fds_h.assign(b->nsolves, f);
    BCK(cudaMemcpyAsync(b->fds, b->fds_h.data(), sizeof(FireDev) * b->nsolves, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemsetAsync(b->V, 0, 5 * (size_t)b->P * b->esz, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->fire_ready = true;
    return QMIN_OK;
}

template <class T> static int batch_fire_impl(qmin_batch_ctx *b, int max_iterations)
{
    BatchArgs<T> B = batch_args<T>(b);
    // every solve's minimize() starts with its forces (energyMinimizerFIRE.cpp:157)
    b->launches += launch_b_force<T>(B, b->fds, b->partials, 0, 0, b->stream);
    if (b->cap < 0) {
        // autotune the force + kick register cap on the live batch (velocities restored)
        cudaEvent_t e0, e1;
        BCK(cudaEventCreate(&e0));
        BCK(cudaEventCreate(&e1));
        void *vb = nullptr;
        const size_t bytes = 5 * (size_t)b->P * b->esz;
        if (cudaMalloc(&vb, bytes) != cudaSuccess) {
            cudaGetLastError();
            return bfail(QMIN_ENOMEM, "batch tuner: scratch allocation failed");
        }
        BCK(cudaMemcpyAsync(vb, b->V, bytes, cudaMemcpyDeviceToDevice, b->stream));
        float best = 1e30f;
        for (int cap = 0; cap < 3; ++cap) {
            launch_b_force<T>(B, b->fds, b->partials, 1, cap, b->stream);
            cudaEventRecord(e0, b->stream);
            for (int r = 0; r < 3; ++r) launch_b_force<T>(B, b->fds, b->partials, 1, cap, b->stream);
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                b->cap = cap;
            }
        }
        BCK(cudaMemcpyAsync(b->V, vb, bytes, cudaMemcpyDeviceToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        cudaFree(vb);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b->launches += 12;
    }
    if (!b->graph || b->graph_cap != b->cap) {
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t g = nullptr;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < kBatchChunk; ++k) launch_b_iteration<T>(b, B, b->cap);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess) return bfail(QMIN_ECUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return bfail(QMIN_ECUDA, std::string("batch graph: ") + cudaGetErrorString(e));
        b->graph_cap = b->cap;
    }
    const int per_iter = 3 + (B.L.multi ? 1 : 0);
    const int max_chunks = max_iterations / kBatchChunk + 2;
    for (int c = 0; c < max_chunks; ++c) {
        BCK(cudaGraphLaunch(b->graph, b->stream));
        b->launches += (long long)kBatchChunk * per_iter;
        BCK(cudaMemcpyAsync(b->any_h, b->any, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        if (!*b->any_h) break;
    }
    k_b_finish<T><<<grid_for(b->nchunks), kBlock, 0, b->stream>>>(B, b->fds);
    k_b_clear_pending<<<(b->nsolves + 255) / 256, 256, 0, b->stream>>>(b->fds, b->nsolves);
    b->launches += 2;
    BCK(cudaGetLastError());
    return QMIN_OK;
}

int qmin_batch_fire_run(qmin_batch b, int max_iterations, int *iterations, double *force_max, int *converged)
{
    if (!b) return bfail(QMIN_EINVAL, "qmin_batch_fire_run: null handle");
    if (!b->have_params || !b->fire_ready)
        return bfail(QMIN_ESTATE, "qmin_batch_fire_run: set_params and fire_init must come first");
    BCK(cudaMemcpyAsync(b->fds_h.data(), b->fds, sizeof(FireDev) * b->nsolves, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    for (int s = 0; s < b->nsolves; ++s) {
        FireDev &f = b->fds_h[s];
        f.max_iters = max_iterations;
        f.active = 1;  // minimize() iterates at least once
        f.status = 0;
        f.nTotal = b->ntotal_h[s];
    }
    BCK(cudaMemcpyAsync(b->fds, b->fds_h.data(), sizeof(FireDev) * b->nsolves, cudaMemcpyHostToDevice, b->stream));
    int r = b->prec == QMIN_FP64 ? batch_fire_impl<double>(b, max_iterations) : batch_fire_impl<float>(b, max_iterations);
    if (r) return r;
    BCK(cudaMemcpyAsync(b->fds_h.data(), b->fds, sizeof(FireDev) * b->nsolves, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    int conv = 0, bad = 0;
    for (int s = 0; s < b->nsolves; ++s) {
        const FireDev &f = b->fds_h[s];
        if (iterations) iterations[s] = f.iterations;
        if (force_max) force_max[s] = f.forceMax;
        if (f.forceMax <= f.fcut) ++conv;
        bad |= f.status;
    }
    if (converged) *converged = conv;
    if (bad) return bfail(QMIN_ENONFINITE, "qmin_batch_fire_run: a solve produced a non-finite force norm");
    return QMIN_OK;
}

int qmin_batch_kernel_launches(qmin_batch b, long long *count)
{
    if (!b || !count) return bfail(QMIN_EINVAL, "qmin_batch_kernel_launches: null argument");
    *count = b->launches;
    return QMIN_OK;
}

