// Batched minimisation: many independent lattices of uneven sizes minimised
// together.  Every solve is an independent energyMinimizerFIRE::minimize
// (energyMinimizerFIRE.cpp:151-170) on its own lattice; the batch packs all of
// them into one set of SoA planes, cut into chunks of 256 sites that never
// straddle two solves (256 consecutive sites, or tiles of the solve's box; the
// tuner picks the shape by timing the force + kick).  qmin_batch_fire_run runs
// every iteration of every solve in one persistent cooperative launch: per
// iteration the predictor, the force + half kick + per-chunk FIRE sums and the
// per-solve FIRE control, separated by bounded grid barriers (FP32
// one-constant batches: predictor, force and kick as one phase from one state
// set into the other, then the control).  Per-solve FIRE
// scalars live on the device; a solve that converged or ran out of iterations
// retires, and the phases then cover only the chunks of the solves still
// active.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "qmin_force_core.cuh"

namespace qmin {

struct __align__(16) SolveDesc {
    int Lx, Ly, Lz;
    int off;      // first packed site of this solve
    int chunk0;   // first chunk of this solve
    int nchunks;  // chunks of this solve
    int obj_base; // first object-table entry of this solve
    int pad;
    unsigned mx, my;  // division multipliers for Lx and Ly (div_magic)
    int pad2[2];
};

// multiplier m = ceil(2^32 / d) for udiv (d >= 2; 0 marks d = 1)
inline unsigned div_magic(unsigned d) { return d < 2 ? 0u : (unsigned)(((1ull << 32) + d - 1) / d); }

// n / d for n < 2^31: the multiply-high estimate is floor(n / d) or one more
// (m d - 2^32 < d, so the excess n (m d - 2^32) / (d 2^32) stays below 1)
__device__ __forceinline__ unsigned udiv(unsigned n, unsigned d, unsigned m)
{
    if (m == 0) return n;
    const unsigned q = __umulhi(n, m);
    return q * d > n ? q - 1 : q;
}

struct ChunkDesc {
    int solve;
    int start;  // solve-local index of the chunk's first site (a tile's lowest corner)
};

template <class T> struct BatchArgs {
    Lat<T> L;  // packed planes (L.N = total sites, L.P = plane stride) and shared force parameters
    const SolveDesc *solves;
    const ChunkDesc *chunks;
    int nchunks;
    // chunk shape: tx = 0: 256 consecutive sites of the solve; else a tx x ty x tz
    // tile of its box (tx ty tz = 256, powers of two: lx = log2 tx, lxy = log2 tx ty)
    // cut where it overhangs the box
    int tx, ty, tz, lx, lxy;
    // multi-constant: site classes (0 deep bulk, 1 other LC site, 2 object) and
    // the sites whose derivative planes the class-1 forms read
    const uint8_t *cls, *needd;
};

// solve-local site (index li, coordinates x y z) of thread t in chunk ch,
// false where the chunk's tile overhangs the solve's box
template <class T>
__device__ __forceinline__ bool chunk_site(const BatchArgs<T> &B, const SolveDesc &sd, const ChunkDesc &ch, int t,
                                           int &li, int &x, int &y, int &z)
{
    if (B.tx == 0) {
        li = ch.start + t;
        if (li >= sd.Lx * sd.Ly * sd.Lz) return false;
        const int r = (int)udiv((unsigned)li, (unsigned)sd.Lx, sd.mx);
        x = li - r * sd.Lx;
        z = (int)udiv((unsigned)r, (unsigned)sd.Ly, sd.my);
        y = r - z * sd.Ly;
        return true;
    }
    const int r = (int)udiv((unsigned)ch.start, (unsigned)sd.Lx, sd.mx);
    const int x0 = ch.start - r * sd.Lx;
    const int z0 = (int)udiv((unsigned)r, (unsigned)sd.Ly, sd.my);
    const int y0 = r - z0 * sd.Ly;
    x = x0 + (t & (B.tx - 1));
    y = y0 + ((t >> B.lx) & (B.ty - 1));
    z = z0 + (t >> B.lxy);
    if (x >= sd.Lx || y >= sd.Ly || z >= sd.Lz) return false;
    li = x + sd.Lx * (y + sd.Ly * z);
    return true;
}
template <class T>
__device__ __forceinline__ bool chunk_site(const BatchArgs<T> &B, const SolveDesc &sd, const ChunkDesc &ch, int t,
                                           int &li)
{
    int x, y, z;
    return chunk_site(B, sd, ch, t, li, x, y, z);
}

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
        : BatchAcc(L, sd, li, li % sd.Lx, (li / sd.Lx) % sd.Ly, li / (sd.Lx * sd.Ly))
    {
    }
    __device__ __forceinline__ BatchAcc(const Lat<T> &L, const SolveDesc &sd, int li, int x, int y, int z)
        : Q(L.Q), D(L.D), types(L.types), objs(L.objs + sd.obj_base), P(L.P), i(sd.off + li)
    {
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

constexpr int kBatchWarps = kBlock / 32;  // warp partial sums per chunk

// one set of packed state planes (Q, V, F)
template <class T> struct BatchSet {
    T *Q, *V, *F;
};

// accessor over the predicted Q of a packed solve, formed on the fly from an
// input state set (one-constant forms: no derivative planes)
template <class T> struct BatchPredAcc {
    const T *Q, *V, *F;
    const int8_t *types;
    const ObjDev<T> *objs;
    long long P;
    int i;
    int nb[6];
    PredCoef<T> c;
    __device__ __forceinline__ BatchPredAcc(const Lat<T> &L, const BatchSet<T> &in, const PredCoef<T> &c_,
                                            const SolveDesc &sd, int li, int x, int y, int z)
        : Q(in.Q), V(in.V), F(in.F), types(L.types), objs(L.objs + sd.obj_base), P(L.P), i(sd.off + li), c(c_)
    {
        const int sx = sd.Lx, sy = sd.Lx * sd.Ly;
        nb[0] = i + (x == 0 ? sd.Lx - 1 : -1);
        nb[1] = i + (x == sd.Lx - 1 ? -(sd.Lx - 1) : 1);
        nb[2] = i + (y == 0 ? (sd.Ly - 1) * sx : -sx);
        nb[3] = i + (y == sd.Ly - 1 ? -(sd.Ly - 1) * sx : sx);
        nb[4] = i + (z == 0 ? (sd.Lz - 1) * sy : -sy);
        nb[5] = i + (z == sd.Lz - 1 ? -(sd.Lz - 1) * sy : sy);
    }
    __device__ __forceinline__ T at(int j, int k) const
    {
        const long long o = (long long)k * P + j;
        return pred_q(c, ld(Q + o), pred_v(c, ld(V + o), ld(F + o)));
    }
    __device__ __forceinline__ int tn(int s) const { return types[nb[s]]; }
    __device__ __forceinline__ T q(int k) const { return at(i, k); }
    __device__ __forceinline__ T nq(int s, int k) const { return at(nb[s], k); }
    __device__ __forceinline__ T dn(int, int) const { return T(0); }  // multi-constant forms only
    __device__ __forceinline__ ObjDev<T> obj(int t) const { return objs[t - 1]; }
};

// ----------------------------------------------------- per-chunk phases
// The deferred mix folded into the Verlet coefficients, as k_fire_pred does:
// v' = cvv v + cvf f, q' = q + dt v' (chunk c of an active solve)
template <class T> __device__ __forceinline__ void b_pred_chunk(const BatchArgs<T> &B, const FireDev *fds, int c)
{
    const ChunkDesc ch = B.chunks[c];
    const FireDev &fd = fds[ch.solve];
    if (!fd.active) return;  // uniform per block
    // formed in FP64 by one lane per warp
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
    int li;
    if (!chunk_site(B, sd, ch, threadIdx.x, li)) return;
    const int i = sd.off + li;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const long long j = (long long)k * B.L.P + i;
        const T vn = cvv * B.L.V[j] + cvf * B.L.F[j];
        B.L.V[j] = vn;
        B.L.Q[j] += tdt * vn;
    }
}

// twice the first derivatives of the LC sites the class-1 forms read (see qmin_force_core.cuh)
template <class T> __device__ __forceinline__ void b_derivs_chunk(const BatchArgs<T> &B, const FireDev *fds, int c)
{
    const ChunkDesc ch = B.chunks[c];
    if (fds && !fds[ch.solve].active) return;
    const SolveDesc sd = B.solves[ch.solve];
    int li, x, y, z;
    if (!chunk_site(B, sd, ch, threadIdx.x, li, x, y, z)) return;
    if (B.needd && !B.needd[sd.off + li]) return;
    BatchAcc<T> a(B.L, sd, li, x, y, z);
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

// force (KICK = 0) or force + half kick + the chunk's FIRE reductions (KICK =
// 1): each warp's sums of its 32 sites into partials[3 (kWarps c + warp) ..],
// so that the warps of a block go through their chunks without waiting for
// one another; ONE_CONST: the one-constant form only
template <class T, int KICK, bool ONE_CONST>
__device__ __forceinline__ void b_force_chunk(const BatchArgs<T> &B, const FireDev *fds, double *partials, int c)
{
    const ChunkDesc ch = B.chunks[c];
    if (KICK && !fds[ch.solve].active) return;  // uniform per block
    const SolveDesc sd = B.solves[ch.solve];
    int li, x, y, z;
    const bool in = chunk_site(B, sd, ch, threadIdx.x, li, x, y, z);
    // the site's three dot products in the site precision (FP32 warp sums for
    // the FP32 form, FP64 across warps and chunks)
    T acc[3] = {T(0), T(0), T(0)};
    if (in) {
        const int gi = sd.off + li;
        T f[5];
        if (!ONE_CONST && B.cls && B.cls[gi] == 0) {
            // deep bulk site: the 25-point form over Q, no derivative planes
            deep_force_box(B.L, sd.off, sd.Lx, sd.Ly, sd.Lz, li, (long long)gi, f);
        } else {
            BatchAcc<T> a(B.L, sd, li, x, y, z);
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
        // the warp's sums in the site precision (32 terms), FP64 from there on
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
        if ((threadIdx.x & 31) == 0) {
            double *p = partials + 3 * ((long long)kBatchWarps * c + threadIdx.x / 32);
            p[0] = (double)acc[0];
            p[1] = (double)acc[1];
            p[2] = (double)acc[2];
        }
    }
}

// One fused FIRE iteration of chunk c (one-constant forms): the predicted Q of
// the site and of its six neighbours formed on the fly from the input set, the
// force there, the half kick, the output set written (Q', V', F) and each
// warp's FIRE sums, as b_force_chunk lays them out
template <class T>
__device__ __forceinline__ void b_fused_chunk(const BatchArgs<T> &B, const BatchSet<T> &in, const BatchSet<T> &out,
                                              const FireDev *fds, double *partials, int c)
{
    const ChunkDesc ch = B.chunks[c];
    // coefficients formed in FP64 by one lane per warp
    double cf[3] = {0.0, 0.0, 0.0};
    if ((threadIdx.x & 31) == 0) {
        const FireDev &fd = fds[ch.solve];
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
    const PredCoef<T> pc{T(cf[0]), T(cf[1]), T(cf[2])};
    const T hdt = T(0.5) * T(cf[2]);  // the kick's half step, as b_force_chunk forms it
    const SolveDesc sd = B.solves[ch.solve];
    int li, x, y, z;
    const bool inb = chunk_site(B, sd, ch, threadIdx.x, li, x, y, z);
    T acc[3] = {T(0), T(0), T(0)};
    if (inb) {
        const int gi = sd.off + li;
        const BatchPredAcc<T> a(B.L, in, pc, sd, li, x, y, z);
        T f[5], v[5];
        site_force_core<T, BatchPredAcc<T>, false, false, true>(B.L, a, B.L.types[gi], f);
        const long long P = B.L.P;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const long long o = k * P + gi;
            const T vp = pred_v(pc, ld(in.V + o), ld(in.F + o));
            out.Q[o] = pred_q(pc, ld(in.Q + o), vp);
            v[k] = vp + hdt * f[k];
            out.V[o] = v[k];
            out.F[o] = f[k];
        }
        acc[0] = dot_qt(f, f);
        acc[1] = dot_qt(v, v);
        acc[2] = dot_qt(f, v);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    if ((threadIdx.x & 31) == 0) {
        double *p = partials + 3 * ((long long)kBatchWarps * c + threadIdx.x / 32);
        p[0] = (double)acc[0];
        p[1] = (double)acc[1];
        p[2] = (double)acc[2];
    }
}

// one warp, solve w: deterministic sum of its chunks' partials, then the
// fireStepCPU scalar logic (energyMinimizerFIRE.cpp:104-144) and the loop
// condition of minimize(); returns (in lane 0) whether the solve retired now
__device__ __forceinline__ bool b_control_solve(FireDev *fds, const SolveDesc *solves, int w, const double *partials)
{
    const int lane = threadIdx.x & 31;
    FireDev *fd = fds + w;
    if (!fd->active) return false;  // uniform per warp
    const SolveDesc sd = solves[w];
    double v[3] = {0.0, 0.0, 0.0};
    // eight strides' loads in flight; each lane adds its entries in index order
    constexpr int U = 8;
    const int n = kBatchWarps * sd.nchunks;
    const double *p = partials + 3LL * kBatchWarps * sd.chunk0;
    for (int c0 = lane; c0 < n; c0 += 32 * U) {
        double x[U][3];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int k = 0; k < 3; ++k) x[u][k] = c0 + 32 * u < n ? p[3 * (c0 + 32 * u) + k] : 0.0;
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (c0 + 32 * u < n)
#pragma unroll
                for (int k = 0; k < 3; ++k) v[k] += x[u][k];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane != 0) return false;
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
        return true;
    }
    fd->active = (it < fd->max_iters && fd->forceMax > fd->fcut) ? 1 : 0;
    return !fd->active;
}

// ----------------------------------------------- launch-per-phase kernels
// (the entry force evaluation of every minimize() call, the tuner's timings)
template <class T, int KICK, bool ONE_CONST>
__global__ void __launch_bounds__(kBlock) k_b_force(BatchArgs<T> B, const FireDev *fds, double *partials)
{
    for (int c = blockIdx.x; c < B.nchunks; c += gridDim.x) b_force_chunk<T, KICK, ONE_CONST>(B, fds, partials, c);
}

template <class T> __global__ void __launch_bounds__(kBlock) k_b_derivs(BatchArgs<T> B, const FireDev *fds)
{
    for (int c = blockIdx.x; c < B.nchunks; c += gridDim.x) b_derivs_chunk<T>(B, fds, c);
}

// apply each solve's last deferred velocity mix
template <class T> __global__ void __launch_bounds__(kBlock) k_b_finish(BatchArgs<T> B, FireDev *fds)
{
    for (int c = blockIdx.x; c < B.nchunks; c += gridDim.x) {
        const ChunkDesc ch = B.chunks[c];
        const FireDev &fd = fds[ch.solve];
        if (!fd.pending) continue;
        const SolveDesc sd = B.solves[ch.solve];
        int li;
        if (!chunk_site(B, sd, ch, threadIdx.x, li)) continue;
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

// after a fused run: the solves whose last iteration wrote the second state
// set get their Q, V, F copied back into the first
template <class T>
__global__ void __launch_bounds__(kBlock) k_b_settle(BatchArgs<T> B, BatchSet<T> s1, const int *in_second)
{
    for (int c = blockIdx.x; c < B.nchunks; c += gridDim.x) {
        const ChunkDesc ch = B.chunks[c];
        if (!in_second[ch.solve]) continue;
        const SolveDesc sd = B.solves[ch.solve];
        int li;
        if (!chunk_site(B, sd, ch, threadIdx.x, li)) continue;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const long long j = (long long)k * B.L.P + sd.off + li;
            B.L.Q[j] = s1.Q[j];
            B.L.V[j] = s1.V[j];
            B.L.F[j] = s1.F[j];
        }
    }
}

// ---------------------------------------------------- persistent FIRE loop
// Run state of one persistent launch: grid barrier (arrival count, generation,
// abort flag, spin limit) and, per iteration, the number of solves that retired.
struct BatchRun {
    unsigned count, gen;
    int abort;
    int pad;
    long long spin_limit;
    int retired[3];
    int pad2;
};


// grid-wide barrier between two phases; bounded: a block that has waited
// spin_limit polls raises the abort flag, and every block leaves at its next
// barrier once the flag is up.  Returns false on abort.
__device__ __forceinline__ bool b_grid_sync(BatchRun *run)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &run->gen;
        volatile int *vabort = &run->abort;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&run->count, 1u) == gridDim.x - 1) {
            atomicExch(&run->count, 0u);
            __threadfence();
            atomicAdd(&run->gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                if (*vabort) break;
                if (++spins > run->spin_limit) {
                    atomicExch(&run->abort, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = *vabort == 0;
    }
    __syncthreads();
    return ok != 0;
}

// Every FIRE iteration of every solve in one cooperative launch: predictor,
// (derivative planes,) force + half kick + per-chunk sums, per-solve control,
// a grid barrier after each phase.  The work of a phase is the chunks of the
// active solves: each block holds the same list of active solves and the
// prefix sums of their chunk counts in shared memory, rebuilt (in solve order)
// when a solve retires, so retired solves cost nothing.
constexpr int kMaxBatchSolves = 16384;  // the lists take 8 (nsolves + 1) bytes of shared memory

// (the one-constant forms ask for three blocks per SM, the FP32 multi-constant
// form for two: the force phase would otherwise hold the registers of fewer)
//
// FUSED (FP32 one-constant forms; in FP64 the neighbours' predictions formed
// again at every site cost more FP64 FMAs than the separate predictor phase
// saves): one phase per iteration instead of predictor and force: iteration it reads state set it & 1 (0: B.L's planes, 1: s1) and
// writes the other, forming the predicted Q of every neighbour on the fly
// (b_fused_chunk); a solve that retires leaves in_second[solve] = 1 when its
// final state is in s1 (k_b_settle copies it back)
template <class T, bool ONE_CONST, bool FUSED = false>
__global__ void __launch_bounds__(kBlock, ONE_CONST ? 3 : (sizeof(T) == 4 ? 2 : 1))
    k_b_fire_persistent(BatchArgs<T> B, BatchSet<T> s1, FireDev *fds, double *partials, int *in_second,
                        int nsolves, BatchRun *run)
{
    static_assert(!FUSED || (ONE_CONST && sizeof(T) == 4), "the fused iteration covers the FP32 one-constant forms");
    extern __shared__ int b_lists[];
    int *act = b_lists;                // active solve ids, in solve order
    int *pre = b_lists + nsolves + 1;  // prefix sums of their chunk counts
    __shared__ int n_act;
    __shared__ int all_act;  // every solve active: work item w is chunk w
    auto rebuild = [&]() {
        // one warp: ballot over the solves in order
        if (threadIdx.x < 32) {
            int n = 0, tot = 0;
            for (int s0 = 0; s0 < nsolves; s0 += 32) {
                const int s = s0 + threadIdx.x;
                const bool a = s < nsolves && fds[s].active;
                const int nc = a ? B.solves[s].nchunks : 0;
                const unsigned m = __ballot_sync(0xffffffffu, a);
                int inc = nc;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, inc, o);
                    if (threadIdx.x >= o) inc += v;
                }
                if (a) {
                    const int k = n + __popc(m & ((1u << threadIdx.x) - 1u));
                    act[k] = s;
                    pre[k] = tot + inc - nc;
                }
                n += __popc(m);
                tot += __shfl_sync(0xffffffffu, inc, 31);
            }
            if (threadIdx.x == 0) {
                n_act = n;
                all_act = n == nsolves;
                pre[n] = tot;
            }
        }
        __syncthreads();
    };
    // chunk of work item w: binary search in the prefix sums
    auto chunk_of = [&](int w) {
        if (all_act) return w;
        int lo = 0, hi = n_act - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (pre[mid] <= w) lo = mid;
            else hi = mid - 1;
        }
        return B.solves[act[lo]].chunk0 + (w - pre[lo]);
    };
    rebuild();
    const int nwarps = gridDim.x * (kBlock / 32);
    const int gwarp = blockIdx.x * (kBlock / 32) + threadIdx.x / 32;
    const BatchSet<T> s0{B.L.Q, B.L.V, B.L.F};
    for (int it = 0; n_act > 0; ++it) {
        if (blockIdx.x == 0 && threadIdx.x == 0) run->retired[it % 3] = 0;
        const int nw = pre[n_act];
        if constexpr (FUSED) {
            const BatchSet<T> in = (it & 1) ? s1 : s0, out = (it & 1) ? s0 : s1;
            for (int w = blockIdx.x; w < nw; w += gridDim.x) b_fused_chunk<T>(B, in, out, fds, partials, chunk_of(w));
            if (!b_grid_sync(run)) return;
        } else {
            for (int w = blockIdx.x; w < nw; w += gridDim.x) b_pred_chunk<T>(B, fds, chunk_of(w));
            if (!b_grid_sync(run)) return;
            if (!ONE_CONST && B.L.multi) {
                for (int w = blockIdx.x; w < nw; w += gridDim.x) b_derivs_chunk<T>(B, fds, chunk_of(w));
                if (!b_grid_sync(run)) return;
            }
            for (int w = blockIdx.x; w < nw; w += gridDim.x)
                b_force_chunk<T, 1, ONE_CONST>(B, fds, partials, chunk_of(w));
            if (!b_grid_sync(run)) return;
        }
        // per-solve control, one warp per active solve (its warps' sums added in order)
        for (int k = gwarp; k < n_act; k += nwarps)
            if (b_control_solve(fds, B.solves, act[k], partials) && (threadIdx.x & 31) == 0) {
                atomicAdd(&run->retired[it % 3], 1);
                if (FUSED) in_second[act[k]] = (it & 1) == 0;
            }
        if (!b_grid_sync(run)) return;
        if (*(volatile int *)&run->retired[it % 3] > 0) rebuild();
    }
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
// chunk shapes the tuner tries: 256 consecutive sites, then tiles of the box
constexpr int kShapes = 5;
constexpr int kShape[kShapes][3] = {{0, 0, 0}, {32, 8, 1}, {16, 16, 1}, {16, 4, 4}, {8, 8, 4}};
constexpr long long kDefaultSpinLimit = 1LL << 24;  // about a second of polling at one barrier

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
    void *Q2 = nullptr, *V2 = nullptr, *F2 = nullptr;  // second state set of the fused iteration
    int *in_second = nullptr;                          // per solve: final state in the second set
    int8_t *types = nullptr;
    uint8_t *cls = nullptr, *needd = nullptr;  // per packed site (multi-constant split of the force)
    void *cbd = nullptr;                       // merged boundary coefficients (multi-constant)
    double *partials = nullptr, *stage = nullptr;
    int32_t *stage_t = nullptr;
    FireDev *fds = nullptr;
    std::vector<FireDev> fds_h;
    cudaStream_t stream = nullptr;
    qmin_ldg_params params{};
    bool have_params = false, fire_ready = false;
    int shape = -1;  // chunk shape chosen by the tuner (-1: not tuned; chunks laid out as shape 0)
    int pinned_shape = -1;  // chunk shape the caller pinned (-1: the tuner picks)
    int layout = 0;  // chunk shape the device chunk list is laid out in
    double shape_ms[kShapes] = {-1, -1, -1, -1, -1};
    int max_chunks = 0;  // partials capacity (chunks of the largest layout)
    BatchRun *run = nullptr;
    long long spin_limit = kDefaultSpinLimit;
    long long launches = 0;
};

// chunk list of shape k: every solve's chunks in solve order, tiles in x-fastest order
static void chunk_layout(int k, std::vector<SolveDesc> &solves, std::vector<ChunkDesc> *chunks)
{
    if (chunks) chunks->clear();
    int c0 = 0;
    for (size_t s = 0; s < solves.size(); ++s) {
        SolveDesc &sd = solves[s];
        const int n = sd.Lx * sd.Ly * sd.Lz;
        int nc = 0;
        if (k == 0) {
            nc = (n + kBlock - 1) / kBlock;
            if (chunks)
                for (int c = 0; c < nc; ++c) chunks->push_back({(int)s, c * kBlock});
        } else {
            const int tx = kShape[k][0], ty = kShape[k][1], tz = kShape[k][2];
            for (int z = 0; z < sd.Lz; z += tz)
                for (int y = 0; y < sd.Ly; y += ty)
                    for (int x = 0; x < sd.Lx; x += tx) {
                        if (chunks) chunks->push_back({(int)s, x + sd.Lx * (y + sd.Ly * z)});
                        ++nc;
                    }
        }
        sd.chunk0 = c0;
        sd.nchunks = nc;
        c0 += nc;
    }
}

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
    B.tx = kShape[b->layout][0];
    B.ty = kShape[b->layout][1];
    B.tz = kShape[b->layout][2];
    if (B.tx > 0) {
        B.lx = __builtin_ctz(B.tx);
        B.lxy = __builtin_ctz(B.tx * B.ty);
    }
    return B;
}

// lay the device chunk list out in shape k (solve descriptors included)
static int set_layout(qmin_batch_ctx *b, int k)
{
    if (b->layout == k && b->nchunks > 0) return QMIN_OK;
    chunk_layout(k, b->solves_h, &b->chunks_h);
    b->nchunks = (int)b->chunks_h.size();
    b->layout = k;
    BCK(cudaMemcpyAsync(b->solves, b->solves_h.data(), sizeof(SolveDesc) * b->nsolves, cudaMemcpyHostToDevice,
                        b->stream));
    BCK(cudaMemcpyAsync(b->chunks, b->chunks_h.data(), sizeof(ChunkDesc) * b->nchunks, cudaMemcpyHostToDevice,
                        b->stream));
    return QMIN_OK;
}

static int grid_for(int nchunks) { return std::min(nchunks, 152 * 8); }

// forces (kick = 0: every solve, object sites zero) or force + half kick +
// per-chunk sums of the active solves (kick = 1), launch per phase
template <class T> static int launch_b_force(const BatchArgs<T> &B, const FireDev *fds, double *partials, int kick,
                                             cudaStream_t s)
{
    const int g = grid_for(B.nchunks);
    int n = 0;
    if (B.L.multi) {
        k_b_derivs<T><<<g, kBlock, 0, s>>>(B, kick ? fds : nullptr);
        ++n;
    }
    if (!B.L.multi) {
        if (kick) k_b_force<T, 1, true><<<g, kBlock, 0, s>>>(B, fds, partials);
        else k_b_force<T, 0, true><<<g, kBlock, 0, s>>>(B, fds, partials);
    } else {
        if (kick) k_b_force<T, 1, false><<<g, kBlock, 0, s>>>(B, fds, partials);
        else k_b_force<T, 0, false><<<g, kBlock, 0, s>>>(B, fds, partials);
    }
    return n + 1;
}

// the chunk shape for the force + kick: each shape's launch timed with CUDA
// events on the live batch (mean of three after a warm-up), the velocities the
// kicks change restored afterwards
template <class T> static int tune_shape(qmin_batch_ctx *b)
{
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
    int best_k = 0;
    for (int k = 0; k < kShapes; ++k) {
        int r = set_layout(b, k);
        if (r) return r;
        BatchArgs<T> B = batch_args<T>(b);
        b->launches += launch_b_force<T>(B, b->fds, b->partials, 1, b->stream);
        cudaEventRecord(e0, b->stream);
        for (int rep = 0; rep < 3; ++rep) b->launches += launch_b_force<T>(B, b->fds, b->partials, 1, b->stream);
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        b->shape_ms[k] = ms / 3;
        if (ms < best) {
            best = ms;
            best_k = k;
        }
    }
    BCK(cudaMemcpyAsync(b->V, vb, bytes, cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    cudaFree(vb);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->shape = best_k;
    return set_layout(b, best_k);
}

// the persistent FIRE loop as one cooperative launch of as many blocks as can
// be resident together
template <class T, bool ONE_CONST, bool FUSED>
static int launch_persistent(qmin_batch_ctx *b, const BatchArgs<T> &B)
{
    const size_t smem = sizeof(int) * 2 * ((size_t)b->nsolves + 1);
    auto kern = k_b_fire_persistent<T, ONE_CONST, FUSED>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return bfail(QMIN_ECUDA, "batch: shared memory for the active-solve lists");
    int per_sm = 0, nsm = 0, dev = 0;
    BCK(cudaGetDevice(&dev));
    BCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, smem));
    if (per_sm < 1) return bfail(QMIN_ECUDA, "batch: the persistent kernel does not fit on an SM");
    const int grid = per_sm * nsm;
    BatchArgs<T> a = B;
    BatchSet<T> s1{(T *)b->Q2, (T *)b->V2, (T *)b->F2};
    FireDev *fds = b->fds;
    double *partials = b->partials;
    int *in_second = b->in_second;
    int ns = b->nsolves;
    BatchRun *run = b->run;
    void *args[] = {&a, &s1, &fds, &partials, &in_second, &ns, &run};
    BCK(cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(kBlock), args, smem, b->stream));
    return QMIN_OK;
}

// The API functions below take C linkage from their declarations in qmin_gb300.h.

int qmin_batch_create(int nsolves, const int32_t *dims, int precision, int metric_mode, qmin_batch *out)
{
    if (!out || !dims || nsolves < 1) return bfail(QMIN_EINVAL, "qmin_batch_create: bad argument");
    if (nsolves > kMaxBatchSolves) return bfail(QMIN_EINVAL, "qmin_batch_create: at most 16384 solves per batch");
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
        SolveDesc sd{Lx, Ly, Lz, (int)off, 0, 0, s * kObjPerSolve, 0, div_magic(Lx), div_magic(Ly), {0, 0}};
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
    for (int k = kShapes - 1; k >= 0; --k) {
        chunk_layout(k, b->solves_h, nullptr);
        b->max_chunks = std::max(b->max_chunks, b->solves_h.back().chunk0 + b->solves_h.back().nchunks);
    }
    chunk_layout(0, b->solves_h, &b->chunks_h);
    b->nchunks = (int)b->chunks_h.size();
    b->ntotal_h.assign(nsolves, 0);
    const size_t plane = (size_t)b->P * b->esz;
    bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&b->Q, 5 * plane) == cudaSuccess && cudaMalloc(&b->V, 5 * plane) == cudaSuccess &&
              cudaMalloc(&b->F, 5 * plane) == cudaSuccess && cudaMalloc(&b->types, (size_t)b->P) == cudaSuccess &&
              cudaMalloc(&b->objs, sizeof(ObjDev<double>) * kObjPerSolve * nsolves) == cudaSuccess &&
              cudaMalloc(&b->solves, sizeof(SolveDesc) * nsolves) == cudaSuccess &&
              cudaMalloc(&b->chunks, sizeof(ChunkDesc) * b->max_chunks) == cudaSuccess &&
              cudaMalloc(&b->partials, sizeof(double) * 3 * kBatchWarps * (size_t)b->max_chunks) == cudaSuccess &&
              cudaMalloc(&b->run, sizeof(BatchRun)) == cudaSuccess &&
              cudaMalloc(&b->stage, sizeof(double) * 5 * (size_t)b->maxN) == cudaSuccess &&
              cudaMalloc(&b->stage_t, sizeof(int32_t) * (size_t)b->maxN) == cudaSuccess &&
              cudaMalloc(&b->fds, sizeof(FireDev) * nsolves) == cudaSuccess &&
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
    void *bufs[] = {b->Q, b->V, b->F, b->D, b->objs, b->types, b->partials, b->stage, b->stage_t, b->fds,
                    b->solves, b->chunks, b->cls, b->needd, b->cbd, b->run, b->Q2, b->V2, b->F2, b->in_second};
    for (void *p : bufs)
        if (p) cudaFree(p);
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
    b->shape = -1;  // the chunk shape is tuned afresh for the new force form
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

template <class T> static int batch_fire_impl(qmin_batch_ctx *b, bool *timed_out)
{
    // every solve's minimize() starts with its forces (energyMinimizerFIRE.cpp:157)
    b->launches += launch_b_force<T>(batch_args<T>(b), b->fds, b->partials, 0, b->stream);
    if (b->shape < 0) {
        int r = b->pinned_shape >= 0 ? (b->shape = b->pinned_shape, set_layout(b, b->pinned_shape)) : tune_shape<T>(b);
        if (r) return r;
    }
    BatchRun run;
    memset(&run, 0, sizeof run);
    run.spin_limit = b->spin_limit;
    BCK(cudaMemcpyAsync(b->run, &run, sizeof run, cudaMemcpyHostToDevice, b->stream));
    const BatchArgs<T> B = batch_args<T>(b);
    const bool fused = !B.L.multi && sizeof(T) == 4;
    if (fused && !b->Q2) {
        // the second state set, on the first one-constant run
        const size_t bytes = 5 * (size_t)b->P * b->esz;
        if (cudaMalloc(&b->Q2, bytes) != cudaSuccess || cudaMalloc(&b->V2, bytes) != cudaSuccess ||
            cudaMalloc(&b->F2, bytes) != cudaSuccess ||
            cudaMalloc(&b->in_second, sizeof(int) * (size_t)b->nsolves) != cudaSuccess) {
            cudaGetLastError();
            return bfail(QMIN_ENOMEM, "qmin_batch_fire_run: second state set allocation failed");
        }
    }
    if (fused) BCK(cudaMemsetAsync(b->in_second, 0, sizeof(int) * (size_t)b->nsolves, b->stream));
    int r;
    if constexpr (sizeof(T) == 4)
        r = B.L.multi ? launch_persistent<T, false, false>(b, B) : launch_persistent<T, true, true>(b, B);
    else
        r = B.L.multi ? launch_persistent<T, false, false>(b, B) : launch_persistent<T, true, false>(b, B);
    if (r) return r;
    b->launches += 1;
    BCK(cudaMemcpyAsync(&run, b->run, sizeof run, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    *timed_out = run.abort != 0;
    if (fused) {
        k_b_settle<T><<<grid_for(b->nchunks), kBlock, 0, b->stream>>>(B, BatchSet<T>{(T *)b->Q2, (T *)b->V2,
                                                                                     (T *)b->F2}, b->in_second);
        b->launches += 1;
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
    bool timed_out = false;
    int r = b->prec == QMIN_FP64 ? batch_fire_impl<double>(b, &timed_out) : batch_fire_impl<float>(b, &timed_out);
    if (r) return r;
    BCK(cudaMemcpyAsync(b->fds_h.data(), b->fds, sizeof(FireDev) * b->nsolves, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    if (timed_out) {
        // every solve still active records the timeout in its status word and stops
        for (int s = 0; s < b->nsolves; ++s) {
            FireDev &f = b->fds_h[s];
            if (f.active) {
                f.status = QMIN_ETIMEOUT;
                f.active = 0;
            }
            if (iterations) iterations[s] = f.iterations;
            if (force_max) force_max[s] = f.forceMax;
        }
        BCK(cudaMemcpyAsync(b->fds, b->fds_h.data(), sizeof(FireDev) * b->nsolves, cudaMemcpyHostToDevice,
                            b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        return bfail(QMIN_ETIMEOUT, "qmin_batch_fire_run: a grid barrier of the persistent FIRE loop gave up "
                                    "(solves still running are marked; their state is that of an unfinished "
                                    "iteration: set them again before another run)");
    }
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

int qmin_batch_set_barrier_limit(qmin_batch b, long long spins)
{
    if (!b || spins < 0) return bfail(QMIN_EINVAL, "qmin_batch_set_barrier_limit: bad argument");
    b->spin_limit = spins == 0 ? kDefaultSpinLimit : spins;
    return QMIN_OK;
}

int qmin_batch_set_chunk_shape(qmin_batch b, int shape)
{
    if (!b || shape < -1 || shape >= kShapes) return bfail(QMIN_EINVAL, "qmin_batch_set_chunk_shape: bad argument");
    b->pinned_shape = shape;
    b->shape = -1;  // applied (or tuned) at the next run
    return QMIN_OK;
}

int qmin_batch_tuning(qmin_batch b, int *shape, int tile[3], double ms[5])
{
    if (!b) return bfail(QMIN_EINVAL, "qmin_batch_tuning: null handle");
    if (shape) *shape = b->shape;
    if (tile)
        for (int k = 0; k < 3; ++k) tile[k] = b->shape >= 0 ? kShape[b->shape][k] : 0;
    if (ms)
        for (int k = 0; k < kShapes; ++k) ms[k] = b->shape_ms[k];
    return QMIN_OK;
}

int qmin_batch_kernel_launches(qmin_batch b, long long *count)
{
    if (!b || !count) return bfail(QMIN_EINVAL, "qmin_batch_kernel_launches: null argument");
    *count = b->launches;
    return QMIN_OK;
}

