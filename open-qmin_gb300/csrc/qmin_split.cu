// Split force + kick for the multi-constant form: deep bulk sites without
// derivative planes, every other LC site through the derivative-plane path.
//
// A deep bulk site (type 0 with six type-0 neighbours) sees central
// differences in all six neighbours' derivatives, so its combined bulk form
// (L1-L4, landauDeGennesLCDistortionTerms.cpp:113-198 with lcForces.h's
// bulk forms) is the same linear form written over Q at the 25 sites within
// two steps (qmin_bulk_q25.h); no derivative plane is read.  The remaining LC
// sites (next to an object, or next to such a site) are a short list that
// keeps the plane-based forms; their derivative planes are refreshed only at
// the sites that list reads.  Results equal the separate kernels' to rounding.
#include <algorithm>
#include <type_traits>

#include "qmin_force_core.cuh"

namespace qmin {

namespace {

// force at the predicted Q of a deep bulk site of the lattice
template <class T>
__device__ __forceinline__ void deep_force(const Lat<T> &L, int i, T *f)
{
    deep_force_box(L, 0, L.Lx, L.Ly, L.Lz, i, (long long)i, f);
}

template <class T>
__device__ __forceinline__ void kick_and_sum(const Lat<T> &L, long long i, T hdt, const T *f, double *acc)
{
    T v[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        v[k] = L.V[k * L.P + i] + hdt * f[k];
        L.F[k * L.P + i] = f[k];
        L.V[k * L.P + i] = v[k];
    }
    if constexpr (sizeof(T) == 8) {
        dot3_acc(f, v, acc);
    } else {
        acc[0] += (double)dot_qt(f, f);
        acc[1] += (double)dot_qt(v, v);
        acc[2] += (double)dot_qt(f, v);
    }
}

int list_grid(int n) { return std::max(1, std::min((n + kBlock - 1) / kBlock, 152 * 4)); }

// the device's greatest stream priority (the lowest number)
int high_priority()
{
    static int prio = [] {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        return greatest;
    }();
    return prio;
}

// A list kernel launched with the greatest priority as a launch attribute: the
// block scheduler then places its blocks ahead of the deep-site kernel's pending
// blocks, so that the two overlap.  Graphs keep the attribute on the kernel
// node (they are instantiated to honour per-node priorities).
template <class... P, class... A>
void launch_high(void (*kern)(P...), int grid, cudaStream_t s, A &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kBlock);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = high_priority();
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

}  // namespace

// every deep bulk site (cls == 0); partials[0 .. gridDim.x).  KICK = false:
// forces only (no FIRE state), object sites' forces set to zero
template <class T, int CAP, bool KICK = true>
__global__ void __launch_bounds__(kBlock, CAP + 1)
    k_force_kick_deep(Lat<T> L, const uint8_t *__restrict__ cls, const FireDev *__restrict__ fd, double *partials)
{
    if (KICK && !fd->active) return;
    const T hdt = KICK ? T(0.5) * T(fd->dt) : T(0);
    double acc[3] = {0.0, 0.0, 0.0};
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        const int c = cls[i];
        if (!KICK && c == 2)
#pragma unroll
            for (int k = 0; k < 5; ++k) L.F[k * L.P + i] = T(0);
        if (c != 0) continue;
        T f[5];
        deep_force(L, i, f);
        if constexpr (KICK) {
            kick_and_sum(L, i, hdt, f, acc);
        } else {
#pragma unroll
            for (int k = 0; k < 5; ++k) L.F[k * L.P + i] = f[k];
        }
    }
    if constexpr (KICK) {
        block_sum<3>(acc);
        if (threadIdx.x == 0)
#pragma unroll
            for (int k = 0; k < 3; ++k) partials[3 * blockIdx.x + k] = acc[k];
    }
}

// the listed LC sites through the derivative-plane forms (KICK = false: forces only)
template <class T, bool KICK = true>
__global__ void __launch_bounds__(kBlock)
    k_force_kick_list(Lat<T> L, const int *__restrict__ list, int n, const FireDev *__restrict__ fd, double *partials)
{
    if (KICK && !fd->active) return;
    const T hdt = KICK ? T(0.5) * T(fd->dt) : T(0);
    double acc[3] = {0.0, 0.0, 0.0};
    for (int e = blockIdx.x * kBlock + threadIdx.x; e < n; e += gridDim.x * kBlock) {
        const int i = list[e];
        T f[5];
        site_force<T, false, true>(L, i, f);
        if constexpr (KICK) {
            kick_and_sum(L, i, hdt, f, acc);
        } else {
#pragma unroll
            for (int k = 0; k < 5; ++k) L.F[k * L.P + i] = f[k];
        }
    }
    if constexpr (KICK) {
        block_sum<3>(acc);
        if (threadIdx.x == 0)
#pragma unroll
            for (int k = 0; k < 3; ++k) partials[3 * blockIdx.x + k] = acc[k];
    }
}

// twice the first derivatives (k_derivs' rules) at the listed sites only
template <class T>
__global__ void __launch_bounds__(kBlock)
    k_derivs_list(Lat<T> L, const int *__restrict__ list, int n, const FireDev *__restrict__ fd)
{
    if (fd && !fd->active) return;  // fd null: a force-only evaluation
    const long long P = L.P;
    for (int e = blockIdx.x * kBlock + threadIdx.x; e < n; e += gridDim.x * kBlock) {
        const int i = list[e];
        const int t = L.types[i];
        const Nb b = neighbours(L, i);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int dn = b.n[2 * ax], up = b.n[2 * ax + 1];
            const int td = t < 0 ? L.types[dn] : 0, tu = t < 0 ? L.types[up] : 0;
#pragma unroll
            for (int k = 0; k < 5; ++k)
                L.D[(5 * ax + k) * P + i] =
                    deriv2_rule(t, td, tu, ld(L.Q + k * P + dn), ld(L.Q + k * P + i), ld(L.Q + k * P + up));
        }
    }
}

// Deep bulk sites from shared memory: a block owns a TX x TY column and walks
// zc planes, keeping Q of the tile plus a two-site halo in a ring of six planes
// (z-2 .. z+2 in use, z+3 arriving by cp.async while z is computed).
namespace {
template <class T> __device__ __forceinline__ void cp_async_q(T *smem, const T *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ int wrap_any(int v, int m)
{
    int r = v % m;
    return r < 0 ? r + m : r;
}
constexpr int kDeepNS = 6, kDeepZc = 8;
template <class T, int TX, int TY> constexpr size_t deep_tiled_smem()
{
    return (size_t)kDeepNS * 5 * (TX + 4) * (TY + 4) * sizeof(T);
}
// FP64 keeps 2 blocks (16 warps) per SM, FP32 4 (32 warps)
template <class T> constexpr int deep_tiled_minb() { return sizeof(T) == 4 ? 4 : 2; }
}  // namespace

// site of thread t in a TX-wide tile.  A warp covers 32 x 1 sites of a 32-wide
// tile, 4 x 8 sites of a 16-wide one: with the staged rows TX + 4 = 20 words
// apart, the 8 rows of 4 fall into disjoint shared-memory banks for every
// stencil offset (a 16 x 2 footprint would put 4 banks of its two rows together).
template <int TX> __device__ __forceinline__ void tile_site(int t, int &lx, int &ly)
{
    constexpr int WX = TX >= 32 ? 32 : 4, WY = 32 / WX, NWX = TX / WX;
    const int lane = t & 31, w = t >> 5;
    lx = (w % NWX) * WX + lane % WX;
    ly = (w / NWX) * WY + lane / WX;
}

// force of a deep bulk site from its Q and its combined bulk form s2, M
// applied as for type-0 sites (twice in CPU mode, the fields between the two)
template <class T>
__device__ __forceinline__ void deep_force_finish(const Lat<T> &L, const T *q, const T *s2, long long i, T *f)
{
    phase_force_sub(L.a, L.b, L.c, q, s2, f);
    if (L.metric_mode == 0 && !L.efield && !L.hfield && !L.Hv) {
        metric2(f);
        return;
    }
    if (L.metric_mode == 0) metric(f);
    if (L.efield)
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] -= L.fE[k];
    if (L.hfield)
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] -= L.fH[k];
    T h[3];
    if (const T *hs = site_field(L, i, h)) {
        const T hx = hs[0], hy = hs[1], hz = hs[2], fp = L.hvp;
        f[0] -= T(-0.5) * fp * (hx * hx - hz * hz);
        f[1] -= -fp * hx * hy;
        f[2] -= -fp * hx * hz;
        f[3] -= T(-0.5) * fp * (hy * hy - hz * hz);
        f[4] -= -fp * hy * hz;
    }
    metric(f);
}

// force of a deep bulk site from Q staged in shared memory: plane dz of the
// site's column starts at sb[dz + 2], components TS apart, rows SX apart
template <class T, int TS, int SX>
__device__ __forceinline__ void deep_force_tile(const Lat<T> &L, const T *sQ, const int (&sb)[5], long long i, T *f)
{
#define QQ(dx, dy, dz, c) sQ[sb[(dz) + 2] + (c) * TS + (dy) * SX + (dx)]
    T q[5], s2[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) q[k] = QQ(0, 0, 0, k);
    if (L.L4 == T(0)) {
        QMIN_BULK_Q25_NO_L4(L.cq, s2);
    } else {
        QMIN_BULK_Q25(L.cq, s2);
    }
#undef QQ
    deep_force_finish(L, q, s2, i, f);
}

// the same for the two x-adjacent sites of an even-aligned pair (site indices
// i and ib): every value comes from a float2 load of an aligned pair of x
// positions (one load serves both sites wherever their stencils overlap)
template <int TS, int SX>
__device__ __forceinline__ void deep_force_pair_tile(const Lat<float> &L, const float *sQ, const int (&sb)[5],
                                                     long long i, long long ib, float *fa, float *fb)
{
#define QMIN_LD2(dz, off) (*reinterpret_cast<const float2 *>(sQ + sb[(dz) + 2] + (off)))
#define QMIN_EVEN(dx) ((dx) >= 0 ? ((dx) & ~1) : -((1 - (dx)) & ~1))
#define QMIN_PICK(v, e) ((e) ? (v).y : (v).x)
#define QQ(dx, dy, dz, c) QMIN_PICK(QMIN_LD2(dz, (c) * TS + (dy) * SX + QMIN_EVEN(dx)), (dx) & 1)
    float qa[5], sa[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) qa[k] = QQ(0, 0, 0, k);
    if (L.L4 == 0.f) {
        QMIN_BULK_Q25_NO_L4(L.cq, sa);
    } else {
        QMIN_BULK_Q25(L.cq, sa);
    }
#undef QQ
#define QQ(dx, dy, dz, c) QMIN_PICK(QMIN_LD2(dz, (c) * TS + (dy) * SX + QMIN_EVEN((dx) + 1)), ((dx) + 1) & 1)
    float qb[5], sbv[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) qb[k] = QQ(0, 0, 0, k);
    if (L.L4 == 0.f) {
        QMIN_BULK_Q25_NO_L4(L.cq, sbv);
    } else {
        QMIN_BULK_Q25(L.cq, sbv);
    }
#undef QQ
#undef QMIN_PICK
#undef QMIN_EVEN
#undef QMIN_LD2
    deep_force_finish(L, qa, sa, i, fa);
    deep_force_finish(L, qb, sbv, ib, fb);
}

template <class T, int TX, int TY>
__global__ void __launch_bounds__(TX *TY, deep_tiled_minb<T>())
    k_force_kick_deep_tiled(Lat<T> L, const uint8_t *__restrict__ cls, const FireDev *__restrict__ fd,
                            double *partials, int zc)
{
    constexpr int NT = TX * TY, SX = TX + 4, TS = SX * (TY + 4), NS = kDeepNS;
    constexpr int NPOS = (TS + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sQ = reinterpret_cast<T *>(smem_raw);  // [NS][5][TS]
    if (!fd->active) return;
    const T hdt = T(0.5) * T(fd->dt);
    const int ntx = (L.Lx + TX - 1) / TX;
    const int gx0 = (blockIdx.x % ntx) * TX, gy0 = (blockIdx.x / ntx) * TY;
    const int zs = blockIdx.y * zc, ze = min(L.Lz, zs + zc);
    const long long P = L.P;
    const int sxy = L.Lx * L.Ly;
    int off[NPOS];
#pragma unroll
    for (int j = 0; j < NPOS; ++j) {
        const int pp = threadIdx.x + j * NT;
        off[j] = pp < TS ? wrap_any(gx0 + pp % SX - 2, L.Lx) + L.Lx * wrap_any(gy0 + pp / SX - 2, L.Ly) : -1;
    }
    auto slot_of = [&](int z) { return (z - zs + 2) % NS; };  // z >= zs - 2
    auto issue = [&](int z) {
        const int sl = slot_of(z);
        const long long base = (long long)sxy * wrap_any(z, L.Lz);
#pragma unroll
        for (int j = 0; j < NPOS; ++j) {
            if (off[j] < 0) continue;
            const int pp = threadIdx.x + j * NT;
#pragma unroll
            for (int k = 0; k < 5; ++k) cp_async_q(&sQ[(sl * 5 + k) * TS + pp], L.Q + k * P + base + off[j]);
        }
    };
    // per-thread sums over the column in the site precision (at most a few
    // tens of terms, each already rounded to it), FP64 across threads and blocks
    using Acc = typename std::conditional<sizeof(T) == 4, float, double>::type;
    Acc sacc[3] = {Acc(0), Acc(0), Acc(0)};
    if (zs < L.Lz) {
        for (int z = zs - 2; z <= zs + 2; ++z) {
            issue(z);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        int lx, ly;
        tile_site<TX>(threadIdx.x, lx, ly);
        const int gx = gx0 + lx, gy = gy0 + ly;
        const bool inside = gx < L.Lx && gy < L.Ly;
        const long long i0 = (long long)gx + (long long)L.Lx * gy;
        const int p = (ly + 2) * SX + (lx + 2);
        // class and velocity of the next plane's site, loaded one plane ahead
        uint8_t c_next = 1;
        T v_next[5];
        auto fetch = [&](int z) {
            c_next = 1;
            if (inside && z < ze) {
                const long long i = i0 + (long long)sxy * z;
                c_next = cls[i];
#pragma unroll
                for (int k = 0; k < 5; ++k) v_next[k] = L.V[k * P + i];
            }
        };
        fetch(zs);
        for (int z = zs; z < ze; ++z) {
            if (z + 3 <= ze + 1) issue(z + 3);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            const uint8_t c_here = c_next;
            T v_here[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) v_here[k] = v_next[k];
            fetch(z + 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            __syncthreads();
            const long long i = i0 + (long long)sxy * z;
            if (c_here == 0) {
                int sb[5];
#pragma unroll
                for (int d = 0; d < 5; ++d) sb[d] = slot_of(z + d - 2) * 5 * TS + p;
                T f[5];
                deep_force_tile<T, TS, SX>(L, sQ, sb, i, f);
                T v[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    v[k] = v_here[k] + hdt * f[k];
                    L.F[k * P + i] = f[k];
                    L.V[k * P + i] = v[k];
                }
                sacc[0] += (Acc)dot_qt(f, f);
                sacc[1] += (Acc)dot_qt(v, v);
                sacc[2] += (Acc)dot_qt(f, v);
            }
            __syncthreads();
        }
    }
    double acc[3] = {(double)sacc[0], (double)sacc[1], (double)sacc[2]};
    block_sum<3, NT>(acc);
    if (threadIdx.x == 0) {
        const int b = blockIdx.y * gridDim.x + blockIdx.x;
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[3 * b + k] = acc[k];
    }
}

// FP32 deep sites two per thread: thread (px, ly) of a TX x TY tile owns the
// x-adjacent sites 2 px and 2 px + 1, reads every staged value as an aligned
// float2 (a half-warp reads one 32-word row: no bank conflicts) and shares the
// loads where the two stencils overlap.  Staging and plane ring as in
// k_force_kick_deep_tiled.
template <int TX, int TY, int MINB, bool KICK = true>
__global__ void __launch_bounds__(TX / 2 * TY, MINB)
    k_force_kick_deep_pair(Lat<float> L, const uint8_t *__restrict__ cls, const FireDev *__restrict__ fd,
                           double *partials, int zc)
{
    static_assert(TX % 2 == 0 && (TX + 4) % 2 == 0, "pairs need even rows");
    constexpr int NT = TX / 2 * TY, SX = TX + 4, TS = SX * (TY + 4), NS = kDeepNS;
    constexpr int NPOS = (TS + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sQ = reinterpret_cast<float *>(smem_raw);  // [NS][5][TS]
    if (KICK && !fd->active) return;
    const float hdt = KICK ? 0.5f * float(fd->dt) : 0.f;
    const int ntx = (L.Lx + TX - 1) / TX;
    const int gx0 = (blockIdx.x % ntx) * TX, gy0 = (blockIdx.x / ntx) * TY;
    const int zs = blockIdx.y * zc, ze = min(L.Lz, zs + zc);
    const long long P = L.P;
    const int sxy = L.Lx * L.Ly;
    int off[NPOS];
#pragma unroll
    for (int j = 0; j < NPOS; ++j) {
        const int pp = threadIdx.x + j * NT;
        off[j] = pp < TS ? wrap_any(gx0 + pp % SX - 2, L.Lx) + L.Lx * wrap_any(gy0 + pp / SX - 2, L.Ly) : -1;
    }
    auto slot_of = [&](int z) { return (z - zs + 2) % NS; };  // z >= zs - 2
    auto issue = [&](int z) {
        const int sl = slot_of(z);
        const long long base = (long long)sxy * wrap_any(z, L.Lz);
#pragma unroll
        for (int j = 0; j < NPOS; ++j) {
            if (off[j] < 0) continue;
            const int pp = threadIdx.x + j * NT;
#pragma unroll
            for (int k = 0; k < 5; ++k) cp_async_q(&sQ[(sl * 5 + k) * TS + pp], L.Q + k * P + base + off[j]);
        }
    };
    float sacc[3] = {0.f, 0.f, 0.f};
    if (zs < L.Lz) {
        for (int z = zs - 2; z <= zs + 2; ++z) {
            issue(z);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        const int px = threadIdx.x % (TX / 2), ly = threadIdx.x / (TX / 2);
        const int gx = gx0 + 2 * px, gy = gy0 + ly;
        // sites a = (gx, gy) and b = (gx + 1, gy); b may lie past an odd Lx
        const bool in_a = gx < L.Lx && gy < L.Ly, in_b = gx + 1 < L.Lx && gy < L.Ly;
        const long long i0 = (long long)gx + (long long)L.Lx * gy;
        const int p = (ly + 2) * SX + (2 * px + 2);
        uint8_t ca_next = 1, cb_next = 1;
        float va_next[5], vb_next[5];
        auto fetch = [&](int z) {
            ca_next = cb_next = 1;
            if (z < ze) {
                const long long i = i0 + (long long)sxy * z;
                if (in_a) {
                    ca_next = cls[i];
                    if (KICK)
#pragma unroll
                        for (int k = 0; k < 5; ++k) va_next[k] = L.V[k * P + i];
                }
                if (in_b) {
                    cb_next = cls[i + 1];
                    if (KICK)
#pragma unroll
                        for (int k = 0; k < 5; ++k) vb_next[k] = L.V[k * P + i + 1];
                }
            }
        };
        fetch(zs);
        for (int z = zs; z < ze; ++z) {
            if (z + 3 <= ze + 1) issue(z + 3);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            const uint8_t ca = ca_next, cb = cb_next;
            float va[5], vb[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                va[k] = va_next[k];
                vb[k] = vb_next[k];
            }
            fetch(z + 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            __syncthreads();
            if (!KICK) {
                // forces only: object sites get zero force
                const long long i = i0 + (long long)sxy * z;
                if (ca == 2)
#pragma unroll
                    for (int k = 0; k < 5; ++k) L.F[k * P + i] = 0.f;
                if (cb == 2)
#pragma unroll
                    for (int k = 0; k < 5; ++k) L.F[k * P + i + 1] = 0.f;
            }
            if (ca == 0 || cb == 0) {
                const long long i = i0 + (long long)sxy * z;
                int sb[5];
#pragma unroll
                for (int d = 0; d < 5; ++d) sb[d] = slot_of(z + d - 2) * 5 * TS + p;
                float fa[5], fb[5];
                // b past the lattice's x edge: computed and dropped, its field read at a
                deep_force_pair_tile<TS, SX>(L, sQ, sb, i, in_b ? i + 1 : i, fa, fb);
                if (ca == 0) {
#pragma unroll
                    for (int k = 0; k < 5; ++k) L.F[k * P + i] = fa[k];
                    if (KICK) {
#pragma unroll
                        for (int k = 0; k < 5; ++k) {
                            va[k] += hdt * fa[k];
                            L.V[k * P + i] = va[k];
                        }
                        sacc[0] += dot_qt(fa, fa);
                        sacc[1] += dot_qt(va, va);
                        sacc[2] += dot_qt(fa, va);
                    }
                }
                if (cb == 0) {
#pragma unroll
                    for (int k = 0; k < 5; ++k) L.F[k * P + i + 1] = fb[k];
                    if (KICK) {
#pragma unroll
                        for (int k = 0; k < 5; ++k) {
                            vb[k] += hdt * fb[k];
                            L.V[k * P + i + 1] = vb[k];
                        }
                        sacc[0] += dot_qt(fb, fb);
                        sacc[1] += dot_qt(vb, vb);
                        sacc[2] += dot_qt(fb, vb);
                    }
                }
            }
            __syncthreads();
        }
    }
    if constexpr (KICK) {
        double acc[3] = {(double)sacc[0], (double)sacc[1], (double)sacc[2]};
        block_sum<3, NT>(acc);
        if (threadIdx.x == 0) {
            const int b = blockIdx.y * gridDim.x + blockIdx.x;
#pragma unroll
            for (int k = 0; k < 3; ++k) partials[3 * b + k] = acc[k];
        }
    }
}

// TMA staging for the two-sites-per-thread kernel.  An interior tile (its
// halo inside the lattice, no periodic wrap) takes each plane of Q as one
// cp.async.bulk.tensor box of (TX + 8) x (TY + 4) sites x 5 components,
// starting at x = gx0 - 4 so that the box's x coordinate is 16-byte aligned;
// one thread issues it against an mbarrier per ring slot.  Tiles on the
// lattice's x or y faces stage the same box with cp.async and the periodic
// wrap.  Waits are bounded: a wait that gives up sets *err, lets the copies in
// flight land (bounded again) and leaves the block's partials unwritten.
namespace {
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait (about a second at most at the default poll count); the ring's
// waits for the next planes poll g_split_wait_limit times (split_set_wait_limit)
__device__ int g_split_wait_limit = kSplitWaitPolls;
__device__ __forceinline__ bool mbar_wait(uint64_t *b, unsigned parity, int polls = kSplitWaitPolls)
{
    for (int it = 0; it < polls; ++it)
        if (mbar_try_wait(b, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(smem_addr(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}
template <int TX, int TY> constexpr size_t deep_pair_tma_smem()
{
    return (size_t)kDeepNS * 5 * (TX + 8) * (TY + 4) * sizeof(float) + kDeepNS * sizeof(uint64_t) + 128;
}
}  // namespace

template <int TX, int TY, int MINB, bool KICK>
__global__ void __launch_bounds__(TX / 2 * TY, MINB)
    k_force_kick_deep_pair_tma(Lat<float> L, const __grid_constant__ CUtensorMap tmap, const uint8_t *__restrict__ cls,
                               const FireDev *__restrict__ fd, double *partials, int zc, int *err)
{
    constexpr int NT = TX / 2 * TY, SX = TX + 8, ROWS = TY + 4, TS = SX * ROWS, NS = kDeepNS;
    constexpr int NPOS = (TS + NT - 1) / NT;
    constexpr unsigned kSlotBytes = 5u * TS * sizeof(float);
    static_assert(kSlotBytes % 128 == 0, "ring slots stay 128-byte aligned");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // TMA boxes land on 128-byte boundaries: round the dynamic area up (128 bytes spare are allocated)
    unsigned char *smem_al = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    float *sQ = reinterpret_cast<float *>(smem_al);                   // [NS][5][ROWS][SX]
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_al + NS * kSlotBytes);
    if (KICK && !fd->active) return;
    const float hdt = KICK ? 0.5f * float(fd->dt) : 0.f;
    const int polls = *(volatile int *)&g_split_wait_limit;
    const int ntx = (L.Lx + TX - 1) / TX;
    const int gx0 = (blockIdx.x % ntx) * TX, gy0 = (blockIdx.x / ntx) * TY;
    const int zs = blockIdx.y * zc, ze = min(L.Lz, zs + zc);
    const long long P = L.P;
    const int sxy = L.Lx * L.Ly;
    // the box [gx0 - 4, gx0 + TX + 4) x [gy0 - 2, gy0 + TY + 2) lies inside the lattice
    const bool use_tma = gx0 >= 4 && gx0 + TX + 4 <= L.Lx && gy0 >= 2 && gy0 + TY + 2 <= L.Ly;
    if (zs >= L.Lz) return;
    if (use_tma && threadIdx.x == 0) {
        for (int k = 0; k < NS; ++k) mbar_init(&bar[k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    int off[NPOS];
#pragma unroll
    for (int j = 0; j < NPOS; ++j) {
        const int pp = threadIdx.x + j * NT;
        off[j] = (!use_tma && pp < TS)
                     ? wrap_any(gx0 - 4 + pp % SX, L.Lx) + L.Lx * wrap_any(gy0 - 2 + pp / SX, L.Ly)
                     : -1;
    }
    auto slot_of = [&](int z) { return (z - zs + 2) % NS; };            // z >= zs - 2
    auto parity_of = [&](int z) { return (unsigned)((z - zs + 2) / NS) & 1u; };
    auto issue = [&](int z) {
        const int sl = slot_of(z);
        if (use_tma) {
            if (threadIdx.x == 0) {
                mbar_expect_tx(&bar[sl], kSlotBytes);
                tma_load_4d(sQ + sl * 5 * TS, &tmap, gx0 - 4, gy0 - 2, wrap_any(z, L.Lz), 0, &bar[sl]);
            }
        } else {
            const long long base = (long long)sxy * wrap_any(z, L.Lz);
#pragma unroll
            for (int j = 0; j < NPOS; ++j) {
                if (off[j] < 0) continue;
                const int pp = threadIdx.x + j * NT;
#pragma unroll
                for (int k = 0; k < 5; ++k) cp_async_q(&sQ[(sl * 5 + k) * TS + pp], L.Q + k * P + base + off[j]);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    int issued = zs + 2, waited = zs - 3;  // planes issued / known complete (TMA)
    float sacc[3] = {0.f, 0.f, 0.f};
    bool aborted = false;
    for (int z = zs - 2; z <= zs + 2; ++z) issue(z);
    const int px = threadIdx.x % (TX / 2), ly = threadIdx.x / (TX / 2);
    const int gx = gx0 + 2 * px, gy = gy0 + ly;
    const bool in_a = gx < L.Lx && gy < L.Ly, in_b = gx + 1 < L.Lx && gy < L.Ly;
    const long long i0 = (long long)gx + (long long)L.Lx * gy;
    const int p = (ly + 2) * SX + (2 * px + 4);
    uint8_t ca_next = 1, cb_next = 1;
    float va_next[5], vb_next[5];
    auto fetch = [&](int z) {
        ca_next = cb_next = 1;
        if (z < ze) {
            const long long i = i0 + (long long)sxy * z;
            if (in_a) {
                ca_next = cls[i];
                if (KICK)
#pragma unroll
                    for (int k = 0; k < 5; ++k) va_next[k] = L.V[k * P + i];
            }
            if (in_b) {
                cb_next = cls[i + 1];
                if (KICK)
#pragma unroll
                    for (int k = 0; k < 5; ++k) vb_next[k] = L.V[k * P + i + 1];
            }
        }
    };
    fetch(zs);
    for (int z = zs; z < ze; ++z) {
        if (z + 3 <= ze + 1) {
            issue(z + 3);
            issued = z + 3;
        } else {
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        const uint8_t ca = ca_next, cb = cb_next;
        float va[5], vb[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            va[k] = va_next[k];
            vb[k] = vb_next[k];
        }
        fetch(z + 1);
        bool ok = true;
        if (use_tma) {
            for (int w = waited + 1; w <= z + 2 && ok; ++w) ok = mbar_wait(&bar[slot_of(w)], parity_of(w), polls);
            if (ok) waited = z + 2;
        } else {
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        }
        if (__syncthreads_or(!ok)) {
            aborted = true;
            break;
        }
        if (!KICK) {
            const long long i = i0 + (long long)sxy * z;
            if (ca == 2)
#pragma unroll
                for (int k = 0; k < 5; ++k) L.F[k * P + i] = 0.f;
            if (cb == 2)
#pragma unroll
                for (int k = 0; k < 5; ++k) L.F[k * P + i + 1] = 0.f;
        }
        if (ca == 0 || cb == 0) {
            const long long i = i0 + (long long)sxy * z;
            int sb[5];
#pragma unroll
            for (int d = 0; d < 5; ++d) sb[d] = slot_of(z + d - 2) * 5 * TS + p;
            float fa[5], fb[5];
            deep_force_pair_tile<TS, SX>(L, sQ, sb, i, in_b ? i + 1 : i, fa, fb);
            if (ca == 0) {
#pragma unroll
                for (int k = 0; k < 5; ++k) L.F[k * P + i] = fa[k];
                if (KICK) {
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        va[k] += hdt * fa[k];
                        L.V[k * P + i] = va[k];
                    }
                    sacc[0] += dot_qt(fa, fa);
                    sacc[1] += dot_qt(va, va);
                    sacc[2] += dot_qt(fa, va);
                }
            }
            if (cb == 0) {
#pragma unroll
                for (int k = 0; k < 5; ++k) L.F[k * P + i + 1] = fb[k];
                if (KICK) {
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        vb[k] += hdt * fb[k];
                        L.V[k * P + i + 1] = vb[k];
                    }
                    sacc[0] += dot_qt(fb, fb);
                    sacc[1] += dot_qt(vb, vb);
                    sacc[2] += dot_qt(fb, vb);
                }
            }
        }
        __syncthreads();
    }
    if (aborted) {
        // let the boxes still in flight land before the block's shared memory
        // goes away (at the default poll count, whatever the limit)
        if (use_tma && threadIdx.x == 0) {
            for (int w = waited + 1; w <= issued; ++w) mbar_wait(&bar[slot_of(w)], parity_of(w));
            atomicExch(err, 1);
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        return;
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if constexpr (KICK) {
        double acc[3] = {(double)sacc[0], (double)sacc[1], (double)sacc[2]};
        block_sum<3, NT>(acc);
        if (threadIdx.x == 0) {
            const int b = blockIdx.y * gridDim.x + blockIdx.x;
#pragma unroll
            for (int k = 0; k < 3; ++k) partials[3 * b + k] = acc[k];
        }
    }
}

// ------------------------------------------------ fused predictor + force + kick
// One launch per FIRE iteration for the deep bulk sites, the velocity-Verlet
// predictor included: a block owns a TX x TY column of the lattice and walks
// zc planes.  For each plane it loads raw Q, V, F of the tile plus a one-site
// halo (every deep site's combined L1-L4 form reads only the 19 sites within
// one step along an axis or a face diagonal: the two-step axis terms of the
// 25-point form all have zero coefficients), applies the predictor (the
// deferred FIRE mix and the Verlet step, k_fire_pred's arithmetic) and keeps
// the predicted Q in a ring of four planes in shared memory; the force of the
// plane below then reads planes z-1, z, z+1 of the ring.  Each thread owns one
// site of the tile; threads 0 .. NH-1 also own one halo position.  Input is
// one buffer set (L.Q, L.V, L.F), output the other (Qo, Vo, Fo): predicted Q
// of every site of the tile, V and F of the deep sites (object sites:
// V = F = 0; listed sites: k_force_kick_list_pred).
template <int TX, int TY> __host__ __device__ constexpr int fused_halo_count() { return 2 * (TX + 2) + 2 * TY; }

// position of halo entry h (< fused_halo_count) in the (TX + 2) x (TY + 2) staged plane
template <int TX, int TY> __device__ __forceinline__ void fused_halo_pos(int h, int &rx, int &ry)
{
    constexpr int SX = TX + 2, SY = TY + 2;
    if (h < SX) {
        rx = h;
        ry = 0;
    } else if (h < 2 * SX) {
        rx = h - SX;
        ry = SY - 1;
    } else if (h < 2 * SX + TY) {
        rx = 0;
        ry = 1 + (h - 2 * SX);
    } else {
        rx = SX - 1;
        ry = 1 + (h - 2 * SX - TY);
    }
}

// the halo entry of thread t, or -1: entries go to the first threads of the
// block, so that they occupy as few warps as possible (a warp issues its halo
// loads and predictor once whatever number of its lanes take part)
template <int TX, int TY> __device__ __forceinline__ int fused_halo_entry(int t)
{
    return t < fused_halo_count<TX, TY>() ? t : -1;
}

// the fused kernels' per-thread staging geometry: the owned site's position in
// the staged plane and its (wrapped) column, the halo position and column
template <int TX, int TY> struct FusedPos {
    int po, colo, ph, colh;
    bool own_in, has_h;
    template <class T> __device__ __forceinline__ FusedPos(const Lat<T> &L, int gx0, int gy0, int t)
    {
        constexpr int SX = TX + 2;
        const int lx = t % TX, ly = t / TX;
        po = (ly + 1) * SX + (lx + 1);
        const int gxo = gx0 + lx, gyo = gy0 + ly;
        own_in = gxo < L.Lx && gyo < L.Ly;
        // a tile that overhangs the lattice still stages the wrapped sites: its
        // positions past the edge are the halo of the last column or row
        colo = wrap_any(gxo, L.Lx) + L.Lx * wrap_any(gyo, L.Ly);
        const int h = fused_halo_entry<TX, TY>(t);
        has_h = h >= 0;
        ph = 0;
        colh = 0;
        if (has_h) {
            int rx, ry;
            fused_halo_pos<TX, TY>(h, rx, ry);
            ph = ry * SX + rx;
            colh = wrap_any(gx0 + rx - 1, L.Lx) + L.Lx * wrap_any(gy0 + ry - 1, L.Ly);
        }
    }
};

// force of a deep bulk site from the predicted-Q ring, its own column (planes
// z-1, z, z+1) from registers
template <class T, int TS, int SX>
__device__ __forceinline__ void deep_force_ring(const Lat<T> &L, const T *sQ, const int (&sb)[3],
                                                const T (&qc)[3][5], long long i, T *f)
{
    // one pointer per plane, every stencil offset a compile-time displacement from it
    const T *r0 = sQ + sb[0], *r1 = sQ + sb[1], *r2 = sQ + sb[2];
#define QQ(dx, dy, dz, c)                                                                     \
    (((dx) == 0 && (dy) == 0) ? qc[(dz) + 1][c]                                               \
                              : ((dz) < 0 ? r0 : (dz) == 0 ? r1 : r2)[(c) * TS + (dy) * SX + (dx)])
    T s2[5];
    if (L.L4 == T(0)) {
        QMIN_BULK_Q25_NO_L4(L.cq, s2);
    } else {
        QMIN_BULK_Q25(L.cq, s2);
    }
#undef QQ
    deep_force_finish(L, qc[1], s2, i, f);
}

// the owned site of plane z: force from the ring, kick, writes to the output
// set (32-bit component offsets from the site's address), FIRE sums
template <class T, int TS, int SX, class Acc>
__device__ __forceinline__ void fused_site_out(const Lat<T> &L, const T *sQ, const int (&sb)[3],
                                               const T (&qc)[3][5], unsigned Pu, unsigned i, uint8_t c,
                                               const T (&vn)[5], T hdt, T *Qo, T *Vo, T *Fo, Acc *sacc)
{
    // component k of site i at (X + k P)[i]: the plane bases are the same for every
    // thread, the site index a 32-bit offset (the launcher requires 5 P < 2^31)
    auto qo = [&](int k) -> T & { return (Qo + (size_t)k * Pu)[i]; };
    auto vo = [&](int k) -> T & { return (Vo + (size_t)k * Pu)[i]; };
    auto fo = [&](int k) -> T & { return (Fo + (size_t)k * Pu)[i]; };
    if (c == 0) {
        T f[5], v[5];
        deep_force_ring<T, TS, SX>(L, sQ, sb, qc, i, f);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            v[k] = vn[k] + hdt * f[k];
            qo(k) = qc[1][k];
            vo(k) = v[k];
            fo(k) = f[k];
        }
        sacc[0] += (Acc)dot_qt(f, f);
        sacc[1] += (Acc)dot_qt(v, v);
        sacc[2] += (Acc)dot_qt(f, v);
    } else {
#pragma unroll
        for (int k = 0; k < 5; ++k) qo(k) = qc[1][k];
        if (c == 2)
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                vo(k) = T(0);
                fo(k) = T(0);
            }
    }
}

template <class T, int TX, int TY> constexpr size_t fused_deep_smem()
{
    return (size_t)4 * 5 * (TX + 2) * (TY + 2) * sizeof(T);
}

// raw planes prefetched into registers one plane ahead.  Component offsets are
// 32-bit (the launcher requires 5 P < 2^31).
template <class T, int TX, int TY, int MINB>
__global__ void __launch_bounds__(TX *TY, MINB)
    k_fire_deep_fused(Lat<T> L, T *__restrict__ Qo, T *__restrict__ Vo, T *__restrict__ Fo,
                      const uint8_t *__restrict__ cls, const FireDev *__restrict__ fd, double *partials, int zc)
{
    constexpr int NT = TX * TY, SX = TX + 2, SY = TY + 2, TS = SX * SY;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sQ = reinterpret_cast<T *>(smem_raw);  // [4][5][TS]: predicted Q of planes z-1 .. z+2
    if (!fd->active) return;
    const PredCoef<T> pc = pred_coef<T>(fd);
    const T hdt = T(0.5) * T(fd->dt);
    const int ntx = (L.Lx + TX - 1) / TX;
    const int gx0 = (blockIdx.x % ntx) * TX, gy0 = (blockIdx.x / ntx) * TY;
    const int zs = blockIdx.y * zc, ze = min(L.Lz, zs + zc);
    const unsigned Pu = (unsigned)L.P;
    const int sxy = L.Lx * L.Ly;
    const FusedPos<TX, TY> fp(L, gx0, gy0, threadIdx.x);
    auto slot = [&](int z) { return ((z - zs + 1) & 3) * 5 * TS; };
    T ro[15], rh[15];
    uint8_t c_next = 1;
    // component k of site j at (X + k P)[j]: plane bases shared by every thread,
    // 32-bit site offsets
    auto load = [&](int z) {
        const unsigned base = (unsigned)(sxy * wrap_near(z, L.Lz));
        const unsigned io = base + fp.colo;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            ro[k] = ld(L.Q + (size_t)k * Pu + io);
            ro[5 + k] = ld(L.V + (size_t)k * Pu + io);
            ro[10 + k] = ld(L.F + (size_t)k * Pu + io);
        }
        if (fp.has_h) {
            const unsigned ih = base + fp.colh;
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                rh[k] = ld(L.Q + (size_t)k * Pu + ih);
                rh[5 + k] = ld(L.V + (size_t)k * Pu + ih);
                rh[10 + k] = ld(L.F + (size_t)k * Pu + ih);
            }
        }
        c_next = (fp.own_in && z >= zs && z < ze) ? cls[io] : uint8_t(1);
    };
    // predicted Q of plane z into the ring; the owned site's predicted velocity and Q
    auto predict = [&](int z, T(&vn)[5], T(&qn)[5]) {
        T *s = sQ + slot(z);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            vn[k] = pred_v(pc, ro[5 + k], ro[10 + k]);
            qn[k] = pred_q(pc, ro[k], vn[k]);
            s[k * TS + fp.po] = qn[k];
        }
        if (fp.has_h)
#pragma unroll
            for (int k = 0; k < 5; ++k) s[k * TS + fp.ph] = pred_q(pc, rh[k], pred_v(pc, rh[5 + k], rh[10 + k]));
    };
    using Acc = typename std::conditional<sizeof(T) == 4, float, double>::type;
    Acc sacc[3] = {Acc(0), Acc(0), Acc(0)};
    if (zs < L.Lz) {
        T vn_cur[5], vn_nxt[5], qc[3][5];
        load(zs - 1);
        predict(zs - 1, vn_cur, qc[1]);
        load(zs);
        uint8_t c_cur = c_next;
        predict(zs, vn_cur, qc[2]);
        load(zs + 1);
        for (int z = zs; z < ze; ++z) {
            const uint8_t c_here = c_cur;
            c_cur = c_next;
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                qc[0][k] = qc[1][k];
                qc[1][k] = qc[2][k];
            }
            predict(z + 1, vn_nxt, qc[2]);
            if (z + 2 <= ze) load(z + 2);
            __syncthreads();
            if (fp.own_in) {
                const int sb[3] = {slot(z - 1) + fp.po, slot(z) + fp.po, slot(z + 1) + fp.po};
                fused_site_out<T, TS, SX, Acc>(L, sQ, sb, qc, Pu, (unsigned)(sxy * z + fp.colo), c_here, vn_cur,
                                               hdt, Qo, Vo, Fo, sacc);
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) vn_cur[k] = vn_nxt[k];
        }
    }
    double acc[3] = {(double)sacc[0], (double)sacc[1], (double)sacc[2]};
    block_sum<3, NT>(acc);
    if (threadIdx.x == 0) {
        const int b = blockIdx.y * gridDim.x + blockIdx.x;
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[3 * b + k] = acc[k];
    }
}

// The same iteration with the raw Q, V, F of each plane staged cooperatively:
// every component row of the tile plus halo is copied as a 40-float segment
// (x = gx0 - 4 .. gx0 + 35) by 16-byte cp.async, two planes ahead, into a
// ring of three raw planes, wrapping across the periodic faces chunk by chunk
// (needs Lx % 4 == 0, so that every chunk is 16-byte aligned and a wrapped
// chunk stays one).  Each step then predicts plane z + 2 and computes the
// force of plane z after one barrier: the predicted-Q ring holds planes
// z - 1 .. z + 2.  The owned site's predicted velocity and Q of the planes in
// flight stay in registers.
template <int TY> constexpr int fused_v_rows() { return TY + 2; }
constexpr int kFusedVRow = 40;  // floats per staged row segment
template <class T, int TX, int TY> constexpr size_t fused_deep_cp_smem()
{
    return (size_t)4 * 5 * (TX + 2) * (TY + 2) * sizeof(T) + (size_t)3 * 15 * (TY + 2) * kFusedVRow * sizeof(T);
}

template <class T, int TX, int TY, int MINB>
__global__ void __launch_bounds__(TX *TY, MINB)
    k_fire_deep_fused_cp(Lat<T> L, T *__restrict__ Qo, T *__restrict__ Vo, T *__restrict__ Fo,
                         const uint8_t *__restrict__ cls, const FireDev *__restrict__ fd, double *partials, int zc)
{
    static_assert(sizeof(T) == 4 && TX == 32, "16-byte row chunks of the 32-wide FP32 tile");
    constexpr int NT = TX * TY, SX = TX + 2, SY = TY + 2, TS = SX * SY;
    constexpr int RW = kFusedVRow, RC = RW / 4;           // row floats, 16-byte chunks per row
    constexpr int RPLANE = 15 * SY * RW;                  // floats per raw plane: [15][SY][RW]
    constexpr int NCH = 15 * SY * RC;                     // chunks per raw plane
    constexpr int CPT = (NCH + NT - 1) / NT;              // chunks per thread
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sQ = reinterpret_cast<T *>(smem_raw);  // [4][5][TS]: predicted Q of planes z-1 .. z+2
    T *sR = sQ + 4 * 5 * TS;                   // [3][15][SY][RW]: raw Q, V, F of planes in flight
    if (!fd->active) return;
    const PredCoef<T> pc = pred_coef<T>(fd);
    const T hdt = T(0.5) * T(fd->dt);
    const int ntx = (L.Lx + TX - 1) / TX;
    const int gx0 = (blockIdx.x % ntx) * TX, gy0 = (blockIdx.x / ntx) * TY;
    const int zs = blockIdx.y * zc, ze = min(L.Lz, zs + zc);
    const unsigned Pu = (unsigned)L.P;
    const int sxy = L.Lx * L.Ly;
    const FusedPos<TX, TY> fp(L, gx0, gy0, threadIdx.x);
    // raw staging position of a staged-plane position (rx, ry): row ry, column rx + 3
    auto raw_of = [&](int p) { return (p / SX) * RW + (p % SX) + 3; };
    const int ro_own = raw_of(fp.po), ro_h = raw_of(fp.ph);
    // this thread's chunks: field, component, row, chunk -> source offset within the
    // field's planes (without the z plane) and destination within a raw plane
    unsigned coff[CPT];
    int cfield[CPT], cdst[CPT];
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
        const int c = threadIdx.x + j * NT;
        cfield[j] = -1;
        if (c < NCH) {
            const int ch = c % RC, row = (c / RC) % SY, fk = c / (RC * SY);  // fk = 5 field + component
            const int x = wrap_any(gx0 - 4 + 4 * ch, L.Lx), y = wrap_any(gy0 - 1 + row, L.Ly);
            cfield[j] = fk / 5;
            coff[j] = (unsigned)(fk % 5) * Pu + (unsigned)(x + L.Lx * y);
            cdst[j] = (fk * SY + row) * RW + 4 * ch;
        }
    }
    auto rslot = [&](int z) { return sR + ((z - zs + 1) % 3) * RPLANE; };
    auto slot = [&](int z) { return ((z - zs + 1) & 3) * 5 * TS; };
    // one commit group per plane (an empty one past the chunk's upper halo plane)
    auto issue = [&](int z) {
        if (z <= ze) {
            const unsigned zoff = (unsigned)(sxy * wrap_near(z, L.Lz));
            T *r = rslot(z);
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                if (cfield[j] < 0) continue;
                const T *src = (cfield[j] == 0 ? L.Q : cfield[j] == 1 ? L.V : L.F) + (coff[j] + zoff);
                const unsigned sa = (unsigned)__cvta_generic_to_shared(r + cdst[j]);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    auto predict = [&](int z, T(&vn)[5], T(&qn)[5]) {
        T *s = sQ + slot(z);
        const T *r = rslot(z);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            vn[k] = pred_v(pc, r[((5 + k) * SY) * RW + ro_own], r[((10 + k) * SY) * RW + ro_own]);
            qn[k] = pred_q(pc, r[(k * SY) * RW + ro_own], vn[k]);
            s[k * TS + fp.po] = qn[k];
        }
        if (fp.has_h)
#pragma unroll
            for (int k = 0; k < 5; ++k)
                s[k * TS + fp.ph] = pred_q(pc, r[(k * SY) * RW + ro_h],
                                           pred_v(pc, r[((5 + k) * SY) * RW + ro_h], r[((10 + k) * SY) * RW + ro_h]));
    };
    auto cls_at = [&](int z) -> uint8_t {
        return (fp.own_in && z >= zs && z < ze) ? cls[(unsigned)(sxy * z + fp.colo)] : uint8_t(1);
    };
    using Acc = float;
    Acc sacc[3] = {0.f, 0.f, 0.f};
    if (zs < L.Lz) {
        // prologue: planes zs-1 .. zs+1 predicted; zs+2 and zs+3 in flight
        T vn0[5], vn1[5], vn2[5], qc[3][5], qn[5];
        issue(zs - 1);
        issue(zs);
        issue(zs + 1);
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
        predict(zs - 1, vn0, qc[0]);
        predict(zs, vn0, qc[1]);
        predict(zs + 1, vn1, qc[2]);
        __syncthreads();
        issue(zs + 2);
        issue(zs + 3);
        uint8_t c_cur = cls_at(zs);
        for (int z = zs; z < ze; ++z) {
            const uint8_t c_here = c_cur;
            c_cur = cls_at(z + 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this thread's copies of plane z + 2
            __syncthreads();  // every copy of plane z + 2; plane z + 1's raw slot and plane z - 2's ring slot free
            issue(z + 4);     // into the raw slot of plane z + 1
            if (z + 2 <= ze) predict(z + 2, vn2, qn);
            if (fp.own_in) {
                const int sb[3] = {slot(z - 1) + fp.po, slot(z) + fp.po, slot(z + 1) + fp.po};
                fused_site_out<T, TS, SX, Acc>(L, sQ, sb, qc, Pu, (unsigned)(sxy * z + fp.colo), c_here, vn0,
                                               hdt, Qo, Vo, Fo, sacc);
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                vn0[k] = vn1[k];
                vn1[k] = vn2[k];
                qc[0][k] = qc[1][k];
                qc[1][k] = qc[2][k];
                qc[2][k] = qn[k];
            }
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    double acc[3] = {(double)sacc[0], (double)sacc[1], (double)sacc[2]};
    block_sum<3, NT>(acc);
    if (threadIdx.x == 0) {
        const int b = blockIdx.y * gridDim.x + blockIdx.x;
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[3 * b + k] = acc[k];
    }
}

// Q at the predicted step, formed on the fly from the input buffer set
template <class T>
__device__ __forceinline__ T pred_q_at(const Lat<T> &L, const PredCoef<T> &c, long long j, int k)
{
    const long long o = (long long)k * L.P + j;
    return pred_q(c, ld(L.Q + o), pred_v(c, ld(L.V + o), ld(L.F + o)));
}

// twice the first derivatives (k_derivs' rules) of the predicted Q at the listed
// sites' neighbours, formed from the input buffer set
template <class T>
__global__ void __launch_bounds__(kBlock)
    k_derivs_list_pred(Lat<T> L, const int *__restrict__ list, int n, const FireDev *__restrict__ fd)
{
    if (!fd->active) return;
    const PredCoef<T> pc = pred_coef<T>(fd);
    const long long P = L.P;
    for (int e = blockIdx.x * kBlock + threadIdx.x; e < n; e += gridDim.x * kBlock) {
        const int i = list[e];
        const int t = L.types[i];
        const Nb b = neighbours(L, i);
        T q[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) q[k] = pred_q_at(L, pc, i, k);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            const int dn = b.n[2 * ax], up = b.n[2 * ax + 1];
            const int td = t < 0 ? L.types[dn] : 0, tu = t < 0 ? L.types[up] : 0;
#pragma unroll
            for (int k = 0; k < 5; ++k)
                L.D[(5 * ax + k) * P + i] =
                    deriv2_rule(t, td, tu, pred_q_at(L, pc, dn, k), q[k], pred_q_at(L, pc, up, k));
        }
    }
}

// accessor over the predicted Q of the input buffer set; neighbour derivatives
// from the D planes k_derivs_list_pred wrote
template <class T> struct PredAcc {
    const T *Q, *V, *F, *D;
    const int8_t *types;
    const ObjDev<T> *objs;
    long long P;
    int i;
    Nb b;
    PredCoef<T> c;
    __device__ __forceinline__ PredAcc(const Lat<T> &L, int i_, const PredCoef<T> &c_)
        : Q(L.Q), V(L.V), F(L.F), D(L.D), types(L.types), objs(L.objs), P(L.P), i(i_), b(neighbours(L, i_)), c(c_)
    {
    }
    __device__ __forceinline__ T at(long long j, int k) const
    {
        const long long o = (long long)k * P + j;
        return pred_q(c, ld(Q + o), pred_v(c, ld(V + o), ld(F + o)));
    }
    __device__ __forceinline__ ObjDev<T> obj(int t) const { return objs[t - 1]; }
    __device__ __forceinline__ int tn(int s) const { return types[b.n[s]]; }
    __device__ __forceinline__ T q(int k) const { return at(i, k); }
    __device__ __forceinline__ T nq(int s, int k) const { return at(b.n[s], k); }
    __device__ __forceinline__ T dn(int s, int d) const { return ld(D + (long long)d * P + b.n[s]); }
};

// the listed LC sites' force at the predicted Q and kick, from the input buffer
// set into the output set's V and F (their predicted Q: the fused deep kernel)
template <class T>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? 2 : 1)
    k_force_kick_list_pred(Lat<T> L, T *__restrict__ Vo, T *__restrict__ Fo, const int *__restrict__ list, int n,
                           const FireDev *__restrict__ fd, double *partials)
{
    if (!fd->active) return;
    const PredCoef<T> pc = pred_coef<T>(fd);
    const T hdt = T(0.5) * T(fd->dt);
    const long long P = L.P;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int e = blockIdx.x * kBlock + threadIdx.x; e < n; e += gridDim.x * kBlock) {
        const int i = list[e];
        const int t = L.types[i];
        PredAcc<T> a(L, i, pc);
        T f[5], h[3], v[5];
        site_force_core<T, PredAcc<T>, false, true>(L, a, t, f, site_field(L, i, h));
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const long long o = (long long)k * P + i;
            v[k] = pred_v(pc, ld(L.V + o), ld(L.F + o)) + hdt * f[k];
            Fo[o] = f[k];
            Vo[o] = v[k];
        }
        if constexpr (sizeof(T) == 8) {
            dot3_acc(f, v, acc);
        } else {
            acc[0] += (double)dot_qt(f, f);
            acc[1] += (double)dot_qt(v, v);
            acc[2] += (double)dot_qt(f, v);
        }
    }
    block_sum<3>(acc);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[3 * blockIdx.x + k] = acc[k];
}

// shared-memory deep kernel over TX x TY columns of kDeepZc planes (more when
// the grid would not fit the partials buffer); returns its block count
template <class T, int TX, int TY>
static int launch_deep_tiled(const Lat<T> &L, const SplitLists &sl, FireDev *fd, double *partials, cudaStream_t s)
{
    constexpr size_t sm = deep_tiled_smem<T, TX, TY>();
    static bool attr_set = false;
    if (!attr_set) {
        // a failure here surfaces as the launch's error
        attr_set = cudaFuncSetAttribute(k_force_kick_deep_tiled<T, TX, TY>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) == cudaSuccess;
    }
    const int ntiles = ((L.Lx + TX - 1) / TX) * ((L.Ly + TY - 1) / TY);
    int zc = kDeepZc;
    while ((long long)ntiles * ((L.Lz + zc - 1) / zc) > kMaxFusedBlocks - 1024) ++zc;
    const int nz = (L.Lz + zc - 1) / zc;
    k_force_kick_deep_tiled<T, TX, TY><<<dim3(ntiles, nz), TX * TY, sm, s>>>(L, sl.cls, fd, partials, zc);
    return ntiles * nz;
}

// the FP32 two-sites-per-thread deep kernel over TX x TY columns
// fitted = true: z chunks sized so that the grid is about two waves of MINB
// blocks on each of the 152 SMs (fewer, longer columns), else kDeepZc planes
template <int TX, int TY, int MINB, bool KICK = true>
static int launch_deep_pair(const Lat<float> &L, const SplitLists &sl, FireDev *fd, double *partials, bool fitted,
                            cudaStream_t s)
{
    constexpr size_t sm = deep_tiled_smem<float, TX, TY>();
    static bool attr_set = false;
    if (!attr_set) {
        // a failure here surfaces as the launch's error
        attr_set = cudaFuncSetAttribute(k_force_kick_deep_pair<TX, TY, MINB, KICK>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) == cudaSuccess;
    }
    const int ntiles = ((L.Lx + TX - 1) / TX) * ((L.Ly + TY - 1) / TY);
    int zc = kDeepZc;
    if (fitted) {
        // about two waves: each block walks a long column
        const long long nz = std::max(1LL, 2LL * 152 * MINB / ntiles);
        zc = std::max(kDeepZc, (int)((L.Lz + nz - 1) / nz));
    }
    while ((long long)ntiles * ((L.Lz + zc - 1) / zc) > kMaxFusedBlocks - 1024) ++zc;
    const int nz = (L.Lz + zc - 1) / zc;
    k_force_kick_deep_pair<TX, TY, MINB, KICK><<<dim3(ntiles, nz), TX / 2 * TY, sm, s>>>(L, sl.cls, fd, partials, zc);
    return ntiles * nz;
}

// the TMA-staged two-sites-per-thread kernel (FP32, z chunks of about two
// waves); -1 when the lattice has no tensor map (x extent not a multiple of 4)
template <int TX, int TY, int MINB, bool KICK = true>
static int launch_deep_pair_tma(const Lat<float> &L, const SplitLists &sl, FireDev *fd, double *partials,
                                cudaStream_t s)
{
    if (!sl.tmap_q || !sl.err) return -1;
    constexpr size_t sm = deep_pair_tma_smem<TX, TY>();
    static bool attr_set = false;
    if (!attr_set) {
        // a failure here surfaces as the launch's error
        attr_set = cudaFuncSetAttribute(k_force_kick_deep_pair_tma<TX, TY, MINB, KICK>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) == cudaSuccess;
    }
    const int ntiles = ((L.Lx + TX - 1) / TX) * ((L.Ly + TY - 1) / TY);
    const long long nzt = std::max(1LL, 2LL * 152 * MINB / ntiles);
    int zc = std::max(kDeepZc, (int)((L.Lz + nzt - 1) / nzt));
    while ((long long)ntiles * ((L.Lz + zc - 1) / zc) > kMaxFusedBlocks - 1024) ++zc;
    const int nz = (L.Lz + zc - 1) / zc;
    k_force_kick_deep_pair_tma<TX, TY, MINB, KICK>
        <<<dim3(ntiles, nz), TX / 2 * TY, sm, s>>>(L, *sl.tmap_q, sl.cls, fd, partials, zc, sl.err);
    return ntiles * nz;
}

// grid of the fused deep kernels over TX x TY columns; zc > 0: z chunks of zc
// planes, zc = 0: chunks long enough that the grid is about two waves of
// MINB blocks on each of the 152 SMs
static inline void fused_grid(int Lx, int Ly, int Lz, int TX, int TY, int MINB, int zc, int &ntiles, int &zc_out,
                              int &nz)
{
    ntiles = ((Lx + TX - 1) / TX) * ((Ly + TY - 1) / TY);
    if (zc <= 0) {
        const long long nzt = std::max(1LL, 2LL * 152 * MINB / ntiles);
        zc = (int)((Lz + nzt - 1) / nzt);
    }
    zc = std::max(1, std::min(zc, Lz));
    while ((long long)ntiles * ((Lz + zc - 1) / zc) > kMaxFusedBlocks - 1024) ++zc;
    zc_out = zc;
    nz = (Lz + zc - 1) / zc;
}

template <class T, int TX, int TY, int MINB>
static int launch_fused_deep(const Lat<T> &L, T *Qo, T *Vo, T *Fo, const SplitLists &sl, FireDev *fd,
                             double *partials, int zc, cudaStream_t s)
{
    constexpr size_t sm = fused_deep_smem<T, TX, TY>();
    static bool attr_set = false;
    if (!attr_set) {
        // a failure here surfaces as the launch's error
        attr_set = cudaFuncSetAttribute(k_fire_deep_fused<T, TX, TY, MINB>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) == cudaSuccess;
    }
    int ntiles, nz;
    fused_grid(L.Lx, L.Ly, L.Lz, TX, TY, MINB, zc, ntiles, zc, nz);
    k_fire_deep_fused<T, TX, TY, MINB><<<dim3(ntiles, nz), TX * TY, sm, s>>>(L, Qo, Vo, Fo, sl.cls, fd, partials, zc);
    return ntiles * nz;
}

template <class T, int TX, int TY, int MINB>
static int launch_fused_deep_cp(const Lat<T> &L, T *Qo, T *Vo, T *Fo, const SplitLists &sl, FireDev *fd,
                                double *partials, int zc, cudaStream_t s)
{
    constexpr size_t sm = fused_deep_cp_smem<T, TX, TY>();
    static bool attr_set = false;
    if (!attr_set) {
        // a failure here surfaces as the launch's error
        attr_set = cudaFuncSetAttribute(k_fire_deep_fused_cp<T, TX, TY, MINB>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) == cudaSuccess;
    }
    int ntiles, nz;
    fused_grid(L.Lx, L.Ly, L.Lz, TX, TY, MINB, zc, ntiles, zc, nz);
    k_fire_deep_fused_cp<T, TX, TY, MINB>
        <<<dim3(ntiles, nz), TX * TY, sm, s>>>(L, Qo, Vo, Fo, sl.cls, fd, partials, zc);
    return ntiles * nz;
}

// Fused split iteration, deep part: variant 0 = 32 x 8 tiles, z chunks of 16;
// 1 = 32 x 8, about two waves; 2 = 32 x 4, z chunks of 16 (raw planes
// prefetched into registers; FP32 at 2, 2, 4 blocks per SM, FP64 at 1, 1, 2);
// 3 = 32 x 8, about two waves, 4 = 32 x 4, about two waves (raw planes
// copied into shared memory by 16-byte row chunks two planes ahead; FP32 with
// Lx % 4 == 0 only, at 2 and 4 blocks per SM).  Returns the block count
// (partials used), -1 for a variant this lattice or precision does not have.
template <class T>
int launch_split_fused_deep(const Lat<T> &Lin, T *Qo, T *Vo, T *Fo, const SplitLists &sl, FireDev *fd,
                            double *partials, int variant, cudaStream_t s)
{
    constexpr bool f32 = sizeof(T) == 4;
    if (5 * Lin.P >= (1LL << 31)) return -1;  // the kernels' component offsets are 32-bit
    switch (variant) {
    case 0: return launch_fused_deep<T, 32, 8, f32 ? 2 : 1>(Lin, Qo, Vo, Fo, sl, fd, partials, 16, s);
    case 1: return launch_fused_deep<T, 32, 8, f32 ? 2 : 1>(Lin, Qo, Vo, Fo, sl, fd, partials, 0, s);
    case 2: return launch_fused_deep<T, 32, 4, f32 ? 4 : 2>(Lin, Qo, Vo, Fo, sl, fd, partials, 16, s);
    case 3:
    case 4:
        // 16-byte row chunks: FP32 with Lx a multiple of 4 only
        if constexpr (f32) {
            if (Lin.Lx % 4 != 0) return -1;
            if (variant == 3) return launch_fused_deep_cp<T, 32, 8, 2>(Lin, Qo, Vo, Fo, sl, fd, partials, 0, s);
            return launch_fused_deep_cp<T, 32, 4, 4>(Lin, Qo, Vo, Fo, sl, fd, partials, 0, s);
        } else {
            return -1;
        }
    default: return -1;
    }
}

// Fused split iteration, listed part: derivative planes of the predicted Q at
// the sites the listed forms read, then the listed sites' force + kick into the
// output set.  Returns its launch count; *nblocks its partials.
template <class T>
int launch_split_fused_list(const Lat<T> &Lin, T *Vo, T *Fo, const SplitLists &sl, FireDev *fd, double *partials,
                            cudaStream_t s, int *nblocks)
{
    int n = 0;
    *nblocks = 0;
    if (sl.n_derivs > 0) {
        launch_high(k_derivs_list_pred<T>, list_grid(sl.n_derivs), s, Lin, (const int *)sl.derivs, sl.n_derivs,
                    (const FireDev *)fd);
        ++n;
    }
    if (sl.n_sites > 0) {
        const int g = list_grid(sl.n_sites);
        launch_high(k_force_kick_list_pred<T>, g, s, Lin, Vo, Fo, (const int *)sl.sites, sl.n_sites, (const FireDev *)fd,
                    partials);
        *nblocks = g;
        ++n;
    }
    return n;
}

template <class T> int launch_split_derivs(const Lat<T> &L, const SplitLists &sl, FireDev *fd, cudaStream_t s)
{
    if (sl.n_derivs == 0) return 0;
    launch_high(k_derivs_list<T>, list_grid(sl.n_derivs), s, L, (const int *)sl.derivs, sl.n_derivs, (const FireDev *)fd);
    return 1;
}

template <class T>
int launch_split_deep(const Lat<T> &L, const SplitLists &sl, FireDev *fd, double *partials, int grid, int cap,
                      cudaStream_t s)
{
    if (cap == 2) return launch_deep_tiled<T, 32, 8>(L, sl, fd, partials, s);
    if (cap == 3) return launch_deep_tiled<T, 16, 16>(L, sl, fd, partials, s);
    if (cap == 4 || cap == 5 || cap == 6) {
        if constexpr (sizeof(T) == 4) {
            if (cap == 6) return launch_deep_pair_tma<32, 8, 3>(L, sl, fd, partials, s);
            return launch_deep_pair<32, 8, 3>(L, sl, fd, partials, cap == 5, s);
        } else {
            return -1;  // FP32 only (the autotuner does not offer it for FP64)
        }
    }
    if (cap == 1) k_force_kick_deep<T, 1><<<grid, kBlock, 0, s>>>(L, sl.cls, fd, partials);
    else k_force_kick_deep<T, 0><<<grid, kBlock, 0, s>>>(L, sl.cls, fd, partials);
    return grid;
}

template <class T>
int launch_split_list(const Lat<T> &L, const SplitLists &sl, FireDev *fd, double *partials, cudaStream_t s)
{
    if (sl.n_sites <= 0) return 0;
    const int g = list_grid(sl.n_sites);
    launch_high(k_force_kick_list<T>, g, s, L, (const int *)sl.sites, sl.n_sites, (const FireDev *)fd, partials);
    return g;
}

template <class T>
int launch_split_force_kick(const Lat<T> &L, const SplitLists &sl, FireDev *fd, double *partials, int grid, int cap,
                            cudaStream_t s, int *nparts)
{
    const int nd = launch_split_deep<T>(L, sl, fd, partials, grid, cap, s);
    if (nd < 0) return -1;
    const int nl = launch_split_list<T>(L, sl, fd, partials + 3 * nd, s);
    *nparts = nd + nl;
    return 1 + (nl > 0 ? 1 : 0);
}

// forces only at Q (no FIRE state): derivative planes at the listed sites'
// neighbours, the deep sites (FP64 from global memory at 2 blocks per SM, FP32
// two per thread on 32x8 tiles), then the listed sites; object sites get zero
template <class T> int launch_split_force(const Lat<T> &L, int grid, cudaStream_t s)
{
    const SplitLists &sl = L.split;
    int n = launch_split_derivs<T>(L, sl, nullptr, s);
    if constexpr (sizeof(T) == 4) launch_deep_pair<32, 8, 3, false>(L, sl, nullptr, nullptr, true, s);
    else k_force_kick_deep<T, 1, false><<<grid, kBlock, 0, s>>>(L, sl.cls, nullptr, nullptr);
    ++n;
    if (sl.n_sites > 0) {
        k_force_kick_list<T, false><<<list_grid(sl.n_sites), kBlock, 0, s>>>(L, sl.sites, sl.n_sites, nullptr, nullptr);
        ++n;
    }
    return n;
}

cudaError_t split_set_wait_limit(int polls)
{
    return cudaMemcpyToSymbol(g_split_wait_limit, &polls, sizeof(int));
}

template int launch_split_derivs<double>(const Lat<double> &, const SplitLists &, FireDev *, cudaStream_t);
template int launch_split_derivs<float>(const Lat<float> &, const SplitLists &, FireDev *, cudaStream_t);
template int launch_split_force_kick<double>(const Lat<double> &, const SplitLists &, FireDev *, double *, int, int,
                                             cudaStream_t, int *);
template int launch_split_force_kick<float>(const Lat<float> &, const SplitLists &, FireDev *, double *, int, int,
                                            cudaStream_t, int *);
template int launch_split_deep<double>(const Lat<double> &, const SplitLists &, FireDev *, double *, int, int,
                                       cudaStream_t);
template int launch_split_deep<float>(const Lat<float> &, const SplitLists &, FireDev *, double *, int, int,
                                      cudaStream_t);
template int launch_split_list<double>(const Lat<double> &, const SplitLists &, FireDev *, double *, cudaStream_t);
template int launch_split_list<float>(const Lat<float> &, const SplitLists &, FireDev *, double *, cudaStream_t);
template int launch_split_force<double>(const Lat<double> &, int, cudaStream_t);
template int launch_split_force<float>(const Lat<float> &, int, cudaStream_t);
template int launch_split_fused_deep<double>(const Lat<double> &, double *, double *, double *, const SplitLists &,
                                             FireDev *, double *, int, cudaStream_t);
template int launch_split_fused_deep<float>(const Lat<float> &, float *, float *, float *, const SplitLists &,
                                            FireDev *, double *, int, cudaStream_t);
template int launch_split_fused_list<double>(const Lat<double> &, double *, double *, const SplitLists &, FireDev *,
                                             double *, cudaStream_t, int *);
template int launch_split_fused_list<float>(const Lat<float> &, float *, float *, const SplitLists &, FireDev *,
                                            double *, cudaStream_t, int *);

}  // namespace qmin
