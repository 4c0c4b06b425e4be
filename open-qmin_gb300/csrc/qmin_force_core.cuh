// The per-site Landau-de Gennes force, written once against an accessor so
// that the global-memory kernels and the shared-memory tile kernels share one
// implementation of the force semantics.
//
// An accessor A provides, for the site being updated:
//   int tn(s)          type of neighbour s (0..5 = x-, x+, y-, y+, z-, z+)
//   T   q(k)           own Q component k
//   T   nq(s, k)       neighbour s's Q component k
//   ObjDev<T> obj(t)   the object whose sites carry type t > 0
//   T   dn(s, d)       TWICE neighbour s's first derivative d = 5*axis + component
//                      (landauDeGennesLC::computeFirstDerivatives rules).  Central
//                      differences are then plain differences; the exact factor 1/2
//                      lives in the coefficients, so results are bit-identical.
#pragma once
#include "qmin_device.cuh"
#include "qmin_distortion_tables.h"
#include "qmin_l6_forms.h"
#include "qmin_internal.h"

namespace qmin {

// sparse multi-constant forms (term, boundary case, component) -> (input, k)
static __device__ const uint16_t g_dt_offset[3 * 64 * 5 + 1] = QMIN_DT_OFFSET_INIT;
static __device__ const uint8_t g_dt_input[QMIN_DT_NPAIRS] = QMIN_DT_INPUT_INIT;
static __device__ const int8_t g_dt_k[QMIN_DT_NPAIRS] = QMIN_DT_K_INIT;
// L6 quadratic forms of the 27 boundary cases: (case, component) -> (i, j, k), value (k/2) x_i x_j
static __device__ const uint16_t g_l6_offset[64 * 5 + 1] = QMIN_L6_OFFSET_INIT;
static __device__ const uint8_t g_l6_i[QMIN_L6_NPAIRS] = QMIN_L6_I_INIT;
static __device__ const uint8_t g_l6_j[QMIN_L6_NPAIRS] = QMIN_L6_J_INIT;
static __device__ const int8_t g_l6_k[QMIN_L6_NPAIRS] = QMIN_L6_K_INIT;

// input x of the 125-input stencils, derivatives as true derivatives
template <class T, class A> __device__ __forceinline__ T stencil_input(const A &acc, int j)
{
    if (j < 5) return acc.q(j);
    if (j < 35) return acc.nq((j - 5) / 5, (j - 5) % 5);
    return T(0.5) * acc.dn((j - 35) / 15, (j - 35) % 15);
}

template <class T>
__device__ __forceinline__ T ld(const T *p)
{
    return __ldg(p);
}

struct Nb {
    int n[6];  // x-, x+, y-, y+, z-, z+ (cubicLattice::getNeighbors, cubicLattice.cpp:179-244)
};

template <class T>
__device__ __forceinline__ Nb neighbours(const Lat<T> &L, int i)
{
    const int x = i % L.Lx;
    const int r = i / L.Lx;
    const int y = r % L.Ly;
    const int z = r / L.Ly;
    const int sx = L.Lx, sy = L.Lx * L.Ly;
    Nb b;
    b.n[0] = x == 0 ? i + (L.Lx - 1) : i - 1;
    b.n[1] = x == L.Lx - 1 ? i - (L.Lx - 1) : i + 1;
    b.n[2] = y == 0 ? i + (L.Ly - 1) * sx : i - sx;
    b.n[3] = y == L.Ly - 1 ? i - (L.Ly - 1) * sx : i + sx;
    b.n[4] = z == 0 ? i + (L.Lz - 1) * sy : i - sy;
    b.n[5] = z == L.Lz - 1 ? i - (L.Lz - 1) * sy : i + sy;
    return b;
}

// block-wide sum of NV doubles over a block of NT threads; result valid in thread 0
template <int NV, int NT = kBlock>
__device__ __forceinline__ void block_sum(double (&v)[NV])
{
    __shared__ double sh[NV][NT / 32];
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sh[k][w] = v[k];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            v[k] = lane < NT / 32 ? sh[k][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        }
    }
    __syncthreads();
}

// the same for FP32 per-thread values: each warp sums its 32 values in FP32
// (terms that are themselves FP32-rounded), the warps' sums are added in FP64;
// result valid in thread 0 of `out`
template <int NV, int NT = kBlock>
__device__ __forceinline__ void block_sum_f32(float (&v)[NV], double (&out)[NV])
{
    __shared__ double shf[NV][NT / 32];
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) shf[k][w] = (double)v[k];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            out[k] = lane < NT / 32 ? shf[k][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) out[k] += __shfl_down_sync(0xffffffffu, out[k], o);
        }
    }
    __syncthreads();
}

// block-wide sum of NV doubles through shared memory: warp 0 adds eight
// consecutive threads' values per lane, then shuffles; about a third of the
// FP64 additions of block_sum (which adds in every lane at every shuffle
// level), for kernels that reduce once per few sites; result in thread 0
template <int NV, int NT = kBlock>
__device__ __forceinline__ void block_sum_smem(double (&v)[NV])
{
    static_assert(NT == 256, "eight values per lane of warp 0");
    __shared__ double shs[NV][NT];
#pragma unroll
    for (int k = 0; k < NV; ++k) shs[k][threadIdx.x] = v[k];
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double a = shs[k][8 * lane];
#pragma unroll
            for (int e = 1; e < 8; ++e) a += shs[k][8 * lane + e];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            v[k] = a;
        }
    }
    __syncthreads();
}

// deterministic sum of partials[NV * nparts] by one block; result in thread 0
template <int NV>
__device__ __forceinline__ void sum_partials(const double *partials, int nparts, double (&v)[NV])
{
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = 0.0;
    // four strides' loads in flight before their adds; each thread still adds
    // its entries b, b + kBlock, b + 2 kBlock, ... in that order
    constexpr int U = 4;
    for (int b0 = threadIdx.x; b0 < nparts; b0 += U * kBlock) {
        double x[U][NV];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int b = b0 + u * kBlock;
#pragma unroll
            for (int k = 0; k < NV; ++k) x[u][k] = b < nparts ? partials[NV * b + k] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (b0 + u * kBlock < nparts)
#pragma unroll
                for (int k = 0; k < NV; ++k) v[k] += x[u][k];
    }
    block_sum<NV>(v);
}

// ---------------------------------------------------- FIRE predictor
// Coefficients of the velocity-Verlet predictor with the deferred velocity mix
// folded in (energyMinimizerFIRE.cpp:104-144 mixes v after the control step;
// the mix is applied here, at the next predictor): v' = cvv v + cvf f,
// q' = q + dt v'.  Kernels that form the predicted Q of a neighbour on the fly
// use pred_v / pred_q, explicit FMAs, so that every kernel gets the same bits.
template <class T> struct PredCoef {
    T cvv, cvf, tdt;
};

// the predictor's coefficients (as k_fire_pred: ve = mv v + mf f folded into the
// Verlet step, v' = cvv v + cvf f, q' = q + dt v')
template <class T> __device__ __forceinline__ PredCoef<T> pred_coef(const FireDev *fd)
{
    const double dt = fd->dt, hdt = 0.5 * dt;
    double mv = 1.0, mf = 0.0;
    if (fd->pending) {
        mv = fd->reset ? 0.0 : 1.0 - fd->mixA;
        mf = fd->reset ? 0.0 : fd->mixA * fd->mixS;
    }
    return PredCoef<T>{T(mv), T(mf + hdt), T(dt)};
}

// predicted velocity and Q of one component: explicit FMAs, so that every
// kernel that recomputes a site's prediction gets the same bits
template <class T> __device__ __forceinline__ T pred_v(const PredCoef<T> &c, T v, T f)
{
    return fma(c.cvf, f, c.cvv * v);
}
template <class T> __device__ __forceinline__ T pred_q(const PredCoef<T> &c, T q, T vn) { return fma(c.tdt, vn, q); }

// first derivative of one component along one axis at a site of type t with
// down/centre/up values and the down/up neighbour types
// (landauDeGennesLCOtherForces.cpp:50-141): central differences; at type < 0
// sites one-sided next to objects, the "up neighbour is an object" branch first
template <class T>
__device__ __forceinline__ T deriv_rule(int t, int td, int tu, T qd, T q, T qu)
{
    if (t > 0) return T(0);
    if (t == 0 || (td <= 0 && tu <= 0)) return T(0.5) * (qu - qd);
    if (tu > 0) return q - qd;
    return qu - q;
}

// the same rule returning twice the derivative (exact: scaling by 2 is exact)
template <class T>
__device__ __forceinline__ T deriv2_rule(int t, int td, int tu, T qd, T q, T qu)
{
    if (t > 0) return T(0);
    if (t == 0 || (td <= 0 && tu <= 0)) return qu - qd;
    if (tu > 0) return T(2) * (q - qd);
    return T(2) * (qu - q);
}

// One site's force, CPU-path semantics by default (multirankSimulation.cpp:462-466):
//   type 0:  F = M( M(-phase - distortion) - fields )
//   type <0: F = M(-phase - distortion + anchoring - fields)
// metric_mode 1 applies M once everywhere (the reference GPU branch).
// WITH_L6 compiles the cubic L6 forms in; kernels without it leave L6 out
// (it is a runtime-zero branch that would still cost registers)
// BND_LINES evaluates the boundary L2-L4 forms as straight-line code per case
// (merged coefficients L.cbd) instead of walking the sparse tables; it needs
// L.cbd and costs code size, so only the listed-site kernel takes it
// ONE_CONST compiles the one-constant form only (the caller guarantees
// !L.multi), which keeps the multi-constant forms' registers out of kernels
// that run one-constant lattices
template <class T, class A, bool WITH_L6 = false, bool BND_LINES = false, bool ONE_CONST = false>
__device__ __forceinline__ void site_force_core(const Lat<T> &L, const A &acc, int t, T *f, const T *hs = nullptr)
{
    if (t > 0) {
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] = T(0);
        return;
    }
    T q[5], nq[6][5];
#pragma unroll
    for (int k = 0; k < 5; ++k) q[k] = acc.q(k);
#pragma unroll
    for (int s = 0; s < 6; ++s)
#pragma unroll
        for (int k = 0; k < 5; ++k) nq[s][k] = acc.nq(s, k);

    const bool boundary = (t == -1);  // type -2 uses the bulk forms (DT:241-279)
    int mask = 0;                     // which neighbours are objects
    if (t < 0) {
#pragma unroll
        for (int s = 0; s < 6; ++s) mask |= (acc.tn(s) > 0) << s;
    }

    T sp[5] = {T(0), T(0), T(0), T(0), T(0)};
    // multi-constant bulk sites carry L1 inside the combined linear form below
    if (ONE_CONST || !L.multi || (boundary && L.L1 != T(0))) {
        // lcForce::bulkL1Force / boundaryL1Force (lcForces.h:26-63)
        T s1[5];
        if (!boundary) {
#pragma unroll
            for (int k = 0; k < 5; ++k)
                s1[k] = L.L1 * (T(6) * q[k] - nq[0][k] - nq[1][k] - nq[2][k] - nq[3][k] - nq[4][k] - nq[5][k]);
        } else {
#pragma unroll
            for (int k = 0; k < 5; ++k) s1[k] = T(0);
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                if (mask & (1 << (2 * ax)))
#pragma unroll
                    for (int k = 0; k < 5; ++k) s1[k] -= (nq[2 * ax + 1][k] - q[k]);
                if (mask & (1 << (2 * ax + 1)))
#pragma unroll
                    for (int k = 0; k < 5; ++k) s1[k] -= (nq[2 * ax][k] - q[k]);
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) s1[k] = s1[k] * L.L1;
        }
        l1_cross(s1);
#pragma unroll
        for (int k = 0; k < 5; ++k) sp[k] += s1[k];
    }
    if (!ONE_CONST && L.multi) {
        if (!boundary) {
            // bulk L1/L2/L3/L4 forms, straight-line over their union pattern
            T s2[5];
#define QIN(c) q[c]
#define QN(slot, c) nq[slot][c]
#define DN(slot, d) acc.dn(slot, d)
            if (L.L4 == T(0)) {
                QMIN_BULK_FORMS_NO_L4(L.cb, s2);
            } else {
                QMIN_BULK_FORMS(L.cb, s2);
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) sp[k] += s2[k];
            if (WITH_L6 && L.L6 != T(0)) {
                // lcForce::bulkL6Force (lcForces.h:801-815): quadratic in the same inputs
                T s6[5];
                QMIN_L6_BULK(T, s6);
#pragma unroll
                for (int k = 0; k < 5; ++k) sp[k] += (T(0.5) * L.L6) * s6[k];
            }
#undef QIN
#undef QN
#undef DN
        } else {
            // boundary forms: lcForce::getBoundaryCase (lcForces.h:13-25), down wins
            int xx = 0, yy = 0, zz = 0;
            if (mask & 2) xx = 1;
            if (mask & 1) xx = 2;
            if (mask & 8) yy = 1;
            if (mask & 4) yy = 2;
            if (mask & 32) zz = 1;
            if (mask & 16) zz = 2;
            const int bcase = xx + 4 * yy + 16 * zz;
            if constexpr (BND_LINES) {
                T s3[5];
                const T *cbd = L.cbd;
#define QIN(c) q[c]
#define QN(slot, c) nq[slot][c]
#define DN(slot, d) acc.dn(slot, d)
                QMIN_BOUNDARY_FORMS(xx + 3 * yy + 9 * zz, cbd, s3);
#undef QIN
#undef QN
#undef DN
#pragma unroll
                for (int k = 0; k < 5; ++k) sp[k] += s3[k];
            }
            const T Lt[3] = {L.L2, L.L3, L.L4};
            for (int term = 0; !BND_LINES && term < 3; ++term) {
                if (Lt[term] == T(0)) continue;
                for (int k = 0; k < 5; ++k) {
                    const int o0 = g_dt_offset[(term * 64 + bcase) * 5 + k];
                    const int o1 = g_dt_offset[(term * 64 + bcase) * 5 + k + 1];
                    T acc_k = T(0);
                    for (int e = o0; e < o1; ++e) {
                        const int j = g_dt_input[e];
                        T x;
                        if (j < 5) x = acc.q(j);
                        else if (j < 35) x = acc.nq((j - 5) / 5, (j - 5) % 5);
                        else x = T(0.5) * acc.dn((j - 35) / 15, (j - 35) % 15);
                        acc_k += T(g_dt_k[e]) * x;
                    }
                    sp[k] += (T(0.5) * Lt[term]) * (acc_k / T(2));
                }
            }
            if (WITH_L6 && L.L6 != T(0)) {
                // lcForce::boundaryL6Force (lcForces.h:818-1047)
                for (int k = 0; k < 5; ++k) {
                    const int o0 = g_l6_offset[bcase * 5 + k], o1 = g_l6_offset[bcase * 5 + k + 1];
                    T acc_k = T(0);
                    for (int e = o0; e < o1; ++e)
                        acc_k += T(g_l6_k[e]) * stencil_input<T>(acc, g_l6_i[e]) * stencil_input<T>(acc, g_l6_j[e]);
                    sp[k] += (T(0.5) * L.L6) * (acc_k / T(2));
                }
            }
        }
    }
    phase_force_sub(L.a, L.b, L.c, q, sp, f);

    if (L.metric_mode == 0 && t == 0) metric(f);
    if (t < 0 && mask) {
        // landauDeGennesLC::computeBoundaryForcesCPU (landauDeGennesLCOtherForces.cpp:314-373)
#pragma unroll
        for (int s = 0; s < 6; ++s) {
            if (mask & (1 << s)) {
                const ObjDev<T> o = acc.obj(acc.tn(s));
                anchoring_force_add(o.kind, o.W, o.S0, q, nq[s], f);
            }
        }
    }
    if (L.efield)
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] -= L.fE[k];
    if (L.hfield)
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] -= L.fH[k];
    if (hs) {
        // landauDeGennesLC::computeSpatiallyVaryingFieldCPU (landauDeGennesLCOtherForces.cpp:254-283):
        // the uniform-field force with this site's H
        const T hx = hs[0], hy = hs[1], hz = hs[2], fp = L.hvp;
        f[0] -= T(-0.5) * fp * (hx * hx - hz * hz);
        f[1] -= -fp * hx * hy;
        f[2] -= -fp * hx * hz;
        f[3] -= T(-0.5) * fp * (hy * hy - hz * hz);
        f[4] -= -fp * hy * hz;
    }
    metric(f);
}

// this site's spatially varying field (3 values) when one is set, else null
template <class T> __device__ __forceinline__ const T *site_field(const Lat<T> &L, long long i, T (&h)[3])
{
    if (!L.Hv) return nullptr;
#pragma unroll
    for (int c = 0; c < 3; ++c) h[c] = L.Hv[c * L.P + i];
    return h;
}

// periodic wrap of a coordinate at most two steps outside [0, m), m >= 2
__device__ __forceinline__ int wrap_near(int v, int m) { return v < 0 ? v + m : (v >= m ? v - m : v); }

// Force at Q of a deep bulk site (type 0 with six type-0 neighbours, so every
// neighbour derivative the bulk forms read is a central difference) through
// the combined L1-L4 form over Q on the 25-point stencil.  The site is li =
// x + Lx (y + Ly z) of a periodic Lx x Ly x Lz box whose planes start at
// element `base` (0 for a lattice, the solve's offset in a batch); i is its
// index in the planes.  M is applied as the reference does for type-0 sites
// (twice in CPU mode, the fields between the two).
template <class T>
__device__ __forceinline__ void deep_force_box(const Lat<T> &L, long long base, int Lx, int Ly, int Lz, int li,
                                               long long i, T *f)
{
    const int x = li % Lx, r = li / Lx, y = r % Ly, z = r / Ly;
    const int sxy = Lx * Ly;
    int xi[5], yo[5], zo[5];
#pragma unroll
    for (int d = 0; d < 5; ++d) {
        xi[d] = wrap_near(x + d - 2, Lx);
        yo[d] = Lx * wrap_near(y + d - 2, Ly);
        zo[d] = sxy * wrap_near(z + d - 2, Lz);
    }
    const T *Q = L.Q + base;
    const long long P = L.P;
#define QQ(dx, dy, dz, c) ld(Q + (long long)(c) * P + (xi[(dx) + 2] + yo[(dy) + 2] + zo[(dz) + 2]))
    T q[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) q[k] = QQ(0, 0, 0, k);
    T s2[5];
    if (L.L4 == T(0)) {
        // FP32 (latency-bound) term by term; FP64 (bound by the FP64 pipe) over shared sums
        if constexpr (sizeof(T) == 4) {
            QMIN_BULK_Q25_NO_L4_PLAIN(L.cqp, s2);
        } else {
            QMIN_BULK_Q25_NO_L4(L.cq, s2);
        }
    } else {
        QMIN_BULK_Q25(L.cq, s2);
    }
#undef QQ
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

// accessor over the global SoA planes; neighbour derivatives from the D planes.
// It copies the few pointers it needs: holding a reference to the kernel's
// parameter block would force that block into local memory.
template <class T> struct GlobalAcc {
    const T *Q;
    const T *D;
    const int8_t *types;
    const ObjDev<T> *objs;
    long long P;
    int i;
    Nb b;
    __device__ __forceinline__ GlobalAcc(const Lat<T> &L, int i_)
        : Q(L.Q), D(L.D), types(L.types), objs(L.objs), P(L.P), i(i_), b(neighbours(L, i_))
    {
    }
    __device__ __forceinline__ ObjDev<T> obj(int t) const { return objs[t - 1]; }
    __device__ __forceinline__ int tn(int s) const { return types[b.n[s]]; }
    __device__ __forceinline__ T q(int k) const { return ld(Q + (long long)k * P + i); }
    __device__ __forceinline__ T nq(int s, int k) const { return ld(Q + (long long)k * P + b.n[s]); }
    __device__ __forceinline__ T dn(int s, int d) const { return ld(D + (long long)d * P + b.n[s]); }
};

template <class T, bool WITH_L6 = false, bool BND_LINES = false>
__device__ __forceinline__ void site_force(const Lat<T> &L, int i, T *f)
{
    const int t = L.types[i];
    if (t > 0) {
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] = T(0);
        return;
    }
    GlobalAcc<T> acc(L, i);
    T h[3];
    site_force_core<T, GlobalAcc<T>, WITH_L6, BND_LINES>(L, acc, t, f, site_field(L, i, h));
}

}  // namespace qmin
