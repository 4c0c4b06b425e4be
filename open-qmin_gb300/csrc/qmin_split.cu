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

#include "qmin_force_core.cuh"

namespace qmin {

namespace {

// periodic wrap of a coordinate at most two steps outside [0, m), m >= 2
__device__ __forceinline__ int wrap_near(int v, int m) { return v < 0 ? v + m : (v >= m ? v - m : v); }

// force at the predicted Q of a deep bulk site; M applied as the reference does
// for type-0 sites (twice in CPU mode, the fields between the two)
template <class T>
__device__ __forceinline__ void deep_force(const Lat<T> &L, int i, T *f)
{
    const int x = i % L.Lx, r = i / L.Lx, y = r % L.Ly, z = r / L.Ly;
    const int sxy = L.Lx * L.Ly;
    int xi[5], yo[5], zo[5];
#pragma unroll
    for (int d = 0; d < 5; ++d) {
        xi[d] = wrap_near(x + d - 2, L.Lx);
        yo[d] = L.Lx * wrap_near(y + d - 2, L.Ly);
        zo[d] = sxy * wrap_near(z + d - 2, L.Lz);
    }
    const T *Q = L.Q;
    const long long P = L.P;
#define QQ(dx, dy, dz, c) ld(Q + (long long)(c) * P + (xi[(dx) + 2] + yo[(dy) + 2] + zo[(dz) + 2]))
    T q[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) q[k] = QQ(0, 0, 0, k);
    T force[5];
    phase_force(L.a, L.b, L.c, q, force);
    T s2[5];
    if (L.L4 == T(0)) {
        QMIN_BULK_Q25_NO_L4(L.cq, s2);
    } else {
        QMIN_BULK_Q25(L.cq, s2);
    }
#undef QQ
#pragma unroll
    for (int k = 0; k < 5; ++k) f[k] = force[k] - s2[k];
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
    acc[0] += (double)dot_qt(f, f);
    acc[1] += (double)dot_qt(v, v);
    acc[2] += (double)dot_qt(f, v);
}

int list_grid(int n) { return std::max(1, std::min((n + kBlock - 1) / kBlock, 152 * 4)); }

}  // namespace

// every deep bulk site (cls == 0); partials[0 .. gridDim.x)
template <class T, int CAP>
__global__ void __launch_bounds__(kBlock, CAP + 1)
    k_force_kick_deep(Lat<T> L, const uint8_t *__restrict__ cls, const FireDev *__restrict__ fd, double *partials)
{
    if (!fd->active) return;
    const T hdt = T(0.5) * T(fd->dt);
    double acc[3] = {0.0, 0.0, 0.0};
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        if (cls[i] != 0) continue;
        T f[5];
        deep_force(L, i, f);
        kick_and_sum(L, i, hdt, f, acc);
    }
    block_sum<3>(acc);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[3 * blockIdx.x + k] = acc[k];
}

// the listed LC sites through the derivative-plane forms
template <class T>
__global__ void __launch_bounds__(kBlock)
    k_force_kick_list(Lat<T> L, const int *__restrict__ list, int n, const FireDev *__restrict__ fd, double *partials)
{
    if (!fd->active) return;
    const T hdt = T(0.5) * T(fd->dt);
    double acc[3] = {0.0, 0.0, 0.0};
    for (int e = blockIdx.x * kBlock + threadIdx.x; e < n; e += gridDim.x * kBlock) {
        const int i = list[e];
        T f[5];
        site_force(L, i, f);
        kick_and_sum(L, i, hdt, f, acc);
    }
    block_sum<3>(acc);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[3 * blockIdx.x + k] = acc[k];
}

// twice the first derivatives (k_derivs' rules) at the listed sites only
template <class T>
__global__ void __launch_bounds__(kBlock)
    k_derivs_list(Lat<T> L, const int *__restrict__ list, int n, const FireDev *__restrict__ fd)
{
    if (!fd->active) return;
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

template <class T> int launch_split_derivs(const Lat<T> &L, const SplitLists &sl, FireDev *fd, cudaStream_t s)
{
    if (sl.n_derivs == 0) return 0;
    k_derivs_list<T><<<list_grid(sl.n_derivs), kBlock, 0, s>>>(L, sl.derivs, sl.n_derivs, fd);
    return 1;
}

template <class T>
int launch_split_force_kick(const Lat<T> &L, const SplitLists &sl, FireDev *fd, double *partials, int grid, int cap,
                            cudaStream_t s, int *nparts)
{
    if (cap == 1) k_force_kick_deep<T, 1><<<grid, kBlock, 0, s>>>(L, sl.cls, fd, partials);
    else k_force_kick_deep<T, 0><<<grid, kBlock, 0, s>>>(L, sl.cls, fd, partials);
    int n = 1, np = grid;
    if (sl.n_sites > 0) {
        const int g2 = list_grid(sl.n_sites);
        k_force_kick_list<T><<<g2, kBlock, 0, s>>>(L, sl.sites, sl.n_sites, fd, partials + 3 * grid);
        np += g2;
        ++n;
    }
    *nparts = np;
    return n;
}

template int launch_split_derivs<double>(const Lat<double> &, const SplitLists &, FireDev *, cudaStream_t);
template int launch_split_derivs<float>(const Lat<float> &, const SplitLists &, FireDev *, cudaStream_t);
template int launch_split_force_kick<double>(const Lat<double> &, const SplitLists &, FireDev *, double *, int, int,
                                             cudaStream_t, int *);
template int launch_split_force_kick<float>(const Lat<float> &, const SplitLists &, FireDev *, double *, int, int,
                                            cudaStream_t, int *);

}  // namespace qmin
