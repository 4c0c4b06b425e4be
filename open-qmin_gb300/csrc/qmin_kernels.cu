// qmin_gb300 CUDA kernels for sm_103a: Landau-de Gennes force/energy on the
// cubic Q-tensor lattice and the FIRE / Adam / Nesterov / L-BFGS updates.
//
// Layout: SoA planes X[k * P + i] (k = 0..4 for Q/V/F, 0..14 for the
// derivative planes), int8 site types.  Reductions are deterministic: a fixed
// grid of blocks writes per-block FP64 partials that one block sums in a
// fixed order.
#include <math.h>

#include <type_traits>

#include "qmin_force_core.cuh"

namespace qmin {

int reduction_grid(int N)
{
    int g = (N + kBlock - 1) / kBlock;
    const int cap = 152 * 8;  // 8 resident blocks per SM on the 152 SMs of a GB300
    return g < cap ? (g > 0 ? g : 1) : cap;
}

// --------------------------------------------------------- first derivatives
// landauDeGennesLC::computeFirstDerivatives (landauDeGennesLCOtherForces.cpp:15-145):
// D[5*axis + k]; central differences, one-sided at type < 0 sites with the
// "up neighbour is an object" branch first; zero at object sites.
template <class T>
__device__ __forceinline__ void site_derivs(const Lat<T> &L, int i, int t, const Nb &b, T *d)
{
    const long long P = L.P;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        const int dn = b.n[2 * ax], up = b.n[2 * ax + 1];
        const int td = t < 0 ? L.types[dn] : 0, tu = t < 0 ? L.types[up] : 0;
#pragma unroll
        for (int k = 0; k < 5; ++k)
            d[5 * ax + k] = deriv_rule(t, td, tu, ld(L.Q + k * P + dn), ld(L.Q + k * P + i), ld(L.Q + k * P + up));
    }
}

// derivative planes for the force: twice the first derivatives (see qmin_force_core.cuh)
template <class T>
__global__ void __launch_bounds__(kBlock) k_derivs(Lat<T> L)
{
    const long long P = L.P;
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        const int t = L.types[i];
        T d[15];
        if (t > 0) {
#pragma unroll
            for (int k = 0; k < 15; ++k) d[k] = T(0);
        } else {
            const Nb b = neighbours(L, i);
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                const int dn = b.n[2 * ax], up = b.n[2 * ax + 1];
                const int td = t < 0 ? L.types[dn] : 0, tu = t < 0 ? L.types[up] : 0;
#pragma unroll
                for (int k = 0; k < 5; ++k)
                    d[5 * ax + k] =
                        deriv2_rule(t, td, tu, ld(L.Q + k * P + dn), ld(L.Q + k * P + i), ld(L.Q + k * P + up));
            }
        }
#pragma unroll
        for (int k = 0; k < 15; ++k) L.D[k * L.P + i] = d[k];
    }
}

// ------------------------------------------------------------------- force
template <class T, bool WITH_L6 = false>
__global__ void __launch_bounds__(kBlock) k_force(Lat<T> L)
{
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        T f[5];
        site_force<T, WITH_L6>(L, i, f);
#pragma unroll
        for (int k = 0; k < 5; ++k) L.F[k * L.P + i] = f[k];
    }
}

// ------------------------------------------------------------------- FIRE
// velocityVerlet::integrateEOMCPU first half (velocityVerlet.cpp:16-25), preceded by
// the deferred FIRE velocity mix of the previous iteration (energyMinimizerFIRE.cpp:116-120, 143)
template <class T>
__global__ void __launch_bounds__(kBlock) k_fire_pred(Lat<T> L, const FireDev *__restrict__ fd)
{
    if (!fd->active) return;
    // With the mix ve = mv v + mf f folded into the Verlet step's coefficients
    // (scalars formed in FP64 once per launch):
    //   v' = cvv v + cvf f,   q' = q + dt v'
    // since dt v' = dt ve + dt^2/2 f is the step d: three FP64 operations per
    // element instead of five (the FP64 pipe bounds this kernel on GB300 about
    // as much as HBM does); the same quantities as q + dt ve + dt^2/2 f and
    // ve + dt/2 f up to rounding.
    const double dt = fd->dt, hdt = 0.5 * dt;
    double mv = 1.0, mf = 0.0;  // ve = mv v + mf f
    if (fd->pending) {
        mv = fd->reset ? 0.0 : 1.0 - fd->mixA;
        mf = fd->reset ? 0.0 : fd->mixA * fd->mixS;
    }
    const T cvv = T(mv), cvf = T(mf + hdt), tdt = T(dt);
    // 16-byte vectors: 5 * P is a multiple of 32 elements and the planes are 256-byte aligned
    using V4 = typename std::conditional<sizeof(T) == 8, double2, float4>::type;
    constexpr int W = 16 / sizeof(T);
    const long long n = 5 * L.P / W;
    V4 *Q4 = reinterpret_cast<V4 *>(L.Q), *Vv4 = reinterpret_cast<V4 *>(L.V);
    const V4 *F4 = reinterpret_cast<const V4 *>(L.F);
    for (long long j = blockIdx.x * (long long)kBlock + threadIdx.x; j < n; j += (long long)gridDim.x * kBlock) {
        V4 vv = Vv4[j], qq = Q4[j];
        const V4 ff = F4[j];
        T *v = reinterpret_cast<T *>(&vv), *q = reinterpret_cast<T *>(&qq);
        const T *f = reinterpret_cast<const T *>(&ff);
#pragma unroll
        for (int e = 0; e < W; ++e) {
            const T vn = cvv * v[e] + cvf * f[e];
            v[e] = vn;
            q[e] += tdt * vn;
        }
        Vv4[j] = vv;
        Q4[j] = qq;
    }
}

// force at the moved Q, second half kick (velocityVerlet.cpp:33-37) and the
// three FIRE reductions F.F, v.v, F.v in the QT metric (energyMinimizerFIRE.cpp:94-103)
// CAP limits registers so that CAP + 1 blocks of 256 threads fit per SM
template <class T, int CAP, bool WITH_L6 = false>
__global__ void __launch_bounds__(kBlock, CAP + 1)
    k_force_kick(Lat<T> L, const FireDev *__restrict__ fd, double *partials)
{
    if (!fd->active) return;
    const T hdt = T(0.5) * T(fd->dt);
    double acc[3] = {0.0, 0.0, 0.0};
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        T f[5], v[5];
        site_force<T, WITH_L6>(L, i, f);
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
    block_sum<3>(acc);
    if (threadIdx.x == 0) {
        partials[3 * blockIdx.x + 0] = acc[0];
        partials[3 * blockIdx.x + 1] = acc[1];
        partials[3 * blockIdx.x + 2] = acc[2];
    }
}

// fireStepCPU scalar logic (energyMinimizerFIRE.cpp:104-144) and the
// minimize() loop condition (:160)
__global__ void __launch_bounds__(kBlock) k_fire_control(FireDev *fd, const double *partials, int nparts)
{
    if (!fd->active) return;
    double v[3];
    sum_partials<3>(partials, nparts, v);
    if (threadIdx.x != 0) return;
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
}

// apply the last deferred velocity mix so the resident velocities match the
// reference's state at the end of minimize()
template <class T>
__global__ void __launch_bounds__(kBlock) k_fire_finish(Lat<T> L, FireDev *fd)
{
    if (!fd->pending) return;
    const bool reset = fd->reset;
    const T ma = T(1.0 - fd->mixA), mb = T(fd->mixA * fd->mixS);
    const long long n = 5 * L.P;
    for (long long j = blockIdx.x * (long long)kBlock + threadIdx.x; j < n; j += (long long)gridDim.x * kBlock)
        L.V[j] = reset ? T(0) : ma * L.V[j] + mb * L.F[j];
}

__global__ void k_fire_clear_pending(FireDev *fd) { fd->pending = 0; }

// ------------------------------------------------------------------ energy
// landauDeGennesLC::computeEnergyCPU (landauDeGennesLC.cpp:204-353): per-site
// phase, distortion, anchoring, E and H densities.  The distortion densities
// are L1/2 dk Qij dk Qij, L2/2 (dj Qij)^2, L3/2 dk Qij dj Qik and
// L4/2 eps_lik Qlj dk Qij, with the same derivative rules as the forces.
template <class T>
__device__ __forceinline__ void sym3(const T *d, T G[3][3])
{
    G[0][0] = d[0]; G[0][1] = d[1]; G[0][2] = d[2];
    G[1][0] = d[1]; G[1][1] = d[3]; G[1][2] = d[4];
    G[2][0] = d[2]; G[2][1] = d[4]; G[2][2] = -d[0] - d[3];
}

// the energy densities of one LC site (type t <= 0), added to acc[5] = phase,
// distortion, anchoring, E field, H field (landauDeGennesLC::computeEnergyCPU,
// landauDeGennesLC.cpp:204-353)
struct FieldArgs {
    double Ex, Ey, Ez, eps, eps0, deps, Hx, Hy, Hz, chi, mu0, dchi;
};
template <class T>
__device__ __forceinline__ void site_energy(const Lat<T> &L, int i, int t, const FieldArgs &fa, double *acc)
{
    const long long P = L.P;
    const double Ex = fa.Ex, Ey = fa.Ey, Ez = fa.Ez, eps = fa.eps, eps0 = fa.eps0, deps = fa.deps;
    const double Hx = fa.Hx, Hy = fa.Hy, Hz = fa.Hz, chi = fa.chi, mu0 = fa.mu0, dchi = fa.dchi;
    T q[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) q[k] = ld(L.Q + k * P + i);
    const T t2 = tr_q2(q);
    acc[0] += (double)(L.a * t2 + L.b * tr_q3(q) + L.c * (t2 * t2));
    if (L.efield) {
        const T ex = T(Ex), ey = T(Ey), ez = T(Ez), e = T(eps), e0 = T(eps0), de = T(deps);
        acc[3] += (double)(e0 * (T(-0.5) * ex * ex * (e + de * q[0]) - de * ex * ey * q[1] - de * ex * ez * q[2] -
                                 T(0.5) * ez * ez * (e - de * q[0] - de * q[3]) -
                                 T(0.5) * ey * ey * (e + de * q[3]) - de * ey * ez * q[4]));
    }
    if (L.hfield) {
        const T hx = T(Hx), hy = T(Hy), hz = T(Hz), c = T(chi), m0 = T(mu0), dc = T(dchi);
        acc[4] += (double)(m0 * (T(-0.5) * hx * hx * (c + dc * q[0]) - dc * hx * hy * q[1] - dc * hx * hz * q[2] -
                                 T(0.5) * hz * hz * (c - dc * q[0] - dc * q[3]) -
                                 T(0.5) * hy * hy * (c + dc * q[3]) - dc * hy * hz * q[4]));
    }
    if (L.Hv) {
        // landauDeGennesLC.cpp:256-265: the H-field density with this site's H
        const T hx = L.Hv[i], hy = L.Hv[P + i], hz = L.Hv[2 * P + i], c = T(chi), m0 = T(mu0), dc = T(dchi);
        acc[4] += (double)(m0 * (T(-0.5) * hx * hx * (c + dc * q[0]) - dc * hx * hy * q[1] - dc * hx * hz * q[2] -
                                 T(0.5) * hz * hz * (c - dc * q[0] - dc * q[3]) -
                                 T(0.5) * hy * hy * (c + dc * q[3]) - dc * hy * hz * q[4]));
    }
    const Nb b = neighbours(L, i);
    T d[15];
    site_derivs(L, i, t, b, d);
    if (t < 0) {
        T anch = T(0);
#pragma unroll
        for (int s = 0; s < 6; ++s) {
            const int ts = L.types[b.n[s]];
            if (ts > 0) {
                T qb[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) qb[k] = ld(L.Q + k * P + b.n[s]);
                const ObjDev<T> o = L.objs[ts - 1];
                anch += anchoring_energy(o.kind, o.W, o.S0, q, qb);
            }
        }
        acc[2] += (double)anch;
    }
    T G[3][3][3];
    sym3(d, G[0]);
    sym3(d + 5, G[1]);
    sym3(d + 10, G[2]);
    T dist = T(0);
    if (L.L1 != T(0)) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int x = 0; x < 3; ++x)
#pragma unroll
                for (int y = 0; y < 3; ++y) s += G[k][x][y] * G[k][x][y];
        dist += T(0.5) * L.L1 * s;
    }
    if (L.L2 != T(0)) {
        T s = T(0);
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            const T dv = G[0][x][0] + G[1][x][1] + G[2][x][2];
            s += dv * dv;
        }
        dist += T(0.5) * L.L2 * s;
    }
    if (L.L3 != T(0)) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int x = 0; x < 3; ++x)
#pragma unroll
                for (int y = 0; y < 3; ++y) s += G[k][x][y] * G[y][x][k];
        dist += T(0.5) * L.L3 * s;
    }
    if (L.L4 != T(0)) {
        T Qm[3][3];
        sym3(q, Qm);
        // eps_lik Q_lj dk Q_ij over the six permutations (l, i, k)
        const int perm[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {2, 1, 0}, {1, 0, 2}};
        T s = T(0);
#pragma unroll
        for (int e = 0; e < 6; ++e) {
            const T sg = e < 3 ? T(1) : T(-1);
#pragma unroll
            for (int y = 0; y < 3; ++y) s += sg * Qm[perm[e][0]][y] * G[perm[e][2]][perm[e][1]][y];
        }
        dist += T(0.5) * L.L4 * s;
    }
    if (L.L6 != T(0)) {
        // cubic term L6/2 Q_ab da Q_ij db Q_ij (landauDeGennesLC.cpp:331-334)
        T Qm[3][3];
        sym3(q, Qm);
        T s = T(0);
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int bb = 0; bb < 3; ++bb) {
                T g = T(0);
#pragma unroll
                for (int x = 0; x < 3; ++x)
#pragma unroll
                    for (int y = 0; y < 3; ++y) g += G[a][x][y] * G[bb][x][y];
                s += Qm[a][bb] * g;
            }
        dist += T(0.5) * L.L6 * s;
    }
    acc[1] += (double)dist;
}

template <class T>
__global__ void __launch_bounds__(kBlock) k_energy(Lat<T> L, double *partials, FieldArgs fa)
{
    double acc[5] = {0, 0, 0, 0, 0};
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        const int t = L.types[i];
        if (t > 0) continue;
        site_energy(L, i, t, fa, acc);
    }
    block_sum<5>(acc);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 5; ++k) partials[5 * blockIdx.x + k] = acc[k];
}

// landauDeGennesLC::computeObjectForces with computeStressTensors, one-constant form
// (landauDeGennesLCOtherForces.cpp:147-251): the force on the object whose sites
// have type j is the sum, over the LC sites next to it, of sigma . a, where
//   sigma_ab = e delta_ab - L1 B(d_a q, d_b q),
//   B(u, v)  = 2 (u0 v0 + u3 v3) + u0 v3 + u3 v0 + 4 (u1 v1 + u2 v2 + u4 v4),
// e is the site's total energy density, d_a q its first derivatives (one-sided
// next to objects) and a the unit direction (+-1 per axis) to its object
// neighbours, the up neighbour taking precedence.
template <class T>
__global__ void __launch_bounds__(kBlock) k_object_force(Lat<T> L, int j, FieldArgs fa, double *partials)
{
    double acc[3] = {0.0, 0.0, 0.0};
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        const int t = L.types[i];
        if (t > 0) continue;
        const Nb b = neighbours(L, i);
        int tn[6];
        bool next_to_j = false;
#pragma unroll
        for (int s = 0; s < 6; ++s) {
            tn[s] = L.types[b.n[s]];
            next_to_j = next_to_j || tn[s] == j;
        }
        if (!next_to_j) continue;
        double e5[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        site_energy(L, i, t, fa, e5);
        const double e = e5[0] + e5[3] + e5[4] + e5[2] + e5[1];  // phase, fields, anchoring, distortion
        T d[15];
        site_derivs(L, i, t, b, d);
        double a[3];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            a[ax] = 0.0;
            if (tn[2 * ax] > 0) a[ax] = -1.0;
            if (tn[2 * ax + 1] > 0) a[ax] = 1.0;
        }
        double sig[3][3];
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const T *u = d + 5 * p, *v = d + 5 * r;
                const double B = 2.0 * ((double)u[0] * v[0] + (double)u[3] * v[3]) + (double)u[0] * v[3] +
                                 (double)u[3] * v[0] +
                                 4.0 * ((double)u[1] * v[1] + (double)u[2] * v[2] + (double)u[4] * v[4]);
                sig[p][r] = -(double)L.L1 * B + (p == r ? e : 0.0);
            }
#pragma unroll
        for (int p = 0; p < 3; ++p) acc[p] += sig[p][0] * a[0] + sig[p][1] * a[1] + sig[p][2] * a[2];
    }
    block_sum<3>(acc);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[3 * blockIdx.x + k] = acc[k];
}

__global__ void __launch_bounds__(kBlock) k_sum3(const double *partials, int nparts, double *out)
{
    double v[3];
    sum_partials<3>(partials, nparts, v);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) out[k] = v[k];
}

__global__ void __launch_bounds__(kBlock) k_sum5(const double *partials, int nparts, double *out)
{
    double v[5];
    sum_partials<5>(partials, nparts, v);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 5; ++k) out[k] = v[k];
}

// ------------------------------------------------------- layout conversion
template <class T>
__global__ void k_aos_to_soa(const double *aos, T *soa, int N, long long P, int layout)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < 5LL * N;
         j += (long long)gridDim.x * blockDim.x) {
        long long i, k;
        if (layout == 0) { i = j / 5; k = j % 5; }
        else { k = j / N; i = j % N; }
        soa[k * P + i] = T(aos[j]);
    }
}

template <class T>
__global__ void k_soa_to_aos(const T *soa, double *aos, int N, long long P, int layout)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < 5LL * N;
         j += (long long)gridDim.x * blockDim.x) {
        long long i, k;
        if (layout == 0) { i = j / 5; k = j % 5; }
        else { k = j / N; i = j % N; }
        aos[j] = (double)soa[k * P + i];
    }
}

__global__ void k_types_to_i8(const int32_t *t32, int8_t *t8, int N)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) t8[i] = (int8_t)t32[i];
}

template <class T>
__global__ void k_fill(T *x, T v, long long n)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x)
        x[j] = v;
}

// ------------------------------------------------------------------- Adam
// energyMinimizerAdam::adamStepCPU (energyMinimizerAdam.cpp:25-54), the force
// already computed at the current Q
template <class T>
__global__ void __launch_bounds__(kBlock) k_adam(Lat<T> L, T *M, T *S, const IterDev *__restrict__ it, T beta1,
                                                 T beta2, T eps, T dt, double *partials)
{
    if (!it->active) return;
    const T c1 = T(1.0 / (1.0 - it->b1t)), c2 = T(1.0 / (1.0 - it->b2t));
    double acc[1] = {0.0};
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        T ff = T(0);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const long long j = k * L.P + i;
            const T f = L.F[j];
            ff += f * f;
            const T m = beta1 * M[j] + (beta1 - T(1)) * f;
            const T s = beta2 * S[j] + (T(1) - beta2) * (f * f);
            M[j] = m;
            S[j] = s;
            const T mc = m * c1, vc = s * c2;
            T root = sqrt(vc);
            if (root == T(0)) root = eps;
            L.Q[j] += -dt * mc / root;
        }
        acc[0] += (double)ff;
    }
    block_sum<1>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

// energyMinimizerNesterovAG::nesterovStepCPU (energyMinimizerNesterovAG.cpp:75-92)
template <class T>
__global__ void __launch_bounds__(kBlock) k_nesterov(Lat<T> L, T *alt, const IterDev *__restrict__ it, T dt, T mu,
                                                     double *partials)
{
    if (!it->active) return;
    double acc[1] = {0.0};
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        T ff = T(0);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const long long j = k * L.P + i;
            const T f = L.F[j];
            ff += f * f;
            const T old = alt[j];
            const T a = L.Q[j] + dt * f;
            alt[j] = a;
            L.Q[j] = a + mu * (a - old);
        }
        acc[0] += (double)ff;
    }
    block_sum<1>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

// energyMinimizerGradientDescent::gradientDescentCPU move (energyMinimizerGradientDescent.cpp:71):
// Q += dt F on every site (object sites carry F = 0)
template <class T>
__global__ void __launch_bounds__(kBlock) k_gd_move(Lat<T> L, const IterDev *__restrict__ it, T dt)
{
    if (!it->active) return;
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock)
#pragma unroll
        for (int k = 0; k < 5; ++k) L.Q[k * L.P + i] += dt * L.F[k * L.P + i];
}

// sum_i F_i . F_i (plain dot, energyMinimizerGradientDescent.cpp:75-79)
template <class T>
__global__ void __launch_bounds__(kBlock) k_ff_dot(Lat<T> L, const IterDev *__restrict__ it, double *partials)
{
    if (!it->active) return;
    double acc[1] = {0.0};
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        T ff = T(0);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const T f = L.F[k * L.P + i];
            ff += f * f;
        }
        acc[0] += (double)ff;
    }
    block_sum<1>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

// determinant of the traceless symmetric Q (Qzz = -Qxx - Qyy)
template <class T> __device__ __forceinline__ double det_q(const T *qt)
{
    const double xx = qt[0], xy = qt[1], xz = qt[2], yy = qt[3], yz = qt[4], zz = -xx - yy;
    return xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz);
}

// qTensorLatticeModel::computeDefectMeasures (qTensorLatticeModel.cpp:95-133) on
// sites with type <= 0 (object sites get 0): 0 the largest eigenvalue
// (trigonometric solution of the characteristic cubic, eigenvaluesOfQ,
// qTensorFunctions.h:215-241), 1 det Q, 2 (tr Q^2)^3 - 54 (det Q)^2
template <class T>
__global__ void __launch_bounds__(kBlock) k_defects(Lat<T> L, int kind, double *out)
{
    const double pi = 3.14159265358979323846;
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < L.N; i += gridDim.x * kBlock) {
        double v = 0.0;
        if (L.types[i] <= 0) {
            T qt[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) qt[k] = L.Q[k * L.P + i];
            if (kind == 0) {
                const double q0 = qt[0], q1 = qt[1], q2 = qt[2], q3 = qt[3], q4 = qt[4];
                const double off = q1 * q1 + q2 * q2 + q4 * q4;
                if (off == 0.0) {
                    v = fmax(fmax(q0, q3), -q0 - q3);
                } else {
                    // eigenvalues 2p cos(phi + 2 pi k / 3), p^2 = tr(Q^2) / 6, cos(3 phi) = det(Q / p) / 2
                    const double p = sqrt((2.0 * (q0 * q0 + q3 * q3 + q0 * q3) + 2.0 * off) / 6.0);
                    const double ip = 1.0 / p;
                    const T b[5] = {T(ip * q0), T(ip * q1), T(ip * q2), T(ip * q3), T(ip * q4)};
                    const double r = 0.5 * det_q(b);
                    const double phi = r <= -1.0 ? pi / 3.0 : (r >= 1.0 ? 0.0 : acos(r) / 3.0);
                    const double e1 = 2.0 * p * cos(phi), e3 = 2.0 * p * cos(phi + 2.0 * pi / 3.0);
                    v = fmax(fmax(e1, -e1 - e3), e3);
                }
            } else {
                const double d = det_q(qt);
                if (kind == 1) {
                    v = d;
                } else {
                    const double t2 = (double)tr_q2(qt);
                    v = t2 * t2 * t2 - 54.0 * d * d;
                }
            }
        }
        out[i] = v;
    }
}

// forceMax = sqrt(F.F) / Ndof and the while-condition of Adam / Nesterov
__global__ void __launch_bounds__(kBlock) k_norm_control(IterDev *it, const double *partials, int nparts, int adam,
                                                         double beta1, double beta2)
{
    if (!it->active) return;
    double v[1];
    sum_partials<1>(partials, nparts, v);
    if (threadIdx.x != 0) return;
    it->forceMax = sqrt(v[0]) / (double)it->ndof;
    if (adam) {
        it->b1t *= beta1;
        it->b2t *= beta2;
    }
    it->iterations += 1;
    if (!isfinite(v[0])) {
        it->status = 1;
        it->active = 0;
        return;
    }
    it->active = (it->iterations < it->max_iters && it->forceMax > it->fcut) ? 1 : 0;
}

// ------------------------------------------------------------------ L-BFGS
// energyMinimizerLoLBFGS::LoLBFGSStepCPU (energyMinimizerLoLBFGS.cpp:105-193)
// as 2m + 1 streaming passes around the force.  Each pass applies one vector
// update of the two-loop recursion and forms the dot product that the next
// update's coefficient needs, so a vector is read once per use:
//   step 2, ii = 0 .. m-2:  p += -alpha_ii y_ii;  dot s_(ii+1).p
//   ii = m-1 with step 3:   p += -alpha_(m-1) y_(m-1);  p += (sy_0 / y_0.y_0) y_0;
//                           dot y_(m-1).p (step 4's first beta)
//   step 4, ii = m-1 .. 1:  p += (alpha_ii - beta_ii) s_ii;  dot y_(ii-1).p
//   ii = 0 with the step:   p += (alpha_0 - beta_0) s_0;  s_cur = eta p;
//                           y_cur = F;  Q += s_cur
//   after the force:        y_cur += -F;  dots F.F, s_cur.y_cur, y_cur.y_cur, s_cur.F
// The vector updates are the reference's, element by element.  A stored
// pair's s.y and y.y never change, so they are formed once, in the pass after
// the force, and kept per slot; alpha_0 of the next iteration (s_0.p / s_0.y_0
// with p the new forces, the reference's unscaledStep = returnForces()) comes
// from the same pass, and the first pass of an iteration reads p from F.
// Pair ii sits in slot (cur - ii - 1 + m) % m, cur = iterations % m.
// lb[0..16): s.y per slot; lb[16..32): y.y per slot; lb[32..48): alpha per ii;
// lb[48]: alpha_ii - beta_ii of the pending step-4 update.
__device__ __forceinline__ int lb_slot(const IterDev *it, int m, int ii)
{
    const int cur = it->iterations % m;
    return (cur - ii - 1 + m) % m;
}

template <class T> struct LbVec;
template <> struct LbVec<float> {
    using V = float4;
};
template <> struct LbVec<double> {
    using V = double2;
};

// a . b over one 16-byte vector, summed in the element type (FP32: four
// products, one FP64 addition per two vectors in the caller)
__device__ __forceinline__ float vdot(const float4 &a, const float4 &b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}
__device__ __forceinline__ double vdot(const double2 &a, const double2 &b) { return a.x * b.x + a.y * b.y; }
// x + c y lane by lane (host_dVec_plusEqual_dVec), c x, x + y
__device__ __forceinline__ float4 vaxpy(const float4 &x, float c, const float4 &y)
{
    return make_float4(x.x + c * y.x, x.y + c * y.y, x.z + c * y.z, x.w + c * y.w);
}
__device__ __forceinline__ double2 vaxpy(const double2 &x, double c, const double2 &y)
{
    return make_double2(x.x + c * y.x, x.y + c * y.y);
}
__device__ __forceinline__ float4 vscale(float c, const float4 &x)
{
    return make_float4(c * x.x, c * x.y, c * x.z, c * x.w);
}
__device__ __forceinline__ double2 vscale(double c, const double2 &x) { return make_double2(c * x.x, c * x.y); }
__device__ __forceinline__ float4 vadd(const float4 &x, const float4 &y)
{
    return make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
}
__device__ __forceinline__ double2 vadd(const double2 &x, const double2 &y) { return make_double2(x.x + y.x, x.y + y.y); }

// KIND 0: step 2 at ii < m - 1;  KIND 1: step 2 at ii = m - 1 with step 3;
// KIND 2: step 4 at ii >= 1.  p_in is F in an iteration's first pass.  Two
// 16-byte vectors per thread per trip; the dot's block partial in partials[b].
template <class T, int KIND>
__global__ void __launch_bounds__(kBlock) k_lb_pass(const IterDev *__restrict__ it, int ii, int m, const T *p_in,
                                                    T *p, const T *__restrict__ sb, const T *__restrict__ yb,
                                                    long long n5, double *partials)
{
    if (!it->active) return;
    using V = typename LbVec<T>::V;
    const double *lb = it->lb;
    const long long n = n5 / (16 / sizeof(T));
    const V *x, *z = nullptr, *w = nullptr;
    T c, cw = T(0);
    bool upd = true;
    if (KIND == 0 || KIND == 1) {
        x = reinterpret_cast<const V *>(yb + lb_slot(it, m, ii) * n5);
        c = T(-lb[32 + ii]);
        if (KIND == 0) {
            z = reinterpret_cast<const V *>(sb + lb_slot(it, m, ii + 1) * n5);
        } else {
            const int t0 = lb_slot(it, m, 0);
            if (lb[16 + t0] != 0) {
                w = reinterpret_cast<const V *>(yb + t0 * n5);
                cw = T(lb[t0] / lb[16 + t0]);
            }
        }
    } else {
        const int t = lb_slot(it, m, ii);
        x = reinterpret_cast<const V *>(sb + t * n5);
        c = T(lb[48]);
        upd = lb[t] != 0;
        z = reinterpret_cast<const V *>(yb + lb_slot(it, m, ii - 1) * n5);
    }
    const V *pi = reinterpret_cast<const V *>(p_in);
    V *po = reinterpret_cast<V *>(p);
    const bool store = upd || p_in != p;
    const long long stride = (long long)gridDim.x * kBlock;
    double acc[1] = {0.0};
    for (long long j0 = blockIdx.x * (long long)kBlock + threadIdx.x; j0 < n; j0 += 2 * stride) {
        T part = T(0);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const long long j = j0 + u * stride;
            if (j < n) {
                V v = pi[j];
                V xv;
                if (upd) {
                    xv = x[j];
                    v = vaxpy(v, c, xv);
                }
                if (KIND == 1 && w) v = vaxpy(v, cw, w[j]);
                if (store) po[j] = v;
                part += vdot(KIND == 1 ? xv : z[j], v);
            }
        }
        acc[0] += (double)part;
    }
    block_sum<1>(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

// step 4 at ii = 0 and the step: p_f = p + (alpha_0 - beta_0) s_0,
// s_cur = eta p_f, y_cur = F (the old forces), Q += s_cur
template <class T>
__global__ void __launch_bounds__(kBlock) k_lb_step(const IterDev *__restrict__ it, int m, T eta, const T *p,
                                                    T *sb, T *yb, const T *F, T *Q, long long n5)
{
    if (!it->active) return;
    using V = typename LbVec<T>::V;
    const double *lb = it->lb;
    const long long n = n5 / (16 / sizeof(T));
    const int t0 = lb_slot(it, m, 0), cur = it->iterations % m;
    const bool upd = lb[t0] != 0;
    const T c = T(lb[48]);
    const V *p4 = reinterpret_cast<const V *>(p), *s0 = reinterpret_cast<const V *>(sb + t0 * n5);
    const V *F4 = reinterpret_cast<const V *>(F);
    V *sc = reinterpret_cast<V *>(sb + cur * n5), *yc = reinterpret_cast<V *>(yb + cur * n5);
    V *Q4 = reinterpret_cast<V *>(Q);
    for (long long j = blockIdx.x * (long long)kBlock + threadIdx.x; j < n; j += (long long)gridDim.x * kBlock) {
        V v = p4[j];
        if (upd) v = vaxpy(v, c, s0[j]);
        const V sv = vscale(eta, v);
        sc[j] = sv;
        yc[j] = F4[j];
        Q4[j] = vadd(Q4[j], sv);
    }
}

// y_cur += -F (F the new forces); dots F.F, s_cur.y_cur, y_cur.y_cur, s_cur.F
template <class T>
__global__ void __launch_bounds__(kBlock) k_lb_post(const IterDev *__restrict__ it, int m, const T *__restrict__ sb,
                                                    T *yb, const T *__restrict__ F, long long n5, double *partials)
{
    if (!it->active) return;
    using V = typename LbVec<T>::V;
    const long long n = n5 / (16 / sizeof(T));
    const int cur = it->iterations % m;
    const V *s = reinterpret_cast<const V *>(sb + cur * n5), *F4 = reinterpret_cast<const V *>(F);
    V *y = reinterpret_cast<V *>(yb + cur * n5);
    const long long stride = (long long)gridDim.x * kBlock;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long j0 = blockIdx.x * (long long)kBlock + threadIdx.x; j0 < n; j0 += 2 * stride) {
        T part[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const long long j = j0 + u * stride;
            if (j < n) {
                const V f = F4[j], sv = s[j];
                const V yv = vaxpy(y[j], T(-1), f);
                y[j] = yv;
                part[0] += vdot(f, f);
                part[1] += vdot(sv, yv);
                part[2] += vdot(yv, yv);
                part[3] += vdot(sv, f);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[k] += (double)part[k];
    }
    block_sum<4>(acc);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 4; ++k) partials[4 * blockIdx.x + k] = acc[k];
}

// op 0: alpha_ii = s_ii.p / s_ii.y_ii (0 when s.y = 0);
// op 1: lb[48] = alpha_ii - y_ii.p / s_ii.y_ii (unused when s.y = 0)
__global__ void __launch_bounds__(kBlock) k_lb_coef(IterDev *it, int op, int ii, int m, const double *partials,
                                                    int nparts)
{
    if (!it->active) return;
    double v[1];
    sum_partials<1>(partials, nparts, v);
    if (threadIdx.x != 0) return;
    double *lb = it->lb;
    const double sy = lb[lb_slot(it, m, ii)];
    if (op == 0) lb[32 + ii] = sy != 0 ? v[0] / sy : 0.0;
    else lb[48] = sy != 0 ? lb[32 + ii] - v[0] / sy : 0.0;
}

// after the post pass: forceMax = sqrt(F.F) / N, the iteration count and the
// stopping test; the new pair's s.y and y.y and the next iteration's alpha_0
__global__ void __launch_bounds__(kBlock) k_lb_close(IterDev *it, int m, const double *partials, int nparts)
{
    if (!it->active) return;
    double v[4];
    sum_partials<4>(partials, nparts, v);
    if (threadIdx.x != 0) return;
    double *lb = it->lb;
    const int cur = it->iterations % m;
    lb[cur] = v[1];
    lb[16 + cur] = v[2];
    lb[32] = v[1] != 0 ? v[3] / v[1] : 0.0;
    it->forceMax = sqrt(v[0]) / (double)it->ndof;
    it->iterations += 1;
    if (!isfinite(v[0])) {
        it->status = 1;
        it->active = 0;
        return;
    }
    it->active = (it->iterations < it->max_iters && it->forceMax > it->fcut) ? 1 : 0;
}

// ---------------------------------------------------------------- launchers
static int elem_grid(long long n)
{
    long long g = (n + kBlock - 1) / kBlock;
    return (int)(g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16);
}

template <class T> int launch_derivs(const Lat<T> &L, cudaStream_t s)
{
    k_derivs<T><<<elem_grid(L.N), kBlock, 0, s>>>(L);
    return 1;
}
template <class T> int launch_force(const Lat<T> &L, int grid, cudaStream_t s)
{
    if (L.multi && L.L6 == T(0) && L.split.cls) return launch_split_force(L, grid, s);
    int n = 0;
    if (L.multi) n += launch_derivs(L, s);
    if (L.L6 != T(0)) k_force<T, true><<<grid, kBlock, 0, s>>>(L);
    else k_force<T><<<grid, kBlock, 0, s>>>(L);
    return n + 1;
}
template <class T> int launch_fire_pred(const Lat<T> &L, FireDev *fd, cudaStream_t s)
{
    k_fire_pred<T><<<elem_grid(5 * L.P / (16 / sizeof(T))), kBlock, 0, s>>>(L, fd);
    return 1;
}
template <class T>
int launch_force_kick(const Lat<T> &L, FireDev *fd, double *partials, int grid, cudaStream_t s, int cap)
{
    int n = 0;
    if (L.multi) n += launch_derivs(L, s);
    return n + launch_force_kick_only(L, fd, partials, grid, s, cap);
}
template <class T>
int launch_force_kick_only(const Lat<T> &L, FireDev *fd, double *partials, int grid, cudaStream_t s, int cap)
{
    // the L6 forms exist only in the uncapped kernel
    if (L.L6 != T(0) && L.multi) k_force_kick<T, 0, true><<<grid, kBlock, 0, s>>>(L, fd, partials);
    else if (cap == 2) k_force_kick<T, 2><<<grid, kBlock, 0, s>>>(L, fd, partials);
    else if (cap == 1) k_force_kick<T, 1><<<grid, kBlock, 0, s>>>(L, fd, partials);
    else k_force_kick<T, 0><<<grid, kBlock, 0, s>>>(L, fd, partials);
    return 1;
}
int launch_fire_control(FireDev *fd, const double *partials, int nparts, cudaStream_t s)
{
    k_fire_control<<<1, kBlock, 0, s>>>(fd, partials, nparts);
    return 1;
}
template <class T> int launch_fire_finish(const Lat<T> &L, FireDev *fd, cudaStream_t s)
{
    k_fire_finish<T><<<elem_grid(5 * L.P), kBlock, 0, s>>>(L, fd);
    k_fire_clear_pending<<<1, 1, 0, s>>>(fd);
    return 2;
}
template <class T> int launch_aos_to_soa(const double *aos, T *soa, int N, long long P, int layout, cudaStream_t s)
{
    k_aos_to_soa<T><<<elem_grid(5LL * N), kBlock, 0, s>>>(aos, soa, N, P, layout);
    return 1;
}
template <class T> int launch_soa_to_aos(const T *soa, double *aos, int N, long long P, int layout, cudaStream_t s)
{
    k_soa_to_aos<T><<<elem_grid(5LL * N), kBlock, 0, s>>>(soa, aos, N, P, layout);
    return 1;
}
int launch_types_to_i8(const int32_t *t32, int8_t *t8, int N, cudaStream_t s)
{
    k_types_to_i8<<<elem_grid(N), kBlock, 0, s>>>(t32, t8, N);
    return 1;
}
template <class T> int launch_fill(T *x, T v, long long n, cudaStream_t s)
{
    k_fill<T><<<elem_grid(n), kBlock, 0, s>>>(x, v, n);
    return 1;
}
template <class T>
int launch_adam_step(const Lat<T> &L, T *M, T *S, IterDev *it, double beta1, double beta2, double eps, double dt,
                     double *partials, int grid, cudaStream_t s)
{
    k_adam<T><<<grid, kBlock, 0, s>>>(L, M, S, it, T(beta1), T(beta2), T(eps), T(dt), partials);
    return 1;
}
template <class T>
int launch_nesterov_step(const Lat<T> &L, T *alt, IterDev *it, double dt, double mu, double *partials, int grid,
                         cudaStream_t s)
{
    k_nesterov<T><<<grid, kBlock, 0, s>>>(L, alt, it, T(dt), T(mu), partials);
    return 1;
}
template <class T>
int launch_object_forces(const Lat<T> &L, int nobj, const double *E, double eps, double eps0, double deps,
                         const double *H, double chi, double mu0, double dchi, double *partials, int grid,
                         double *out, cudaStream_t s)
{
    const FieldArgs fa = {E[0], E[1], E[2], eps, eps0, deps, H[0], H[1], H[2], chi, mu0, dchi};
    for (int j = 1; j <= nobj; ++j) {
        k_object_force<T><<<grid, kBlock, 0, s>>>(L, j, fa, partials);
        k_sum3<<<1, kBlock, 0, s>>>(partials, grid, out + 3 * (j - 1));
    }
    return 2 * nobj;
}
template <class T> int launch_defects(const Lat<T> &L, int kind, double *out, cudaStream_t s)
{
    k_defects<T><<<elem_grid(L.N), kBlock, 0, s>>>(L, kind, out);
    return 1;
}
template <class T> int launch_gd_move(const Lat<T> &L, IterDev *it, double dt, cudaStream_t s)
{
    k_gd_move<T><<<elem_grid(L.N), kBlock, 0, s>>>(L, it, T(dt));
    return 1;
}
template <class T> int launch_ff_dot(const Lat<T> &L, IterDev *it, double *partials, int grid, cudaStream_t s)
{
    k_ff_dot<T><<<grid, kBlock, 0, s>>>(L, it, partials);
    return 1;
}
int launch_norm_control(IterDev *it, const double *partials, int nparts, int adam, double beta1, double beta2,
                        cudaStream_t s)
{
    k_norm_control<<<1, kBlock, 0, s>>>(it, partials, nparts, adam, beta1, beta2);
    return 1;
}
template <class T>
int launch_lbfgs_iteration(const Lat<T> &L, T *p, T *sb, T *yb, IterDev *it, int m, double eta, double *partials,
                           int grid, cudaStream_t s)
{
    const long long n5 = 5 * L.P;
    int n = 0;
    for (int ii = 0; ii < m - 1; ++ii) {
        k_lb_pass<T, 0><<<grid, kBlock, 0, s>>>(it, ii, m, ii == 0 ? L.F : p, p, sb, yb, n5, partials);
        k_lb_coef<<<1, kBlock, 0, s>>>(it, 0, ii + 1, m, partials, grid);
        n += 2;
    }
    k_lb_pass<T, 1><<<grid, kBlock, 0, s>>>(it, m - 1, m, m == 1 ? L.F : p, p, sb, yb, n5, partials);
    k_lb_coef<<<1, kBlock, 0, s>>>(it, 1, m - 1, m, partials, grid);
    n += 2;
    for (int ii = m - 1; ii >= 1; --ii) {
        k_lb_pass<T, 2><<<grid, kBlock, 0, s>>>(it, ii, m, p, p, sb, yb, n5, partials);
        k_lb_coef<<<1, kBlock, 0, s>>>(it, 1, ii - 1, m, partials, grid);
        n += 2;
    }
    k_lb_step<T><<<elem_grid(n5 / (16 / sizeof(T))), kBlock, 0, s>>>(it, m, T(eta), p, sb, yb, L.F, L.Q, n5);
    n += 1;
    // forces at the moved Q (no FIRE state: a force-only launch)
    n += launch_force(L, grid, s);
    k_lb_post<T><<<grid, kBlock, 0, s>>>(it, m, sb, yb, L.F, n5, partials);
    k_lb_close<<<1, kBlock, 0, s>>>(it, m, partials, grid);
    return n + 2;
}

template <class T>
int launch_energy_full(const Lat<T> &L, double *partials, int grid, double *out5, const double *E, double eps,
                       double eps0, double deps, const double *H, double chi, double mu0, double dchi, cudaStream_t s)
{
    const FieldArgs fa = {E[0], E[1], E[2], eps, eps0, deps, H[0], H[1], H[2], chi, mu0, dchi};
    k_energy<T><<<grid, kBlock, 0, s>>>(L, partials, fa);
    k_sum5<<<1, kBlock, 0, s>>>(partials, grid, out5);
    return 2;
}

#define QMIN_INSTANTIATE(T)                                                                                       \
    template int launch_derivs<T>(const Lat<T> &, cudaStream_t);                                                   \
    template int launch_force<T>(const Lat<T> &, int, cudaStream_t);                                               \
    template int launch_fire_pred<T>(const Lat<T> &, FireDev *, cudaStream_t);                                     \
    template int launch_force_kick<T>(const Lat<T> &, FireDev *, double *, int, cudaStream_t, int);                \
    template int launch_force_kick_only<T>(const Lat<T> &, FireDev *, double *, int, cudaStream_t, int);           \
    template int launch_fire_finish<T>(const Lat<T> &, FireDev *, cudaStream_t);                                   \
    template int launch_aos_to_soa<T>(const double *, T *, int, long long, int, cudaStream_t);                     \
    template int launch_soa_to_aos<T>(const T *, double *, int, long long, int, cudaStream_t);                     \
    template int launch_fill<T>(T *, T, long long, cudaStream_t);                                                  \
    template int launch_adam_step<T>(const Lat<T> &, T *, T *, IterDev *, double, double, double, double,          \
                                     double *, int, cudaStream_t);                                                 \
    template int launch_nesterov_step<T>(const Lat<T> &, T *, IterDev *, double, double, double *, int,            \
                                         cudaStream_t);                                                            \
    template int launch_defects<T>(const Lat<T> &, int, double *, cudaStream_t);                                   \
    template int launch_object_forces<T>(const Lat<T> &, int, const double *, double, double, double,               \
                                         const double *, double, double, double, double *, int, double *,          \
                                         cudaStream_t);                                   \
    template int launch_gd_move<T>(const Lat<T> &, IterDev *, double, cudaStream_t);                                 \
    template int launch_ff_dot<T>(const Lat<T> &, IterDev *, double *, int, cudaStream_t);                          \
    template int launch_lbfgs_iteration<T>(const Lat<T> &, T *, T *, T *, IterDev *, int, double, double *, int,   \
                                           cudaStream_t);                                                          \
    template int launch_energy_full<T>(const Lat<T> &, double *, int, double *, const double *, double, double,    \
                                       double, const double *, double, double, double, cudaStream_t);

QMIN_INSTANTIATE(double)
QMIN_INSTANTIATE(float)

}  // namespace qmin
