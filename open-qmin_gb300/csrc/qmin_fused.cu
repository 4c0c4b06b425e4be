// Fused FIRE iteration on shared-memory halo tiles (2.5D z-marching).
//
// One launch performs a whole FIRE iteration for every site:
//   deferred FIRE velocity mix of the previous iteration
//   -> velocity-Verlet predictor (velocityVerlet.cpp:16-25)
//   -> force at the predicted Q (landauDeGennesLC::computeForces)
//   -> second half kick (velocityVerlet.cpp:33-37)
//   -> the three FIRE reductions F.F, v.v, F.v (energyMinimizerFIRE.cpp:94-103).
// A block owns a TX x TY column of sites and walks a range of z planes.  For
// every plane entering the window it loads Q, V, F (and the site types) of the
// tile plus a halo of H sites (H = 1 one-constant, 2 multi-constant), applies
// the mix and the predictor, and keeps the predicted Q in a ring of 2H+1
// shared-memory planes; neighbour first derivatives are formed from that ring
// when the multi-constant forms need them.  State is read from one buffer set
// and written to the other (ping-pong), so no block reads a site another
// block has already advanced.
#include "qmin_force_core.cuh"

namespace qmin {

template <class T, int H, int TX, int TY> struct TileAcc {
    static constexpr int SX = TX + 2 * H, SY = TY + 2 * H, TS = SX * SY, NP = 2 * H + 1;
    const T *sQ;
    const int8_t *sT;
    const ObjDev<T> *objs;
    int slot[NP];  // ring slot of plane dz = -H..H (index dz + H)
    int p;         // centre position inside a plane

    __device__ __forceinline__ ObjDev<T> obj(int t) const { return objs[t - 1]; }
    __device__ __forceinline__ static int ndz(int s) { return s == 4 ? -1 : (s == 5 ? 1 : 0); }
    __device__ __forceinline__ static int ndp(int s)
    {
        return s == 0 ? -1 : (s == 1 ? 1 : (s == 2 ? -SX : (s == 3 ? SX : 0)));
    }
    __device__ __forceinline__ T qv(int dz, int pp, int k) const { return sQ[(slot[dz + H] * 5 + k) * TS + pp]; }
    __device__ __forceinline__ int tv(int dz, int pp) const { return sT[slot[dz + H] * TS + pp]; }
    __device__ __forceinline__ int tn(int s) const { return tv(ndz(s), p + ndp(s)); }
    __device__ __forceinline__ T q(int k) const { return qv(0, p, k); }
    __device__ __forceinline__ T nq(int s, int k) const { return qv(ndz(s), p + ndp(s), k); }
    __device__ __forceinline__ T dn(int s, int d) const
    {
        if constexpr (H < 2) {
            return T(0);
        } else {
            const int dz = ndz(s), pp = p + ndp(s);
            const int t = tv(dz, pp);
            if (t > 0) return T(0);
            const int a = d / 5, c = d % 5;
            const int odz = a == 2 ? 1 : 0, odp = a == 0 ? 1 : (a == 1 ? SX : 0);
            const T qd = qv(dz - odz, pp - odp, c), qu = qv(dz + odz, pp + odp, c);
            int td = 0, tu = 0;
            if (t < 0) {
                td = tv(dz - odz, pp - odp);
                tu = tv(dz + odz, pp + odp);
            }
            return deriv2_rule(t, td, tu, qd, qv(dz, pp, c), qu);
        }
    }
};

// Deep-bulk sites (type 0 with six type-0 neighbours): every neighbour
// derivative is a central difference, so no site types are consulted.
template <class T, int H, int TX, int TY> struct DeepTileAcc : TileAcc<T, H, TX, TY> {
    using B = TileAcc<T, H, TX, TY>;
    __device__ __forceinline__ int tn(int) const { return 0; }
    __device__ __forceinline__ T dn(int s, int d) const
    {
        if constexpr (H < 2) {
            return T(0);
        } else {
            const int dz = B::ndz(s), pp = this->p + B::ndp(s);
            const int a = d / 5, c = d % 5;
            const int odz = a == 2 ? 1 : 0, odp = a == 0 ? 1 : (a == 1 ? B::SX : 0);
            return this->qv(dz + odz, pp + odp, c) - this->qv(dz - odz, pp - odp, c);
        }
    }
};

// running sum: compensated (Kahan) FP32 for the FP32 form, plain FP64 otherwise
template <class T> struct RunSum {
    double s = 0.0;
    __device__ __forceinline__ void add(T x) { s += (double)x; }
    __device__ __forceinline__ double value() const { return s; }
};
template <> struct RunSum<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ int wrapi(int v, int m)
{
    int r = v % m;
    return r < 0 ? r + m : r;
}

template <class T, int H, int TX, int TY, int BY>
__global__ void __launch_bounds__(TX *BY) k_fire_fused(Lat<T> L, T *__restrict__ Qn, T *__restrict__ Vn,
                                                       T *__restrict__ Fn, const FireDev *__restrict__ fd,
                                                       double *partials, int zc)
{
    constexpr int NT = TX * BY, RY = TY / BY;
    using Acc = TileAcc<T, H, TX, TY>;
    constexpr int SX = Acc::SX, TS = Acc::TS, NP = Acc::NP;
    constexpr int NPOS = (TS + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sQ = reinterpret_cast<T *>(smem_raw);
    int8_t *sT = reinterpret_cast<int8_t *>(sQ + NP * 5 * TS);

    if (!fd->active) return;
    const T dt = T(fd->dt);
    const T hdt2 = T(0.5 * fd->dt * fd->dt);
    const T hdt = T(0.5) * dt;
    const bool pend = fd->pending, reset = fd->reset;
    const T ma = T(1.0 - fd->mixA), mb = T(fd->mixA * fd->mixS);

    const int ntx = (L.Lx + TX - 1) / TX;
    const int gx0 = (blockIdx.x % ntx) * TX, gy0 = (blockIdx.x / ntx) * TY;
    const int zs = blockIdx.y * zc;
    const int ze = min(L.Lz, zs + zc);
    const long long P = L.P;
    const int sxy = L.Lx * L.Ly;

    // in-plane global offsets of the positions this thread loads (same for every plane)
    int off[NPOS];
#pragma unroll
    for (int j = 0; j < NPOS; ++j) {
        const int pp = threadIdx.x + j * NT;
        off[j] = -1;
        if (pp < TS) {
            const int px = pp % SX, py = pp / SX;
            off[j] = wrapi(gx0 + px - H, L.Lx) + L.Lx * wrapi(gy0 + py - H, L.Ly);
        }
    }
    auto slot_of = [&](int z) { return (z - zs + H) % NP; };
    auto load_plane = [&](int z) {
        const int s = slot_of(z);
        const long long base = (long long)sxy * wrapi(z, L.Lz);
#pragma unroll
        for (int j = 0; j < NPOS; ++j) {
            if (off[j] < 0) continue;
            const int pp = threadIdx.x + j * NT;
            const long long i = base + off[j];
            sT[s * TS + pp] = L.types[i];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const T q = ld(L.Q + k * P + i), f = ld(L.F + k * P + i);
                T v = ld(L.V + k * P + i);
                if (pend) v = reset ? T(0) : ma * v + mb * f;
                sQ[(s * 5 + k) * TS + pp] = q + (dt * v + hdt2 * f);
            }
        }
    };

    RunSum<T> sff, svv, sfv;
    if (zs < L.Lz) {
        for (int d = -H; d < H; ++d) load_plane(zs + d);
        for (int z = zs; z < ze; ++z) {
            load_plane(z + H);
            __syncthreads();
            DeepTileAcc<T, H, TX, TY> a;
            a.sQ = sQ;
            a.sT = sT;
            a.objs = L.objs;
#pragma unroll
            for (int j = 0; j < NP; ++j) a.slot[j] = slot_of(z - H + j);
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                const int lx = threadIdx.x % TX, ly = threadIdx.x / TX + r * BY;
                const int gx = gx0 + lx, gy = gy0 + ly;
                if (gx < L.Lx && gy < L.Ly) {
                    a.p = (ly + H) * SX + (lx + H);
                    const int t = a.tv(0, a.p);
                    T f[5];
                    bool deep = (t == 0);
#pragma unroll
                    for (int sn = 0; sn < 6; ++sn) deep = deep && (a.B::tn(sn) == 0);
                    const long long i = (long long)gx + (long long)L.Lx * gy + (long long)sxy * z;
                    T hv[3];
                    const T *hp = site_field(L, i, hv);
                    if (deep) site_force_core(L, a, 0, f, hp);
                    else site_force_core(L, static_cast<const Acc &>(a), t, f, hp);
                    T v2[5];
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        const T fo = ld(L.F + k * P + i);
                        T v = ld(L.V + k * P + i);
                        if (pend) v = reset ? T(0) : ma * v + mb * fo;
                        v2[k] = (v + hdt * fo) + hdt * f[k];
                        Qn[k * P + i] = a.q(k);
                        Vn[k * P + i] = v2[k];
                        Fn[k * P + i] = f[k];
                    }
                    sff.add(dot_qt(f, f));
                    svv.add(dot_qt(v2, v2));
                    sfv.add(dot_qt(f, v2));
                }
            }
            __syncthreads();
        }
    }
    double acc[3] = {sff.value(), svv.value(), sfv.value()};
    block_sum<3, NT>(acc);
    if (threadIdx.x == 0) {
        const int b = blockIdx.y * gridDim.x + blockIdx.x;
        partials[3 * b + 0] = acc[0];
        partials[3 * b + 1] = acc[1];
        partials[3 * b + 2] = acc[2];
    }
}

// ----------------------------------------------------------- configurations
template <class T, int H, int TX, int TY, int BY> static size_t fused_smem()
{
    constexpr int TS = (TX + 2 * H) * (TY + 2 * H);
    return (size_t)(2 * H + 1) * TS * (5 * sizeof(T) + 1);
}

template <class T, int H, int TX, int TY, int BY>
static int launch_cfg(const Lat<T> &L, T *Qn, T *Vn, T *Fn, FireDev *fd, double *partials, int zc, cudaStream_t s,
                      int *nblocks)
{
    const size_t sm = fused_smem<T, H, TX, TY, BY>();
    static bool attr_set = false;  // per instantiation, per process
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_fire_fused<T, H, TX, TY, BY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm) != cudaSuccess)
            return -1;
        attr_set = true;
    }
    const int ntiles = ((L.Lx + TX - 1) / TX) * ((L.Ly + TY - 1) / TY);
    const int nz = (L.Lz + zc - 1) / zc;
    *nblocks = ntiles * nz;
    k_fire_fused<T, H, TX, TY, BY><<<dim3(ntiles, nz), TX * BY, sm, s>>>(L, Qn, Vn, Fn, fd, partials, zc);
    return 1;
}

// tile shapes the autotuner chooses from (per precision and halo width)
template <class T, int H>
int launch_fire_fused_cfg(int cfg, const Lat<T> &L, T *Qn, T *Vn, T *Fn, FireDev *fd, double *partials, int zc,
                          cudaStream_t s, int *nblocks)
{
    switch (cfg) {
    case 0: return launch_cfg<T, H, 32, 8, 8>(L, Qn, Vn, Fn, fd, partials, zc, s, nblocks);
    case 1: return launch_cfg<T, H, 32, 16, 8>(L, Qn, Vn, Fn, fd, partials, zc, s, nblocks);
    case 2: return launch_cfg<T, H, 64, 8, 4>(L, Qn, Vn, Fn, fd, partials, zc, s, nblocks);
    default: return launch_cfg<T, H, 32, 4, 4>(L, Qn, Vn, Fn, fd, partials, zc, s, nblocks);
    }
}

template <class T>
int launch_fire_fused(int cfg, const Lat<T> &L, T *Qn, T *Vn, T *Fn, FireDev *fd, double *partials, int zc,
                      cudaStream_t s, int *nblocks)
{
    return L.multi ? launch_fire_fused_cfg<T, 2>(cfg, L, Qn, Vn, Fn, fd, partials, zc, s, nblocks)
                   : launch_fire_fused_cfg<T, 1>(cfg, L, Qn, Vn, Fn, fd, partials, zc, s, nblocks);
}

int fused_tile_shape(int cfg, int *tx, int *ty)
{
    static const int shapes[4][2] = {{32, 8}, {32, 16}, {64, 8}, {32, 4}};
    if (cfg < 0 || cfg >= kFusedConfigs) return -1;
    *tx = shapes[cfg][0];
    *ty = shapes[cfg][1];
    return 0;
}

template int launch_fire_fused<double>(int, const Lat<double> &, double *, double *, double *, FireDev *, double *,
                                       int, cudaStream_t, int *);
template int launch_fire_fused<float>(int, const Lat<float> &, float *, float *, float *, FireDev *, double *, int,
                                      cudaStream_t, int *);

}  // namespace qmin
