// Force + second half kick of a FIRE iteration from shared-memory tiles.
//
// Same work and results per site as k_force_kick (landauDeGennesLC::computeForces
// at the predicted Q, velocityVerlet.cpp:33-37 half kick, the three FIRE
// reductions of energyMinimizerFIRE.cpp:94-103), but every operand the force
// stencil reads comes from shared memory: a block owns a TX x TY column of
// sites and walks a range of z planes, keeping a ring of four planes of
// (Q, the 15 derivative planes, site types) for the tile plus a one-site halo.
// Plane z+2 streams in with cp.async while plane z is computed, so the ~100
// neighbour operands of a multi-constant site are shared-memory loads instead
// of dependent L1/L2 round trips.
#include "qmin_force_core.cuh"

namespace qmin {

namespace {

__device__ __forceinline__ int wrapt(int v, int m)
{
    int r = v % m;
    return r < 0 ? r + m : r;
}

template <class T> __device__ __forceinline__ void cp_async(T *smem, const T *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all_but_newest() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

}  // namespace

// accessor over the staged ring: slot s0 holds plane z, sm plane z-1, sp plane z+1
template <class T, bool MULTI, int TX, int TY> struct StagedAcc {
    static constexpr int SX = TX + 2, TS = SX * (TY + 2);
    const T *sQ;
    const T *sD;
    const int8_t *sT;
    const ObjDev<T> *objs;
    int s0, sm, sp, p;
    __device__ __forceinline__ int slot(int s) const { return s == 4 ? sm : (s == 5 ? sp : s0); }
    __device__ __forceinline__ int pos(int s) const
    {
        return p + (s == 0 ? -1 : (s == 1 ? 1 : (s == 2 ? -SX : (s == 3 ? SX : 0))));
    }
    __device__ __forceinline__ ObjDev<T> obj(int t) const { return objs[t - 1]; }
    __device__ __forceinline__ int tn(int s) const { return sT[slot(s) * TS + pos(s)]; }
    __device__ __forceinline__ T q(int k) const { return sQ[(s0 * 5 + k) * TS + p]; }
    __device__ __forceinline__ T nq(int s, int k) const { return sQ[(slot(s) * 5 + k) * TS + pos(s)]; }
    __device__ __forceinline__ T dn(int s, int d) const
    {
        if constexpr (MULTI) return sD[(slot(s) * 15 + d) * TS + pos(s)];
        else return T(0);
    }
};

template <class T, bool MULTI, int TX, int TY> constexpr size_t tiled_smem()
{
    constexpr int TS = (TX + 2) * (TY + 2);
    constexpr int NC = MULTI ? 20 : 5;
    return ((size_t)4 * TS * (NC * sizeof(T) + 1) + 15) / 16 * 16;
}

template <class T, bool MULTI, int TX, int TY, int BY>
__global__ void __launch_bounds__(TX *BY, (sizeof(T) == 4 && MULTI) ? 2 : 1)
    k_force_kick_tiled(Lat<T> L, const FireDev *__restrict__ fd, double *partials, int zc)
{
    constexpr int NT = TX * BY, RY = TY / BY, NS = 4;
    using Acc = StagedAcc<T, MULTI, TX, TY>;
    constexpr int SX = Acc::SX, TS = Acc::TS;
    constexpr int NPOS = (TS + NT - 1) / NT;
    constexpr int NC = MULTI ? 20 : 5;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sQ = reinterpret_cast<T *>(smem_raw);  // [NS][5][TS]
    T *sD = sQ + NS * 5 * TS;                  // [NS][15][TS] when MULTI
    int8_t *sT = reinterpret_cast<int8_t *>(sQ + NS * NC * TS);  // [NS][TS]

    if (!fd->active) return;
    const T hdt = T(0.5) * T(fd->dt);
    const int ntx = (L.Lx + TX - 1) / TX;
    const int gx0 = (blockIdx.x % ntx) * TX, gy0 = (blockIdx.x / ntx) * TY;
    const int zs = blockIdx.y * zc;
    const int ze = min(L.Lz, zs + zc);
    const long long P = L.P;
    const int sxy = L.Lx * L.Ly;

    // in-plane global offsets of the tile positions this thread stages
    int off[NPOS];
#pragma unroll
    for (int j = 0; j < NPOS; ++j) {
        const int pp = threadIdx.x + j * NT;
        off[j] = -1;
        if (pp < TS) off[j] = wrapt(gx0 + pp % SX - 1, L.Lx) + L.Lx * wrapt(gy0 + pp / SX - 1, L.Ly);
    }
    auto slot_of = [&](int z) { return (z - zs + 1) & 3; };
    auto issue = [&](int z) {
        const int s = slot_of(z);
        const long long base = (long long)sxy * wrapt(z, L.Lz);
#pragma unroll
        for (int j = 0; j < NPOS; ++j) {
            if (off[j] < 0) continue;
            const int pp = threadIdx.x + j * NT;
            const long long i = base + off[j];
#pragma unroll
            for (int k = 0; k < 5; ++k) cp_async(&sQ[(s * 5 + k) * TS + pp], L.Q + k * P + i);
            if constexpr (MULTI) {
#pragma unroll
                for (int d = 0; d < 15; ++d) cp_async(&sD[(s * 15 + d) * TS + pp], L.D + d * P + i);
            }
        }
    };
    auto load_types = [&](int z, int (&tr)[NPOS]) {
        const long long base = (long long)sxy * wrapt(z, L.Lz);
#pragma unroll
        for (int j = 0; j < NPOS; ++j) tr[j] = off[j] >= 0 ? (int)L.types[base + off[j]] : 0;
    };
    auto store_types = [&](int z, const int (&tr)[NPOS]) {
        const int s = slot_of(z);
#pragma unroll
        for (int j = 0; j < NPOS; ++j) {
            const int pp = threadIdx.x + j * NT;
            if (pp < TS) sT[s * TS + pp] = (int8_t)tr[j];
        }
    };

    double acc3[3] = {0.0, 0.0, 0.0};
    if (zs < L.Lz) {
        for (int z = zs - 1; z <= zs + 1; ++z) {
            issue(z);
            cp_async_commit();
            int tr[NPOS];
            load_types(z, tr);
            store_types(z, tr);
        }
        for (int z = zs; z < ze; ++z) {
            const bool more = z + 2 <= ze;
            int tr[NPOS];
            if (more) {
                issue(z + 2);
                load_types(z + 2, tr);
            }
            cp_async_commit();
            cp_async_wait_all_but_newest();
            __syncthreads();
            Acc a;
            a.sQ = sQ;
            a.sD = sD;
            a.sT = sT;
            a.objs = L.objs;
            a.s0 = slot_of(z);
            a.sm = slot_of(z - 1);
            a.sp = slot_of(z + 1);
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                const int lx = threadIdx.x % TX, ly = threadIdx.x / TX + r * BY;
                const int gx = gx0 + lx, gy = gy0 + ly;
                if (gx < L.Lx && gy < L.Ly) {
                    const long long i = (long long)gx + (long long)L.Lx * gy + (long long)sxy * z;
                    T vo[5];
#pragma unroll
                    for (int k = 0; k < 5; ++k) vo[k] = L.V[k * P + i];
                    a.p = (ly + 1) * SX + (lx + 1);
                    T f[5], v[5];
                    T hv[3];
                    site_force_core(L, a, (int)sT[a.s0 * TS + a.p], f, site_field(L, i, hv));
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        v[k] = vo[k] + hdt * f[k];
                        L.F[k * P + i] = f[k];
                        L.V[k * P + i] = v[k];
                    }
                    acc3[0] += (double)dot_qt(f, f);
                    acc3[1] += (double)dot_qt(v, v);
                    acc3[2] += (double)dot_qt(f, v);
                }
            }
            if (more) store_types(z + 2, tr);
            __syncthreads();
        }
    }
    block_sum<3, NT>(acc3);
    if (threadIdx.x == 0) {
        const int b = blockIdx.y * gridDim.x + blockIdx.x;
        partials[3 * b + 0] = acc3[0];
        partials[3 * b + 1] = acc3[1];
        partials[3 * b + 2] = acc3[2];
    }
}

namespace {

template <class T, bool MULTI, int TX, int TY, int BY>
int launch_tiled(const Lat<T> &L, FireDev *fd, double *partials, int zc, cudaStream_t s, int *nblocks)
{
    constexpr size_t sm = tiled_smem<T, MULTI, TX, TY>();
    static bool attr_set = false;  // per instantiation, per process
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_force_kick_tiled<T, MULTI, TX, TY, BY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm) != cudaSuccess)
            return -1;
        attr_set = true;
    }
    const int ntiles = ((L.Lx + TX - 1) / TX) * ((L.Ly + TY - 1) / TY);
    const int nz = (L.Lz + zc - 1) / zc;
    *nblocks = ntiles * nz;
    k_force_kick_tiled<T, MULTI, TX, TY, BY><<<dim3(ntiles, nz), TX * BY, sm, s>>>(L, fd, partials, zc);
    return 1;
}

template <class T, bool MULTI>
int launch_tiled_cfg(int cfg, const Lat<T> &L, FireDev *fd, double *partials, int zc, cudaStream_t s, int *nb)
{
    switch (cfg) {
    case 0: return launch_tiled<T, MULTI, 32, 8, 8>(L, fd, partials, zc, s, nb);
    case 1: return launch_tiled<T, MULTI, 32, 4, 4>(L, fd, partials, zc, s, nb);
    default: return launch_tiled<T, MULTI, 16, 16, 16>(L, fd, partials, zc, s, nb);
    }
}

}  // namespace

// The staged force + kick for the FP32 form (the FP64 form is bound by the
// FP64 pipe, and its doubled tiles would leave one block per SM).
template <class T>
int launch_force_kick_tiled(int cfg, const Lat<T> &L, FireDev *fd, double *partials, int zc, cudaStream_t s,
                            int *nblocks)
{
    if constexpr (sizeof(T) != 4) {
        return -1;
    } else {
        if (cfg < 0 || cfg >= kTiledConfigs) return -1;
        return L.multi ? launch_tiled_cfg<T, true>(cfg, L, fd, partials, zc, s, nblocks)
                       : launch_tiled_cfg<T, false>(cfg, L, fd, partials, zc, s, nblocks);
    }
}

int tiled_tile_shape(int cfg, int *tx, int *ty)
{
    static const int shapes[kTiledConfigs][2] = {{32, 8}, {32, 4}, {16, 16}};
    if (cfg < 0 || cfg >= kTiledConfigs) return -1;
    *tx = shapes[cfg][0];
    *ty = shapes[cfg][1];
    return 0;
}

template int launch_force_kick_tiled<double>(int, const Lat<double> &, FireDev *, double *, int, cudaStream_t, int *);
template int launch_force_kick_tiled<float>(int, const Lat<float> &, FireDev *, double *, int, cudaStream_t, int *);

}  // namespace qmin
