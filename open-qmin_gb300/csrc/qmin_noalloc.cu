// qmin_energy_noalloc: the Landau-de Gennes energy of a Q field that lives in
// the caller's own device buffers, computed without allocating any memory.
//
// Who needs it: callers that cannot call cudaMalloc, for example code that
// runs inside a host framework whose device memory is all owned by its own
// pool allocator, or a caller that has already committed every byte of HBM to
// its lattice.  Such a caller passes its device arrays in and receives the
// energy in a device array it owns; the only scratch this call needs (the
// per-block partial sums of the reduction, the object table and the site
// count) sits in one file-scope static device array below.
//
// When that array exists: CUDA loads a library's device code and its static
// device arrays lazily by default (CUDA_MODULE_LOADING=LAZY), so the array
// (about 1.6 MB) and the kernels this call launches are placed on a device by
// the first call made on it, and stay there until the process exits.  A caller
// that will later commit all of its device memory makes one call on each
// device first (any small lattice), or runs with CUDA_MODULE_LOADING=EAGER.
//
// All calls share the array, so calls that overlap on the GPU (two streams,
// two host threads, or a call made while a previous call's kernels still run
// on another stream) race on it and give wrong results: serialise them.  Every
// scratch slot a call reads is first written by the same call (the object
// table is rewritten in full, the slots past nobj with a NaN sentinel), so
// nothing needs clearing between calls.
//
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/qmin_gb300.h"
#include "qmin_internal.h"

using namespace qmin;

namespace {

constexpr int kMaxBlocks = QMIN_NOALLOC_MAX_SITES / kBlock;  // one reduction block per 256 sites
constexpr int kPartials = 5 * kMaxBlocks;                    // energy partials (doubles)
constexpr int kCounts = kMaxBlocks;                          // active-site counts per block (doubles)
constexpr int kSums = 8;                                     // summed energy components
constexpr int kObjDoubles = 3 * 128;                         // object table, 128 ObjDev<double> slots
constexpr int kScratchDoubles = kPartials + kCounts + kSums + kObjDoubles;

static_assert(sizeof(ObjDev<double>) == 24, "object record layout");

// The scratch: partials | counts | sums | object table.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_addr_mutex;
double *g_addr[64] = {};  // cached device address of g_noalloc_scratch per device ordinal

// The whole object table as a kernel argument (128 x 24 B): the table reaches
// the scratch without a host-to-device copy from a host buffer.
struct ObjTable {
    ObjDev<double> o[128];
};

int noalloc_fail(int code, const std::string &m)
{
    qmin::g_last_error = m;  // reported by qmin_last_error_string
    return code;
}

// Writes all 128 slots: the caller's nobj objects, then a sentinel whose
// anchoring energy is NaN, so a site type naming an object past nobj (which
// this entry point cannot see on the host: the types are in device memory)
// turns the anchoring energy and the total into NaN instead of reading a slot
// left by an earlier call.
__global__ void k_noalloc_objects(ObjTable t, int nobj, ObjDev<double> *dst)
{
    const int k = threadIdx.x;
    if (k < 128) {
        ObjDev<double> o = t.o[k];
        if (k >= nobj) o = {0, __longlong_as_double(0x7ff8000000000000LL), __longlong_as_double(0x7ff8000000000000LL)};
        dst[k] = o;
    }
}

__global__ void __launch_bounds__(kBlock) k_count_active(const int8_t *types, int N, double *counts)
{
    const int i = blockIdx.x * kBlock + threadIdx.x;
    int c = (i < N && types[i] <= 0) ? 1 : 0;
    c = __syncthreads_count(c);
    if (threadIdx.x == 0) counts[blockIdx.x] = (double)c;
}

// E / NActive and the five components (multirankSimulation::computePotentialEnergy,
// multirankSimulation.cpp:475-490)
__global__ void __launch_bounds__(kBlock) k_noalloc_finish(const double *counts, int nblocks, const double *sums,
                                                          double *out)
{
    __shared__ double sh[kBlock];
    double c = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kBlock) c += counts[b];
    sh[threadIdx.x] = c;
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double nact = sh[0];
        const double total = sums[0] + sums[1] + sums[2] + sums[3] + sums[4];
        out[0] = nact != 0 ? total / (1.0 * nact) : total;
        for (int k = 0; k < 5; ++k) out[1 + k] = sums[k];
    }
}

}  // namespace

int qmin_energy_noalloc(const qmin_lattice_desc *desc, const qmin_ldg_params *p, const qmin_object *objs, int nobj,
                        const double *Q_dev, long long plane_stride, const int8_t *types_dev, double *out_dev,
                        void *stream)
{
    if (!desc || !p || !Q_dev || !types_dev || !out_dev || (nobj > 0 && !objs) || nobj < 0)
        return noalloc_fail(QMIN_EINVAL, "qmin_energy_noalloc: null or negative argument");
    if (desc->precision != QMIN_FP64)
        return noalloc_fail(QMIN_EINVAL, "qmin_energy_noalloc: only QMIN_FP64 (double planes) is supported");
    if (desc->Lx < 3 || desc->Ly < 3 || desc->Lz < 3)
        return noalloc_fail(QMIN_EINVAL, "qmin_energy_noalloc: every lattice side must be >= 3");
    const long long N = (long long)desc->Lx * desc->Ly * desc->Lz;
    if (N > QMIN_NOALLOC_MAX_SITES)
        return noalloc_fail(QMIN_EINVAL, "qmin_energy_noalloc: lattice has " + std::to_string(N) +
                                             " sites; this entry point's static scratch covers at most " +
                                             std::to_string(QMIN_NOALLOC_MAX_SITES) + " sites");
    if (plane_stride < N) return noalloc_fail(QMIN_EINVAL, "qmin_energy_noalloc: plane_stride < number of sites");
    if (nobj > 127) return noalloc_fail(QMIN_EINVAL, "qmin_energy_noalloc: at most 127 objects");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return noalloc_fail(QMIN_ECUDA, std::string("qmin_energy_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64)
        return noalloc_fail(QMIN_EINVAL, "qmin_energy_noalloc: device ordinal " + std::to_string(dev) +
                                             " not supported (ordinals 0..63)");
    double *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_addr_mutex);
        if (!g_addr[dev]) {
            // set-up, once per device with that device current: the host-side name of
            // g_noalloc_scratch is not a device address, so look the address up
            e = cudaGetSymbolAddress((void **)&g_addr[dev], g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_addr[dev] = nullptr;
                return noalloc_fail(QMIN_ECUDA, std::string("qmin_energy_noalloc: cudaGetSymbolAddress: ") +
                                                    cudaGetErrorString(e));
            }
        }
        base = g_addr[dev];
    }
    double *partials = base;
    double *counts = base + kPartials;
    double *sums = counts + kCounts;
    ObjDev<double> *dobjs = reinterpret_cast<ObjDev<double> *>(sums + kSums);
    cudaStream_t s = (cudaStream_t)stream;

    // object table into the scratch, as a kernel argument
    ObjTable tbl;
    memset(&tbl, 0, sizeof tbl);
    for (int k = 0; k < nobj; ++k) tbl.o[k] = {objs[k].kind, objs[k].W, objs[k].S0};
    k_noalloc_objects<<<1, 128, 0, s>>>(tbl, nobj, dobjs);

    Lat<double> L;
    memset(&L, 0, sizeof L);
    L.Lx = desc->Lx;
    L.Ly = desc->Ly;
    L.Lz = desc->Lz;
    L.N = (int)N;
    L.P = plane_stride;
    L.Q = const_cast<double *>(Q_dev);
    L.types = types_dev;
    L.objs = dobjs;
    L.a = 0.5 * p->A;
    L.b = p->B / 3.0;
    L.c = 0.25 * p->C;
    L.L1 = p->L1;
    L.L2 = p->L2;
    L.L3 = p->L3;
    L.L4 = p->L4;
    L.L6 = p->L6;
    L.multi = p->multi_constant;
    L.efield = p->efield;
    L.hfield = p->hfield;
    const int grid = (int)((N + kBlock - 1) / kBlock);
    double E0[3] = {0, 0, 0}, H0[3] = {0, 0, 0};
    launch_energy_full<double>(L, partials, grid, sums, p->efield ? p->E : E0, p->eps, p->eps0, p->deps,
                               p->hfield ? p->H : H0, p->chi, p->mu0, p->dchi, s);
    k_count_active<<<grid, kBlock, 0, s>>>(types_dev, (int)N, counts);
    k_noalloc_finish<<<1, kBlock, 0, s>>>(counts, grid, sums, out_dev);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return noalloc_fail(QMIN_ECUDA, std::string("qmin_energy_noalloc: launch: ") + cudaGetErrorString(e));
    return QMIN_OK;
}
