// Site-type scan and the split path's site classes and lists, built on the GPU
// from the device copy of the site types (qmin_set_state, qmin_checkpoint_load).
//
// Classes: 0 = deep bulk site (type 0 with six type-0 neighbours), 1 = listed
// LC site (any other type <= 0), 2 = object site.  Lists: the listed sites
// grouped by the form their force takes (0: bulk-like; 1 + xx + 3 yy + 9 zz:
// lcForce::getBoundaryCase with the down neighbour winning, lcForces.h:13-25),
// in site order within a form; and, in site order, the sites whose derivative
// planes the listed forms read (the listed sites' neighbours).  Both lists come
// from a deterministic bucket compaction (per-chunk histograms, an exclusive
// scan, then a one-warp-per-chunk scatter that ranks equal keys with
// __match_any_sync), so they are the same on every run.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "qmin_internal.h"

namespace qmin {

namespace {

constexpr int kScanBlock = 256;
constexpr int kBucketChunk = 4096;  // sites per compaction chunk (one warp each)
constexpr uint8_t kNoBucket = 255;

// per-block min and max type, count of types <= 0, count of sites whose type
// differs from the previous device types (when old8 is given)
template <class TT>
__global__ void __launch_bounds__(kScanBlock)
    k_types_scan(const TT *__restrict__ t32, const int8_t *__restrict__ old8, int N, int *part)
{
    int mn = 1 << 30, mx = -(1 << 30), act = 0, chg = 0;
    for (int i = blockIdx.x * kScanBlock + threadIdx.x; i < N; i += gridDim.x * kScanBlock) {
        const int t = t32[i];
        mn = min(mn, t);
        mx = max(mx, t);
        act += t <= 0;
        if (old8) chg += (int)old8[i] != t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        act += __shfl_xor_sync(0xffffffffu, act, o);
        chg += __shfl_xor_sync(0xffffffffu, chg, o);
    }
    __shared__ int sh[4][kScanBlock / 32];
    const int w = threadIdx.x / 32;
    if ((threadIdx.x & 31) == 0) {
        sh[0][w] = mn;
        sh[1][w] = mx;
        sh[2][w] = act;
        sh[3][w] = chg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kScanBlock / 32; ++k) {
            mn = min(mn, sh[0][k]);
            mx = max(mx, sh[1][k]);
            act += sh[2][k];
            chg += sh[3][k];
        }
        part[4 * blockIdx.x + 0] = mn;
        part[4 * blockIdx.x + 1] = mx;
        part[4 * blockIdx.x + 2] = act;
        part[4 * blockIdx.x + 3] = chg;
    }
}

__global__ void k_types_scan_finish(const int *part, int nparts, int *out)
{
    if (threadIdx.x != 0) return;
    int mn = 1 << 30, mx = -(1 << 30), act = 0, chg = 0;
    for (int b = 0; b < nparts; ++b) {
        mn = min(mn, part[4 * b]);
        mx = max(mx, part[4 * b + 1]);
        act += part[4 * b + 2];
        chg += part[4 * b + 3];
    }
    out[0] = mn;
    out[1] = mx;
    out[2] = act;
    out[3] = chg;
}

__device__ __forceinline__ void site_xyz(int i, int Lx, int Ly, int &x, int &y, int &z)
{
    x = i % Lx;
    const int r = i / Lx;
    y = r % Ly;
    z = r / Ly;
}

// class of every site and the form key of the listed sites (kNoBucket otherwise)
__global__ void __launch_bounds__(kScanBlock)
    k_split_classify(const int8_t *__restrict__ t8, int Lx, int Ly, int Lz, uint8_t *cls, uint8_t *key)
{
    const int N = Lx * Ly * Lz;
    for (int i = blockIdx.x * kScanBlock + threadIdx.x; i < N; i += gridDim.x * kScanBlock) {
        const int t = t8[i];
        if (t > 0) {
            cls[i] = 2;
            key[i] = kNoBucket;
            continue;
        }
        int x, y, z;
        site_xyz(i, Lx, Ly, x, y, z);
        const int xm = (x == 0 ? Lx - 1 : x - 1) + Lx * (y + Ly * z);
        const int xp = (x == Lx - 1 ? 0 : x + 1) + Lx * (y + Ly * z);
        const int ym = x + Lx * ((y == 0 ? Ly - 1 : y - 1) + Ly * z);
        const int yp = x + Lx * ((y == Ly - 1 ? 0 : y + 1) + Ly * z);
        const int zm = x + Lx * (y + Ly * (z == 0 ? Lz - 1 : z - 1));
        const int zp = x + Lx * (y + Ly * (z == Lz - 1 ? 0 : z + 1));
        const int txm = t8[xm], txp = t8[xp], tym = t8[ym], typ = t8[yp], tzm = t8[zm], tzp = t8[zp];
        const bool deep = t == 0 && txm == 0 && txp == 0 && tym == 0 && typ == 0 && tzm == 0 && tzp == 0;
        cls[i] = deep ? 0 : 1;
        if (deep) {
            key[i] = kNoBucket;
            continue;
        }
        int form = 0;
        if (t == -1) {
            int xx = 0, yy = 0, zz = 0;  // the down neighbour wins
            if (txp > 0) xx = 1;
            if (txm > 0) xx = 2;
            if (typ > 0) yy = 1;
            if (tym > 0) yy = 2;
            if (tzp > 0) zz = 1;
            if (tzm > 0) zz = 2;
            form = 1 + xx + 3 * yy + 9 * zz;
        }
        key[i] = (uint8_t)form;
    }
}

// key 0 at every LC site one of whose six neighbours is a listed site (an
// object site's derivative planes are zero, and stay so: they are never listed)
__global__ void __launch_bounds__(kScanBlock)
    k_split_need(const uint8_t *__restrict__ cls, int Lx, int Ly, int Lz, uint8_t *key)
{
    const int N = Lx * Ly * Lz;
    for (int i = blockIdx.x * kScanBlock + threadIdx.x; i < N; i += gridDim.x * kScanBlock) {
        int x, y, z;
        site_xyz(i, Lx, Ly, x, y, z);
        const bool need = cls[i] != 2 && (cls[(x == 0 ? Lx - 1 : x - 1) + Lx * (y + Ly * z)] == 1 ||
                          cls[(x == Lx - 1 ? 0 : x + 1) + Lx * (y + Ly * z)] == 1 ||
                          cls[x + Lx * ((y == 0 ? Ly - 1 : y - 1) + Ly * z)] == 1 ||
                          cls[x + Lx * ((y == Ly - 1 ? 0 : y + 1) + Ly * z)] == 1 ||
                          cls[x + Lx * (y + Ly * (z == 0 ? Lz - 1 : z - 1))] == 1 ||
                          cls[x + Lx * (y + Ly * (z == Lz - 1 ? 0 : z + 1))] == 1);
        key[i] = need ? 0 : kNoBucket;
    }
}

// per-chunk histogram of the keys below NB
template <int NB>
__global__ void __launch_bounds__(kScanBlock) k_bucket_count(const uint8_t *__restrict__ key, int N, int *counts)
{
    __shared__ int h[NB];
    for (int b = threadIdx.x; b < NB; b += kScanBlock) h[b] = 0;
    __syncthreads();
    const int i0 = blockIdx.x * kBucketChunk, i1 = min(N, i0 + kBucketChunk);
    for (int i = i0 + threadIdx.x; i < i1; i += kScanBlock) {
        const int k = key[i];
        if (k < NB) atomicAdd(&h[k], 1);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < NB; b += kScanBlock) counts[blockIdx.x * NB + b] = h[b];
}

// offsets[chunk][bucket]: the list is bucket-major, chunk order within a bucket;
// totals[bucket] the bucket sizes.  One block; each bucket is an exclusive scan
// over the chunks, in fixed order.
template <int NB>
__global__ void __launch_bounds__(1024) k_bucket_offsets(const int *counts, int nchunks, int *offsets, int *totals)
{
    __shared__ int carry;
    __shared__ int warp_sums[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < NB; ++b) {
        for (int c0 = 0; c0 < nchunks; c0 += 1024) {
            const int c = c0 + threadIdx.x;
            const int v = c < nchunks ? counts[c * NB + b] : 0;
            // inclusive scan within the block
            int s = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int n = __shfl_up_sync(0xffffffffu, s, o);
                if ((threadIdx.x & 31) >= o) s += n;
            }
            if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x / 32] = s;
            __syncthreads();
            if (threadIdx.x < 32) {
                int ws = warp_sums[threadIdx.x];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int n = __shfl_up_sync(0xffffffffu, ws, o);
                    if (threadIdx.x >= o) ws += n;
                }
                warp_sums[threadIdx.x] = ws;
            }
            __syncthreads();
            const int before = (threadIdx.x >= 32 ? warp_sums[threadIdx.x / 32 - 1] : 0) + s - v;
            if (c < nchunks) offsets[c * NB + b] = carry + before;
            __syncthreads();
            if (threadIdx.x == 1023) carry += before + v;
            __syncthreads();
        }
        if (threadIdx.x == 0) totals[b] = carry;  // the running end of bucket b
        __syncthreads();
    }
    // running ends to sizes
    if (threadIdx.x == 0)
        for (int b = NB - 1; b > 0; --b) totals[b] -= totals[b - 1];
}

// one warp per chunk: every site with key k < NB goes to offsets[chunk][k] +
// (its rank among the chunk's earlier sites with key k)
template <int NB>
__global__ void __launch_bounds__(32)
    k_bucket_scatter(const uint8_t *__restrict__ key, int N, const int *__restrict__ offsets, int *out)
{
    __shared__ int run[NB];
    for (int b = threadIdx.x; b < NB; b += 32) run[b] = offsets[blockIdx.x * NB + b];
    __syncwarp();
    const int lane = threadIdx.x;
    const unsigned lt = (1u << lane) - 1u;
    const int i0 = blockIdx.x * kBucketChunk, i1 = min(N, i0 + kBucketChunk);
    for (int base = i0; base < i1; base += 32) {
        const int i = base + lane;
        const int k = i < i1 ? (int)key[i] : (int)kNoBucket;
        const unsigned same = __match_any_sync(0xffffffffu, k);
        const int rank = __popc(same & lt);
        int pos = 0;
        if (k < NB) pos = run[k] + rank;
        __syncwarp();
        if (k < NB) {
            out[pos] = i;
            if (rank == __popc(same) - 1) run[k] += __popc(same);  // the group's last lane advances it
        }
        __syncwarp();
    }
}

constexpr int kForms = 28;  // listed-site forms: bulk-like and the 27 boundary cases

}  // namespace

template <class TT>
int scan_types(const TT *t, const int8_t *old8, int N, int *part, int *out_dev, int *out_host, cudaStream_t s)
{
    const int grid = std::max(1, std::min((N + kScanBlock - 1) / kScanBlock, 152 * 4));
    k_types_scan<TT><<<grid, kScanBlock, 0, s>>>(t, old8, N, part);
    k_types_scan_finish<<<1, 32, 0, s>>>(part, grid, out_dev);
    if (cudaMemcpyAsync(out_host, out_dev, 4 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    return 2;
}

template int scan_types<int32_t>(const int32_t *, const int8_t *, int, int *, int *, int *, cudaStream_t);
template int scan_types<int8_t>(const int8_t *, const int8_t *, int, int *, int *, int *, cudaStream_t);

size_t split_scratch_bytes(int N)
{
    const size_t nch = ((size_t)N + kBucketChunk - 1) / kBucketChunk;
    return 2 * (size_t)N + 4 * nch * kForms * sizeof(int) + 64 * sizeof(int);
}

int build_split_lists_dev(const int8_t *t8, int Lx, int Ly, int Lz, uint8_t *cls, void *scratch, int *host_totals,
                          int **sites, int *sites_cap, int *n_sites, int **derivs, int *derivs_cap, int *n_derivs,
                          cudaStream_t s)
{
    const int N = Lx * Ly * Lz;
    const int nch = (N + kBucketChunk - 1) / kBucketChunk;
    uint8_t *key = reinterpret_cast<uint8_t *>(scratch);
    uint8_t *key2 = key + N;
    int *ib = reinterpret_cast<int *>(reinterpret_cast<uintptr_t>(key2 + N + 15) & ~(uintptr_t)15);
    int *counts = ib, *offsets = counts + (size_t)nch * kForms, *counts2 = offsets + (size_t)nch * kForms,
        *offsets2 = counts2 + nch, *totals = offsets2 + nch;  // totals: kForms + 1 ints
    const int grid = std::max(1, std::min((N + kScanBlock - 1) / kScanBlock, 152 * 8));
    int n = 0;
    k_split_classify<<<grid, kScanBlock, 0, s>>>(t8, Lx, Ly, Lz, cls, key);
    k_split_need<<<grid, kScanBlock, 0, s>>>(cls, Lx, Ly, Lz, key2);
    k_bucket_count<kForms><<<nch, kScanBlock, 0, s>>>(key, N, counts);
    k_bucket_count<1><<<nch, kScanBlock, 0, s>>>(key2, N, counts2);
    k_bucket_offsets<kForms><<<1, 1024, 0, s>>>(counts, nch, offsets, totals);
    k_bucket_offsets<1><<<1, 1024, 0, s>>>(counts2, nch, offsets2, totals + kForms);
    n += 6;
    if (cudaMemcpyAsync(host_totals, totals, (kForms + 1) * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return -1;
    int ns = 0;
    for (int b = 0; b < kForms; ++b) ns += host_totals[b];
    const int nd = host_totals[kForms];
    auto ensure = [&](int **p, int *cap, int need) -> bool {
        if (need <= *cap && *p) return true;
        if (*p) cudaFree(*p);
        *p = nullptr;
        *cap = 0;
        if (cudaMalloc(p, sizeof(int) * (size_t)std::max(need, 1)) != cudaSuccess) return false;
        *cap = std::max(need, 1);
        return true;
    };
    if (!ensure(sites, sites_cap, ns) || !ensure(derivs, derivs_cap, nd)) return -2;
    if (ns > 0) {
        k_bucket_scatter<kForms><<<nch, 32, 0, s>>>(key, N, offsets, *sites);
        ++n;
    }
    if (nd > 0) {
        k_bucket_scatter<1><<<nch, 32, 0, s>>>(key2, N, offsets2, *derivs);
        ++n;
    }
    *n_sites = ns;
    *n_derivs = nd;
    if (cudaGetLastError() != cudaSuccess) return -1;
    return n;
}

}  // namespace qmin
