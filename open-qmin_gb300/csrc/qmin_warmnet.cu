// Learned warm start: a small 3-D U-Net that maps (random initial Q, object
// and boundary masks, anchoring kind and strength) to a near-minimal Q field,
// which FIRE then finishes.  No reference counterpart: the reference has no
// learned component.
//
// Layout: activations channels-last, [sample][z][y][x][channel]; every
// tensor-core operand BF16, every accumulator and gradient FP32.  Each
// convolution (3x3x3 or 1x1x1, stride 1 or 2, zero padding) is an implicit
// GEMM on the BF16 tensor cores: by default tcgen05.mma with tensor-memory
// accumulators (a direct kernel with TMA-staged halo planes for the 3^3
// stride-1 layers of 32 and 48 output channels, a gathering kernel
// otherwise), or mma.sync m16n8k16 (tensor path 0; the weight gradient
// always), FP32 accumulate:
//   forward:      out[v][co]      = sum_{tap,ci} in[src(v,tap)][ci] * W[co][tap][ci]
//   data grad:    din[u][ci]      = sum_{tap,co} dout[src'(u,tap)][co] * W'[ci][tap][co]
//   weight grad:  dW[co][tap][ci] = sum_v dout[v][co] * in[src(v,tap)][ci]
//
// Network (levels l = 0..3 have grid (Lx, Ly, Lz) >> l):
//   0 enc0  3^3 s1 16->32 (l0) | 1 enc1 3^3 s2 32->48 (l1) | 2 enc2 3^3 s2 48->64 (l2)
//   3 enc3  3^3 s2 64->128 (l3)
//   4 dec2a 1^3 128->64 (l3), x2 nearest up + enc2 -> 5 dec2b 3^3 64->64 (l2)
//   6 dec1a 1^3 64->48 (l2),  x2 up + enc1        -> 7 dec1b 3^3 48->48 (l1)
//   8 dec0a 1^3 48->32 (l1),  x2 up + enc0        -> 9 dec0b 3^3 32->32 (l0)
//  10 head  1^3 32->16 (l0), no ReLU; channels 0..4 are the predicted Q
// ReLU after every 3^3 convolution; the 1^3 convolutions before an
// upsampling are linear, so they run on the coarse grid (they commute with
// nearest upsampling).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/qmin_gb300.h"
#include "qmin_internal.h"

namespace qmin {
namespace nn {

typedef __nv_bfloat16 bf16;

constexpr int kIn = 16;     // input channels (10 used)
constexpr int kOut = 16;    // head channels (5 used)
constexpr int kLayers = 11;
constexpr int kMaxObj = 64;

struct Geo {
    int Di, Hi, Wi;  // gathered (input) grid: z, y, x
    int Do, Ho, Wo;  // GEMM-row (output) grid
    int cin;         // channels of the gathered tensor (multiple of 16)
    int cout;        // GEMM columns (multiple of 8)
    int taps;        // 27 or 1
    int stride;      // 1 or 2
    int mode;        // 0 forward gather; 1 the transposed gather of a stride-2 conv
    int nb;          // samples (rows = nb * Do * Ho * Wo)
};

// flat source voxel (sample offset included) of GEMM row r for one tap, or -1
__device__ __forceinline__ int gather_src(const Geo &g, int r, int tap)
{
    const int vo = g.Do * g.Ho * g.Wo;
    const int b = r / vo;
    int rem = r - b * vo;
    const int ox = rem % g.Wo;
    rem /= g.Wo;
    const int oy = rem % g.Ho;
    const int oz = rem / g.Ho;
    int kx = 0, ky = 0, kz = 0, pad = 0;
    if (g.taps == 27) {
        kx = tap % 3;
        ky = (tap / 3) % 3;
        kz = tap / 9;
        pad = 1;
    }
    int ix, iy, iz;
    if (g.mode == 0) {
        ix = ox * g.stride + kx - pad;
        iy = oy * g.stride + ky - pad;
        iz = oz * g.stride + kz - pad;
    } else {
        const int tx = ox + pad - kx, ty = oy + pad - ky, tz = oz + pad - kz;
        if ((tx | ty | tz) & 1) return -1;
        ix = tx >> 1;
        iy = ty >> 1;
        iz = tz >> 1;
    }
    if (ix < 0 || iy < 0 || iz < 0 || ix >= g.Wi || iy >= g.Hi || iz >= g.Di) return -1;
    return ((b * g.Di + iz) * g.Hi + iy) * g.Wi + ix;
}

__device__ __forceinline__ uint32_t ld32(const bf16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// C[rows][NT*8] = gather(in)[rows][taps*cin] x W^T with W row-major
// [NT*8][taps*cin] (BF16).  One warp owns 16 rows and every column; 4 warps a
// block.  Epilogue: + bias, ReLU, + addend (FP32 outputs), store FP32 or BF16.
template <int NT, bool OUT_BF16>
__global__ void __launch_bounds__(128) k_conv_gemm(Geo g, const bf16 *__restrict__ in, const bf16 *__restrict__ w,
                                                   const float *__restrict__ bias, const float *__restrict__ addend,
                                                   void *out, int relu, int rows)
{
    const int warp = blockIdx.x * 4 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
    if (warp * 16 >= rows) return;
    const int r0 = warp * 16 + gq, r1 = r0 + 8;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int K = g.taps * g.cin;
    for (int tap = 0; tap < g.taps; ++tap) {
        const int s0 = r0 < rows ? gather_src(g, r0, tap) : -1;
        const int s1 = r1 < rows ? gather_src(g, r1, tap) : -1;
        const bf16 *p0 = in + (size_t)(s0 < 0 ? 0 : s0) * g.cin + 2 * t4;
        const bf16 *p1 = in + (size_t)(s1 < 0 ? 0 : s1) * g.cin + 2 * t4;
        const bf16 *wt = w + (size_t)gq * K + tap * g.cin + 2 * t4;
        for (int c0 = 0; c0 < g.cin; c0 += 16) {
            const uint32_t a0 = s0 >= 0 ? ld32(p0 + c0) : 0u;
            const uint32_t a1 = s1 >= 0 ? ld32(p1 + c0) : 0u;
            const uint32_t a2 = s0 >= 0 ? ld32(p0 + c0 + 8) : 0u;
            const uint32_t a3 = s1 >= 0 ? ld32(p1 + c0 + 8) : 0u;
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                const bf16 *wr = wt + (size_t)(8 * j) * K + c0;
                mma_bf16(acc[j], a0, a1, a2, a3, ld32(wr), ld32(wr + 8));
            }
        }
    }
    constexpr int cout = NT * 8;
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const int col = 8 * j + 2 * t4;
        const float bb0 = bias ? bias[col] : 0.f, bb1 = bias ? bias[col + 1] : 0.f;
        float v[4] = {acc[j][0] + bb0, acc[j][1] + bb1, acc[j][2] + bb0, acc[j][3] + bb1};
        if (relu)
#pragma unroll
            for (int e = 0; e < 4; ++e) v[e] = fmaxf(v[e], 0.f);
        if (OUT_BF16) {
            bf16 *o = reinterpret_cast<bf16 *>(out);
            if (r0 < rows)
                *reinterpret_cast<__nv_bfloat162 *>(o + (size_t)r0 * cout + col) = __floats2bfloat162_rn(v[0], v[1]);
            if (r1 < rows)
                *reinterpret_cast<__nv_bfloat162 *>(o + (size_t)r1 * cout + col) = __floats2bfloat162_rn(v[2], v[3]);
        } else {
            float *o = reinterpret_cast<float *>(out);
            if (addend) {
                if (r0 < rows) {
                    const float2 a = *reinterpret_cast<const float2 *>(addend + (size_t)r0 * cout + col);
                    v[0] += a.x;
                    v[1] += a.y;
                }
                if (r1 < rows) {
                    const float2 a = *reinterpret_cast<const float2 *>(addend + (size_t)r1 * cout + col);
                    v[2] += a.x;
                    v[3] += a.y;
                }
            }
            if (r0 < rows) *reinterpret_cast<float2 *>(o + (size_t)r0 * cout + col) = make_float2(v[0], v[1]);
            if (r1 < rows) *reinterpret_cast<float2 *>(o + (size_t)r1 * cout + col) = make_float2(v[2], v[3]);
        }
    }
}

// ---- the same implicit GEMM on the 5th-generation tensor cores (tcgen05)
//
// A CTA computes 128 GEMM rows x all cout columns.  Per tap, the 128
// gathered activation rows (A, 128 x cin) and the tap's weights (B, cout x
// cin) are staged in shared memory in the canonical no-swizzle K-major
// layout: 8-row x 16-byte core matrices, core matrix (m8, k8) at
// (m8 * cin/8 + k8) * 128 bytes, so the descriptors' leading (K) byte offset is
// 128 and their stride (M/N) byte offset cin/8 * 128.  One thread issues
// cin/16 tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128, N = cout,
// K = 16) into an accumulator in tensor memory and commits them to the
// stage's mbarrier; two stage buffers let the next tap's gather overlap the
// MMAs.  The epilogue reads each warp's 32 accumulator rows with tcgen05.ld.
// Every wait is bounded; a wait that gives up sets g_conv_err, and the CTA
// still frees its tensor memory.
__device__ int g_conv_err;
// polls of the TMA direct kernel's waits for its copies and MMAs before it
// gives up (qmin_set_wait_limit); the waits that let copies and MMAs in
// flight land before a CTA that gave up exits always poll kWaitPolls times
constexpr int kWaitPolls = 1 << 22;
__device__ int g_conv_wait_limit = kWaitPolls;

namespace {
__device__ __forceinline__ unsigned s_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle, K-major (SM100 format: version 1 at bits 46-47)
__device__ __forceinline__ uint64_t umma_desc(unsigned saddr, unsigned lbo, unsigned sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major, N, M = 128
__host__ __device__ constexpr uint32_t umma_idesc(int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity, int polls = kWaitPolls)
{
    for (int it = 0; it < polls; ++it) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
}  // namespace

// tensor-memory columns for an accumulator of n FP32 columns (a power of two >= 32)
static int umma_cols(int n)
{
    int c = 32;
    while (c < n) c <<= 1;
    return c;
}
// dynamic shared memory of k_conv_umma: two stages of A and B, two mbarriers,
// the tensor-memory address; padded so that at most 512 / cols CTAs share an SM
// and a tcgen05.alloc never waits
static size_t umma_smem(int cin, int n)
{
    const size_t need = 2 * (size_t)(128 + n) * cin * 2 + 64;
    const int per_sm = 512 / umma_cols(n);
    const size_t floor_bytes = (size_t)(232448 / per_sm) - 1024 + 1;  // more than 1/(per_sm+1) of the SM's 227 KB
    return std::max(need, std::min<size_t>(floor_bytes, 232448 - 1024));
}

template <int N, bool OUT_BF16>
__global__ void __launch_bounds__(128) k_conv_umma(Geo g, const bf16 *__restrict__ in, const bf16 *__restrict__ w,
                                                   const float *__restrict__ bias, const float *__restrict__ addend,
                                                   void *out, int relu, int rows)
{
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "tcgen05 M=128 needs N a multiple of 16 in [16, 256]");
    constexpr int COLS = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int cin = g.cin, kc8 = cin >> 3, K = g.taps * cin;
    const size_t a_bytes = (size_t)128 * cin * 2, b_bytes = (size_t)N * cin * 2;
    unsigned char *bufA[2] = {smem_raw, smem_raw + a_bytes + b_bytes};
    unsigned char *bufB[2] = {smem_raw + a_bytes, smem_raw + 2 * a_bytes + b_bytes};
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + 2 * (a_bytes + b_bytes));
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = blockIdx.x * 128 + tid;
    // an earlier CTA's wait gave up: the launch's results are void, do no more work
    if (*(volatile int *)&g_conv_err) return;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_addr(tmem_slot)),
                     "r"(COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(&bar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(&bar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    bool ok = true;
    for (int tap = 0; tap < g.taps; ++tap) {
        const int b = tap & 1;
        if (tap >= 2) {
            // the MMAs of tap - 2 have read this buffer
            const bool w_ok = mbar_wait_bounded(s_addr(&bar[b]), (unsigned)((tap - 2) >> 1) & 1u);
            if (__syncthreads_or(!w_ok)) {
                ok = false;
                break;
            }
        }
        // A: this thread's row, cin channels of the tap's source voxel (zeros outside)
        {
            const int src = row < rows ? gather_src(g, row, tap) : -1;
            const uint4 *sp = reinterpret_cast<const uint4 *>(in + (size_t)(src < 0 ? 0 : src) * cin);
            unsigned char *dst = bufA[b] + (size_t)(tid >> 3) * kc8 * 128 + (tid & 7) * 16;
            for (int k8 = 0; k8 < kc8; ++k8) {
                const uint4 v = src >= 0 ? sp[k8] : make_uint4(0, 0, 0, 0);
                *reinterpret_cast<uint4 *>(dst + k8 * 128) = v;
            }
        }
        // B: the tap's weights, N x cin
        for (int e = tid; e < N * kc8; e += 128) {
            const int co = e / kc8, k8 = e - co * kc8;
            const uint4 v = *reinterpret_cast<const uint4 *>(w + (size_t)co * K + (size_t)tap * cin + k8 * 8);
            *reinterpret_cast<uint4 *>(bufB[b] + ((size_t)(co >> 3) * kc8 + k8) * 128 + (co & 7) * 16) = v;
        }
        // generic-proxy stores -> visible to the tensor cores' async proxy
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const unsigned sa = s_addr(bufA[b]), sb = s_addr(bufB[b]);
            const unsigned sbo = (unsigned)kc8 * 128u;
            for (int kk = 0; kk < (cin >> 4); ++kk) {
                const uint64_t da = umma_desc(sa + kk * 256, 128, sbo);
                const uint64_t db = umma_desc(sb + kk * 256, 128, sbo);
                const unsigned acc = (tap > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(umma_idesc(N)), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             s_addr(&bar[b]))
                         : "memory");
        }
    }
    if (ok) {
        // the last commit covers every MMA this CTA issued
        const int last = g.taps - 1;
        const bool w_ok = mbar_wait_bounded(s_addr(&bar[last & 1]), (unsigned)(last >> 1) & 1u);
        ok = !__syncthreads_or(!w_ok);
    }
    if (ok) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 8) {
            uint32_t r[8];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7])
                         : "r"(taddr + c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                v[e] = __uint_as_float(r[e]) + (bias ? bias[c0 + e] : 0.f);
                if (relu) v[e] = fmaxf(v[e], 0.f);
            }
            if (row < rows) {
                if (OUT_BF16) {
                    bf16 *o = reinterpret_cast<bf16 *>(out) + (size_t)row * N + c0;
                    __nv_bfloat162 h[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) h[e] = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
                    *reinterpret_cast<uint4 *>(o) = *reinterpret_cast<const uint4 *>(h);
                } else {
                    float *o = reinterpret_cast<float *>(out) + (size_t)row * N + c0;
                    if (addend) {
                        const float *a = addend + (size_t)row * N + c0;
#pragma unroll
                        for (int e = 0; e < 8; ++e) v[e] += a[e];
                    }
                    *reinterpret_cast<float4 *>(o) = make_float4(v[0], v[1], v[2], v[3]);
                    *reinterpret_cast<float4 *>(o + 4) = make_float4(v[4], v[5], v[6], v[7]);
                }
            }
        }
    } else if (tid == 0) {
        // a wait gave up: let the MMAs in flight finish (bounded) before the buffers go away
        for (int b = 0; b < 2; ++b) mbar_wait_bounded(s_addr(&bar[b]), 0u), mbar_wait_bounded(s_addr(&bar[b]), 1u);
        atomicExch(&g_conv_err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(COLS) : "memory");
}

// ---- direct 3x3x3 stride-1 convolution on tcgen05 (no per-tap gather)
//
// A CTA computes 8 (x) x 16 (y) output voxels = 128 GEMM rows, row r = (x0 +
// r % 8, y0 + r / 8), for each of ZT consecutive output planes.  8 consecutive
// x voxels of one 8-channel group of a staged input halo plane form a
// canonical 8-row x 16-byte core matrix, so for tap (dx, dy, dz) the A operand
// is the staged plane z - 1 + dz seen from (dx, dy): the start address moves
// by the tap, the stride (M) byte offset is one halo row (160 bytes, the next
// output y) and the leading (K) byte offset one 8-channel group (180 * 16
// bytes).  The 27 taps' weights stay resident in shared memory for the whole
// column, the input halo planes (18 x 10 voxels, zero outside the volume) pass
// through a ring of four slots ([cin/8][18][10][8 channels] each), and two
// tensor-memory accumulators alternate: the MMAs of plane p run while the
// epilogue of plane p - 1 reads the other accumulator and the halo plane z + 2
// is loaded into the slot that the MMAs of plane p - 1 have finished reading.
// Every wait is bounded and reports through g_conv_err; the CTA always frees
// its tensor memory.
static size_t direct_z_smem(int cin, int n)
{
    const size_t need = (size_t)27 * n * cin * 2 + (size_t)4 * 180 * cin * 2 + 64;
    const int per_sm = 512 / umma_cols(2 * n);
    const size_t floor_bytes = (size_t)(232448 / per_sm) - 1024 + 1;
    return std::max(need, std::min<size_t>(floor_bytes, 232448 - 1024));
}

template <int N>
__global__ void __launch_bounds__(128) k_conv3_direct_z(Geo g, const bf16 *__restrict__ in,
                                                        const bf16 *__restrict__ w, const float *__restrict__ bias,
                                                        bf16 *__restrict__ out, int relu, int zt)
{
    static_assert(N % 16 == 0 && N >= 16 && 2 * N <= 256, "two M=128 accumulators of N columns");
    constexpr int COLS = 2 * N <= 32 ? 32 : (2 * N <= 64 ? 64 : (2 * N <= 128 ? 128 : 256));
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int cin = g.cin, kc8 = cin >> 3, K = 27 * cin;
    const int W = g.Wo, H = g.Ho, D = g.Do;
    const size_t w_bytes = (size_t)27 * N * cin * 2, slot_bytes = (size_t)180 * cin * 2;
    unsigned char *wts = smem_raw;
    unsigned char *ring = smem_raw + w_bytes;
    uint64_t *bar = reinterpret_cast<uint64_t *>(ring + 4 * slot_bytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 2);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int tx = (W + 7) >> 3, ty = (H + 15) >> 4, tz = (D + zt - 1) / zt;
    int bidx = blockIdx.x;
    const int x0 = (bidx % tx) * 8;
    bidx /= tx;
    const int y0 = (bidx % ty) * 16;
    bidx /= ty;
    const int z0 = (bidx % tz) * zt, b = bidx / tz;
    const int nz = min(zt, D - z0);
    if (*(volatile int *)&g_conv_err) return;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_addr(tmem_slot)),
                     "r"(COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(&bar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(&bar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // all 27 taps' weights, [tap][co][cin] with each tap's [co][cin] in the canonical layout
    for (int e = tid; e < 27 * N * kc8; e += 128) {
        const int tap = e / (N * kc8), rem = e - tap * N * kc8, co = rem / kc8, k8 = rem - co * kc8;
        const uint4 v = *reinterpret_cast<const uint4 *>(w + (size_t)co * K + (size_t)tap * cin + k8 * 8);
        *reinterpret_cast<uint4 *>(wts + (size_t)tap * N * cin * 2 + ((size_t)(co >> 3) * kc8 + k8) * 128 +
                                   (co & 7) * 16) = v;
    }
    auto slot_of = [&](int iz) { return ((iz - z0 + 1) & 3); };  // iz >= z0 - 1
    // input plane iz (zero outside the volume) into its ring slot
    auto load_plane = [&](int iz) {
        unsigned char *dst = ring + (size_t)slot_of(iz) * slot_bytes;
        const bool zin = iz >= 0 && iz < D;
        for (int e = tid; e < 180 * kc8; e += 128) {
            const int vox = e / kc8, k8 = e - vox * kc8;
            const int hx = vox % 10, hy = vox / 10;
            const int ix = x0 - 1 + hx, iy = y0 - 1 + hy;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (zin && ix >= 0 && iy >= 0 && ix < W && iy < H)
                v = *reinterpret_cast<const uint4 *>(in + ((((size_t)b * D + iz) * H + iy) * W + ix) * cin + k8 * 8);
            *reinterpret_cast<uint4 *>(dst + ((size_t)k8 * 180 + hy * 10 + hx) * 16) = v;
        }
    };
    auto issue = [&](int z, int acc_idx) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const unsigned sw = s_addr(wts), sbo_b = (unsigned)kc8 * 128u;
        const uint32_t dst = *tmem_slot + (uint32_t)(acc_idx * N);
        for (int tap = 0; tap < 27; ++tap) {
            const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
            const unsigned sa = s_addr(ring + (size_t)slot_of(z - 1 + dz) * slot_bytes);
            for (int kk = 0; kk < (cin >> 4); ++kk) {
                const unsigned a0 = sa + ((unsigned)(2 * kk * 180 + dy * 10 + dx) * 16u);
                const unsigned b0 = sw + (unsigned)tap * (unsigned)(N * cin * 2) + (unsigned)kk * 256u;
                const uint64_t da = umma_desc(a0, 2880, 160), db = umma_desc(b0, 128, sbo_b);
                const unsigned acc = (tap > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dst),
                    "l"(da), "l"(db), "r"(umma_idesc(N)), "r"(acc)
                    : "memory");
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         s_addr(&bar[acc_idx]))
                     : "memory");
    };
    auto epilogue = [&](int z, int acc_idx, uint32_t tmem) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(acc_idx * N);
        const int ox = x0 + (tid & 7), oy = y0 + (tid >> 3);
        const bool inside = ox < W && oy < H;
        bf16 *o = out + ((((size_t)b * D + z) * H + oy) * W + ox) * N;
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 8) {
            uint32_t r[8];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7])
                         : "r"(taddr + c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (inside) {
                __nv_bfloat162 hh[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    float v0 = __uint_as_float(r[2 * e]) + bias[c0 + 2 * e];
                    float v1 = __uint_as_float(r[2 * e + 1]) + bias[c0 + 2 * e + 1];
                    if (relu) {
                        v0 = fmaxf(v0, 0.f);
                        v1 = fmaxf(v1, 0.f);
                    }
                    hh[e] = __floats2bfloat162_rn(v0, v1);
                }
                *reinterpret_cast<uint4 *>(o + c0) = *reinterpret_cast<const uint4 *>(hh);
            }
        }
    };
    load_plane(z0 - 1);
    load_plane(z0);
    load_plane(z0 + 1);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    bool ok = true;
    for (int p = 0; p < nz; ++p) {
        const int z = z0 + p;
        if (tid == 0) issue(z, p & 1);
        if (p >= 1) {
            // the MMAs of plane p - 1: done with their accumulator and with slot z - 2
            const bool w_ok = mbar_wait_bounded(s_addr(&bar[(p - 1) & 1]), (unsigned)((p - 1) >> 1) & 1u);
            if (__syncthreads_or(!w_ok)) {
                ok = false;
                break;
            }
            epilogue(z - 1, (p - 1) & 1, tmem);
        }
        if (p + 1 < nz) load_plane(z + 2);
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
    }
    if (ok) {
        const int last = nz - 1;
        const bool w_ok = mbar_wait_bounded(s_addr(&bar[last & 1]), (unsigned)(last >> 1) & 1u);
        ok = !__syncthreads_or(!w_ok);
        if (ok) epilogue(z0 + last, last & 1, tmem);
    }
    if (!ok && tid == 0) {
        // a wait gave up: let the MMAs in flight finish (bounded) before the buffers go away
        for (int k = 0; k < 2; ++k) mbar_wait_bounded(s_addr(&bar[k]), 0u), mbar_wait_bounded(s_addr(&bar[k]), 1u);
        atomicExch(&g_conv_err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(COLS) : "memory");
}

// The same column walk with each halo plane staged by the tensor-memory-access
// unit: one cp.async.bulk.tensor.5d box of 8 channels x 10 x 18 voxels x 1
// plane per 8-channel group (the box's channel coordinate is a multiple of 8
// BF16 elements, 16 bytes; the spatial coordinates start one voxel before the
// tile and may be negative or past the volume, where the box reads zeros,
// which is the convolution's zero padding in x, y and z).  A group's box lands
// as [18][10][8 channels], the canonical K-major core-matrix layout the
// descriptors read, in a slab padded to 2944 bytes so that every box starts on
// a 128-byte boundary; the leading byte offset of the A descriptor is that
// slab pitch.  One thread issues the boxes against one mbarrier per ring slot
// (the expected bytes count the whole box, zero fill included), waits for
// plane z + 1 before it issues the MMAs of plane z, and reloads a slot only
// after the MMAs that read it have committed.  All waits are bounded; a wait
// that gives up leaves the copies and MMAs in flight to land (bounded again)
// before the CTA frees its tensor memory and reports through g_conv_err.
constexpr int kTmaSlab = 2944;  // 2880 bytes of box, padded to a multiple of 128
static size_t direct_z_tma_smem(int cin, int n)
{
    const size_t need = (size_t)27 * n * cin * 2 + (size_t)4 * (cin / 8) * kTmaSlab + 128 + 128;
    const int per_sm = 512 / umma_cols(2 * n);
    const size_t floor_bytes = (size_t)(232448 / per_sm) - 1024 + 1;
    return std::max(need, std::min<size_t>(floor_bytes, 232448 - 1024));
}

namespace {
__device__ __forceinline__ void tma_box_5d(unsigned dst, const CUtensorMap *map, int c, int x, int y, int z, int b,
                                           unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];\n" ::"r"(dst),
        "l"(map), "r"(c), "r"(x), "r"(y), "r"(z), "r"(b), "r"(bar)
        : "memory");
}
}  // namespace

template <int N, int CIN>
__global__ void __launch_bounds__(128) k_conv3_direct_z_tma(Geo g, const __grid_constant__ CUtensorMap tmap,
                                                            const bf16 *__restrict__ w,
                                                            const float *__restrict__ bias, bf16 *__restrict__ out,
                                                            int relu, int zt)
{
    static_assert(N % 16 == 0 && N >= 16 && 2 * N <= 256, "two M=128 accumulators of N columns");
    static_assert(CIN % 16 == 0 && CIN >= 16, "input channels a multiple of 16");
    constexpr int COLS = 2 * N <= 32 ? 32 : (2 * N <= 64 ? 64 : (2 * N <= 128 ? 128 : 256));
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int cin = CIN, kc8 = CIN / 8, K = 27 * CIN;
    const int W = g.Wo, H = g.Ho, D = g.Do;
    constexpr size_t w_bytes = (size_t)27 * N * cin * 2;  // a multiple of 128 (27 * 2 * 16 * 16 divides it)
    constexpr unsigned slot_bytes = (unsigned)kc8 * kTmaSlab;
    // the boxes start on 128-byte boundaries: the dynamic area rounded up (128 bytes spare are allocated)
    unsigned char *base = smem_raw + ((128u - (s_addr(smem_raw) & 127u)) & 127u);
    unsigned char *wts = base;
    unsigned char *ring = base + w_bytes;
    uint64_t *bar = reinterpret_cast<uint64_t *>(ring + 4 * (size_t)slot_bytes);  // [0..1] MMAs, [2..5] ring slots
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 6);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int tx = (W + 7) >> 3, ty = (H + 15) >> 4, tz = (D + zt - 1) / zt;
    int bidx = blockIdx.x;
    const int x0 = (bidx % tx) * 8;
    bidx /= tx;
    const int y0 = (bidx % ty) * 16;
    bidx /= ty;
    const int z0 = (bidx % tz) * zt, b = bidx / tz;
    const int nz = min(zt, D - z0);
    if (*(volatile int *)&g_conv_err) return;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s_addr(tmem_slot)),
                     "r"(COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < 6; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(s_addr(&bar[k])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    auto slot_of = [&](int iz) { return (iz - z0 + 1) & 3; };            // iz >= z0 - 1
    auto use_of = [&](int iz) { return (unsigned)((iz - z0 + 1) >> 2); };  // how many loads the slot had before
    // plane iz's boxes into its ring slot (one thread)
    auto load_plane = [&](int iz) {
        const int sl = slot_of(iz);
        const unsigned bs = s_addr(&bar[2 + sl]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bs), "r"(kc8 * 2880u)
                     : "memory");
        const unsigned dst = s_addr(ring) + (unsigned)sl * slot_bytes;
        for (int k8 = 0; k8 < kc8; ++k8) tma_box_5d(dst + (unsigned)k8 * kTmaSlab, &tmap, k8 * 8, x0 - 1, y0 - 1, iz, b, bs);
    };
    const int polls = *(volatile int *)&g_conv_wait_limit;
    auto wait_plane = [&](int iz, int lim) {
        return mbar_wait_bounded(s_addr(&bar[2 + slot_of(iz)]), use_of(iz) & 1u, lim);
    };
    int issued_hi = z0 - 2;  // the last plane whose boxes were issued
    __syncthreads();         // the barriers are initialised
    if (tid == 0) {
        for (int iz = z0 - 1; iz <= z0 + 1; ++iz) load_plane(iz);
        issued_hi = z0 + 1;
    }
    // all 27 taps' weights, [tap][co][cin] with each tap's [co][cin] in the canonical layout
    for (int e = tid; e < 27 * N * kc8; e += 128) {
        const int tap = e / (N * kc8), rem = e - tap * N * kc8, co = rem / kc8, k8 = rem - co * kc8;
        const uint4 v = *reinterpret_cast<const uint4 *>(w + (size_t)co * K + (size_t)tap * cin + k8 * 8);
        *reinterpret_cast<uint4 *>(wts + (size_t)tap * N * cin * 2 + ((size_t)(co >> 3) * kc8 + k8) * 128 +
                                   (co & 7) * 16) = v;
    }
    // descriptors of the ring's and the weights' first core matrices; a
    // descriptor's address field is the byte address / 16 in its low 14 bits,
    // so an offset (a multiple of 16 bytes, the sum below 256 KB) is added to
    // the descriptor itself: the issuing thread does one add per operand per MMA
    const uint64_t da0 = umma_desc(s_addr(ring), kTmaSlab, 160);
    const uint64_t db0 = umma_desc(s_addr(wts), 128, (unsigned)kc8 * 128u);
    auto issue = [&](int z, int acc_idx) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t dst = *tmem_slot + (uint32_t)(acc_idx * N);
        const uint64_t das[3] = {da0 + ((uint64_t)slot_of(z - 1) * slot_bytes >> 4),
                                 da0 + ((uint64_t)slot_of(z) * slot_bytes >> 4),
                                 da0 + ((uint64_t)slot_of(z + 1) * slot_bytes >> 4)};
#pragma unroll
        for (int tap = 0; tap < 27; ++tap) {
            const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
#pragma unroll
            for (int kk = 0; kk < CIN / 16; ++kk) {
                const uint64_t da = das[dz] + (uint64_t)((2 * kk * kTmaSlab + (dy * 10 + dx) * 16) >> 4);
                const uint64_t db = db0 + (uint64_t)((tap * N * CIN * 2 + kk * 256) >> 4);
                const unsigned acc = (tap > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dst),
                    "l"(da), "l"(db), "r"(umma_idesc(N)), "r"(acc)
                    : "memory");
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         s_addr(&bar[acc_idx]))
                     : "memory");
    };
    auto epilogue = [&](int z, int acc_idx, uint32_t tmem) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(acc_idx * N);
        const int ox = x0 + (tid & 7), oy = y0 + (tid >> 3);
        const bool inside = ox < W && oy < H;
        bf16 *o = out + ((((size_t)b * D + z) * H + oy) * W + ox) * N;
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 8) {
            uint32_t r[8];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7])
                         : "r"(taddr + c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (inside) {
                __nv_bfloat162 hh[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    float v0 = __uint_as_float(r[2 * e]) + bias[c0 + 2 * e];
                    float v1 = __uint_as_float(r[2 * e + 1]) + bias[c0 + 2 * e + 1];
                    if (relu) {
                        v0 = fmaxf(v0, 0.f);
                        v1 = fmaxf(v1, 0.f);
                    }
                    hh[e] = __floats2bfloat162_rn(v0, v1);
                }
                *reinterpret_cast<uint4 *>(o + c0) = *reinterpret_cast<const uint4 *>(hh);
            }
        }
    };
    // the weights (generic-proxy stores) become visible to the MMAs (async proxy)
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    bool ok = true;
    int committed = 0;  // planes whose MMAs were committed
    for (int p = 0; p < nz; ++p) {
        const int z = z0 + p;
        bool good = true;
        if (tid == 0) {
            // planes z - 1 and z were waited for by earlier steps (all three at the first)
            if (p == 0) good = wait_plane(z - 1, polls) && wait_plane(z, polls);
            good = good && wait_plane(z + 1, polls);
            if (good) issue(z, p & 1);
        }
        if (__syncthreads_or(!good)) {
            ok = false;
            break;
        }
        committed = p + 1;
        if (p >= 1) {
            // the MMAs of plane p - 1: done with their accumulator and with slot z - 2
            const bool w_ok = mbar_wait_bounded(s_addr(&bar[(p - 1) & 1]), (unsigned)((p - 1) >> 1) & 1u, polls);
            if (__syncthreads_or(!w_ok)) {
                ok = false;
                break;
            }
            epilogue(z - 1, (p - 1) & 1, tmem);
        }
        if (tid == 0 && p + 1 < nz) {
            load_plane(z + 2);
            issued_hi = z + 2;
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
    }
    if (ok) {
        const int last = nz - 1;
        const bool w_ok = mbar_wait_bounded(s_addr(&bar[last & 1]), (unsigned)(last >> 1) & 1u, polls);
        ok = !__syncthreads_or(!w_ok);
        if (ok) epilogue(z0 + last, last & 1, tmem);
    }
    if (!ok && tid == 0) {
        // a wait gave up: let the boxes and the MMAs in flight land (bounded,
        // at the full poll count) before the buffers go away
        for (int iz = max(z0 - 1, issued_hi - 3); iz <= issued_hi; ++iz) wait_plane(iz, kWaitPolls);
        for (int q = max(0, committed - 2); q < committed; ++q)
            mbar_wait_bounded(s_addr(&bar[q & 1]), (unsigned)(q >> 1) & 1u);
        atomicExch(&g_conv_err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(COLS) : "memory");
}

// dW[co][tap][ci] += sum_v dout[v][co] * in[src(v,tap)][ci] over rows
// [blockIdx.x * chunk, +chunk): block tile 64 co x 64 ci for one tap, the
// row dimension staged through shared memory 16 rows at a time; each block
// adds its partial tile into dW with FP32 atomics.
__global__ void __launch_bounds__(128) k_conv_wgrad(Geo g, const bf16 *__restrict__ dout, const bf16 *__restrict__ in,
                                                    float *__restrict__ dw, int rows, int chunk)
{
    __shared__ __align__(16) bf16 sA[16][72];  // dout slab [row][co]
    __shared__ __align__(16) bf16 sB[16][72];  // gathered input slab [row][ci]
    const int tap = blockIdx.y;
    const int ntc = (g.cout + 63) / 64;
    const int co0 = (blockIdx.z % ntc) * 64, ci0 = (blockIdx.z / ntc) * 64;
    const int vbeg = blockIdx.x * chunk, vend = min(rows, vbeg + chunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t4 = lane & 3;
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int rr = threadIdx.x >> 3, cc = (threadIdx.x & 7) * 8;
    const bool coin = co0 + cc < g.cout, ciin = ci0 + cc < g.cin;  // channel counts are multiples of 8
    for (int v0 = vbeg; v0 < vend; v0 += 16) {
        const int v = v0 + rr;
        const int src = v < vend ? gather_src(g, v, tap) : -1;
        uint4 a = make_uint4(0u, 0u, 0u, 0u), b = make_uint4(0u, 0u, 0u, 0u);
        if (v < vend && coin) a = *reinterpret_cast<const uint4 *>(dout + (size_t)v * g.cout + co0 + cc);
        if (src >= 0 && ciin) b = *reinterpret_cast<const uint4 *>(in + (size_t)src * g.cin + ci0 + cc);
        *reinterpret_cast<uint4 *>(&sA[rr][cc]) = a;
        *reinterpret_cast<uint4 *>(&sB[rr][cc]) = b;
        __syncthreads();
        auto pk = [](bf16 lo, bf16 hi) {
            return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
        };
        const int m = 16 * warp;
        const uint32_t a0 = pk(sA[2 * t4][m + gq], sA[2 * t4 + 1][m + gq]);
        const uint32_t a1 = pk(sA[2 * t4][m + gq + 8], sA[2 * t4 + 1][m + gq + 8]);
        const uint32_t a2 = pk(sA[2 * t4 + 8][m + gq], sA[2 * t4 + 9][m + gq]);
        const uint32_t a3 = pk(sA[2 * t4 + 8][m + gq + 8], sA[2 * t4 + 9][m + gq + 8]);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = 8 * j + gq;
            const uint32_t b0 = pk(sB[2 * t4][n], sB[2 * t4 + 1][n]);
            const uint32_t b1 = pk(sB[2 * t4 + 8][n], sB[2 * t4 + 9][n]);
            mma_bf16(acc[j], a0, a1, a2, a3, b0, b1);
        }
        __syncthreads();
    }
    const int K = g.taps * g.cin;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int ci = ci0 + 8 * j + 2 * t4;
        const int coA = co0 + 16 * warp + gq, coB = coA + 8;
        if (ci < g.cin) {
            if (coA < g.cout) {
                atomicAdd(dw + (size_t)coA * K + tap * g.cin + ci, acc[j][0]);
                atomicAdd(dw + (size_t)coA * K + tap * g.cin + ci + 1, acc[j][1]);
            }
            if (coB < g.cout) {
                atomicAdd(dw + (size_t)coB * K + tap * g.cin + ci, acc[j][2]);
                atomicAdd(dw + (size_t)coB * K + tap * g.cin + ci + 1, acc[j][3]);
            }
        }
    }
}

// ------------------------------------------------------------ elementwise
#define GRID_STRIDE(i, n) \
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

__global__ void k_f32_to_bf16(const float *x, bf16 *y, long long n)
{
    GRID_STRIDE(i, n) y[i] = __float2bfloat16(x[i]);
}

// gradient through the ReLU (mask from the stored BF16 activation), as BF16
__global__ void k_relu_grad_bf16(const float *g, const bf16 *act, bf16 *y, long long n)
{
    GRID_STRIDE(i, n) y[i] = __float2bfloat16(__bfloat162float(act[i]) > 0.f ? g[i] : 0.f);
}

// data-gradient weights: Wd[ci][tap'][co] = W[co][tap][ci], tap' = 26 - tap
// for a stride-1 3^3 convolution (flip), tap' = tap otherwise
__global__ void k_dgrad_weights(const bf16 *w, bf16 *wd, int cout, int cin, int taps, int flip)
{
    const long long n = (long long)cout * cin * taps;
    GRID_STRIDE(i, n)
    {
        const int ci = (int)(i % cin), tap = (int)((i / cin) % taps), co = (int)(i / ((long long)cin * taps));
        const int tp = flip ? taps - 1 - tap : tap;
        wd[((size_t)ci * taps + tp) * cout + co] = w[i];
    }
}

struct Dims {
    int B, x, y, z;  // coarse grid
};

// nearest x2 upsampling of h (coarse, FP32) plus a BF16 skip on the fine grid, into BF16
__global__ void k_up2_add(const float *h, const bf16 *skip, bf16 *out, Dims d, int c)
{
    // one thread per 8 channels of a fine voxel (c is a multiple of 8): 16-byte
    // loads and stores, the voxel's coordinates decoded once per 8 channels
    const int X = 2 * d.x, Y = 2 * d.y, Z = 2 * d.z, cg = c >> 3;
    const long long n = (long long)d.B * X * Y * Z * cg;
    GRID_STRIDE(t, n)
    {
        const int g = (int)(t % cg);
        long long v = t / cg;
        const long long vf = v;
        const int x = (int)(v % X);
        v /= X;
        const int y = (int)(v % Y);
        v /= Y;
        const int z = (int)(v % Z);
        const int b = (int)(v / Z);
        const long long src = (((long long)b * d.z + z / 2) * d.y + y / 2) * d.x + x / 2;
        const float4 *hp = reinterpret_cast<const float4 *>(h + src * c + 8 * g);
        const float4 h0 = hp[0], h1 = hp[1];
        const uint4 sk = *reinterpret_cast<const uint4 *>(skip + vf * c + 8 * g);
        const __nv_bfloat162 *s2 = reinterpret_cast<const __nv_bfloat162 *>(&sk);
        const float hv[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
        __nv_bfloat162 o[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float2 f = __bfloat1622float2(s2[e]);
            o[e] = __floats2bfloat162_rn(hv[2 * e] + f.x, hv[2 * e + 1] + f.y);
        }
        *reinterpret_cast<uint4 *>(out + vf * c + 8 * g) = *reinterpret_cast<const uint4 *>(o);
    }
}

// gradient of nearest x2 upsampling: the sum over the 8 children
__global__ void k_up2_grad(const float *g2, float *g, Dims d, int c)
{
    const int X = 2 * d.x, Y = 2 * d.y, Z = 2 * d.z;
    const long long n = (long long)d.B * d.x * d.y * d.z * c;
    GRID_STRIDE(i, n)
    {
        const int ch = (int)(i % c);
        long long v = i / c;
        const int x = (int)(v % d.x);
        v /= d.x;
        const int y = (int)(v % d.y);
        v /= d.y;
        const int z = (int)(v % d.z);
        const int b = (int)(v / d.z);
        float s = 0.f;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx)
                    s += g2[((((long long)b * Z + 2 * z + dz) * Y + 2 * y + dy) * X + 2 * x + dx) * c + ch];
        g[i] = s;
    }
}

// bias gradient db[c] += sum_v g[v][c] (masked by the ReLU when act != NULL);
// one block per (row chunk, 32-channel group), a thread per channel and row lane
__global__ void k_bias_grad(const float *g, const bf16 *act, float *db, long long rows, int c)
{
    const int ch = blockIdx.y * 32 + (threadIdx.x & 31);
    const int lanes = blockDim.x >> 5;
    float s = 0.f;
    if (ch < c) {
        for (long long v = blockIdx.x * (long long)lanes + (threadIdx.x >> 5); v < rows; v += (long long)gridDim.x * lanes) {
            const float x = g[v * c + ch];
            s += (act == nullptr || __bfloat162float(act[v * c + ch]) > 0.f) ? x : 0.f;
        }
        atomicAdd(db + ch, s);
    }
}

__global__ void k_count_mask(const uint8_t *mask, long long n, unsigned long long *count)
{
    unsigned long long s = 0;
    GRID_STRIDE(i, n) s += mask[i] ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(count, s);
}

// masked mean-squared error over the 5 Q channels of y [rows][16]:
// loss = sum_{masked v, k<5} (y - t)^2 / count; dy = 2 (y - t) / count (0 elsewhere)
__global__ void k_mse(const float *y, const float *t, const uint8_t *mask, const unsigned long long *count, float *dy,
                      double *loss, long long rows)
{
    const double inv = 1.0 / (double)max(*count, 1ull);
    double s = 0.0;
    GRID_STRIDE(v, rows)
    {
        const bool m = mask[v] != 0;
#pragma unroll
        for (int k = 0; k < kOut; ++k) {
            float d = 0.f;
            if (k < 5 && m) d = y[v * kOut + k] - t[v * 5 + k];
            dy[v * kOut + k] = (float)(2.0 * d * inv);
            s += (double)d * d;
        }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv);
}

// Adam on the FP32 master parameters, refreshing their BF16 copies
__global__ void k_adam_params(float *p, const float *g, float *m, float *v, bf16 *pb, long long n, float lr, float b1,
                              float b2, float eps, float c1, float c2)
{
    GRID_STRIDE(i, n)
    {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        p[i] = pi;
        pb[i] = __float2bfloat16(pi);
    }
}

struct ObjTab {
    int n;
    int kind[kMaxObj];
    float W[kMaxObj];
};

// input features of one sample: channels 0..4 Q (the initial field, which on
// object sites is the imposed anchoring Q), 5 object site, 6 boundary site
// (type -1), 7 W/10 of the site's object, 8 homeotropic object, 9 degenerate
// planar object, 10..15 zero; mask = 1 on the sites the minimiser moves (type <= 0)
template <class T>
__global__ void k_features(const T *Q, long long P, const int8_t *types, int N, ObjTab objs, bf16 *x, uint8_t *mask)
{
    GRID_STRIDE(i, (long long)N)
    {
        const int t = types[i];
        float f[kIn];
#pragma unroll
        for (int k = 0; k < kIn; ++k) f[k] = 0.f;
#pragma unroll
        for (int k = 0; k < 5; ++k) f[k] = (float)Q[k * P + i];
        if (t > 0) {
            f[5] = 1.f;
            if (t - 1 < objs.n) {
                f[7] = 0.1f * objs.W[t - 1];
                f[8] = objs.kind[t - 1] == QMIN_HOMEOTROPIC ? 1.f : 0.f;
                f[9] = objs.kind[t - 1] == QMIN_DEGENERATE_PLANAR ? 1.f : 0.f;
            }
        } else if (t == -1) {
            f[6] = 1.f;
        }
        uint4 pk[2];
        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(pk);
#pragma unroll
        for (int k = 0; k < kIn / 2; ++k) h[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
        uint4 *dst = reinterpret_cast<uint4 *>(x + (size_t)i * kIn);
        dst[0] = pk[0];
        dst[1] = pk[1];
        if (mask) mask[i] = t <= 0 ? 1 : 0;
    }
}

// predicted Q (channels 0..4 of y) into the SoA planes on the sites the
// minimiser moves; object sites keep their imposed Q
template <class T>
__global__ void k_write_state(const float *y, T *Q, long long P, const int8_t *types, int N)
{
    GRID_STRIDE(i, (long long)N)
    {
        if (types[i] > 0) continue;
#pragma unroll
        for (int k = 0; k < 5; ++k) Q[k * P + i] = (T)y[(size_t)i * kOut + k];
    }
}

static int grid1(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 16)); }

template <int N, bool OB>
static void conv_umma(const Geo &g, const bf16 *in, const bf16 *w, const float *bias, const float *addend, void *out,
                      int relu, int rows, cudaStream_t s)
{
    static int attr_bytes = 0;
    const size_t sm = umma_smem(g.cin, N);
    if ((int)sm > attr_bytes) {
        // a failure here surfaces as the launch's error
        if (cudaFuncSetAttribute(k_conv_umma<N, OB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) ==
            cudaSuccess)
            attr_bytes = (int)sm;
    }
    k_conv_umma<N, OB><<<(rows + 127) / 128, 128, sm, s>>>(g, in, w, bias, addend, out, relu, rows);
}

template <int N>
static void conv3_direct_z(const Geo &g, const bf16 *in, const bf16 *w, const float *bias, bf16 *out, int relu,
                           cudaStream_t s)
{
    static int attr_bytes = 0;
    const size_t sm = direct_z_smem(g.cin, N);
    if ((int)sm > attr_bytes) {
        // a failure here surfaces as the launch's error
        if (cudaFuncSetAttribute(k_conv3_direct_z<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) ==
            cudaSuccess)
            attr_bytes = (int)sm;
    }
    const int zt = std::min(g.Do, 16);
    const long long tiles = (long long)((g.Wo + 7) / 8) * ((g.Ho + 15) / 16) * ((g.Do + zt - 1) / zt) * g.nb;
    k_conv3_direct_z<N><<<(unsigned)tiles, 128, sm, s>>>(g, in, w, bias, out, relu, zt);
}

// the driver's tensor-map encoder (fetched at run time: no link-time dependency), or null
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

// the TMA-staged direct kernel; false (nothing launched) where its tensor map
// cannot describe the input: no encoder, an input not 16-byte aligned, or a
// grid smaller than one halo box (10 x 18)
template <int N, int CIN>
static bool conv3_direct_z_tma(const Geo &g, const bf16 *in, const bf16 *w, const float *bias, bf16 *out, int relu,
                               cudaStream_t s)
{
    auto enc = tmap_encoder();
    if (!enc || (reinterpret_cast<uintptr_t>(in) & 15) || g.Wi < 10 || g.Hi < 18 || g.cin != CIN) return false;
    CUtensorMap map;
    const cuuint64_t es = 2;  // BF16
    const cuuint64_t dims[5] = {(cuuint64_t)g.cin, (cuuint64_t)g.Wi, (cuuint64_t)g.Hi, (cuuint64_t)g.Di,
                                (cuuint64_t)g.nb};
    const cuuint64_t strides[4] = {(cuuint64_t)g.cin * es, (cuuint64_t)g.Wi * g.cin * es,
                                   (cuuint64_t)g.Hi * g.Wi * g.cin * es, (cuuint64_t)g.Di * g.Hi * g.Wi * g.cin * es};
    const cuuint32_t box[5] = {8, 10, 18, 1, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(in), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    static int attr_bytes = 0;
    const size_t sm = direct_z_tma_smem(CIN, N);
    if (sm > 232448 - 1024) return false;
    if ((int)sm > attr_bytes) {
        // a failure here surfaces as the launch's error
        if (cudaFuncSetAttribute(k_conv3_direct_z_tma<N, CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm) == cudaSuccess)
            attr_bytes = (int)sm;
    }
    const int zt = std::min(g.Do, 16);
    const long long tiles = (long long)((g.Wo + 7) / 8) * ((g.Ho + 15) / 16) * ((g.Do + zt - 1) / zt) * g.nb;
    k_conv3_direct_z_tma<N, CIN><<<(unsigned)tiles, 128, sm, s>>>(g, map, w, bias, out, relu, zt);
    return true;
}

// path 1 or 2: the 5th-generation tensor-core kernels above (the direct kernel
// for 3x3x3 stride-1 forward convolutions with BF16 output, its halo planes
// staged by TMA on path 1 where the tensor map applies, by the threads on path
// 2; the gathering kernel otherwise); path 0: mma.sync
template <bool OB>
static void conv_gemm(const Geo &g, const bf16 *in, const bf16 *w, const float *bias, const float *addend, void *out,
                      int relu, int rows, cudaStream_t s, int path)
{
    const bool tcgen05 = path != 0;
    // the direct kernel wins where a dz plane's weights are small (measured at
    // 128^3: 16->32 0.29 ms vs 0.49 gathering, 32->32 0.77 vs 0.95; at 48->48
    // and 64->64 the 135-216 KB of staging leave one CTA per SM and it loses)
    if (tcgen05 && OB && g.mode == 0 && g.taps == 27 && g.stride == 1 && !addend && bias &&
        direct_z_smem(g.cin, g.cout) <= 232448 - 1024) {
        if (g.cout == 32) {
            // the network's direct layers: 16 -> 32 and 32 -> 32 (TMA kernel per input width)
            if (path == 1 && g.cin == 16 &&
                conv3_direct_z_tma<32, 16>(g, in, w, bias, reinterpret_cast<bf16 *>(out), relu, s))
                return;
            if (path == 1 && g.cin == 32 &&
                conv3_direct_z_tma<32, 32>(g, in, w, bias, reinterpret_cast<bf16 *>(out), relu, s))
                return;
            conv3_direct_z<32>(g, in, w, bias, reinterpret_cast<bf16 *>(out), relu, s);
            return;
        }
        if (g.cout == 48) {
            if (path == 1 && g.cin == 48 &&
                conv3_direct_z_tma<48, 48>(g, in, w, bias, reinterpret_cast<bf16 *>(out), relu, s))
                return;
            conv3_direct_z<48>(g, in, w, bias, reinterpret_cast<bf16 *>(out), relu, s);
            return;
        }
    }
    if (tcgen05) {
        switch (g.cout) {
        case 16: conv_umma<16, OB>(g, in, w, bias, addend, out, relu, rows, s); return;
        case 32: conv_umma<32, OB>(g, in, w, bias, addend, out, relu, rows, s); return;
        case 48: conv_umma<48, OB>(g, in, w, bias, addend, out, relu, rows, s); return;
        case 64: conv_umma<64, OB>(g, in, w, bias, addend, out, relu, rows, s); return;
        case 128: conv_umma<128, OB>(g, in, w, bias, addend, out, relu, rows, s); return;
        default: break;
        }
    }
    const int blocks = (rows + 63) / 64;
    switch (g.cout / 8) {
    case 2: k_conv_gemm<2, OB><<<blocks, 128, 0, s>>>(g, in, w, bias, addend, out, relu, rows); break;
    case 4: k_conv_gemm<4, OB><<<blocks, 128, 0, s>>>(g, in, w, bias, addend, out, relu, rows); break;
    case 6: k_conv_gemm<6, OB><<<blocks, 128, 0, s>>>(g, in, w, bias, addend, out, relu, rows); break;
    case 8: k_conv_gemm<8, OB><<<blocks, 128, 0, s>>>(g, in, w, bias, addend, out, relu, rows); break;
    case 16: k_conv_gemm<16, OB><<<blocks, 128, 0, s>>>(g, in, w, bias, addend, out, relu, rows); break;
    default: break;
    }
}

struct Layer {
    int cin, cout, taps, stride, level;  // level of the input grid
    bool relu;
    size_t woff, boff;  // offsets into the flat parameter vector
};

}  // namespace nn
}  // namespace qmin

using namespace qmin::nn;

struct qmin_warmnet_ctx {
    int B = 1, Lx = 0, Ly = 0, Lz = 0;
    bool train = false;
    Layer layers[kLayers];
    size_t nparams = 0;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 master, gradients, Adam moments
    bf16 *pb = nullptr;                                           // BF16 weights
    bf16 *wd = nullptr;                                           // data-gradient weights (scratch)
    bf16 *x = nullptr;                                            // input features [B][sites][16]
    uint8_t *mask = nullptr;                                      // [B][sites]
    float *y = nullptr;                                           // output [B][sites][16]
    bf16 *act[kLayers] = {};                                      // BF16 layer outputs (0..9)
    float *pre[kLayers] = {};                                     // FP32 outputs of 4, 6, 8
    float *sk[3] = {};                                            // skip gradients of levels 0..2
    float *gA = nullptr, *gB = nullptr;
    bf16 *gbf = nullptr;
    double *loss = nullptr;
    unsigned long long *count = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    long long adam_t = 0;
    long long launches = 0;
    int path = 1;  // convolutions: 1 tcgen05 (TMA-staged direct kernel), 2 tcgen05 (thread-staged), 0 mma.sync
};

namespace {

int nfail(int code, const std::string &m)
{
    qmin::g_last_error = m;
    return code;
}

long long sites(const qmin_warmnet_ctx *n, int level)
{
    return (long long)(n->Lx >> level) * (n->Ly >> level) * (n->Lz >> level);
}
long long rows_at(const qmin_warmnet_ctx *n, int level) { return n->B * sites(n, level); }
Dims dims_at(const qmin_warmnet_ctx *n, int level) { return Dims{n->B, n->Lx >> level, n->Ly >> level, n->Lz >> level}; }

void build_layers(qmin_warmnet_ctx *n)
{
    struct Spec {
        int cin, cout, taps, stride, level;
        bool relu;
    };
    const Spec s[kLayers] = {{kIn, 32, 27, 1, 0, true}, {32, 48, 27, 2, 0, true},  {48, 64, 27, 2, 1, true},
                             {64, 128, 27, 2, 2, true}, {128, 64, 1, 1, 3, false}, {64, 64, 27, 1, 2, true},
                             {64, 48, 1, 1, 2, false},  {48, 48, 27, 1, 1, true},  {48, 32, 1, 1, 1, false},
                             {32, 32, 27, 1, 0, true},  {32, kOut, 1, 1, 0, false}};
    size_t off = 0;
    for (int i = 0; i < kLayers; ++i) {
        Layer &L = n->layers[i];
        L.cin = s[i].cin;
        L.cout = s[i].cout;
        L.taps = s[i].taps;
        L.stride = s[i].stride;
        L.level = s[i].level;
        L.relu = s[i].relu;
        L.woff = off;
        off += (size_t)L.cout * L.taps * L.cin;
        L.boff = off;
        off += L.cout;
    }
    n->nparams = off;
}

int out_level(const Layer &L) { return L.level + (L.stride == 2 ? 1 : 0); }

Geo fwd_geo(const qmin_warmnet_ctx *n, const Layer &L)
{
    const Dims di = dims_at(n, L.level), dd = dims_at(n, out_level(L));
    Geo g;
    g.Di = di.z;
    g.Hi = di.y;
    g.Wi = di.x;
    g.Do = dd.z;
    g.Ho = dd.y;
    g.Wo = dd.x;
    g.cin = L.cin;
    g.cout = L.cout;
    g.taps = L.taps;
    g.stride = L.stride;
    g.mode = 0;
    g.nb = n->B;
    return g;
}

int check_launch(qmin_warmnet_ctx *n, const char *what, int nk)
{
    n->launches += nk;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return nfail(QMIN_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return QMIN_OK;
}

// forward of layer i: BF16 output into act[i], or FP32 into `f32out`
void run_layer(qmin_warmnet_ctx *n, int i, const bf16 *in, float *f32out)
{
    const Layer &L = n->layers[i];
    const Geo g = fwd_geo(n, L);
    const int rows = (int)rows_at(n, out_level(L));
    if (f32out)
        conv_gemm<false>(g, in, n->pb + L.woff, n->p + L.boff, nullptr, f32out, L.relu, rows, n->stream, n->path);
    else
        conv_gemm<true>(g, in, n->pb + L.woff, n->p + L.boff, nullptr, n->act[i], L.relu, rows, n->stream,
                        n->path);
}

// backward of layer i: gout is the FP32 gradient w.r.t. the layer's output
// (after its ReLU); accumulates the weight and bias gradients and, if gin is
// given, writes the gradient w.r.t. the layer's input (+ addend) into gin
void layer_backward(qmin_warmnet_ctx *n, int i, const float *gout, const bf16 *act_in, float *gin, const float *addend)
{
    cudaStream_t s = n->stream;
    const Layer &L = n->layers[i];
    const long long rows_out = rows_at(n, out_level(L)), rows_in = rows_at(n, L.level);
    const bf16 *act_out = L.relu ? n->act[i] : nullptr;
    const long long ne = rows_out * L.cout;
    if (act_out) k_relu_grad_bf16<<<grid1(ne), 256, 0, s>>>(gout, act_out, n->gbf, ne);
    else k_f32_to_bf16<<<grid1(ne), 256, 0, s>>>(gout, n->gbf, ne);
    k_bias_grad<<<dim3((unsigned)std::min<long long>((rows_out + 7) / 8, 1024), (unsigned)((L.cout + 31) / 32)), 256, 0,
                  s>>>(gout, act_out, n->g + L.boff, rows_out, L.cout);
    const Geo g = fwd_geo(n, L);
    {
        const int tiles = ((L.cout + 63) / 64) * ((L.cin + 63) / 64);
        const long long want = std::max<long long>(1, 152 * 8 / (L.taps * tiles));
        long long chunk = (rows_out + want - 1) / want;
        chunk = std::max<long long>(256, (chunk + 15) / 16 * 16);
        const dim3 grid((unsigned)((rows_out + chunk - 1) / chunk), (unsigned)L.taps, (unsigned)tiles);
        k_conv_wgrad<<<grid, 128, 0, s>>>(g, n->gbf, act_in, n->g + L.woff, (int)rows_out, (int)chunk);
    }
    n->launches += 3;
    if (!gin) return;
    Geo d;
    d.Di = g.Do;
    d.Hi = g.Ho;
    d.Wi = g.Wo;
    d.Do = g.Di;
    d.Ho = g.Hi;
    d.Wo = g.Wi;
    d.cin = L.cout;
    d.cout = L.cin;
    d.taps = L.taps;
    d.stride = L.stride;
    d.mode = L.stride == 2 ? 1 : 0;
    d.nb = n->B;
    const int flip = (L.stride == 1 && L.taps == 27) ? 1 : 0;
    k_dgrad_weights<<<grid1((long long)L.cout * L.cin * L.taps), 256, 0, s>>>(n->pb + L.woff, n->wd, L.cout, L.cin,
                                                                              L.taps, flip);
    conv_gemm<false>(d, n->gbf, n->wd, nullptr, addend, gin, 0, (int)rows_in, s, n->path);
    n->launches += 2;
}

template <class T>
int features_impl(qmin_warmnet_ctx *n, int sample, const T *Q, long long P, const int8_t *types,
                  const qmin_object *objs, int nobj)
{
    ObjTab tab;
    tab.n = nobj;
    for (int k = 0; k < nobj; ++k) {
        tab.kind[k] = objs[k].kind;
        tab.W[k] = (float)objs[k].W;
    }
    const long long N = sites(n, 0);
    k_features<T><<<grid1(N), 256, 0, n->stream>>>(Q, P, types, (int)N, tab, n->x + (size_t)sample * N * kIn,
                                                   n->mask ? n->mask + (size_t)sample * N : nullptr);
    return check_launch(n, "qmin_warmnet_features", 1);
}

}  // namespace

int qmin_warmnet_create(int batch, int Lx, int Ly, int Lz, int train, qmin_warmnet *out)
{
    if (!out) return nfail(QMIN_EINVAL, "qmin_warmnet_create: null output handle");
    *out = nullptr;
    if (batch < 1 || Lx < 8 || Ly < 8 || Lz < 8 || (Lx | Ly | Lz) % 8 != 0)
        return nfail(QMIN_EINVAL, "qmin_warmnet_create: batch >= 1 and every side a positive multiple of 8");
    if ((long long)batch * Lx * Ly * Lz > (1ll << 30))
        return nfail(QMIN_EINVAL, "qmin_warmnet_create: batch x sites above 2^30");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return nfail(QMIN_ENODEVICE, "qmin_warmnet_create: no CUDA device available");
    }
    auto *n = new qmin_warmnet_ctx();
    n->B = batch;
    n->Lx = Lx;
    n->Ly = Ly;
    n->Lz = Lz;
    n->train = train != 0;
    build_layers(n);
    bool ok = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) == cudaSuccess;
    n->own_stream = ok;
    auto al = [&](void **p, size_t bytes) {
        if (ok && cudaMalloc(p, bytes) != cudaSuccess) ok = false;
        if (ok) ok = cudaMemsetAsync(*p, 0, bytes, n->stream) == cudaSuccess;
    };
    const size_t R0 = (size_t)rows_at(n, 0);
    al((void **)&n->p, n->nparams * 4);
    al((void **)&n->pb, n->nparams * 2);
    al((void **)&n->x, R0 * kIn * 2);
    al((void **)&n->y, R0 * kOut * 4);
    al((void **)&n->mask, R0);
    for (int i = 0; i < kLayers - 1; ++i) {
        const Layer &L = n->layers[i];
        const size_t ro = (size_t)rows_at(n, out_level(L));
        if (i == 4 || i == 6 || i == 8) {
            // the FP32 output on the coarse grid, and the BF16 upsampled sum on the fine one
            al((void **)&n->pre[i], ro * L.cout * 4);
            al((void **)&n->act[i], (size_t)rows_at(n, L.level - 1) * L.cout * 2);
        } else {
            al((void **)&n->act[i], ro * L.cout * 2);
        }
    }
    if (n->train) {
        size_t maxw = 0, maxg = 0;
        for (const Layer &L : n->layers) {
            maxw = std::max(maxw, (size_t)L.cout * L.taps * L.cin);
            maxg = std::max(maxg, (size_t)rows_at(n, L.level) * L.cin);
            maxg = std::max(maxg, (size_t)rows_at(n, out_level(L)) * L.cout);
        }
        al((void **)&n->g, n->nparams * 4);
        al((void **)&n->m, n->nparams * 4);
        al((void **)&n->v, n->nparams * 4);
        al((void **)&n->wd, maxw * 2);
        al((void **)&n->gA, maxg * 4);
        al((void **)&n->gB, maxg * 4);
        al((void **)&n->gbf, maxg * 2);
        al((void **)&n->sk[0], (size_t)rows_at(n, 0) * 32 * 4);
        al((void **)&n->sk[1], (size_t)rows_at(n, 1) * 48 * 4);
        al((void **)&n->sk[2], (size_t)rows_at(n, 2) * 64 * 4);
        al((void **)&n->loss, sizeof(double));
        al((void **)&n->count, sizeof(unsigned long long));
    }
    if (ok) ok = cudaStreamSynchronize(n->stream) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        qmin_warmnet_destroy(n);
        return nfail(QMIN_ENOMEM, "qmin_warmnet_create: device allocation failed");
    }
    *out = n;
    return QMIN_OK;
}

int qmin_warmnet_destroy(qmin_warmnet n)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_destroy: null handle");
    if (n->stream) cudaStreamSynchronize(n->stream);
    void *bufs[] = {n->p, n->g, n->m, n->v, n->pb, n->wd, n->x, n->mask, n->y, n->gA, n->gB, n->gbf, n->loss, n->count,
                    n->sk[0], n->sk[1], n->sk[2]};
    for (void *b : bufs)
        if (b) cudaFree(b);
    for (int i = 0; i < kLayers; ++i) {
        if (n->act[i]) cudaFree(n->act[i]);
        if (n->pre[i]) cudaFree(n->pre[i]);
    }
    if (n->own_stream) cudaStreamDestroy(n->stream);
    delete n;
    return QMIN_OK;
}

int qmin_warmnet_set_stream(qmin_warmnet n, void *stream)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_set_stream: null handle");
    cudaStreamSynchronize(n->stream);
    if (n->own_stream) cudaStreamDestroy(n->stream);
    n->own_stream = false;
    n->stream = (cudaStream_t)stream;
    return QMIN_OK;
}

int qmin_warmnet_param_count(qmin_warmnet n, long long *count)
{
    if (!n || !count) return nfail(QMIN_EINVAL, "qmin_warmnet_param_count: null argument");
    *count = (long long)n->nparams;
    return QMIN_OK;
}

int qmin_warmnet_shape(qmin_warmnet n, int *batch, int *Lx, int *Ly, int *Lz)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_shape: null handle");
    if (batch) *batch = n->B;
    if (Lx) *Lx = n->Lx;
    if (Ly) *Ly = n->Ly;
    if (Lz) *Lz = n->Lz;
    return QMIN_OK;
}

int qmin_warmnet_buffers(qmin_warmnet n, void **x, float **y, uint8_t **mask)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_buffers: null handle");
    if (x) *x = n->x;
    if (y) *y = n->y;
    if (mask) *mask = n->mask;
    return QMIN_OK;
}

int qmin_warmnet_set_params(qmin_warmnet n, const float *host)
{
    if (!n || !host) return nfail(QMIN_EINVAL, "qmin_warmnet_set_params: null argument");
    cudaStream_t s = n->stream;
    if (cudaMemcpyAsync(n->p, host, n->nparams * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return nfail(QMIN_ECUDA, "qmin_warmnet_set_params: copy failed");
    k_f32_to_bf16<<<grid1(n->nparams), 256, 0, s>>>(n->p, n->pb, (long long)n->nparams);
    if (n->train) {
        cudaMemsetAsync(n->m, 0, n->nparams * 4, s);
        cudaMemsetAsync(n->v, 0, n->nparams * 4, s);
    }
    n->adam_t = 0;
    const int rc = check_launch(n, "qmin_warmnet_set_params", 1);
    if (rc) return rc;
    return cudaStreamSynchronize(s) == cudaSuccess ? QMIN_OK : nfail(QMIN_ECUDA, "qmin_warmnet_set_params: sync");
}

int qmin_warmnet_get_params(qmin_warmnet n, float *params, float *grads)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_get_params: null handle");
    if (grads && !n->train) return nfail(QMIN_ESTATE, "qmin_warmnet_get_params: gradients need a training net");
    if (params) cudaMemcpyAsync(params, n->p, n->nparams * 4, cudaMemcpyDeviceToHost, n->stream);
    if (grads) cudaMemcpyAsync(grads, n->g, n->nparams * 4, cudaMemcpyDeviceToHost, n->stream);
    return cudaStreamSynchronize(n->stream) == cudaSuccess ? QMIN_OK : nfail(QMIN_ECUDA, "qmin_warmnet_get_params");
}

int qmin_warmnet_features(qmin_warmnet n, int sample, const void *Q_dev, int precision, long long plane_stride,
                          const int8_t *types_dev, const qmin_object *objs, int nobj)
{
    if (!n || !Q_dev || !types_dev || (nobj > 0 && !objs)) return nfail(QMIN_EINVAL, "qmin_warmnet_features: null argument");
    if (sample < 0 || sample >= n->B) return nfail(QMIN_EINVAL, "qmin_warmnet_features: sample out of range");
    if (nobj < 0 || nobj > kMaxObj) return nfail(QMIN_EINVAL, "qmin_warmnet_features: at most 64 objects");
    if (plane_stride < sites(n, 0)) return nfail(QMIN_EINVAL, "qmin_warmnet_features: plane stride below the site count");
    if (precision == QMIN_FP64)
        return features_impl(n, sample, (const double *)Q_dev, plane_stride, types_dev, objs, nobj);
    if (precision == QMIN_FP32)
        return features_impl(n, sample, (const float *)Q_dev, plane_stride, types_dev, objs, nobj);
    return nfail(QMIN_EINVAL, "qmin_warmnet_features: precision must be QMIN_FP64 or QMIN_FP32");
}

int qmin_warmnet_forward(qmin_warmnet n)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_forward: null handle");
    cudaStream_t s = n->stream;
    run_layer(n, 0, n->x, nullptr);
    run_layer(n, 1, n->act[0], nullptr);
    run_layer(n, 2, n->act[1], nullptr);
    run_layer(n, 3, n->act[2], nullptr);
    run_layer(n, 4, n->act[3], n->pre[4]);
    k_up2_add<<<grid1(rows_at(n, 2) * 8), 256, 0, s>>>(n->pre[4], n->act[2], n->act[4], dims_at(n, 3), 64);
    run_layer(n, 5, n->act[4], nullptr);
    run_layer(n, 6, n->act[5], n->pre[6]);
    k_up2_add<<<grid1(rows_at(n, 1) * 6), 256, 0, s>>>(n->pre[6], n->act[1], n->act[6], dims_at(n, 2), 48);
    run_layer(n, 7, n->act[6], nullptr);
    run_layer(n, 8, n->act[7], n->pre[8]);
    k_up2_add<<<grid1(rows_at(n, 0) * 4), 256, 0, s>>>(n->pre[8], n->act[0], n->act[8], dims_at(n, 1), 32);
    run_layer(n, 9, n->act[8], nullptr);
    run_layer(n, 10, n->act[9], n->y);
    return check_launch(n, "qmin_warmnet_forward", 14);
}

int qmin_warmnet_backward(qmin_warmnet n, const float *target_dev, double *loss)
{
    if (!n || !target_dev) return nfail(QMIN_EINVAL, "qmin_warmnet_backward: null argument");
    if (!n->train) return nfail(QMIN_ESTATE, "qmin_warmnet_backward: the net was created without training buffers");
    cudaStream_t s = n->stream;
    const long long R = rows_at(n, 0);
    cudaMemsetAsync(n->g, 0, n->nparams * 4, s);
    cudaMemsetAsync(n->loss, 0, sizeof(double), s);
    cudaMemsetAsync(n->count, 0, sizeof(unsigned long long), s);
    k_count_mask<<<grid1(R), 256, 0, s>>>(n->mask, R, n->count);
    k_mse<<<grid1(R), 256, 0, s>>>(n->y, target_dev, n->mask, n->count, n->gA, n->loss, R);
    n->launches += 2;
    float *gA = n->gA, *gB = n->gB;
    layer_backward(n, 10, gA, n->act[9], gB, nullptr);        // d act9
    layer_backward(n, 9, gB, n->act[8], n->sk[0], nullptr);   // d act8 = d skip of enc0
    k_up2_grad<<<grid1(rows_at(n, 1) * 32), 256, 0, s>>>(n->sk[0], gB, dims_at(n, 1), 32);
    layer_backward(n, 8, gB, n->act[7], gA, nullptr);         // d act7
    layer_backward(n, 7, gA, n->act[6], n->sk[1], nullptr);   // d act6 = d skip of enc1
    k_up2_grad<<<grid1(rows_at(n, 2) * 48), 256, 0, s>>>(n->sk[1], gA, dims_at(n, 2), 48);
    layer_backward(n, 6, gA, n->act[5], gB, nullptr);         // d act5
    layer_backward(n, 5, gB, n->act[4], n->sk[2], nullptr);   // d act4 = d skip of enc2
    k_up2_grad<<<grid1(rows_at(n, 3) * 64), 256, 0, s>>>(n->sk[2], gA, dims_at(n, 3), 64);
    layer_backward(n, 4, gA, n->act[3], gB, nullptr);         // d act3
    layer_backward(n, 3, gB, n->act[2], gA, n->sk[2]);        // d act2 (+ skip)
    layer_backward(n, 2, gA, n->act[1], gB, n->sk[1]);        // d act1 (+ skip)
    layer_backward(n, 1, gB, n->act[0], gA, n->sk[0]);        // d act0 (+ skip)
    layer_backward(n, 0, gA, n->x, nullptr, nullptr);
    n->launches += 3;
    int rc = check_launch(n, "qmin_warmnet_backward", 0);
    if (rc) return rc;
    if (loss) {
        if (cudaMemcpyAsync(loss, n->loss, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return nfail(QMIN_ECUDA, "qmin_warmnet_backward: loss read-back failed");
        if (!std::isfinite(*loss)) return nfail(QMIN_ENONFINITE, "qmin_warmnet_backward: non-finite loss");
    }
    return QMIN_OK;
}

int qmin_warmnet_adam_step(qmin_warmnet n, double lr, double beta1, double beta2, double eps)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_adam_step: null handle");
    if (!n->train) return nfail(QMIN_ESTATE, "qmin_warmnet_adam_step: the net was created without training buffers");
    n->adam_t += 1;
    const double c1 = 1.0 / (1.0 - std::pow(beta1, (double)n->adam_t));
    const double c2 = 1.0 / (1.0 - std::pow(beta2, (double)n->adam_t));
    k_adam_params<<<grid1(n->nparams), 256, 0, n->stream>>>(n->p, n->g, n->m, n->v, n->pb, (long long)n->nparams,
                                                            (float)lr, (float)beta1, (float)beta2, (float)eps,
                                                            (float)c1, (float)c2);
    return check_launch(n, "qmin_warmnet_adam_step", 1);
}

int qmin_warmnet_write_state(qmin_warmnet n, int sample, void *Q_dev, int precision, long long plane_stride,
                             const int8_t *types_dev)
{
    if (!n || !Q_dev || !types_dev) return nfail(QMIN_EINVAL, "qmin_warmnet_write_state: null argument");
    if (sample < 0 || sample >= n->B) return nfail(QMIN_EINVAL, "qmin_warmnet_write_state: sample out of range");
    if (plane_stride < sites(n, 0)) return nfail(QMIN_EINVAL, "qmin_warmnet_write_state: plane stride below the site count");
    const long long N = sites(n, 0);
    const float *y = n->y + (size_t)sample * N * kOut;
    if (precision == QMIN_FP64)
        k_write_state<double><<<grid1(N), 256, 0, n->stream>>>(y, (double *)Q_dev, plane_stride, types_dev, (int)N);
    else if (precision == QMIN_FP32)
        k_write_state<float><<<grid1(N), 256, 0, n->stream>>>(y, (float *)Q_dev, plane_stride, types_dev, (int)N);
    else
        return nfail(QMIN_EINVAL, "qmin_warmnet_write_state: precision must be QMIN_FP64 or QMIN_FP32");
    return check_launch(n, "qmin_warmnet_write_state", 1);
}

int qmin_warmnet_sync(qmin_warmnet n)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_sync: null handle");
    const cudaError_t e = cudaStreamSynchronize(n->stream);
    if (e != cudaSuccess) return nfail(QMIN_ECUDA, std::string("qmin_warmnet_sync: ") + cudaGetErrorString(e));
    int err = 0;
    if (cudaMemcpyFromSymbol(&err, g_conv_err, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return QMIN_OK;
    }
    if (err) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_conv_err, &zero, sizeof(int));
        return nfail(QMIN_ETIMEOUT, "qmin_warmnet_sync: a tensor-core or TMA wait in a convolution gave up "
                                    "(the pass's outputs are void)");
    }
    return QMIN_OK;
}

int qmin_set_wait_limit(long long polls)
{
    const int conv = polls < 0 ? kWaitPolls : (int)std::min<long long>(polls, 1LL << 30);
    const int split = polls < 0 ? qmin::kSplitWaitPolls : conv;
    cudaError_t e = cudaMemcpyToSymbol(g_conv_wait_limit, &conv, sizeof(int));
    if (e == cudaSuccess) e = qmin::split_set_wait_limit(split);
    if (e != cudaSuccess) return nfail(QMIN_ECUDA, std::string("qmin_set_wait_limit: ") + cudaGetErrorString(e));
    return QMIN_OK;
}

int qmin_warmnet_set_tensor_path(qmin_warmnet n, int path)
{
    if (!n) return nfail(QMIN_EINVAL, "qmin_warmnet_set_tensor_path: null handle");
    if (path < 0 || path > 2) return nfail(QMIN_EINVAL, "qmin_warmnet_set_tensor_path: path must be 0, 1 or 2");
    n->path = path;
    return QMIN_OK;
}

int qmin_warmnet_kernel_launches(qmin_warmnet n, long long *count)
{
    if (!n || !count) return nfail(QMIN_EINVAL, "qmin_warmnet_kernel_launches: null argument");
    *count = n->launches;
    return QMIN_OK;
}
