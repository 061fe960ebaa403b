// 3D convolution kernels of the learned preconditioner: 3x3x3 periodic
// convolutions with 16 channels, BF16 operands and FP32 accumulation, over a
// batch of n^3 grids (n a multiple of 8).
//
// Layouts
//   act   [sys][z][y][x][16] bfloat16 (channels last, 32 B per point);
//   field [sys][z][y][x] float64 (the residual r, the output z, gradients);
//   wt    [27][16 cout][16 cin] bfloat16, tap t = (dx+1) + 3(dy+1) + 9(dz+1),
//         output(p) = sum_t W_t act(p + d_t)  (cross-correlation);
//   bias  [16] float32.
// Sources (the 16-channel rows a kernel stages): an act tensor; a field
// scaled per system with the system's shift eps as a second channel (the
// network input); a field scaled per system (single channel).
//
// Work decomposition: one 8x8x8 output tile per CTA iteration (persistent
// CTAs), its 10x10x10 halo staged in shared memory as 16-channel BF16 rows
// (two 16-byte chunks per point, XOR-swizzled on bit 2 of the point index so
// the eight rows of an ldmatrix hit distinct banks); the 27 taps are 27
// K = 16 steps of an implicit GEMM whose A rows are gathered by ldmatrix row
// addresses (output point + tap offset in the halo), mma.sync m16n8k16 BF16.
//
// forward / input-gradient: D[point][cout] = sum_t A_t[point][cin] W_t[cout][cin]
// weight-gradient:          dW_t[cout][cin] = sum_point G[point][cout] X[point + d_t][cin]
//
// For n >= 16 the forward / input-gradient convolution runs on the 5th-
// generation tensor cores instead (conv_tc_kernel below): the halo is laid
// out so that every tap's A operand is one shared-memory descriptor, the
// accumulators live in TMEM.  The mma.sync kernel remains for n = 8 and for
// the weight gradient (a reduction over points, training only).
#include <cuda_bf16.h>
#include <stdint.h>

#include "../../include/libconv_gb300.h"
#include "lcg_plan.cuh"

namespace {

constexpr int kT = 8;                 // output tile edge
constexpr int kH = kT + 2;            // halo tile edge
constexpr int kHalo = kH * kH * kH;   // 1000 points
constexpr int kThreads = 256;

enum Src { SRC_ACT = 0, SRC_FIELD_EPS = 1, SRC_FIELD = 2 };
enum Dst { DST_ACT_RELU = 0, DST_FIELD = 1, DST_ACT_MASK = 2 };

struct ConvArgs {
    int n, nsys;
    // source
    const __nv_bfloat16 *src_act;
    const double *src_field;
    const double *src_fac;     // per system factor applied to the field
    const double *eps;         // per system shift (SRC_FIELD_EPS channel 1)
    // weights
    const __nv_bfloat16 *wt;   // [27][16][16]
    const float *bias;         // [16] (forward)
    // destination
    __nv_bfloat16 *dst_act;
    double *dst_field;
    const double *dst_fac;     // per system factor of DST_FIELD
    const __nv_bfloat16 *mask; // DST_ACT_MASK: keep where mask > 0
    int nout_tiles;            // 1 (cout 0-7) or 2 (cout 0-15)
    const int *active;         // per system: 0 = skip its tiles (or null: all)
};

__device__ __forceinline__ uint32_t saddr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Byte offset of 16-byte chunk c (channels 8c..8c+7) of staged point h.
__device__ __forceinline__ uint32_t row_off(int h, int c) {
    return (uint32_t)(h * 32 + ((c ^ ((h >> 2) & 1)) << 4));
}

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// Stage the 16-channel rows of `count` points of system s into smem rows
// 0..count-1; point i of the staged box sits at global (x0 + i % ex,
// y0 + (i / ex) % ey, z0 + i / (ex ey)) with periodic wrap.
template <int SRC>
__device__ __forceinline__ void stage(const ConvArgs &A, uint8_t *sm, int s, int x0, int y0, int z0,
                                      int ex, int ey, int count) {
    const int n = A.n;
    const long long base = (long long)s * n * n * n;
    if (SRC == SRC_ACT) {
        for (int idx = threadIdx.x; idx < 2 * count; idx += kThreads) {
            const int i = idx >> 1, c = idx & 1;
            const int gx = wrap(x0 + i % ex, n), gy = wrap(y0 + (i / ex) % ey, n),
                      gz = wrap(z0 + i / (ex * ey), n);
            const long long p = base + gx + (long long)n * (gy + (long long)n * gz);
            const uint4 v = *reinterpret_cast<const uint4 *>(A.src_act + p * 16 + c * 8);
            *reinterpret_cast<uint4 *>(sm + row_off(i, c)) = v;
        }
    } else {
        const double fac = A.src_fac[s];
        const float e = SRC == SRC_FIELD_EPS ? (float)A.eps[s] : 0.f;
        for (int i = threadIdx.x; i < count; i += kThreads) {
            const int gx = wrap(x0 + i % ex, n), gy = wrap(y0 + (i / ex) % ey, n),
                      gz = wrap(z0 + i / (ex * ey), n);
            const long long p = base + gx + (long long)n * (gy + (long long)n * gz);
            const float v = (float)(A.src_field[p] * fac);
            __nv_bfloat162 h01 = __floats2bfloat162_rn(v, e);
            uint4 lo = make_uint4(*reinterpret_cast<uint32_t *>(&h01), 0u, 0u, 0u);
            *reinterpret_cast<uint4 *>(sm + row_off(i, 0)) = lo;
            *reinterpret_cast<uint4 *>(sm + row_off(i, 1)) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
}

// Forward / input-gradient convolution.  Warp w owns m-tiles w, w+8, w+16,
// w+24 (16 consecutive tile points each, x fastest).
template <int SRC, int DST>
__global__ void __launch_bounds__(kThreads) conv_kernel(const ConvArgs A) {
    __shared__ __align__(128) uint8_t halo[kHalo * 32];
    __shared__ __align__(128) uint8_t wsm[27 * 16 * 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // weights: row (tap, cout) = 16 cin = two 16-byte chunks, swizzled like the halo
    for (int i = threadIdx.x; i < 27 * 16 * 2; i += kThreads) {
        const int row = i >> 1, c = i & 1;
        *reinterpret_cast<uint4 *>(wsm + row_off(row, c)) =
            *reinterpret_cast<const uint4 *>(A.wt + row * 16 + c * 8);
    }
    const int tpa = A.n / kT;
    const long long ntiles = (long long)A.nsys * tpa * tpa * tpa;
    const int g = lane >> 2, q = lane & 3;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int s = (int)(tile / (tpa * tpa * tpa));
        const int tr = (int)(tile % (tpa * tpa * tpa));
        const int tx = (tr % tpa) * kT, ty = ((tr / tpa) % tpa) * kT, tz = (tr / (tpa * tpa)) * kT;
        if (A.active && !A.active[s]) continue;   // uniform over the CTA
        __syncthreads();   // previous tile's halo fully consumed
        stage<SRC>(A, halo, s, tx - 1, ty - 1, tz - 1, kH, kH, kHalo);
        __syncthreads();
        float acc[4][2][4];
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[m][j][e] = 0.f;
        // this lane's ldmatrix row: A row (tile point) and chunk
        const int arow = (lane & 7) + 8 * ((lane >> 3) & 1), achunk = lane >> 4;
        const int brow = (lane & 7) + 8 * (lane >> 4), bchunk = (lane >> 3) & 1;
        for (int t = 0; t < 27; ++t) {
            const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
            uint32_t b[4];
            ldsm_x4(saddr(wsm) + row_off(t * 16 + brow, bchunk), b);
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int pt = (warp + 8 * m) * 16 + arow;               // tile point
                const int ox = pt & 7, oy = (pt >> 3) & 7, oz = pt >> 6;
                const int h = (ox + 1 + dx) + kH * ((oy + 1 + dy) + kH * (oz + 1 + dz));
                uint32_t a[4];
                ldsm_x4(saddr(halo) + row_off(h, achunk), a);
                mma_bf16(acc[m][0], a, b[0], b[1]);
                if (A.nout_tiles > 1) mma_bf16(acc[m][1], a, b[2], b[3]);
            }
        }
        // epilogue: rows g, g+8 of each m-tile; columns 2q, 2q+1 of each n-tile
        const int n = A.n;
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int hr = 0; hr < 2; ++hr) {
                const int pt = (warp + 8 * m) * 16 + g + 8 * hr;
                const int gx = tx + (pt & 7), gy = ty + ((pt >> 3) & 7), gz = tz + (pt >> 6);
                const long long p = (long long)s * n * n * n + gx + (long long)n * (gy + (long long)n * gz);
                if (DST == DST_FIELD) {
                    if (q == 0)
                        A.dst_field[p] = A.dst_fac[s] * (double)(acc[m][0][2 * hr] + A.bias[0]);
                } else {
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const int c = 8 * j + 2 * q;
                        float v0 = acc[m][j][2 * hr], v1 = acc[m][j][2 * hr + 1];
                        if (DST == DST_ACT_RELU) {
                            v0 = fmaxf(v0 + A.bias[c], 0.f);
                            v1 = fmaxf(v1 + A.bias[c + 1], 0.f);
                        } else {
                            const __nv_bfloat162 mk =
                                *reinterpret_cast<const __nv_bfloat162 *>(A.mask + p * 16 + c);
                            if (!(__low2float(mk) > 0.f)) v0 = 0.f;
                            if (!(__high2float(mk) > 0.f)) v1 = 0.f;
                        }
                        *reinterpret_cast<__nv_bfloat162 *>(A.dst_act + p * 16 + c) =
                            __floats2bfloat162_rn(v0, v1);
                    }
                }
            }
    }
}

// Weight gradient: per CTA partial sums over its tiles of
//   dW_t[cout][cin] = sum_p G[p][cout] X[p + d_t][cin],  db[cout] = sum_p G[p][cout]
// written to part[blockIdx.x][27*256 + 16] (float); warp w owns taps w, w+8,
// w+16, w+24.  G is the output gradient (source kind GSRC, no halo), X the
// layer input (source kind XSRC, halo).
template <int GSRC, int XSRC>
__global__ void __launch_bounds__(kThreads) wgrad_kernel(const ConvArgs G, const ConvArgs X,
                                                         float *part) {
    __shared__ __align__(128) uint8_t halo[kHalo * 32];
    __shared__ __align__(128) uint8_t gsm[kT * kT * kT * 32];
    __shared__ float bsum[16];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < 16) bsum[threadIdx.x] = 0.f;
    const int tpa = G.n / kT;
    const long long ntiles = (long long)G.nsys * tpa * tpa * tpa;
    float acc[4][2][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
    float bacc = 0.f;   // threads 0..15: bias gradient of cout = threadIdx.x
    // ldmatrix.trans rows: A (G^T) stored rows = points, chunk = cout half;
    // B (X) stored rows = points, chunk = cin half
    const int a_pt = (lane & 7) + 8 * (lane >> 4), a_ch = (lane >> 3) & 1;
    const int b_pt = (lane & 7) + 8 * ((lane >> 3) & 1), b_ch = lane >> 4;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int s = (int)(tile / (tpa * tpa * tpa));
        const int tr = (int)(tile % (tpa * tpa * tpa));
        const int tx = (tr % tpa) * kT, ty = ((tr / tpa) % tpa) * kT, tz = (tr / (tpa * tpa)) * kT;
        __syncthreads();
        stage<XSRC>(X, halo, s, tx - 1, ty - 1, tz - 1, kH, kH, kHalo);
        stage<GSRC>(G, gsm, s, tx, ty, tz, kT, kT, kT * kT * kT);
        __syncthreads();
        if (threadIdx.x < 16) {
            float b = 0.f;
            for (int p = 0; p < kT * kT * kT; ++p) {
                const __nv_bfloat16 *row = reinterpret_cast<const __nv_bfloat16 *>(
                    gsm + row_off(p, threadIdx.x >> 3));
                b += __bfloat162float(row[threadIdx.x & 7]);
            }
            bacc += b;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int t = warp + 8 * i;
            if (t >= 27) break;
            const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
            for (int k0 = 0; k0 < kT * kT * kT; k0 += 16) {
                uint32_t a[4], b[4];
                ldsm_x4_t(saddr(gsm) + row_off(k0 + a_pt, a_ch), a);
                const int pt = k0 + b_pt;
                const int ox = pt & 7, oy = (pt >> 3) & 7, oz = pt >> 6;
                const int h = (ox + 1 + dx) + kH * ((oy + 1 + dy) + kH * (oz + 1 + dz));
                ldsm_x4_t(saddr(halo) + row_off(h, b_ch), b);
                mma_bf16(acc[i][0], a, b[0], b[1]);
                mma_bf16(acc[i][1], a, b[2], b[3]);
            }
        }
    }
    // partials: rows (cout) g, g+8; columns (cin) 2q, 2q+1 of each n-tile
    float *out = part + (long long)blockIdx.x * (27 * 256 + 16);
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int t = warp + 8 * i;
        if (t >= 27) break;
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int hr = 0; hr < 2; ++hr) {
                const int co = g + 8 * hr, ci = 8 * j + 2 * q;
                out[t * 256 + co * 16 + ci] = acc[i][j][2 * hr];
                out[t * 256 + co * 16 + ci + 1] = acc[i][j][2 * hr + 1];
            }
    }
    if (threadIdx.x < 16) out[27 * 256 + threadIdx.x] = bacc;
}

// Sum of the per-CTA partials: out[i] = sum_b part[b][i], i < len.
__global__ void reduce_parts(const float *part, int nparts, int len, float *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= len) return;
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += part[(long long)b * len + i];
    out[i] = (float)s;
}

// ---------------------------------------------------------------------------
// Tensor-core (tcgen05) forward / input-gradient convolution, n >= 16.
//
// Output tile: 8 (x) x 16 (y) x TZ (z) points.  Its 10 x 18 x (TZ + 2) halo
// sits in shared memory as two planes of 8-channel chunks,
// [chunk][z][y][x] x 16 B.  For halo z-plane h and in-plane tap (dx, dy) the
// A operand (M = 128 rows = 16 y-rows of 8 x-points, K = 16 input channels)
// is one K-major, unswizzled descriptor into that buffer: a core matrix is 8
// consecutive x-points x 16 B starting at halo point (dx, dy, h), the 8-row
// groups (successive y) one halo row (160 B) apart, the two channel chunks
// one plane apart.  The three z-taps of (dx, dy) read that same A: their
// weights are stacked along N (rows 16 (2 - dz) + cout, dz = 0..2 the tap's
// z offset + 1), and the contribution of halo plane h through tap dz belongs
// to output plane h - dz, whose FP32 accumulators sit at TMEM columns
// 16 (h - dz) + cout.  Stacked in that order, one MMA at column 16 (h - dz_max)
// with N = 16 x (number of valid dz) adds every z-tap of (dx, dy) for plane
// h to its own output plane; the first MMA of a plane that opens output
// plane h is split so that block starts from zero (accumulate off) while the
// older planes' blocks accumulate.  Per tile: 9 (TZ + 2) + TZ - 1 MMAs of
// kind::f16 (BF16 operands, M = 128, N = 16 / 32 / 48, K = 16); each A tile
// read from shared memory serves up to 48 output columns instead of 16.
// Weights: per (dx, dy) a 48 x 16 K-major tile, 8-row groups 128 B apart,
// the two K chunks 768 B apart.
//
// One CTA of 8 warps per tile at a time: all threads stage the halo
// (cp.async for activations), thread 0 issues the MMAs and commits them to
// an mbarrier, then warp w drains TMEM lanes 32 (w % 4) .. + 31 of half of
// the output planes (bias + ReLU / mask / field scale, 32 B stored per
// point).  Several CTAs reside per SM (three at TZ = 8), so one CTA's
// staging overlaps another's MMAs and epilogue; on GB300 one M = 128 MMA of
// this shape costs about 80 cycles whatever N (16-48), following its 4 KB A
// tile, so the layer is bound by the number of A tiles read, which is what
// the z-tap stacking cuts.  Every wait is bounded; a wait that gives up sets
// the device status word.
namespace tcc {
constexpr int kTX = 8, kTY = 16;
constexpr int kHX = kTX + 2, kHY = kTY + 2;
constexpr uint32_t kRowB = kHX * 16;              // one halo row (8-row group stride, SBO)
constexpr uint32_t kJB = 48 * 32;                 // one (dx, dy) stack of 3 taps x 16 x 16 BF16
constexpr uint32_t kWB = 9 * kJB;
constexpr int kThreads = 256;
constexpr long long kWaitCycles = 4000000000LL;   // ~2 s of SM clock

template <int TZ>
struct Geo {
    static constexpr int HZ = TZ + 2;
    static constexpr int HPTS = kHX * kHY * HZ;                  // halo points
    static constexpr uint32_t PLANE = HPTS * 16;                 // one 8-channel chunk plane
    static constexpr uint32_t HALO = 2 * PLANE;
    static constexpr uint32_t SMEM = HALO + kWB + 16 * 4 + 16;   // + bias, mbarrier, TMEM slot
    static constexpr uint32_t TMEM_COLS = TZ * 16 <= 32 ? 32 : TZ * 16 <= 64 ? 64 : 128;
    static constexpr int CTAS = SMEM <= 50 * 1024 ? 4 : 3;       // resident CTAs per SM
    static_assert(TZ % 2 == 0 && TZ * 16 <= 128, "tile depth");
    static_assert(CTAS * TMEM_COLS <= 512, "TMEM columns");
    static_assert(CTAS * (SMEM + 1024) <= 228 * 1024, "shared memory");
    static_assert(2 * PLANE <= (0x3FFFu << 4), "descriptor offsets");
};

// kind::f16 instruction descriptor: D F32 (bits 4-5 = 1), A and B BF16 (bits
// 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc(int nn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nn >> 3) << 17) | ((128u >> 4) << 24);
}

// Shared-memory matrix descriptor, K-major without swizzle: start address,
// leading (K-direction) and stride (8-row group) byte offsets in 16-byte
// units, descriptor version 1 at bits 46-47.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(accum)
        : "memory");
}

__device__ __forceinline__ bool bar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase of the given parity; false after ~2 s.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    if (bar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (!bar_try(bar, parity)) {
        __nanosleep(64);
        if (clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}

// Stage the halo of the tile whose first halo point is (x0, y0, z0) of
// system s (periodic wrap; n >= 16 so one wrap suffices on every axis).
template <int SRC, int TZ>
__device__ __forceinline__ void stage(const ConvArgs &A, uint8_t *halo, int s, int x0, int y0,
                                      int z0) {
    using G = Geo<TZ>;
    const int n = A.n;
    const long long base = (long long)s * n * n * n;
    if (SRC == SRC_ACT) {
        const uint32_t hb = saddr(halo);
        for (int idx = threadIdx.x; idx < 2 * G::HPTS; idx += kThreads) {
            const int i = idx >> 1, c = idx & 1;
            const int hx = i % kHX, hy = (i / kHX) % kHY, hz = i / (kHX * kHY);
            const int gx = wrap(x0 + hx, n), gy = wrap(y0 + hy, n), gz = wrap(z0 + hz, n);
            const long long p = base + gx + (long long)n * (gy + (long long)n * gz);
            cp_async16(hb + c * G::PLANE + i * 16, A.src_act + p * 16 + c * 8);
        }
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;\n" ::: "memory");
    } else {
        // channels 0 (field x factor) and 1 (eps or 0) in chunk 0; chunk 1
        // stays zero from the kernel's start
        const double fac = A.src_fac[s];
        const float e = SRC == SRC_FIELD_EPS ? (float)A.eps[s] : 0.f;
        for (int i = threadIdx.x; i < G::HPTS; i += kThreads) {
            const int hx = i % kHX, hy = (i / kHX) % kHY, hz = i / (kHX * kHY);
            const int gx = wrap(x0 + hx, n), gy = wrap(y0 + hy, n), gz = wrap(z0 + hz, n);
            const long long p = base + gx + (long long)n * (gy + (long long)n * gz);
            __nv_bfloat162 h01 = __floats2bfloat162_rn((float)(A.src_field[p] * fac), e);
            *reinterpret_cast<uint4 *>(halo + i * 16) =
                make_uint4(*reinterpret_cast<uint32_t *>(&h01), 0u, 0u, 0u);
        }
    }
}

// The MMAs of one tile (thread 0).
template <int TZ>
__device__ __forceinline__ void issue_tile(uint32_t tmem, uint32_t hb, uint32_t wb) {
    using G = Geo<TZ>;
#pragma unroll 1
    for (int h = 0; h < TZ + 2; ++h) {
        const int dmax = h < 2 ? h : 2, dmin = h > TZ - 1 ? h - (TZ - 1) : 0;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const int dx = j % 3, dy = j / 3;
            const uint64_t a = sdesc(hb + (h * kHY + dy) * kRowB + dx * 16, G::PLANE, kRowB);
            const uint32_t bj = wb + j * kJB;
            if (j == 0 && h < TZ) {
                // output plane h opens here (tap dz = 0, stack rows 32..47)
                mma(tmem + 16 * h, a, sdesc(bj + 32 * 16, 768, 128), idesc(16), 0u);
                if (dmax > 0)
                    mma(tmem + 16 * (h - dmax), a, sdesc(bj + 16 * (2 - dmax) * 16, 768, 128),
                        idesc(16 * dmax), 1u);
            } else {
                mma(tmem + 16 * (h - dmax), a, sdesc(bj + 16 * (2 - dmax) * 16, 768, 128),
                    idesc(16 * (dmax - dmin + 1)), 1u);
            }
        }
    }
}

}  // namespace tcc

template <int SRC, int DST, int TZ>
__global__ void __launch_bounds__(tcc::kThreads, tcc::Geo<TZ>::CTAS)
    conv_tc_kernel(const ConvArgs A, int *status) {
    using namespace tcc;
    using G = Geo<TZ>;
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t *halo = sm;
    uint8_t *wsm = sm + G::HALO;
    float *bsm = reinterpret_cast<float *>(wsm + kWB);
    uint64_t *bar = reinterpret_cast<uint64_t *>(bsm + 16);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = A.n;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         saddr(tslot)),
                     "r"(G::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // weights: 16-byte piece (tap t, cout co, cin chunk kc) to stack j = t % 9,
    // row 16 (2 - dz) + co with dz = t / 9
    for (int i = tid; i < 27 * 16 * 2; i += tcc::kThreads) {
        const int t = i >> 5, co = (i >> 1) & 15, kc = i & 1;
        const int row = 16 * (2 - t / 9) + co;
        *reinterpret_cast<uint4 *>(wsm + (t % 9) * kJB + kc * 768 + row * 16) =
            *reinterpret_cast<const uint4 *>(A.wt + (t * 16 + co) * 16 + kc * 8);
    }
    if (tid < 16) bsm[tid] = DST == DST_ACT_MASK ? 0.f : A.bias[tid];
    if (SRC != SRC_ACT)
        for (int i = tid; i < G::HPTS; i += tcc::kThreads)
            *reinterpret_cast<uint4 *>(halo + G::PLANE + i * 16) = make_uint4(0u, 0u, 0u, 0u);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    const uint32_t hb = saddr(halo), wb = saddr(wsm), barA = saddr(bar);

    const int tpx = n / kTX, tpy = (n + kTY - 1) / kTY, tpz = n / TZ;
    const long long per = (long long)tpx * tpy * tpz;
    const long long ntiles = per * A.nsys;
    const int q = warp & 3, mh = warp >> 2;
    const int ox = lane & 7, oy = 4 * q + (lane >> 3);   // this thread's tile row 32 q + lane
    uint32_t phase = 0;
    bool alive = true;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int s = (int)(tile / per);
        if (A.active && !A.active[s]) continue;   // uniform over the CTA
        int r = (int)(tile % per);
        const int xt = r % tpx;
        r /= tpx;
        const int yt = r % tpy, zt = r / tpy;
        const int tx = xt * kTX, tz = zt * TZ;
        // the last y tile of a grid with n % 16 == 8 overlaps the one before
        // it; rows below ybeg were written by that tile
        const int ty = min(yt * kTY, n - kTY), ybeg = yt * kTY - ty;
        tcc::stage<SRC, TZ>(A, halo, s, tx - 1, ty - 1, tz - 1);
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            issue_tile<TZ>(tmem, hb, wb);
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                    barA)
                : "memory");
        }
        __syncwarp();
        const bool ok = bar_wait(barA, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) {
            alive = false;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const long long pbase = (long long)s * n * n * n + (tx + ox) + (long long)n * (ty + oy);
        const bool store = oy >= ybeg;
#pragma unroll 1
        for (int mm = 0; mm < TZ / 2; ++mm) {
            const int m = (TZ / 2) * mh + mm;
            uint32_t v[16];
            __syncwarp();
            tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + m * 16, v);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (!store) continue;   // uniform per warp (ybeg is 0 or 8, a warp holds 4 rows)
            const long long p = pbase + (long long)n * n * (tz + m);
            float f[16];
#pragma unroll
            for (int c = 0; c < 16; ++c)
                f[c] = (A.nout_tiles == 1 && c >= 8) ? 0.f : __uint_as_float(v[c]);
            if (DST == DST_FIELD) {
                A.dst_field[p] = A.dst_fac[s] * (double)(f[0] + bsm[0]);
            } else {
                if (DST == DST_ACT_RELU) {
#pragma unroll
                    for (int c = 0; c < 16; ++c) f[c] = fmaxf(f[c] + bsm[c], 0.f);
                } else {
                    const uint4 *mk4 = reinterpret_cast<const uint4 *>(A.mask + p * 16);
                    const uint4 mk[2] = {mk4[0], mk4[1]};
                    const __nv_bfloat162 *mk2 = reinterpret_cast<const __nv_bfloat162 *>(mk);
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        if (!(__low2float(mk2[c]) > 0.f)) f[2 * c] = 0.f;
                        if (!(__high2float(mk2[c]) > 0.f)) f[2 * c + 1] = 0.f;
                    }
                }
                uint32_t o[8];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    __nv_bfloat162 hv = __floats2bfloat162_rn(f[2 * c], f[2 * c + 1]);
                    o[c] = *reinterpret_cast<uint32_t *>(&hv);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(A.dst_act + p * 16);
                dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
                dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    }
    if (!alive && tid == 0) atomicExch(status, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(G::TMEM_COLS)
                     : "memory");
}

// Tile depth of the tensor-core kernel (z-planes per tile).
constexpr int kConvTZ = 8;

int g_sms = 0;
int sm_count() {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 148;
    }
    return g_sms;
}

template <int SRC, int DST>
cudaError_t launch_conv(const ConvArgs &A, int *status, cudaStream_t st) {
    if (A.n >= tcc::kTY) {
        using G = tcc::Geo<kConvTZ>;
        static bool attr = false;   // the dynamic shared memory opt-in, once per instantiation
        if (!attr) {
            cudaError_t e = cudaFuncSetAttribute(conv_tc_kernel<SRC, DST, kConvTZ>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)G::SMEM);
            if (e != cudaSuccess) return e;
            attr = true;
        }
        const long long tiles = (long long)A.nsys * (A.n / tcc::kTX) *
                                ((A.n + tcc::kTY - 1) / tcc::kTY) * (A.n / kConvTZ);
        const long long cap = (long long)G::CTAS * sm_count();
        conv_tc_kernel<SRC, DST, kConvTZ>
            <<<(unsigned)(tiles < cap ? tiles : cap), tcc::kThreads, G::SMEM, st>>>(A, status);
        return cudaGetLastError();
    }
    const int tpa = A.n / kT;
    const long long tiles = (long long)A.nsys * tpa * tpa * tpa;
    const long long grid = tiles < 4LL * sm_count() ? tiles : 4LL * sm_count();
    conv_kernel<SRC, DST><<<(unsigned)grid, kThreads, 0, st>>>(A);
    return cudaGetLastError();
}

int check_common(int n, int nsys) {
    if (n < 8 || n % 8 || nsys < 1) return LIBCONV_EARG;
    return LIBCONV_OK;
}

}  // namespace

extern "C" {

int libconv_cnn_wgrad_parts(int n, int nsys) {
    (void)n; (void)nsys;
    return sm_count();
}

int libconv_cnn_conv(int n, int nsys, int src_kind, int dst_kind, const void *src, const double *src_fac,
                     const double *eps, const void *wt, const float *bias, void *dst,
                     const double *dst_fac, const void *mask, int cout, const int *active,
                     void *stream) {
    if (check_common(n, nsys) || !src || !wt || !dst) return LIBCONV_EARG;
    ConvArgs A{};
    A.n = n;
    A.nsys = nsys;
    A.src_act = (const __nv_bfloat16 *)src;
    A.src_field = (const double *)src;
    A.src_fac = src_fac;
    A.eps = eps;
    A.wt = (const __nv_bfloat16 *)wt;
    A.bias = bias;
    A.dst_act = (__nv_bfloat16 *)dst;
    A.dst_field = (double *)dst;
    A.dst_fac = dst_fac;
    A.mask = (const __nv_bfloat16 *)mask;
    A.nout_tiles = cout > 8 ? 2 : 1;
    A.active = active;
    if ((src_kind != 0 && !src_fac) || (src_kind == 1 && !eps)) return LIBCONV_EARG;
    if ((dst_kind == 0 && !bias) || (dst_kind == 1 && (!dst_fac || !bias)) || (dst_kind == 2 && !mask))
        return LIBCONV_EARG;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = LIBCONV_OK;
    int *status = lcg::device_status(rc);
    if (!status) return rc;
    cudaError_t e;
    if (src_kind == 0 && dst_kind == 0) e = launch_conv<SRC_ACT, DST_ACT_RELU>(A, status, st);
    else if (src_kind == 1 && dst_kind == 0) e = launch_conv<SRC_FIELD_EPS, DST_ACT_RELU>(A, status, st);
    else if (src_kind == 0 && dst_kind == 1) e = launch_conv<SRC_ACT, DST_FIELD>(A, status, st);
    else if (src_kind == 0 && dst_kind == 2) e = launch_conv<SRC_ACT, DST_ACT_MASK>(A, status, st);
    else if (src_kind == 2 && dst_kind == 2) e = launch_conv<SRC_FIELD, DST_ACT_MASK>(A, status, st);
    else return LIBCONV_EARG;
    return e == cudaSuccess ? LIBCONV_OK : LIBCONV_ECUDA;
}

int libconv_cnn_wgrad(int n, int nsys, int g_kind, const void *g, const double *g_fac, int x_kind,
                      const void *x, const double *x_fac, const double *eps, float *part,
                      float *out, void *stream) {
    if (check_common(n, nsys) || !g || !x || !part || !out) return LIBCONV_EARG;
    ConvArgs G{}, X{};
    G.n = X.n = n;
    G.nsys = X.nsys = nsys;
    G.src_act = (const __nv_bfloat16 *)g;
    G.src_field = (const double *)g;
    G.src_fac = g_fac;
    X.src_act = (const __nv_bfloat16 *)x;
    X.src_field = (const double *)x;
    X.src_fac = x_fac;
    X.eps = eps;
    if ((g_kind == 2 && !g_fac) || (x_kind == 1 && (!x_fac || !eps))) return LIBCONV_EARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = sm_count();
    if (g_kind == 0 && x_kind == 0) wgrad_kernel<SRC_ACT, SRC_ACT><<<grid, kThreads, 0, st>>>(G, X, part);
    else if (g_kind == 0 && x_kind == 1) wgrad_kernel<SRC_ACT, SRC_FIELD_EPS><<<grid, kThreads, 0, st>>>(G, X, part);
    else if (g_kind == 2 && x_kind == 0) wgrad_kernel<SRC_FIELD, SRC_ACT><<<grid, kThreads, 0, st>>>(G, X, part);
    else return LIBCONV_EARG;
    const int len = 27 * 256 + 16;
    reduce_parts<<<(len + 255) / 256, 256, 0, st>>>(part, grid, len, out);
    return cudaGetLastError() == cudaSuccess ? LIBCONV_OK : LIBCONV_ECUDA;
}

}  // extern "C"
