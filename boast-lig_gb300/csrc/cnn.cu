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
#include <cuda_bf16.h>
#include <stdint.h>

#include "../../include/libconv_gb300.h"

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
cudaError_t launch_conv(const ConvArgs &A, cudaStream_t st) {
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
    cudaError_t e;
    if (src_kind == 0 && dst_kind == 0) e = launch_conv<SRC_ACT, DST_ACT_RELU>(A, st);
    else if (src_kind == 1 && dst_kind == 0) e = launch_conv<SRC_FIELD_EPS, DST_ACT_RELU>(A, st);
    else if (src_kind == 0 && dst_kind == 1) e = launch_conv<SRC_ACT, DST_FIELD>(A, st);
    else if (src_kind == 0 && dst_kind == 2) e = launch_conv<SRC_ACT, DST_ACT_MASK>(A, st);
    else if (src_kind == 2 && dst_kind == 2) e = launch_conv<SRC_FIELD, DST_ACT_MASK>(A, st);
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
