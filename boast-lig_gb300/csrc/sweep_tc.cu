// Host side of the tensor-core sweeps: filter operand planes, support test,
// grid size and scheme dispatch.  The kernel itself is tc_kernel.cuh.
#include <cuda_fp16.h>
#include <math.h>
#include <string.h>

#include "lcg_tc.cuh"

namespace lcg {
namespace tck {

namespace {
int g_sms[64] = {0};
}

int sm_count() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 148;
    if (!g_sms[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_sms[dev] = n > 0 ? n : 148;
    }
    return g_sms[dev];
}

// 128-line x qp-output-position tiles of one sweep (all narr arrays).
long long tile_count_for(const Sweep &S, int qp) {
    const long long nlines = (long long)S.nL * S.nR;
    const long long nq = S.qhi - S.qlo + 1;
    return ((nlines + 127) / 128) * ((nq + qp - 1) / qp) * S.narr;
}

// Largest exponent field over the elements each line of S uses (positions
// 0..plen-1 of every channel; ld padding is not read), one int per line of
// every array.  Contiguous lines (nL == 1): a warp per line, lanes along the
// line; strided lines: a thread per line, consecutive lines in a warp.
__device__ __forceinline__ void line_exp_lines(const Sweep &S, int plen, int *out, long long first,
                                               long long step) {
    const int nchan = S.kind == KCONV ? 1 : 2;
    const long long nlines = (long long)S.nL * S.nR, total = nlines * S.narr;
    const long long pext = (long long)S.in_ext * nchan;
    auto offset = [&](int e) -> long long {          // element e of the used run
        if (S.kind == KCONV || S.kind == KDEC) return e;   // interleaved pairs: contiguous
        return e < plen ? e : (long long)(e - plen) + S.in_ext;   // blocked channels
    };
    const long long *xb = reinterpret_cast<const long long *>(S.x);
    const int count = plen * nchan;
    if (S.nL == 1) {
        const int lane = threadIdx.x & 31;
        for (long long w = first >> 5; w < total; w += step >> 5) {
            const long long arr = w / nlines, r = w % nlines;
            const long long *base = xb + arr * S.x_arr + pext * r;
            int mx = 0;
            for (int e = lane; e < count; e += 32)
                mx = max(mx, (int)(((unsigned long long)base[offset(e)] >> 52) & 0x7FF));
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            if (lane == 0) out[w] = mx;
        }
    } else {
        for (long long t = first; t < total; t += step) {
            const long long arr = t / nlines, g = t % nlines;
            const long long l = g % S.nL, r = g / S.nL;
            const long long *base = xb + arr * S.x_arr + l + (long long)S.nL * pext * r;
            int mx = 0;
            for (int e = 0; e < count; ++e)
                mx = max(mx, (int)(((unsigned long long)base[offset(e) * S.nL] >> 52) & 0x7FF));
            out[t] = mx;
        }
    }
}

__global__ void line_exp_kernel(const Sweep S, int plen, int *out) {
    line_exp_lines(S, plen, out, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                   (long long)gridDim.x * blockDim.x);
}

// Input positions 0..plen-1 a sweep's outputs read along its line: the whole
// line, or the used part of a shrink input.
__host__ __device__ __forceinline__ int line_exp_plen(const Sweep &S) {
    const int up = S.lowfil + S.ntaps - 1;
    return S.bc == BC_SHRINK ? S.qhi + up - S.in_lo + 1 : S.n;
}

// The same maxima for a batch of sweeps: blockIdx.y = sweep, its lines'
// maxima written from out + le_off on.
__global__ void line_exp_batch_kernel(const Sweep *__restrict__ descs, int *out) {
    const Sweep &S = descs[blockIdx.y];
    line_exp_lines(S, line_exp_plen(S), out + S.le_off,
                   (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// Per-line exponent maxima of one n0 x n1 x n2 grid (narr of them, back to
// back) along all three axes in one read: e0[i1 + n1 (i2 + n2 a)] over i0,
// e1[i0 + n0 (i2 + n2 a)] over i1, e2[i0 + n0 (i1 + n1 a)] over i2 -- the
// line orders of the three non-rotating sweeps of the grid.  Block: 32 i0 x
// 8 i1 threads over one segment of i2 (blockIdx.z = a nseg + segment), in
// chunks of 8 planes (the next chunk's 8 loads in flight while one chunk is
// reduced).  e2 is a thread's own maximum; each chunk is staged in shared
// memory (rows padded to 33 words, so the row and the column reads below are
// free of bank conflicts), where 4 threads per (plane, i1) row reduce the 32
// i0 values for e0 and one thread per (plane, i0) column the 8 i1 values for
// e1.  Partial maxima are
// combined across blocks with atomicMax (e0, e1 and, with several segments,
// e2 zeroed first).
constexpr int kExpChunk = 8;
__global__ void __launch_bounds__(256)
line_exp3_kernel(const double *__restrict__ x, int n0, int n1, int n2, int nseg,
                 int *__restrict__ e0, int *__restrict__ e1, int *__restrict__ e2,
                 const int *__restrict__ active) {
    __shared__ int ys[kExpChunk][8][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i0 = blockIdx.x * 32 + tx, i1 = blockIdx.y * 8 + ty;
    const long long a = blockIdx.z / nseg;
    if (active && !active[a]) return;                   // grid skipped (uniform over the block)
    const int seg = blockIdx.z % nseg, seglen = (n2 + nseg - 1) / nseg;
    const int zb = seg * seglen, ze = min(n2, zb + seglen);
    const bool valid = i0 < n0 && i1 < n1;
    const long long plane = (long long)n0 * n1;
    const unsigned long long *xa =
        reinterpret_cast<const unsigned long long *>(x) + a * plane * n2 + i0 + (long long)n0 * i1;
    // e1 reader: column (c1, tx) of the chunk; e0 reader: quarter q0 of row (c0r, r0)
    const int c1 = ty, row = threadIdx.x >> 2, q0 = threadIdx.x & 3;
    const int c0r = row >> 3, r0 = row & 7;
    const int i1r = blockIdx.y * 8 + r0;
    int zmax = 0;
    // the next chunk's loads are in flight while this chunk is reduced
    unsigned long long raw[kExpChunk];
#pragma unroll
    for (int c = 0; c < kExpChunk; ++c) raw[c] = (valid && zb + c < ze) ? xa[plane * (zb + c)] : 0ull;
    for (int c0 = zb; c0 < ze; c0 += kExpChunk) {
        int e[kExpChunk];
#pragma unroll
        for (int c = 0; c < kExpChunk; ++c) e[c] = (int)((raw[c] >> 52) & 0x7FF);
        const int c1n = c0 + kExpChunk;
#pragma unroll
        for (int c = 0; c < kExpChunk; ++c) raw[c] = (valid && c1n + c < ze) ? xa[plane * (c1n + c)] : 0ull;
#pragma unroll
        for (int c = 0; c < kExpChunk; ++c) {
            zmax = max(zmax, e[c]);
            ys[c][ty][tx] = e[c];
        }
        __syncthreads();
        if (c0 + c1 < ze && i0 < n0) {
            int m = ys[c1][0][tx];
#pragma unroll
            for (int r = 1; r < 8; ++r) m = max(m, ys[c1][r][tx]);
            atomicMax(e1 + i0 + (long long)n0 * (c0 + c1 + (long long)n2 * a), m);
        }
        {
            int m = ys[c0r][r0][8 * q0];
#pragma unroll
            for (int k = 1; k < 8; ++k) m = max(m, ys[c0r][r0][8 * q0 + k]);
            m = max(m, __shfl_xor_sync(0xffffffffu, m, 1));
            m = max(m, __shfl_xor_sync(0xffffffffu, m, 2));
            if (q0 == 0 && c0 + c0r < ze && i1r < n1)
                atomicMax(e0 + i1r + (long long)n1 * (c0 + c0r + (long long)n2 * a), m);
        }
        __syncthreads();
    }
    if (valid) {
        int *const p = e2 + i0 + (long long)n0 * (i1 + (long long)n1 * a);
        if (nseg == 1) *p = zmax;
        else atomicMax(p, zmax);
    }
}

}  // namespace tck

constexpr int kExpChunkHost = tck::kExpChunk;

long long sweep_tc_lines(const Sweep &S) { return (long long)S.nL * S.nR * S.narr; }

cudaError_t launch_line_exp3(const double *x, int n0, int n1, int n2, int narr, int *e0, int *e1,
                             int *e2, cudaStream_t st, const int *active) {
    if (n0 < 1 || n1 < 1 || n2 < 1 || narr < 1 || narr > 65535) return cudaErrorInvalidValue;
    const long long gx = (n0 + 31) / 32, gy = (n1 + 7) / 8;
    // segments of i2 so that a few grids still give the GPU about 8 blocks per SM
    const long long want = 8LL * tck::sm_count();
    long long nseg = (want + gx * gy * narr - 1) / (gx * gy * narr);
    const long long most = (n2 + kExpChunkHost - 1) / kExpChunkHost;
    if (nseg > most) nseg = most;
    if (nseg > 65535 / narr) nseg = 65535 / narr;
    if (nseg < 1) nseg = 1;
    cudaError_t e = cudaMemsetAsync(e0, 0, (size_t)n1 * n2 * narr * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(e1, 0, (size_t)n0 * n2 * narr * sizeof(int), st);
    if (e == cudaSuccess && nseg > 1)
        e = cudaMemsetAsync(e2, 0, (size_t)n0 * n1 * narr * sizeof(int), st);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)(narr * nseg));
    tck::line_exp3_kernel<<<grid, 256, 0, st>>>(x, n0, n1, n2, (int)nseg, e0, e1, e2, active);
    return cudaGetLastError();
}

// Divisor d with its inverse for n < 2^31: s = 31 + ceil(log2 d),
// m = ceil(2^s / d) < 2^32, floor(n / d) = (n m) >> s (the error term
// n (m - 2^s / d) / 2^s stays below 1 / d).
static void fast_div(unsigned int d, unsigned int &dd, unsigned int &m, unsigned int &s) {
    unsigned int l = 0;
    while ((1ull << l) < d) ++l;
    dd = d;
    s = 31 + l;
    m = (unsigned int)(((1ull << s) + d - 1) / d);
}

bool tc_prepare(Sweep &S) {
    const int qp = S.kind == KCONV ? 64 : 32;
    const long long nlines = (long long)S.nL * S.nR;
    const long long nch = (S.qhi - S.qlo + qp) / qp, nlb = (nlines + 127) / 128;
    if (nlines < 1 || nlines >= (1LL << 31) || nch * nlb * S.narr >= (1LL << 31)) return false;
    fast_div((unsigned int)nch, S.tdiv_d[0], S.tdiv_m[0], S.tdiv_s[0]);
    fast_div((unsigned int)nlb, S.tdiv_d[1], S.tdiv_m[1], S.tdiv_s[1]);
    fast_div((unsigned int)S.nL, S.tdiv_d[2], S.tdiv_m[2], S.tdiv_s[2]);
    return true;
}

bool sweep_tc_supported(const Sweep &S) {
    if (S.kind == KCONV) return S.ntaps == 16 || S.ntaps == 17 || S.ntaps == 29;
    return (S.kind == KDEC || S.kind == KREC) && (S.ntaps == 8 || S.ntaps == 16);
}

long long sweep_tc_blocks(const Sweep &S) {
    const long long tiles = tck::tile_count_for(S, S.kind == KCONV ? 64 : 32);
    const int sms = tck::sm_count();
    return tiles < sms ? tiles : sms;
}

// Filter digits with the operator scalar folded in exactly: a*f is formed as
// the 106-bit product of the two mantissas, then rounded once to the signed
// fixed point F = a f 2^(62 - ef), |F| <= 2^62 (ef: power of two above the
// largest |a f| of the whole flat filter, so every channel pair shares one
// scale; raised further while the sum of |a f| reaches 8 * 2^ef, which keeps
// the kernel's recombined 64-bit result below 2^61).  F is cut into 8
// balanced byte digits e_0 (top) .. e_7 in [-128, 127]:
// F = sum_t e_t 256^(7-t), the bytes of F + 0x8080808080808080 minus 128.
void tc_filter_digits(const double *taps, int ntaps, double a, TcFilter &F) {
    memset(&F, 0, sizeof(F));
    int ea = 0;
    const double fa = frexp(fabs(a), &ea);                          // |a| = fa 2^ea
    const unsigned long long ma = (unsigned long long)ldexp(fa, 53);  // 53-bit integer
    unsigned __int128 prod[TcFilter::kMaxTaps];
    int ep[TcFilter::kMaxTaps];
    int ef = -100000;
    double sum = 0.0;
    for (int i = 0; i < ntaps; ++i) {
        int e = 0;
        const double ff = frexp(fabs(taps[i]), &e);
        const unsigned long long mf = (unsigned long long)ldexp(ff, 53);
        prod[i] = (unsigned __int128)ma * mf;
        ep[i] = (ea - 53) + (e - 53);                               // |a f| = prod 2^ep
        sum += fabs(a * taps[i]);
        if (prod[i]) {
            int bl = 0;
            for (unsigned __int128 t = prod[i]; t; t >>= 1) ++bl;
            if (bl + ep[i] > ef) ef = bl + ep[i];                   // |a f| < 2^(bl + ep)
        }
    }
    if (ef == -100000) ef = 0;
    while (sum >= ldexp(8.0, ef)) ++ef;
    F.ef = ef;
    for (int i = 0; i < ntaps; ++i) {
        const int sh = ep[i] + 62 - ef;                             // |F| = prod 2^sh <= 2^62
        const unsigned __int128 v = prod[i];
        unsigned long long M;
        if (sh >= 0) M = (unsigned long long)(v << sh);
        else if (-sh >= 127) M = 0;
        else M = (unsigned long long)((v + ((unsigned __int128)1 << (-sh - 1))) >> (-sh));
        const bool neg = (a < 0) != (taps[i] < 0);
        const unsigned long long X = neg ? 0ull - M : M;           // two's complement
        const unsigned long long U = X + 0x8080808080808080ull;
        for (int t = 0; t < TcFilter::kSlices; ++t) {
            const int digit = (int)((U >> (8 * (7 - t))) & 0xFF) - 128;
            F.dig[t][i] = __half_as_ushort(__int2half_rn(digit));
        }
    }
}

// bfloat16 x 3 or tf32 x 2 terms of the FP32 value of a*f (rounded to
// nearest); each term is its remainder rounded to nearest (ties away from
// zero), each remainder exact in FP32 -- the split the kernel applies to x.
void tc_filter_split(const double *taps, int ntaps, double a, int sch, TcFilter &F) {
    memset(&F, 0, sizeof(F));
    const int nsplit = sch == SCH_BF16X3 ? 3 : 2;
    const uint32_t mask = sch == SCH_BF16X3 ? 0xFFFF0000u : 0xFFFFE000u;
    const uint32_t half = (~mask + 1u) >> 1;
    for (int i = 0; i < ntaps; ++i) {
        float r = (float)(a * taps[i]);
        for (int s = 0; s < nsplit; ++s) {
            uint32_t b;
            memcpy(&b, &r, 4);
            const uint32_t h = (b + half) & mask;
            float hf;
            memcpy(&hf, &h, 4);
            F.dig[s][i] = sch == SCH_BF16X3 ? (h >> 16) : h;
            r = r - hf;
        }
    }
}

long long sweep_tc_tiles(const Sweep &S) {
    return tck::tile_count_for(S, S.kind == KCONV ? 64 : 32);
}

bool sweep_tc_batch_supported(int kind, int ntaps) {
    return kind == KCONV && (ntaps == 16 || ntaps == 29);
}

int line_exp_batch_blocks(long long max_lines, bool contiguous) {
    const long long threads = contiguous ? max_lines * 32 : max_lines;
    const long long want = (threads + 255) / 256;
    return (int)(want < 1 ? 1 : want > 64 ? 64 : want);
}

cudaError_t launch_sweep_tc_batch(int kind, int ntaps, const Sweep *descs, const long long *prefix,
                                  int nsweeps, const TcFilter &F, int sch, int *status,
                                  int *lineE, int exp_blocks, cudaStream_t st) {
    if (sch == SCH_EXACT) {
        if (lineE) {
            if (exp_blocks < 1 || nsweeps > 65535) return cudaErrorInvalidValue;
            tck::line_exp_batch_kernel<<<dim3(exp_blocks, nsweeps), 256, 0, st>>>(descs, lineE);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        return tck::launch_exact_batch(kind, ntaps, descs, prefix, nsweeps, F, status, lineE, st);
    }
    if (sch == SCH_BF16X3) return tck::launch_bf16x3_batch(kind, ntaps, descs, prefix, nsweeps, F, status, st);
    if (sch == SCH_TF32X3) return tck::launch_tf32x3_batch(kind, ntaps, descs, prefix, nsweeps, F, status, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_sweep_tc(const Sweep &S, const TcFilter &F, int sch, int *status, int *lineE,
                            cudaStream_t st, bool lineE_ready) {
    if (sch == SCH_EXACT) {
        // Periodic convolution lines at least one tile window long: the
        // producers load each 8-element group as one or two runs (vectors on
        // contiguous lines, one coalesced load per element across the warp's
        // lines otherwise), and a first pass over those loads gives each tile
        // window's largest exponent at less cost than a pass over the array
        // (32 x 128^3: MagicFilter3D 2.00 -> 1.93 ms; a 1D MagicFilter sweep
        // along axis 1 0.686 -> 0.613 ms).  The window's scale is the line's
        // or a finer one.
        if (lineE && !lineE_ready && S.kind == KCONV && S.bc == BC_PERIODIC &&
            S.n >= tck::exact_conv_window(S.ntaps))
            lineE = nullptr;
        if (lineE && !lineE_ready) {
            const int plen = tck::line_exp_plen(S);
            const long long total = sweep_tc_lines(S);
            const long long threads = S.nL == 1 ? total * 32 : total;
            const long long want = (threads + 255) / 256;
            const int grid = (int)(want < 8LL * tck::sm_count() ? want : 8LL * tck::sm_count());
            tck::line_exp_kernel<<<grid > 0 ? grid : 1, 256, 0, st>>>(S, plen, lineE);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        return tck::launch_exact(S, F, status, lineE, st);
    }
    if (sch == SCH_BF16X3) return tck::launch_bf16x3(S, F, status, nullptr, st);
    if (sch == SCH_TF32X3) return tck::launch_tf32x3(S, F, status, nullptr, st);
    return cudaErrorInvalidValue;
}

}  // namespace lcg
