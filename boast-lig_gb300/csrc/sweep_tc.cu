// FP64-accurate convolution sweep on the tcgen05 tensor cores.
//
// Exact integer arithmetic on FP16 operands:
//   * each line of a 128-line x KT-position tile is scaled by one power of two
//     (the line segment's largest exponent) to integers X with |X| < 2^62, and
//     X is cut into 7 balanced base-512 digits d_0..d_6 (|d| <= 256, exact in
//     FP16).  Lines never share a scale, so a line's result does not depend on
//     the magnitudes of the other lines of its tile; a line segment holding an
//     Inf or NaN yields NaN for the outputs of that tile row;
//   * the filter taps are scaled by the power of two above their largest
//     magnitude and cut the same way into digits e_0..e_6;
//   * every digit-pair product is an integer of magnitude <= 2^16 and every
//     partial sum over <= 29 taps x 7 pairs stays below 2^24, so the FP32
//     accumulation of tcgen05.mma (kind::f16) is exact;
//   * the pairs of order k = s + t <= 5 (21 pairs) and of order 6 (all 7 for
//     the 29-tap filters, whose large alternating taps cancel; the leading
//     (0,6) and (6,0) for the 16-tap MagicFilter) are accumulated in TMEM, one
//     accumulator per order; the epilogue recombines
//     Y = sum_{k<=5} Acc_k 512^(5-k) + Acc_6 / 512 in int64 and scales it back
//     to FP64 together with the operator scalar a.
// The dropped orders weigh <= 2^-63 of the tile scale: the result is at least
// as accurate as the FP64 FMA chain.
//
// The convolution of one 16-output block is a banded Toeplitz product
//   D[line, n] = sum_kk A[line, kk] * B[kk, n],   B[kk, n] = f(kk - n + lowfil)
// with K = 32 (16 taps) or 48 (29 taps); A is a digit plane of the tile,
// addressed at an offset of 16 positions per output block.
#include <cuda_fp16.h>
#include <stdint.h>

#include "lcg_sweep.cuh"
#include "lcg_tc.cuh"

namespace lcg {
namespace {

constexpr int kM = 128;          // lines per tile (MMA M)
constexpr int kQC = 64;          // outputs per tile (4 blocks of N = 16)
constexpr int kNB = kQC / 16;
constexpr int kS = TcFilter::kSlices;   // digits per operand (7)
constexpr int kG = 7;                   // accumulated orders k = 0..6

// Digit pairs (s, t) accumulated, in issue order; order 6 is complete for the
// 29-tap filters and reduced to its two leading pairs for 16 taps.
template <int NT> struct Pairs {
    static constexpr int N = NT > 16 ? 28 : 23;
};
__host__ __device__ constexpr int pair_s(int NT, int i) {
    return i < 21 ? (i < 1 ? 0 : i < 3 ? i - 1 : i < 6 ? i - 3 : i < 10 ? i - 6 : i < 15 ? i - 10 : i - 15)
                  : (NT > 16 ? i - 21 : (i == 21 ? 0 : 6));
}
__host__ __device__ constexpr int pair_k(int NT, int i) {
    return i < 1 ? 0 : i < 3 ? 1 : i < 6 ? 2 : i < 10 ? 3 : i < 15 ? 4 : i < 21 ? 5 : 6;
}
constexpr int kThreads = 256;
constexpr uint32_t kTmemCols = 512;

template <int NT> struct TcGeom {
    static constexpr int KB = ((16 + NT - 1) + 15) / 16 * 16;   // K per output block
    static constexpr int KT = 16 * (kNB - 1) + KB;              // positions per tile
    static constexpr int A_PLANE = kM * KT * 2;                 // bytes per digit plane
    static constexpr int B_PLANE = 16 * KB * 2;
    static constexpr int A_BYTES = kS * A_PLANE;
    static constexpr int B_BYTES = kS * B_PLANE;
    static constexpr int SMEM = A_BYTES + B_BYTES + 256 + 4 * kM + 1024;  // + slots, row exponents, alignment
};

// ---- PTX wrappers ----------------------------------------------------------------
__device__ __forceinline__ uint32_t saddr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    // K-major, no swizzle: start, leading (K-direction) and stride (8-row)
    // byte offsets in 16-byte units; bits 46-47 = 1 (descriptor version).
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: D F32, A/B F16, both K-major, N = 16, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((16u >> 3) << 17) |
                            ((uint32_t)(kM >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
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

__device__ __forceinline__ int imod(int a, int n) {
    int r = a % n;
    return r < 0 ? r + n : r;
}

// Input element of line g at logical processed index p (conv filters), with
// the boundary condition applied; 0 outside the data of a free boundary.
__device__ __forceinline__ double fetch_conv(const Sweep &S, const double *__restrict__ x,
                                             long long g, int p) {
    int pos;
    if (S.bc == BC_PERIODIC) pos = imod(p, S.n);
    else if (S.bc == BC_SHRINK) pos = p - S.in_lo;
    else {
        if (p < 0 || p >= S.n) return 0.0;
        pos = p;
    }
    const long long l = g % S.nL, r = g / S.nL;
    return x[l + (long long)S.nL * ((long long)pos + (long long)S.in_ext * r)];
}

// Balanced base-512 digits of X = round(x 2^(62-E)) (|x| < 2^E, |X| < 2^62).
__device__ __forceinline__ void digits(double x, int E, int (&d)[kS]) {
    const long long bits = __double_as_longlong(x);
    int ex = (int)((bits >> 52) & 0x7FF);
    long long mant = bits & 0xFFFFFFFFFFFFFLL;
    if (ex) mant |= 1LL << 52;
    else ex = 1;
    const int r = E - (ex - 1022) - 9;      // X = mant * 2^-r
    long long X;
    if (r <= 0) X = mant << (-r);
    else if (r >= 63) X = 0;
    else X = (mant + (1LL << (r - 1))) >> r;
    if (bits < 0) X = -X;
#pragma unroll
    for (int s = kS - 1; s >= 1; --s) {
        const long long u = X + 256;
        d[s] = (int)(u & 511) - 256;
        X = u >> 9;
    }
    d[0] = (int)X;
}

template <int NT>
__global__ void __launch_bounds__(kThreads, 1)
sweep_tc_kernel(const Sweep S, const TcFilter F, int *status) {
    using G = TcGeom<NT>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *A = smem;
    uint8_t *B = smem + G::A_BYTES;
    uint64_t *bar = (uint64_t *)(B + G::B_BYTES);
    uint32_t *tslot = (uint32_t *)(bar + 1);
    double *red = (double *)(tslot + 4);   // 8 doubles, 8-byte aligned
    int *rowmax = (int *)(red + 8);        // largest biased exponent of each tile row

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int arr = blockIdx.z;
    const long long nlines = (long long)S.nL * S.nR;
    const long long g0 = (long long)blockIdx.x * kM;
    const int qc0 = S.qlo + blockIdx.y * kQC;
    const int upfil = S.lowfil + NT - 1;
    const int plast = S.qhi + upfil;            // last input index any output needs
    const int kneed = kQC + NT - 1;             // positions the tile's outputs use
    const double *__restrict__ x = S.x + (long long)arr * S.x_arr;
    double *__restrict__ y = S.y + (long long)arr * S.y_arr;
    const double *__restrict__ x2 = S.x2 ? S.x2 + (long long)arr * S.x_arr : nullptr;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         saddr(tslot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    for (int i = tid; i < kM; i += kThreads) rowmax[i] = 0;

    // ---- Toeplitz filter tiles B_t[n][kk] = e_t(kk - n), K-major core matrices
    for (int idx = tid; idx < kS * 16 * G::KB; idx += kThreads) {
        const int t = idx / (16 * G::KB), rem = idx % (16 * G::KB);
        const int n = rem / G::KB, kk = rem % G::KB;
        const int tap = kk - n;
        const unsigned short v = (tap >= 0 && tap < NT) ? F.dig[t][tap] : (unsigned short)0;
        *(unsigned short *)(B + t * G::B_PLANE + (kk >> 3) * 256 + (n >> 3) * 128 + (n & 7) * 16 +
                            (kk & 7) * 2) = v;
    }
    __syncthreads();

    // ---- pass 1: largest exponent of each line segment (a thread always owns
    // the same row: row = tid % 128)
    constexpr int kChunks = G::KT / 8;
    int mx = 0;
    for (int id = tid; id < kM * kChunks; id += kThreads) {
        const int row = id % kM, chunk = id / kM;
        const long long g = g0 + row;
        if (g >= nlines) continue;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int kk = chunk * 8 + e;
            const int p = qc0 + S.lowfil + kk;
            if (kk < kneed && p <= plast) {
                const double v = fetch_conv(S, x, g, p);
                const int ex = (int)((__double_as_longlong(v) >> 52) & 0x7FF);
                mx = max(mx, ex);
            }
        }
    }
    atomicMax(&rowmax[tid % kM], mx);
    __syncthreads();
    const int E = (rowmax[tid % kM] ? rowmax[tid % kM] : 1) - 1022;   // |x| < 2^E on the row

    // ---- pass 2: digit planes, 8 positions (one core-matrix row) per task
    for (int id = tid; id < kM * kChunks; id += kThreads) {
        const int row = id % kM, chunk = id / kM;
        const long long g = g0 + row;
        __half h[kS][8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int kk = chunk * 8 + e;
            const int p = qc0 + S.lowfil + kk;
            double v = 0.0;
            if (g < nlines && kk < kneed && p <= plast) v = fetch_conv(S, x, g, p);
            int d[kS];
            digits(v, E, d);
#pragma unroll
            for (int s = 0; s < kS; ++s) h[s][e] = __int2half_rn(d[s]);
        }
        const int off = chunk * 2048 + (row >> 3) * 128 + (row & 7) * 16;
#pragma unroll
        for (int s = 0; s < kS; ++s) {
            uint4 v;
            v.x = (uint32_t)__half_as_ushort(h[s][0]) | ((uint32_t)__half_as_ushort(h[s][1]) << 16);
            v.y = (uint32_t)__half_as_ushort(h[s][2]) | ((uint32_t)__half_as_ushort(h[s][3]) << 16);
            v.z = (uint32_t)__half_as_ushort(h[s][4]) | ((uint32_t)__half_as_ushort(h[s][5]) << 16);
            v.w = (uint32_t)__half_as_ushort(h[s][6]) | ((uint32_t)__half_as_ushort(h[s][7]) << 16);
            *(uint4 *)(A + s * G::A_PLANE + off) = v;
        }
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;

    // ---- MMA issue: one thread; pairs are ordered by k, so the first pair of
    // each order overwrites its accumulator and the others add to it
    if (tid == 0) {
        const uint32_t a0 = saddr(A), b0 = saddr(B);
        for (int j = 0; j < kNB; ++j)
            for (int i = 0; i < Pairs<NT>::N; ++i) {
                const int k = pair_k(NT, i), s = pair_s(NT, i), t = k - s;
                const bool first = i == 0 || pair_k(NT, i - 1) != k;
                const uint32_t d = tmem + (uint32_t)((j * kG + k) * 16);
                for (int ks = 0; ks < G::KB / 16; ++ks) {
                    const uint64_t ad =
                        umma_desc(a0 + s * G::A_PLANE + (2 * j + 2 * ks) * 2048, 2048, 128);
                    const uint64_t bd = umma_desc(b0 + t * G::B_PLANE + 2 * ks * 256, 256, 128);
                    mma_f16(d, ad, bd, (first && ks == 0) ? 0u : 1u);
                }
            }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                saddr(bar))
            : "memory");
    }

    // ---- wait for the accumulators (bounded)
    // give up after ~2 s of SM clock: report through *status, free TMEM, return
    bool ok = false;
    const long long t0 = clock64();
    while (!(ok = mbar_try_wait(saddr(bar), 0)))
        if (clock64() - t0 > 4000000000LL) break;
    if (!ok && lane == 0) atomicExch(status, 1);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

    // ---- epilogue: warp (w%4) owns TMEM lanes 32(w%4).., warps 0-3 / 4-7 split the blocks
    const int lq = warp & 3, jb = warp >> 2;
    const int row = lq * 32 + lane;
    const long long g = g0 + row;
    const long long l = g % S.nL, rr = g / S.nL;
    const long long out_ext = S.out_ext;
    const int rmax = rowmax[row];
    const double scale = rmax == 0x7FF ? __longlong_as_double(0x7FF8000000000000LL)
                                       : (S.has_a ? S.a : 1.0) * ldexp(1.0, (rmax ? rmax : 1) - 1022 + F.ef - 61);
    double dot = 0.0;
    for (int jj = 0; jj < kNB / 2; ++jj) {
        const int j = jb * (kNB / 2) + jj;
        uint32_t acc[kG][16];
#pragma unroll
        for (int k = 0; k < kG; ++k)
            tmem_ld16(tmem + ((uint32_t)(lq * 32) << 16) + (uint32_t)((j * kG + k) * 16), acc[k]);
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (!ok || g >= nlines) continue;
#pragma unroll
        for (int n = 0; n < 16; ++n) {
            const int q = qc0 + 16 * j + n;
            if (q > S.qhi) break;
            long long Y = 0;
#pragma unroll
            for (int k = 0; k < 6; ++k)
                Y += (long long)__float2int_rn(__uint_as_float(acc[k][n])) << (9 * (5 - k));
            Y += ((long long)__float2int_rn(__uint_as_float(acc[6][n])) + 256) >> 9;
            double out = __ll2double_rn(Y) * scale;
            const long long pos = q - S.out_lo;
            const long long yi = S.transpose ? rr + (long long)S.nR * pos
                                             : l + (long long)S.nL * (pos + out_ext * rr);
            if ((S.has_dot || S.has_ax) && (S.bc != BC_GROW || (q >= 0 && q < S.n))) {
                const double xq = fetch_conv(S, x, g, q);
                if (S.has_dot) dot = fma(xq, out, dot);
                if (S.has_ax) out = fma(xq, S.a_x, out);
            }
            if (x2) {
                const long long x2i = S.bc == BC_GROW
                    ? yi : l + (long long)S.nL * ((long long)(q - S.in_lo) + (long long)S.in_ext * rr);
                out += x2[x2i];
            }
            if (S.ay_mode == 2) out += y[yi];
            else if (S.ay_mode == 1) out = fma(S.a_y, y[yi], out);
            y[yi] = out;
        }
    }
    if (S.has_dot) {
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if (lane == 0) red[warp] = dot;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    if (S.has_dot && tid == 0) {
        double s = 0.0;
        for (int i = 0; i < kThreads / 32; ++i) s += red[i];
        const long long b = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        S.dot_part[b] = s;
    }
}

template <int NT>
cudaError_t launch_t(const Sweep &S, const TcFilter &F, int *status, cudaStream_t st) {
    using G = TcGeom<NT>;
    static bool attr[64] = {};   // the attribute is set once per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !attr[dev]) {
        cudaError_t e = cudaFuncSetAttribute(sweep_tc_kernel<NT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) attr[dev] = true;
    }
    const long long nlines = (long long)S.nL * S.nR;
    const int nq = S.qhi - S.qlo + 1;
    dim3 grid((unsigned)((nlines + kM - 1) / kM), (unsigned)((nq + kQC - 1) / kQC), (unsigned)S.narr);
    sweep_tc_kernel<NT><<<grid, kThreads, G::SMEM, st>>>(S, F, status);
    return cudaGetLastError();
}

}  // namespace

bool sweep_tc_supported(const Sweep &S) {
    return S.kind == KCONV && (S.ntaps == 16 || S.ntaps == 29);
}

long long sweep_tc_blocks(const Sweep &S) {
    const long long nlines = (long long)S.nL * S.nR;
    const long long nq = S.qhi - S.qlo + 1;
    return ((nlines + kM - 1) / kM) * ((nq + kQC - 1) / kQC) * S.narr;
}

void tc_filter_digits(const double *taps, int ntaps, TcFilter &F) {
    double m = 0.0;
    for (int i = 0; i < ntaps; ++i) m = fmax(m, fabs(taps[i]));
    int ef = 0;
    frexp(m, &ef);                       // m < 2^ef
    F.ef = ef;
    for (int s = 0; s < TcFilter::kSlices; ++s)
        for (int i = 0; i < TcFilter::kMaxTaps; ++i) F.dig[s][i] = 0;
    for (int i = 0; i < ntaps; ++i) {
        const double v = taps[i];
        long long X = llround(ldexp(fabs(v), 62 - ef));   // exact: 53-bit taps shifted up
        if (v < 0) X = -X;
        int d[TcFilter::kSlices];
        for (int s = TcFilter::kSlices - 1; s >= 1; --s) {
            const long long u = X + 256;
            d[s] = (int)(u & 511) - 256;
            X = u >> 9;
        }
        d[0] = (int)X;
        for (int s = 0; s < TcFilter::kSlices; ++s)
            F.dig[s][i] = __half_as_ushort(__int2half_rn(d[s]));
    }
}

cudaError_t launch_sweep_tc(const Sweep &S, const TcFilter &F, int *status, cudaStream_t st) {
    if (S.ntaps == 16) return launch_t<16>(S, F, status, st);
    if (S.ntaps == 29) return launch_t<29>(S, F, status, st);
    return cudaErrorInvalidValue;
}

}  // namespace lcg
