// tcgen05 tensor-core sweep, shared by the exact-digit and split-precision
// forms (instantiated in sweep_tc_exact.cu and sweep_tc_split.cu).
//
// One sweep = one banded Toeplitz product per 16-output block:
//   D[line, n] = sum_kk A[line, kk] * B[kk, n]
// A holds the tile's input elements (128 lines x KT elements), B the filter:
// B[kk, n] = f_{c,c'}(kk/NCH - n/NCH) with c = n mod NCH, c' = kk mod NCH, where
// NCH = 1 for a convolution and 2 for the wavelet polyphase pairs (elements are
// (pair, channel), interleaved), so K = 32 or 48 for every filter here.
//
// Scheme SCH_EXACT (FP64-accurate, exact integer arithmetic on FP16 operands)
//   * each line segment of a tile is scaled by the power of two above its
//     largest magnitude to signed 62-bit integers X = x 2^(62-E) (|X| <=
//     2^62, truncated toward zero); X is cut into 8 balanced byte digits
//     d_0 (top) .. d_7 in [-128, 127], X = sum_s d_s 256^(7-s): the bytes
//     of X + 0x8080808080808080 minus 128, exact in FP16;
//   * the filter, with the operator scalar a folded in exactly (128-bit
//     product of the two mantissas), is cut the same way into e_0..e_7;
//   * byte-pair products are at most 2^14 in magnitude and every partial
//     sum over <= 32 products x 8 pairs stays within 2^22; every TMEM
//     accumulator starts at 1.5 * 2^23 (one MMA of a constant tile per output
//     block), so all its values are integers in [2^23, 2^24], where FP32 is
//     exact, and its bits are 0x4B400000 plus the sum;
//   * the 36 pairs of order k = s + t <= 7 are accumulated, one TMEM
//     accumulator per order; the epilogue recombines
//     Y = sum_k Acc_k 2^(46-8k) in int64 (the orders 6-7 rounded to an
//     integer first), converts once and rescales the exponent.
//   Dropped orders (k >= 8) weigh below 2^-70 of the product of the line and
//   filter scales; the data truncation (2^-62 of the line scale) and the
//   final roundings stay below the rounding of an FP64 FMA chain.
//   Lines never share a scale; a line segment holding an Inf or NaN gives
//   NaN on that tile row.
//
// Split-precision schemes (FP32-class accuracy, reported per operator)
//   * every element is rounded to FP32 (magnitudes outside the normal float
//     range flush to zero / infinity), every filter tap times a likewise;
//   * SCH_BF16X3: three bfloat16 terms x = x0 + x1 + x2 (exact split of the
//     24-bit value), the 6 products of order <= 2, kind::f16 with BF16 inputs;
//   * SCH_TF32X3: two tf32 terms x = hi + lo (about 23 bits, both rounded to
//     nearest), the 3 products hi.hi + hi.lo + lo.hi, kind::tf32 (4-byte
//     elements, K = 8 per MMA);
//   * one FP32 accumulator per output: relative error near 1e-7.
//
// Persistent, warp-specialised CTA (one per SM), 512 threads at <= 128
// registers, one A buffer used as a ring of three chunk pairs (input elements
// [0, 32), [32, 64), [64, KT)) and two TMEM accumulator halves (output blocks
// 0-1, which read pairs 0-1, and blocks 2-3, which read pairs 1-2):
//   warps 0-7  producers: thread = (row, half of every pair); exact scheme:
//              largest exponent of the row, then its byte digits; split
//              schemes: bfloat16 / tf32 terms; coalesced or vector loads.  The
//              pairs of a tile are written in order, pair 0 as soon as the
//              previous tile's half-0 MMAs completed, pairs 1-2 once both
//              halves' did, so the next tile's production overlaps the MMAs;
//   warps 8-15 epilogue: group 0 (warps 8-11) owns TMEM half 0, group 1
//              (12-15) half 1.  The group's first warp issues its half's MMAs
//              (lane 0, fully unrolled, precomputed descriptors) once the
//              pairs they read are written, then the group drains the half:
//              thread = TMEM lane = tile row; TMEM -> FP64 -> global.
// Every hand-off is an mbarrier whose phase can never run two phases ahead of
// its waiter; every wait gives up after ~2 s of SM clock (status word set,
// TMEM freed, kernel returns).  In single-sweep launches every role skips the
// tiles of an array whose S0.active flag is 0 (flags fixed for the launch), so
// the roles still meet on the same tiles and count only those.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "lcg_sweep.cuh"
#include "lcg_tc.cuh"

namespace lcg {
namespace tck {

constexpr int kM = 128;          // lines per tile (MMA M)
constexpr int kQE = 64;          // output elements per tile
constexpr int kNB = kQE / 16;    // 16-element output blocks per tile
constexpr int kThreads = 512;    // 8 producer warps + 8 epilogue warps
constexpr int kProducers = 256;
constexpr long long kWaitCycles = 4000000000LL;

template <int KIND, int NT, int SCH> struct Geom {
    static constexpr int NCH = KIND == KCONV ? 1 : 2;            // elements per position
    static constexpr int PROD = NCH * NT;                        // products per output
    static constexpr int KB = ((NCH * (16 / NCH + NT - 1)) + 15) / 16 * 16;   // K per block
    static constexpr int KT = 16 * (kNB - 1) + KB;               // input elements per tile
    static constexpr int QP = kQE / NCH;                         // output positions per tile
    static constexpr int ESZ = SCH == SCH_TF32X3 ? 4 : 2;         // operand element bytes
    static constexpr int CE = 16 / ESZ;                          // elements per core-matrix row
    static constexpr int MK = 32 / ESZ;                          // K of one MMA
    static constexpr int ND = SCH == SCH_EXACT ? 8 : SCH == SCH_BF16X3 ? 3 : 2;
    static constexpr int ORD = ND;                               // order accumulators per block
    // operand planes interleaved along K: the exact scheme keeps its digit
    // planes in pairs (K index = 2 * element + plane within the pair), so one
    // byte permute builds both FP16 digits of an element; split schemes one
    // plane per slice
    static constexpr int PL = SCH == SCH_EXACT ? 2 : 1;
    static constexpr int NS = ND / PL;                           // A slices (MMAs per K step)
    static constexpr int BN = 16 * ORD;                          // rows of the stacked filter
    static constexpr int LBO_B = BN * 16;                        // its K-direction chunk stride
    static constexpr int A_SLICE = kM * KT * PL * ESZ;
    static constexpr int A_BYTES = NS * A_SLICE;
    static constexpr int KBP = KB * PL;                          // K of a block window
    static constexpr int B_BYTES = BN * KBP * ESZ;
    // exact scheme: a 128 x 16 FP16 tile holding 2048 at K = 0, 1, 2 of every
    // row; as both operands of an N = 128 MMA it sets an output block's eight
    // order accumulators to 3 * 2048^2 = 1.5 * 2^23
    static constexpr int Z_BYTES = SCH == SCH_EXACT ? kM * 16 * 2 : 0;
    static constexpr int AUX = 1024 + 3 * 4 * kM + 2 * 4 * 32 * 4;   // barriers, slots, row exponents,
                                                                 // next-sweep column maxima
    static constexpr int SMEM = A_BYTES + B_BYTES + Z_BYTES + AUX + 1024;
    static constexpr int HALF_COLS = 2 * ORD * 16;               // one TMEM half (2 blocks)
    static constexpr uint32_t TMEM_COLS = 2 * HALF_COLS <= 32 ? 32 : 2 * HALF_COLS <= 64 ? 64 : 2 * HALF_COLS <= 128 ? 128 : 2 * HALF_COLS <= 256 ? 256 : 512;
    static_assert(2 * HALF_COLS <= 512, "TMEM columns");
    static_assert(ND % PL == 0, "plane slices");
    static_assert(SMEM <= 232448, "shared memory");
    // Instruction descriptor (kind::f16 / kind::tf32): D F32; A and B F16
    // (exact), BF16 or TF32 (formats 0, 1, 2); both K-major; M = 128; N is
    // added per MMA (idesc()).
    static constexpr uint32_t FMT = SCH == SCH_EXACT ? 0u : SCH == SCH_BF16X3 ? 1u : 2u;
    static constexpr uint32_t IDESC0 = (1u << 4) | (FMT << 7) | (FMT << 10) |
                                       ((uint32_t)(kM >> 4) << 24);
    static constexpr uint32_t idesc(int n) { return IDESC0 | ((uint32_t)(n >> 3) << 17); }
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

template <bool TF32>
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t IDESC,
                                    uint32_t accum) {
    if (TF32)
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
            "l"(a), "l"(b), "r"(IDESC), "r"(accum)
            : "memory");
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
            "l"(a), "l"(b), "r"(IDESC), "r"(accum)
            : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void bar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void bar_arrive(uint32_t bar) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(bar)
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

// Bounded wait for the phase of the given parity; false after ~2 s.  Between
// polls the warp sleeps briefly so waiting warps leave the issue slots to the
// working ones.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    if (bar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (!bar_try(bar, parity)) {
        __nanosleep(128);
        if (clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
}

// 32 bytes from global memory (a 32-byte aligned address) in one load.
__device__ __forceinline__ void ld256(const long long *p, long long &a, long long &b, long long &c,
                                      long long &d) {
    asm("ld.global.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p));
}

// 32 bytes to global memory (a 32-byte aligned address) in one store.
__device__ __forceinline__ void st256(double *p, double a, double b, double c, double d) {
    asm volatile("st.global.v4.u64 [%0], {%1, %2, %3, %4};" ::"l"(p), "l"(__double_as_longlong(a)),
                 "l"(__double_as_longlong(b)), "l"(__double_as_longlong(c)), "l"(__double_as_longlong(d))
                 : "memory");
}

__device__ __forceinline__ int imod(int a, int n) {
    int r = a % n;
    return r < 0 ? r + n : r;
}

// Y * 2^se as an FP64, Y rounded to 53 bits to nearest-even (the rounding of
// an int64 -> FP64 conversion), built from bits on the integer pipes: the
// conversion instruction runs on the narrow FP64 pipe of this GPU.  ldexp
// when the result is not a normal number.
__device__ __forceinline__ double ll_scaled(long long Y, int se) {
    if (Y == 0) return 0.0;
    const unsigned long long sg = (unsigned long long)Y & 0x8000000000000000ull;
    unsigned long long a = Y < 0 ? 0ull - (unsigned long long)Y : (unsigned long long)Y;
    int e = 63 - __clzll((long long)a);                         // a in [2^e, 2^(e+1))
    if (e <= 52) {
        a <<= (52 - e);
    } else {
        const int sh = e - 52;                                  // 1..10
        const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        a >>= sh;
        if (rem > half || (rem == half && (a & 1ull))) ++a;
        if (a >> 53) { a >>= 1; ++e; }
    }
    const int be = e + 1023 + se;
    const unsigned long long m = a & 0xFFFFFFFFFFFFFull;
    if (be >= 1 && be <= 2046)
        return __longlong_as_double((long long)(sg | ((unsigned long long)be << 52) | m));
    return ldexp(__longlong_as_double((long long)(sg | (1075ull << 52) | m)), e - 52 + se);
}

// The same conversion without branches, for the common case: `bad` records
// a subnormal-or-infinite result exponent (the caller then redoes the
// conversion with ll_scaled).  |Y| is normalised so its leading one is bit
// 63; the 11 bits below the 53-bit mantissa and its last bit give
// round-to-nearest-even (an increment exactly when low + lsb + 0x3FF carries
// into bit 11), and a carry out of the mantissa moves into the exponent field.
__device__ __forceinline__ double ll_scaled_fast(long long Y, int se, bool &bad) {
    const unsigned long long u = (unsigned long long)Y;
    const unsigned long long s = (unsigned long long)(Y >> 63);
    const unsigned long long a = (u ^ s) - s;                    // |Y|
    const int lz = __clzll((long long)a);                        // 64 when Y == 0
    const unsigned long long nrm = a << (lz & 63);
    const unsigned long long mant = nrm >> 11;                   // leading one at bit 52
    const uint32_t nl = (uint32_t)nrm;
    const uint32_t inc = ((nl & 0x7FFu) + ((nl >> 11) & 1u) + 0x3FFu) >> 11;
    const int be = 1086 - lz + se;                               // exponent field
    bad |= (unsigned)(be - 1) > 2045u;
    const unsigned long long bits = (u & 0x8000000000000000ull) +
                                    (((unsigned long long)(be - 1) << 52) + mant + inc);
    return Y == 0 ? 0.0 : __longlong_as_double((long long)bits);
}

// Y = sum_k Acc_k 2^(46 - 8k) over the 8 order accumulators of one output,
// from their biased bits b_k = Acc_k + 0x4B400000 (the bits of an FP32
// accumulator that started at 1.5 * 2^23, |Acc_k| <= 2^22): orders 0-5 by
// Horner modulo 2^64 (three 32x32+64 multiply-adds for the low terms, a
// 32-bit add into the high word for the two top terms), orders 6-7 as the
// nearest integer of Acc_6 / 4 + Acc_7 / 1024 (one 32-bit multiply-add and
// an arithmetic shift, exact because that sum fits in 31 bits), then the
// bias of every term removed by one 64-bit constant.  The wrap-around is
// exact because the true sum fits in 62 bits.
template <int ORD>
__device__ __forceinline__ long long horner_bal(const uint32_t (&b)[ORD]) {
    static_assert(ORD == 8, "eight order accumulators");
    constexpr unsigned long long kW = (1ull << 46) + (1ull << 38) + (1ull << 30) + (1ull << 22) +
                                      (1ull << 14) + (1ull << 6);
    constexpr unsigned long long kBias = 0x4B400000ull * kW;
    unsigned long long v = (unsigned long long)b[5] << 6;
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(v) : "r"(b[4]), "r"(16384u), "l"(v));
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(v) : "r"(b[3]), "r"(4194304u), "l"(v));
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(v) : "r"(b[2]), "r"(1073741824u), "l"(v));
    v += (unsigned long long)(b[1] * 64u + b[0] * 16384u) << 32;
    // (Acc_6 * 256 + Acc_7 + 512) >> 10, the biases folded into one constant
    const int lo = (int)(b[6] * 256u + b[7] + (512u - 257u * 0x4B400000u)) >> 10;
    return (long long)(v + (unsigned long long)(long long)lo + (0ull - kBias));
}

// FP32 bits -> FP64 value, integer only (normal, zero, subnormal flushed, inf/nan).
__device__ __forceinline__ double f32_to_f64(uint32_t f) {
    const uint32_t sgn = f >> 31, ex = (f >> 23) & 0xFF, man = f & 0x7FFFFF;
    unsigned long long b = (unsigned long long)sgn << 63;
    if (ex == 0xFF) b |= 0x7FF0000000000000ull | ((unsigned long long)man << 29);
    else if (ex != 0) b |= ((unsigned long long)(ex - 127 + 1023) << 52) | ((unsigned long long)man << 29);
    return __longlong_as_double((long long)b);
}

// Balanced fixed point of one FP64 bit pattern against its line's largest
// exponent field mx (>= 1): U = X + 0x8080808080808080 with X = x 2^(62-E),
// E = mx - 1022, truncated toward zero; integer only, no branch: the 53-bit
// mantissa shifted up by 10 (below 2^63), then right by 10 - sh in [0, 63]
// where X = mant 2^sh (sh <= 9 since the element's exponent is at most mx;
// a shift of 63 leaves 0), sign applied in two's complement, bias added.
__device__ __forceinline__ void fixed_bal(long long bits, int mx, uint32_t &ul, uint32_t &uh) {
    const uint32_t lo = (uint32_t)bits, hi = (uint32_t)((unsigned long long)bits >> 32);
    const int ex = (int)((hi >> 20) & 0x7FF);
    const uint32_t mh = (hi & 0xFFFFFu) | (ex ? 0x100000u : 0u);
    const int c = min(max(mx - max(ex, 1) + 1, 0), 63);         // 10 - sh
    const unsigned long long m10 = (((unsigned long long)mh << 32) | lo) << 10;
    const unsigned long long M = m10 >> c;
    const unsigned long long sg = (unsigned long long)(bits >> 63);   // 0 or all ones
    const unsigned long long U = (M ^ sg) + (sg & 1ull) + 0x8080808080808080ull;
    ul = (uint32_t)U;
    uh = (uint32_t)(U >> 32);
}

// FP16 pair of balanced digits 2p, 2p+1 (bytes 7-2p and 6-2p) of one biased
// fixed point (ul/uh): PRMT takes the two bytes with a 0x64 byte above each,
// which makes them 1024 + byte in FP16, and one HADD2 subtracts 1024 + 128
// (exact).  The lower half is plane 2p (the more significant digit).
__device__ __forceinline__ uint32_t digit_pair_elem(int p, uint32_t ul, uint32_t uh) {
    const uint32_t w = p < 2 ? uh : ul;
    // bytes (3, 2) of the word for even p, (1, 0) for odd p; selector 4 = 0x64
    const uint32_t sel = (p & 1) ? 0x4041u : 0x4243u;
    uint32_t t;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(t) : "r"(w), "r"(0x64646464u), "r"(sel));
    const uint32_t off = 0xE480E480u;                            // (-1152, -1152) in FP16
    __half2 h = __hadd2(*reinterpret_cast<__half2 *>(&t), *reinterpret_cast<const __half2 *>(&off));
    return *reinterpret_cast<uint32_t *>(&h);
}

// FP64 bit pattern -> FP32 bit pattern, rounded to nearest (ties away) on the
// magnitude, integer only; magnitudes outside the normal float range flush to
// a signed zero or overflow to infinity.
__device__ __forceinline__ uint32_t f64_to_f32_bits(long long bits) {
    const uint32_t lo = (uint32_t)bits, hi = (uint32_t)((unsigned long long)bits >> 32);
    const uint32_t sg = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FF) - 1023 + 127;
    if (e <= 0) return sg;
    if (e >= 255) return sg | 0x7F800000u;
    // the rounding carry may step into the exponent (and up to infinity): exact
    return sg | ((((uint32_t)e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29)) + ((lo >> 28) & 1u));
}

// Split of an FP32 value into SPLITS terms (bfloat16: 3 x 8 significant bits,
// an exact split; tf32: 2 x 11 bits), as FP32 bit patterns whose low bits are
// zero.  Each term is the remainder rounded to nearest (half an ulp added to
// the magnitude bits, ties away from zero; a carry steps into the exponent),
// and each remainder is formed exactly in FP32.
template <int SPLITS, uint32_t MASK>
__device__ __forceinline__ void split_f32(uint32_t f, uint32_t (&h)[SPLITS]) {
    constexpr uint32_t HALF = (~MASK + 1u) >> 1;
    uint32_t r = f;
#pragma unroll
    for (int i = 0; i < SPLITS; ++i) {
        h[i] = (r + HALF) & MASK;
        if (i + 1 < SPLITS) r = __float_as_uint(__uint_as_float(r) - __uint_as_float(h[i]));
    }
}

// Issue the MMAs of one TMEM half (output blocks 2h, 2h+1) of a tile.  The
// filter planes t = 0..ORD-1 are stacked along N in one matrix (rows 16t + n),
// and the ORD accumulators of a block (order k = s + t at columns 16k) are
// contiguous in TMEM, so ONE MMA per data plane s covers all its pairs:
// D = columns 16s.. of the block, N = 16 (ORD - s) (a prefix of the stacked
// filter), giving pair (s, t) at order s + t.  The s = 0 MMA of the first K
// step initialises every order (split schemes); in the exact scheme one MMA of
// the constant tile (z_desc, N = 128) first sets all eight orders of the block
// to 1.5 * 2^23 and every data MMA accumulates.  Output block j starts 16
// elements into the A planes; one MMA covers 32 bytes of K (two core
// matrices).  Descriptors are advanced by adding the (16-byte unit) offset to
// the start-address field (addresses < 256 KB never carry out of it).
template <int KIND, int NT, int SCH, int H>
__device__ __forceinline__ void issue_half(uint32_t tmem, uint64_t a_desc0, uint64_t b_desc0,
                                           uint64_t z_desc) {
    using G = Geom<KIND, NT, SCH>;
    constexpr bool TF = SCH == SCH_TF32X3;
    constexpr bool EX = SCH == SCH_EXACT;
    constexpr int NKS = G::KBP / G::MK;
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) {
        const int j = 2 * H + jj;
        const int a_blk = (16 * G::PL / G::CE) * j * 2048;
        if (EX) mma<false>(tmem + (uint32_t)(H * G::HALF_COLS + jj * G::ORD * 16), z_desc, z_desc,
                           G::idesc(16 * G::ORD), 0u);
#pragma unroll
        for (int sl = 0; sl < G::NS; ++sl) {
            const int sd = sl * G::PL;                           // first plane (order) of the slice
            const uint32_t d = tmem + (uint32_t)(H * G::HALF_COLS + (jj * G::ORD + sd) * 16);
            const uint32_t id = G::idesc(16 * (G::ORD - sd));
#pragma unroll
            for (int ks = 0; ks < NKS; ++ks) {
                const uint64_t ad = a_desc0 + (uint64_t)((sl * G::A_SLICE + a_blk + 2 * ks * 2048) >> 4);
                const uint64_t bd = b_desc0 + (uint64_t)((2 * ks * G::LBO_B) >> 4);
                mma<TF>(d, ad, bd, id, (EX || sl > 0 || ks > 0) ? 1u : 0u);
            }
        }
    }
}

// Filter of output channel c, input channel c2 within the flat digit table
// (convolution: 0; wavelets: LE | LO | HE | HO, each NT taps).
template <int KIND>
__device__ __forceinline__ int filter_index(int c, int c2) {
    if (KIND == KCONV) return 0;
    if (KIND == KDEC) return c == 0 ? (c2 == 0 ? 0 : 1) : (c2 == 0 ? 2 : 3);
    return c == 0 ? (c2 == 0 ? 1 : 3) : (c2 == 0 ? 0 : 2);          // KREC
}

// floor(n / d) for n < 2^31 with d's multiplicative inverse (tc_prepare).
__device__ __forceinline__ uint32_t fdiv(uint32_t n, uint32_t m, uint32_t s) {
    return (uint32_t)(((unsigned long long)n * m) >> s);
}

// Where tile `tile` of a launch lives: its sweep, its output chunk `ch`
// along the lines, its block of kM lines `lb` and its array.  Tiles are
// numbered chunk fastest, then line block, then array.  A batched launch
// (BATCH) covers a list of sweeps of the same kind and filter, one per grid
// of a batch of uneven grids, whose tiles are numbered consecutively
// (prefix[i] = first tile of sweep i).
struct TileLoc {
    const Sweep *S;
    int ch;
    uint32_t lb;
    int arr;
};

template <bool BATCH>
__device__ __forceinline__ TileLoc locate(const Sweep &S0, const Sweep *descs,
                                          const long long *prefix, int nsweeps, long long tile) {
    const Sweep *S = &S0;
    uint32_t t = (uint32_t)tile;
    if (BATCH) {
        int lo = 0, hi = nsweeps - 1;                    // last i with prefix[i] <= tile
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (prefix[mid] <= tile) lo = mid;
            else hi = mid - 1;
        }
        S = descs + lo;
        t = (uint32_t)(tile - prefix[lo]);
    }
    const uint32_t q = fdiv(t, S->tdiv_m[0], S->tdiv_s[0]);          // t / chunks
    const uint32_t arr = fdiv(q, S->tdiv_m[1], S->tdiv_s[1]);        // / line blocks
    return {S, (int)(t - q * S->tdiv_d[0]), q - arr * S->tdiv_d[1], (int)arr};
}

// Line g of a sweep as (l, r): g = l + nL r.
__device__ __forceinline__ void line_lr(const Sweep &S, uint32_t g, uint32_t &l, uint32_t &r) {
    r = fdiv(g, S.tdiv_m[2], S.tdiv_s[2]);
    l = g - r * S.tdiv_d[2];
}

template <int KIND, int NT, int SCH, bool BATCH>
__global__ void __launch_bounds__(kThreads, 1)
sweep_tc_kernel(const __grid_constant__ Sweep S0, const __grid_constant__ TcFilter F, int *status,
                const Sweep *__restrict__ descs, const long long *__restrict__ prefix, int nsweeps,
                const int *__restrict__ lineE) {
    using G = Geom<KIND, NT, SCH>;
    constexpr int NCH = G::NCH;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *A = smem;
    uint8_t *B = smem + G::A_BYTES;
    uint8_t *Z = B + G::B_BYTES;                      // exact scheme: accumulator bias tile
    uint8_t *aux = Z + G::Z_BYTES;
    uint64_t *bars = (uint64_t *)aux;                 // 9 barriers (16 slots)
    uint32_t *tslot = (uint32_t *)(aux + 128);
    int *rowE3 = (int *)(aux + 1024);                 // row exponents, by tile index mod 3
    int *colE = (int *)(aux + 1024 + 3 * 4 * kM);     // [group][warp][column]: next-sweep line maxima
    // pfull[p]: chunk pair p of the tile is written (producer arrivals);
    // pfree0: pair 0 may be rewritten (the MMAs of TMEM half 0 completed);
    // pfree12: pairs 1 and 2 may be rewritten (both halves' MMAs completed:
    //          one commit from each issuer);
    // bT_full[h]: TMEM half h holds the tile's accumulators;
    // gsync[h]: the 4 warps of epilogue group h have drained TMEM half h.
    const uint32_t pfull[3] = {saddr(&bars[0]), saddr(&bars[1]), saddr(&bars[2])};
    const uint32_t pfree0 = saddr(&bars[3]), pfree12 = saddr(&bars[4]);
    const uint32_t bT_full[2] = {saddr(&bars[5]), saddr(&bars[6])};
    const uint32_t gsync[2] = {saddr(&bars[7]), saddr(&bars[8])};

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long ntiles = BATCH ? prefix[nsweeps]
                                   : ((long long)S0.nL * S0.nR + kM - 1) / kM *
                                         ((S0.qhi - S0.qlo + G::QP) / G::QP) * S0.narr;
    // window offset of the convolution sweeps (0 in batched launches)
    const int woff = (!BATCH && KIND == KCONV) ? S0.woff : 0;
    const int kneed = NCH * (G::QP + NT - 1) + woff;  // window elements the tile's outputs use

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         saddr(tslot)),
                     "r"(G::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int p = 0; p < 3; ++p) bar_init(pfull[p], kProducers);
        bar_init(pfree0, 1);
        bar_init(pfree12, 2);
        for (int h = 0; h < 2; ++h) {
            bar_init(bT_full[h], 1);
            bar_init(gsync[h], 128);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // Toeplitz filter tiles B_t[n][kk], K-major core matrices
    for (int idx = tid; idx < G::ORD * 16 * G::KBP; idx += kThreads) {
        const int t = idx / (16 * G::KBP), rem = idx % (16 * G::KBP);
        const int n = rem / G::KBP, k2 = rem % G::KBP;
        // K index k2 = element kk, data plane pj within the slice: the pair
        // (slice plane pj, filter digit t - pj) lands on order column t
        const int kk = k2 / G::PL, pj = k2 % G::PL;
        const int ti = kk / NCH - n / NCH - woff;
        const uint32_t v = (ti >= 0 && ti < NT && t >= pj)
                               ? F.dig[t - pj][filter_index<KIND>(n % NCH, kk % NCH) * NT + ti] : 0u;
        const int row = 16 * t + n;                      // stacked filter planes
        uint8_t *b = B + (k2 / G::CE) * G::LBO_B + (row >> 3) * 128 + (row & 7) * 16 +
                     (k2 % G::CE) * G::ESZ;
        if (G::ESZ == 4) *(uint32_t *)b = v;
        else *(unsigned short *)b = (unsigned short)v;
    }
    // bias tile, K-major core matrices like A: (row, k) at (k / 8) * 2048 +
    // (row / 8) * 128 + (row % 8) * 16 + (k % 8) * 2; FP16 2048 = 0x6800
    for (int idx = tid; idx < G::Z_BYTES / 2; idx += kThreads) {
        const int k8 = idx / 1024, rem = idx % 1024, k = rem % 8;
        ((unsigned short *)Z)[idx] = (k8 == 0 && k < 3) ? (unsigned short)0x6800 : (unsigned short)0;
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    bool alive = true;

    const uint64_t a_desc0 = umma_desc(saddr(A), 2048, 128);
    const uint64_t b_desc0 = umma_desc(saddr(B), G::LBO_B, 128);
    const uint64_t z_desc = umma_desc(saddr(Z), 2048, 128);
    if (warp < kProducers / 32) {
        // ============ producers: thread = (row, half of every chunk pair);
        // half-warps cover 16 consecutive rows.  The KT elements of a row are
        // 8-element groups in three chunk pairs (elements [0, 32), [32, 64),
        // [64, KT)); lanes 0-15 take the first half of every pair's groups,
        // lanes 16-31 the second half, and both write the pairs in order, so
        // pair 0 of the next tile (read only by the MMAs of TMEM half 0) is
        // written while the MMAs of half 1 still read pairs 1 and 2.
        constexpr int NG = G::KT / 8;                                 // 10 or 12 groups
        constexpr int NGH = NG / 2;                                   // groups per thread
        constexpr int G2 = (NG - 8) / 2;                              // per thread in pair 2
        static_assert(NG == 10 || NG == 12, "three chunk pairs");
        const int half = lane >> 4;
        const int row = warp * 16 + (lane & 15);
        auto group_of = [&](int c) -> int {          // c-th group of this thread
            return c < 2 ? 2 * half + c : c < 4 ? 4 + 2 * half + (c - 2) : 8 + G2 * half + (c - 4);
        };
        uint32_t it = 0;                                  // tiles processed (inactive arrays skipped)
        for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const TileLoc loc = locate<BATCH>(S0, descs, prefix, nsweeps, tile);
            if (!BATCH && S0.active && !S0.active[loc.arr]) continue;
            const Sweep &S = *loc.S;
            const uint32_t nlines = (uint32_t)S.nL * (uint32_t)S.nR;
            const int plast = S.qhi + S.lowfil + NT - 1;                // last input position used
            const long long in_ext = S.in_ext;
            const int p0 = S.qlo + loc.ch * G::QP + S.lowfil - woff;    // window start position
            const int pstart = S.bc == BC_PERIODIC ? imod(p0, S.n) : 0;
            const bool onewrap = S.n >= G::KT;
            // element kk of the tile -> offset (in elements) in the line, -1 for a zero
            auto off_of = [&](int kk) -> long long {
                const int pp = kk / NCH, c = kk % NCH;
                const int p = p0 + pp;
                if (kk >= kneed || p > plast) return -1;
                int ps;
                if (S.bc == BC_PERIODIC) {
                    if (onewrap) { const int q = pstart + pp; ps = q >= S.n ? q - S.n : q; }
                    else ps = imod(p, S.n);
                } else if (S.bc == BC_SHRINK) {
                    ps = p - S.in_lo;
                } else {
                    if (p < 0 || p >= S.n) return -1;
                    ps = p;
                }
                return KIND == KCONV ? ps : KIND == KDEC ? (long long)c + 2LL * ps : ps + in_ext * c;
            };
            const uint32_t g = loc.lb * kM + row;
            const bool valid = g < nlines;
            uint32_t l = 0, r = 0;
            if (valid) line_lr(S, g, l, r);
            const long long *base = reinterpret_cast<const long long *>(S.x) + (long long)loc.arr * S.x_arr +
                                    l + (long long)S.nL * (in_ext * NCH) * r;
            const long long stride = S.nL;
            const int klim = min(kneed, NCH * (plast - p0 + 1));
            // the 8 elements of group gi.  The group's first cnt elements are
            // used (the same for every row of the tile).  Periodic
            // convolution lines (the common case) take their positions as at
            // most two runs (before and after the wrap): contiguous lines by
            // 32- or 16-byte vectors when the group is one aligned run,
            // strided lines by one pointer stepping the stride.  Other
            // boundaries: one pointer when the group's line offsets are one
            // consecutive run, else element by element.
            auto load8 = [&](int gi, long long (&bits)[8]) {
                const int i0 = gi * 8;
                const int cnt = max(0, min(8, klim - i0));
#pragma unroll
                for (int e = 0; e < 8; ++e) bits[e] = 0ll;
                if (cnt <= 0 || !valid) return;
                if (KIND == KCONV && S.bc == BC_PERIODIC && onewrap) {
                    int ps0 = pstart + i0;                           // < 2n
                    if (ps0 >= S.n) ps0 -= S.n;
                    const int w = S.n - ps0;                         // elements before the wrap
                    if (stride == 1) {
                        const long long *q = base + ps0;
                        if (cnt == 8 && w >= 8) {
                            if ((((uintptr_t)q) & 31) == 0) {
                                ld256(q, bits[0], bits[1], bits[2], bits[3]);
                                ld256(q + 4, bits[4], bits[5], bits[6], bits[7]);
                                return;
                            }
                            if ((((uintptr_t)q) & 15) == 0) {
                                const double2 *v = reinterpret_cast<const double2 *>(q);
#pragma unroll
                                for (int e = 0; e < 4; ++e) {
                                    const double2 t = v[e];
                                    bits[2 * e] = __double_as_longlong(t.x);
                                    bits[2 * e + 1] = __double_as_longlong(t.y);
                                }
                                return;
                            }
                        }
#pragma unroll
                        for (int e = 0; e < 8; ++e)
                            if (e < cnt) bits[e] = e < w ? q[e] : base[e - w];
                    } else {
                        const long long *q = base + (long long)ps0 * stride;
                        if (cnt == 8 && w >= 8) {
#pragma unroll
                            for (int e = 0; e < 8; ++e) {
                                bits[e] = *q;
                                q += stride;
                            }
                        } else {
#pragma unroll
                            for (int e = 0; e < 8; ++e) {
                                if (e == w) q = base;
                                if (e < cnt) bits[e] = *q;
                                q += stride;
                            }
                        }
                    }
                    return;
                }
                if (KIND == KREC && S.bc == BC_PERIODIC && S.n * NCH >= G::KT) {
                    // synthesis input: 4 positions x 2 channels, channel c of
                    // position ps at ps + in_ext c: two runs of 4, read as
                    // vectors on contiguous lines, interleaved into the group
                    int ps0 = pstart + i0 / 2;                       // < 2n
                    if (ps0 >= S.n) ps0 -= S.n;
                    const int np = cnt / 2, w = S.n - ps0;           // positions, before the wrap
                    const long long *qL = base + (long long)ps0 * stride, *qH = qL + in_ext * stride;
                    if (np == 4 && w >= 4) {
                        if (stride == 1 && ((((uintptr_t)qL) | ((uintptr_t)qH)) & 31) == 0) {
                            ld256(qL, bits[0], bits[2], bits[4], bits[6]);
                            ld256(qH, bits[1], bits[3], bits[5], bits[7]);
                        } else {
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                bits[2 * j] = qL[j * stride];
                                bits[2 * j + 1] = qH[j * stride];
                            }
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            if (j >= np) break;
                            int ps = ps0 + j;
                            if (ps >= S.n) ps -= S.n;
                            bits[2 * j] = base[(long long)ps * stride];
                            bits[2 * j + 1] = base[((long long)ps + in_ext) * stride];
                        }
                    }
                    return;
                }
                long long oa = -1;
                if (KIND != KREC) {
                    const long long a0 = off_of(i0);
                    if (a0 >= 0 && off_of(i0 + cnt - 1) == a0 + cnt - 1) oa = a0;
                }
                if (oa >= 0) {
                    const long long *q = base + oa * stride;
                    if (stride == 1 && cnt == 8 && ((((uintptr_t)q) & 31) == 0)) {
                        ld256(q, bits[0], bits[1], bits[2], bits[3]);
                        ld256(q + 4, bits[4], bits[5], bits[6], bits[7]);
                    } else if (stride == 1 && ((((uintptr_t)q) & 15) == 0)) {
                        const double2 *v = reinterpret_cast<const double2 *>(q);
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            if (2 * e + 1 < cnt) {
                                const double2 t = v[e];
                                bits[2 * e] = __double_as_longlong(t.x);
                                bits[2 * e + 1] = __double_as_longlong(t.y);
                            } else if (2 * e < cnt) {
                                bits[2 * e] = q[2 * e];
                            }
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            if (e < cnt) bits[e] = *q;
                            q += stride;
                        }
                    }
                } else {
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const long long o = e < cnt ? off_of(i0 + e) : -1;
                        if (o >= 0) bits[e] = base[o * stride];
                    }
                }
            };
            int mx = 0;
            if (SCH == SCH_EXACT && lineE) {
                // largest exponent field of the line (line_exp_kernel)
                mx = valid ? lineE[S.le_off + (long long)loc.arr * nlines + g] : 0;
            } else if (SCH == SCH_EXACT) {
#pragma unroll
                for (int c0 = 0; c0 < NGH; c0 += 2) {            // 16 loads in flight
                    long long b0[8], b1[8];
                    load8(group_of(c0), b0);
                    if (c0 + 1 < NGH) load8(group_of(c0 + 1), b1);
                    else {
#pragma unroll
                        for (int e = 0; e < 8; ++e) b1[e] = 0ll;
                    }
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        mx = max(mx, max((int)(((unsigned long long)b0[e] >> 52) & 0x7FF),
                                         (int)(((unsigned long long)b1[e] >> 52) & 0x7FF)));
                }
                mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
            }
            const int mxe = max(mx, 1);
            // software pipeline: the next group's loads are in flight while the
            // current group is cut into digits
            long long bits[8], nxt[8];
            load8(group_of(0), bits);
            bool ok = true;
#pragma unroll 1
            for (int c = 0; c < NGH; ++c) {
                if (c + 1 < NGH) load8(group_of(c + 1), nxt);
                // pair 0 rewrites what the previous tile's TMEM-half-0 MMAs read,
                // pairs 1 and 2 what both halves read
                if (it > 0 && (c == 0 || c == 2) && !bar_wait(c == 0 ? pfree0 : pfree12, (it - 1) & 1)) {
                    ok = false;
                    break;
                }
                // 8 elements = 8 PL / CE core-matrix chunks of 2048 bytes (128 rows)
                const int off = group_of(c) * (8 * G::PL / G::CE) * 2048 + (row >> 3) * 128 + (row & 7) * 16;
                if (SCH == SCH_EXACT) {
                    uint32_t ul[8], uh[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) fixed_bal(bits[e], mxe, ul[e], uh[e]);
                    // slice p holds digit planes 2p, 2p+1 = bytes 7-2p, 6-2p of
                    // the biased fixed point: one 16-byte core-matrix row per
                    // 4 elements
#pragma unroll
                    for (int sl = 0; sl < G::NS; ++sl) {
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            uint32_t wds[4];
#pragma unroll
                            for (int w = 0; w < 4; ++w)
                                wds[w] = digit_pair_elem(sl, ul[4 * h + w], uh[4 * h + w]);
                            *(uint4 *)(A + sl * G::A_SLICE + off + h * 2048) = make_uint4(wds[0], wds[1], wds[2], wds[3]);
                        }
                    }
                } else if (SCH == SCH_BF16X3) {
                    uint32_t h[8][3];
#pragma unroll
                    for (int e = 0; e < 8; ++e) split_f32<3, 0xFFFF0000u>(f64_to_f32_bits(bits[e]), h[e]);
#pragma unroll
                    for (int sd = 0; sd < 3; ++sd) {
                        uint32_t wds[4];
#pragma unroll
                        for (int w = 0; w < 4; ++w) wds[w] = (h[2 * w][sd] >> 16) | (h[2 * w + 1][sd] & 0xFFFF0000u);
                        *(uint4 *)(A + sd * G::A_SLICE + off) = make_uint4(wds[0], wds[1], wds[2], wds[3]);
                    }
                } else {
                    uint32_t h[8][2];
#pragma unroll
                    for (int e = 0; e < 8; ++e) split_f32<2, 0xFFFFE000u>(f64_to_f32_bits(bits[e]), h[e]);
#pragma unroll
                    for (int sd = 0; sd < 2; ++sd) {
                        *(uint4 *)(A + sd * G::A_SLICE + off) = make_uint4(h[0][sd], h[1][sd], h[2][sd], h[3][sd]);
                        *(uint4 *)(A + sd * G::A_SLICE + off + 2048) = make_uint4(h[4][sd], h[5][sd], h[6][sd], h[7][sd]);
                    }
                }
#pragma unroll
                for (int e = 0; e < 8; ++e) bits[e] = nxt[e];
                if (c == 1 || c == 3 || c == NGH - 1) {          // last group of a pair
                    if (c == 1 && half == 0) rowE3[(it % 3) * kM + row] = mx == 0x7FF ? 0x7FFFFFFF : mxe - 1022;
                    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                    bar_arrive(pfull[c == 1 ? 0 : c == 3 ? 1 : 2]);
                }
            }
            if (!ok) { alive = false; break; }
            ++it;
        }
    } else {
        // ============ epilogue: warp group hf issues and drains TMEM half hf
        // (output blocks 2hf, 2hf+1); thread = TMEM lane = tile row; 8 outputs
        // per step
        const int ew = warp - kProducers / 32;
        const int lq = ew & 3, hf = ew >> 2;
        const int row = lq * 32 + lane;
        // dot products per array: each epilogue warp owns the slot
        // dot_part[(arr * gridDim.x + blockIdx.x) * 8 + ew] of every array it
        // visits (tiles are array-major, so a CTA meets the arrays in order)
        double dot = 0.0;
        int dot_arr = -1;
        auto flush_dot = [&]() {
            for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
            if (lane == 0) S0.dot_part[((long long)dot_arr * gridDim.x + blockIdx.x) * 8 + ew] = dot;
            dot = 0.0;
        };
        uint32_t it = 0;                                  // tiles processed (inactive arrays skipped)
        for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            if (!BATCH && S0.active && !S0.active[locate<BATCH>(S0, descs, prefix, nsweeps, tile).arr])
                continue;                                 // the producers skip the same tiles
            // the group issues its TMEM half's MMAs for this tile (the half was
            // drained by the group at the end of the previous tile) once the
            // chunk pairs they read are written: half 0 pairs 0-1, half 1 pairs 1-2
            if (!bar_wait(pfull[hf], it & 1) || !bar_wait(pfull[hf + 1], it & 1)) { alive = false; break; }
            if (ew == 4 * hf) {
                if (lane == 0) {
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    if (hf == 0) issue_half<KIND, NT, SCH, 0>(tmem, a_desc0, b_desc0, z_desc);
                    else issue_half<KIND, NT, SCH, 1>(tmem, a_desc0, b_desc0, z_desc);
                    commit(bT_full[hf]);
                    if (hf == 0) commit(pfree0);
                    commit(pfree12);
                }
                __syncwarp();
            }
            if (!bar_wait(bT_full[hf], it & 1)) { alive = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int Er = rowE3[(it % 3) * kM + row];
            const TileLoc loc = locate<BATCH>(S0, descs, prefix, nsweeps, tile);
            const Sweep &S = *loc.S;
            const int arr = loc.arr;
            if (!BATCH && S0.has_dot && arr != dot_arr) {
                if (dot_arr >= 0) flush_dot();
                dot_arr = arr;
            }
            const int qc0 = S.qlo + loc.ch * G::QP;
            const long long out_pext = (long long)S.out_ext * NCH;
            const uint32_t nlines = (uint32_t)S.nL * (uint32_t)S.nR;
            const uint32_t g = loc.lb * kM + row;
            const bool valid = g < nlines;
            uint32_t l32 = 0, r32 = 0;
            if (valid) line_lr(S, g, l32, r32);
            const long long l = l32, rr = r32;
            double *__restrict__ y = S.y + (long long)arr * S.y_arr;
            const double *__restrict__ xa = S.x + (long long)arr * S.x_arr;
            const double *__restrict__ x2 = S.x2 ? S.x2 + (long long)arr * S.x_arr : nullptr;
            // this row's output element (position p, channel c) sits at
            // yrow + yps p + ycs c; its x2 partial at x2row + x2s q; its input
            // at xrow + nL ps (row bases formed once per tile)
            const long long ys = S.transpose ? S.nR : S.nL;
            double *const yrow = S.transpose ? y + rr : y + l + (long long)S.nL * out_pext * rr;
            const long long yps = KIND == KREC ? 2 * ys : ys;
            const long long ycs = KIND == KREC ? ys : ys * S.out_ext;
            const bool grow = S.bc == BC_GROW;
            const double *const x2row = !x2 ? nullptr
                : grow ? (S.transpose ? x2 + rr : x2 + l + (long long)S.nL * S.out_ext * rr)
                       : x2 + l + (long long)S.nL * S.in_ext * rr;
            const long long x2s = grow ? ys : S.nL;
            const int x2lo = grow ? S.out_lo : S.in_lo;
            const double *const xrow = xa + l + (long long)S.nL * S.in_ext * rr;
            const int se = Er + F.ef - 58;
            const bool nanrow = SCH == SCH_EXACT && Er == 0x7FFFFFFF;
            // no dot, a_x or a_y term: every output is its value (plus x2), stored
            const bool lean = !S.has_dot && !S.has_ax && S.ay_mode == 0;
#pragma unroll 1
            for (int step = 0; step < 4; ++step) {             // 2 blocks x 2 x 8 outputs
                const int jj = step >> 1, n0 = (step & 1) * 8;
                const int e0 = 16 * (2 * hf + jj) + n0;         // first output element of the step
                const int q0 = qc0 + e0 / NCH;                  // e0 is a multiple of 8
                const int nv = (S.qhi - q0 + 1) * NCH;          // valid elements of the step
                // the x2 partials first, so their loads overlap the TMEM loads
                double add[8];
                if (KIND == KCONV && x2 && valid) {
                    const double *xp = x2row + x2s * (q0 - x2lo);
#pragma unroll
                    for (int n = 0; n < 8; ++n) {
                        add[n] = n < nv ? *xp : 0.0;
                        xp += x2s;
                    }
                }
                uint32_t acc[G::ORD][8];
#pragma unroll
                for (int k = 0; k < G::ORD; ++k)
                    tmem_ld8(tmem + ((uint32_t)(lq * 32) << 16) +
                                 (uint32_t)(hf * G::HALF_COLS + (jj * G::ORD + k) * 16 + n0),
                             acc[k]);
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (!valid || nv <= 0) continue;
                double *const ystep = yrow + yps * (q0 - S.out_lo);
                // the 8 outputs' values first (independent, branch-free chains;
                // one rare fix-up), then their memory side
                double outv[8];
                if constexpr (SCH == SCH_EXACT) {
                    bool bad = false;
                    long long Y[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        uint32_t bb[G::ORD];              // 0x4B400000 + Acc_k (biased start)
#pragma unroll
                        for (int k = 0; k < G::ORD; ++k) bb[k] = acc[k][i];
                        Y[i] = horner_bal<G::ORD>(bb);
                    }
#pragma unroll
                    for (int i = 0; i < 8; ++i) outv[i] = ll_scaled_fast(Y[i], se, bad);
                    if (bad) {                    // result not a normal number
#pragma unroll
                        for (int i = 0; i < 8; ++i) outv[i] = ll_scaled(Y[i], se);
                    }
                    if (nanrow) {
#pragma unroll
                        for (int i = 0; i < 8; ++i) outv[i] = __longlong_as_double(0x7FF8000000000000LL);
                    }
                } else {                          // sum of the order accumulators
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        float f = __uint_as_float(acc[0][i]);
#pragma unroll
                        for (int k = 1; k < G::ORD; ++k) f += __uint_as_float(acc[k][i]);
                        outv[i] = f32_to_f64(__float_as_uint(f));
                    }
                }
                double *yq = ystep;
                if (lean && nv >= 8) {
                    if (KIND == KCONV && x2) {
#pragma unroll
                        for (int i = 0; i < 8; ++i) outv[i] += add[i];
                    }
                    if (!BATCH && KIND == KCONV && S0.le_next) {
                        // the warp's maximum exponent field of each of the 8 output
                        // columns (every lane is here: run_plan hands off only
                        // whole tiles of valid lines); lane i keeps column i's
                        uint32_t mine = 0;
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const uint32_t ex = (uint32_t)((unsigned long long)__double_as_longlong(outv[i]) >> 52) & 0x7FFu;
                            const uint32_t m = __reduce_max_sync(0xffffffffu, ex);
                            if (lane == i) mine = m;
                        }
                        if (lane < 8) colE[(hf * 4 + lq) * 32 + step * 8 + lane] = (int)mine;
                    }
                    // a contiguous output line takes the step's 8 outputs as two
                    // 32-byte runs: elements 0-7 (convolution; synthesis, whose
                    // channels interleave), or channel 0 and channel 1 (analysis)
                    double *const r1 = KIND == KDEC ? ystep + ycs : ystep + 4;
                    if (ys == 1 && ((((uintptr_t)ystep) | ((uintptr_t)r1)) & 31) == 0) {
                        if (KIND == KDEC) {
                            st256(ystep, outv[0], outv[2], outv[4], outv[6]);
                            st256(r1, outv[1], outv[3], outv[5], outv[7]);
                        } else {
                            st256(ystep, outv[0], outv[1], outv[2], outv[3]);
                            st256(r1, outv[4], outv[5], outv[6], outv[7]);
                        }
                    } else {
#pragma unroll
                        for (int n = 0; n < 8; ++n) {
                            const int c = n % NCH;
                            *(c ? yq + ycs * c : yq) = outv[n];
                            if (c == NCH - 1) yq += yps;
                        }
                    }
                    continue;
                }
#pragma unroll
                for (int n = 0; n < 8; ++n) {
                    const int q = q0 + n / NCH, c = n % NCH;
                    if (n >= nv) break;
                    double out = outv[n];
                    double *const yp = c ? yq + ycs * c : yq;
                    if (KIND == KCONV) {
                        const bool want_dot = !BATCH && S.has_dot;   // batched sweeps have no dot
                        if ((want_dot || S.has_ax) && (!grow || (q >= 0 && q < S.n))) {
                            const int ps = S.bc == BC_PERIODIC ? imod(q, S.n) : q - S.in_lo;
                            const double xq = xrow[(long long)S.nL * ps];
                            if (want_dot) dot = fma(xq, out, dot);
                            if (S.has_ax) out = fma(xq, S.a_x, out);
                        }
                        if (x2) out += add[n];
                    }
                    if (S.ay_mode == 2) out += *yp;
                    else if (S.ay_mode == 1) out = fma(S.a_y, *yp, out);
                    *yp = out;
                    if (c == NCH - 1) yq += yps;
                }
            }
            // the whole group has read TMEM half hf: it may be reissued
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            bar_arrive(gsync[hf]);
            if (!bar_wait(gsync[hf], it & 1)) { alive = false; break; }
            if (!BATCH && KIND == KCONV && S0.le_next && lq == 0) {
                // lane c: output column 32 hf + c; the tile's 128 lines form 128 / n1
                // of the next sweep's lines per column, warps (32 lq) / n1 == k the
                // k-th (the group's other warps wrote colE before the barrier, and
                // write it again only after this warp issues the next tile's MMAs)
                const int n1 = S0.le_n1, per = kM / n1;
                const int q = qc0 + 32 * hf + lane;
                for (int k = 0; k < per; ++k) {
                    int m = 0;
                    for (int w = k * n1 / 32; w < (k + 1) * n1 / 32; ++w) m = max(m, colE[(hf * 4 + w) * 32 + lane]);
                    const long long i2 = (long long)loc.lb * per + k;
                    S0.le_next[(long long)arr * S0.le_next_lines + i2 + (long long)S0.le_n2 * (q - S0.out_lo)] = m;
                }
            }
            ++it;
        }
        if (!BATCH && S0.has_dot && dot_arr >= 0) flush_dot();
    }

    if (!alive) atomicExch(status, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(G::TMEM_COLS)
                     : "memory");
}

template <int KIND, int NT, int SCH, bool BATCH>
cudaError_t set_smem_attr() {
    using G = Geom<KIND, NT, SCH>;
    static bool attr[64] = {};   // the attribute is set once per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !attr[dev]) {
        cudaError_t e = cudaFuncSetAttribute(sweep_tc_kernel<KIND, NT, SCH, BATCH>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) attr[dev] = true;
    }
    return cudaSuccess;
}

template <int KIND, int NT, int SCH>
cudaError_t launch(const Sweep &S_in, const TcFilter &F, int *status, const int *lineE,
                   cudaStream_t st) {
    using G = Geom<KIND, NT, SCH>;
    Sweep S = S_in;
    if (!tc_prepare(S)) return cudaErrorInvalidValue;
    // contiguous periodic lines of a filter whose K blocks leave room: start
    // the window on a 4-element boundary (32-byte aligned groups)
    if (KIND == KCONV && G::KB - 15 - NT >= 3 && S.nL == 1 && S.bc == BC_PERIODIC && S.n % 4 == 0 &&
        S.in_ext % 4 == 0 && S.x_arr % 4 == 0 && (((uintptr_t)S.x) & 31) == 0)
        S.woff = ((S.qlo + S.lowfil) % 4 + 4) % 4;
    cudaError_t e = set_smem_attr<KIND, NT, SCH, false>();
    if (e != cudaSuccess) return e;
    const long long tiles = tile_count_for(S, G::QP);
    const int grid = (int)(tiles < sm_count() ? tiles : sm_count());
    sweep_tc_kernel<KIND, NT, SCH, false><<<grid, kThreads, G::SMEM, st>>>(S, F, status, nullptr,
                                                                           nullptr, 0, lineE);
    return cudaGetLastError();
}

// Batched launch over nsweeps descriptors (device arrays); S0 only carries
// has_dot = 0.  One CTA per SM.  lineE (exact scheme, or null): line
// exponent maxima of every sweep's lines, sweep i's at descs[i].le_off.
template <int KIND, int NT, int SCH>
cudaError_t launch_batch(const Sweep *descs, const long long *prefix, int nsweeps,
                         const TcFilter &F, int *status, const int *lineE, cudaStream_t st) {
    using G = Geom<KIND, NT, SCH>;
    cudaError_t e = set_smem_attr<KIND, NT, SCH, true>();
    if (e != cudaSuccess) return e;
    Sweep S0{};
    sweep_tc_kernel<KIND, NT, SCH, true><<<sm_count(), kThreads, G::SMEM, st>>>(S0, F, status, descs,
                                                                                prefix, nsweeps, lineE);
    return cudaGetLastError();
}

}  // namespace tck
}  // namespace lcg
