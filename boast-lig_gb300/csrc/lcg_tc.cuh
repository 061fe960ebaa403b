// Tensor-core (tcgen05) sweeps: operand schemes, filter digits and launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lcg_sweep.cuh"

namespace lcg {

// Operand schemes of the tensor-core sweep.
enum Scheme { SCH_EXACT = 0, SCH_BF16X3 = 1, SCH_TF32X3 = 2 };

// Filter operand planes, one entry per tap of the flat filter (convolution:
// the taps; wavelets: LE | LO | HE | HO), operator scalar folded in.
//   SCH_EXACT: balanced byte digits (in [-128, 127]) of the signed 62-bit
//     fixed point as FP16 bit patterns, a*tap = 2^(ef-62) * sum_s dig[s] 256^(7-s);
//   SCH_BF16X3: three bfloat16 terms (low 16 bits of dig[0..2]);
//   SCH_TF32X3: two tf32 terms (FP32 bit patterns in dig[0..1]).
struct TcFilter {
    static constexpr int kSlices = 8;
    static constexpr int kMaxTaps = 64;
    uint32_t dig[kSlices][kMaxTaps];
    int ef;
};

// Host: operand planes of a * taps[0..ntaps) for scheme sch.
void tc_filter_digits(const double *taps, int ntaps, double a, TcFilter &F);
void tc_filter_split(const double *taps, int ntaps, double a, int sch, TcFilter &F);
bool sweep_tc_supported(const Sweep &S);
// Fill S's tile-index divisors (Sweep::tdiv_*); false when the sweep has
// 2^31 or more tiles or lines (the kernel's 32-bit tile arithmetic).
bool tc_prepare(Sweep &S);
// CTAs of the (non-batched) tensor-core sweep of S.  Its dot partials: 8
// per CTA per array, array-major (sweep_tc_blocks(S) * 8 per array); the
// slots of an array a CTA has no tile of are not written.
long long sweep_tc_blocks(const Sweep &S);
// status (device int) is set non-zero if a tensor-core wait timed out.
// lineE (exact scheme, or null): device scratch of sweep_tc_lines(S) ints; the
// largest exponent of each line is computed into it first (one read of the
// input), so the tensor-core sweep reads its input once.
// lineE_ready: lineE already holds the exponents (launch_line_exp3); no pre-pass.
cudaError_t launch_sweep_tc(const Sweep &S, const TcFilter &F, int sch, int *status, int *lineE,
                            cudaStream_t st, bool lineE_ready = false);
// Line exponents of narr n0 x n1 x n2 grids along all three axes in one read
// of x (e0: n1 n2 narr, e1: n0 n2 narr, e2: n0 n1 narr ints), in the line
// order of the non-rotating sweeps along axes 0, 1, 2.  active (or null):
// grids with active[a] == 0 are skipped (their entries stay 0).
cudaError_t launch_line_exp3(const double *x, int n0, int n1, int n2, int narr, int *e0, int *e1,
                             int *e2, cudaStream_t st, const int *active = nullptr);
long long sweep_tc_lines(const Sweep &S);
// Tiles of one sweep (the unit a batched launch numbers consecutively).
long long sweep_tc_tiles(const Sweep &S);
bool sweep_tc_batch_supported(int kind, int ntaps);
// One persistent launch over nsweeps sweeps (device descriptor array, tile
// prefix sums with prefix[nsweeps] = total) of one kind and filter.  Exact
// scheme with lineE: first one launch computes the largest exponent of every
// line of every sweep into lineE (sweep i's lines from descs[i].le_off on,
// exp_blocks blocks per sweep), so the sweeps read their input once.
cudaError_t launch_sweep_tc_batch(int kind, int ntaps, const Sweep *descs, const long long *prefix,
                                  int nsweeps, const TcFilter &F, int sch, int *status,
                                  int *lineE, int exp_blocks, cudaStream_t st);
// Blocks per sweep of the batched line-exponent pass for sweeps whose largest
// line count (lines x narr) is max_lines, contiguous lines (nL == 1) or not.
int line_exp_batch_blocks(long long max_lines, bool contiguous);

namespace tck {
long long tile_count_for(const Sweep &S, int qp);
// 17-tap convolution (the Poisson finite differences), every scheme; its own
// translation unit.
cudaError_t launch_fd(const Sweep &S, const TcFilter &F, int sch, int *status, const int *lineE,
                      cudaStream_t st);
int sm_count();
// Per-scheme launchers (one translation unit each).
cudaError_t launch_exact(const Sweep &S, const TcFilter &F, int *status, const int *lineE,
                          cudaStream_t st);
cudaError_t launch_bf16x3(const Sweep &S, const TcFilter &F, int *status, const int *lineE,
                          cudaStream_t st);
cudaError_t launch_tf32x3(const Sweep &S, const TcFilter &F, int *status, const int *lineE,
                          cudaStream_t st);
cudaError_t launch_exact_batch(int kind, int ntaps, const Sweep *descs, const long long *prefix,
                               int nsweeps, const TcFilter &F, int *status, const int *lineE,
                               cudaStream_t st);
// Input elements one tile of an exact convolution sweep of ntaps taps reads
// along each line (a huge value for an unsupported filter length).
int exact_conv_window(int ntaps);
cudaError_t launch_bf16x3_batch(int kind, int ntaps, const Sweep *descs, const long long *prefix,
                                int nsweeps, const TcFilter &F, int *status, cudaStream_t st);
cudaError_t launch_tf32x3_batch(int kind, int ntaps, const Sweep *descs, const long long *prefix,
                                int nsweeps, const TcFilter &F, int *status, cudaStream_t st);
}  // namespace tck

}  // namespace lcg
