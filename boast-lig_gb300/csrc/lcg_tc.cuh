// Tensor-core (tcgen05) FP64-accurate sweep: filter digits and launcher.
#pragma once
#include <cuda_runtime.h>

#include "lcg_sweep.cuh"

namespace lcg {

// Signed byte digits of the 64-bit fixed-point filter (operator scalar folded
// in exactly), as FP16 bit patterns: a*tap = 2^(ef-64) * sum_s dig[s] 256^(7-s).
struct TcFilter {
    static constexpr int kSlices = 8;
    static constexpr int kMaxTaps = 32;
    unsigned short dig[kSlices][kMaxTaps];
    int ef;
};

// Host: digits of a * taps[0..ntaps).
void tc_filter_digits(const double *taps, int ntaps, double a, TcFilter &F);
bool sweep_tc_supported(const Sweep &S);
long long sweep_tc_blocks(const Sweep &S);
// status (device int) is set non-zero if a tensor-core wait timed out.
cudaError_t launch_sweep_tc(const Sweep &S, const TcFilter &F, int *status, cudaStream_t st);

}  // namespace lcg
