// Tensor-core sweep of the 17-tap convolution (the Poisson finite-difference
// stencils of order 2..16, zero padded to 17 taps), for every operand scheme.
#include "tc_kernel.cuh"

namespace lcg {
namespace tck {

cudaError_t launch_fd(const Sweep &S, const TcFilter &F, int sch, int *status, const int *lineE,
                      cudaStream_t st) {
    if (S.kind != KCONV || S.ntaps != 17) return cudaErrorInvalidValue;
    if (sch == SCH_EXACT) return launch<KCONV, 17, SCH_EXACT>(S, F, status, lineE, st);
    if (sch == SCH_BF16X3) return launch<KCONV, 17, SCH_BF16X3>(S, F, status, nullptr, st);
    if (sch == SCH_TF32X3) return launch<KCONV, 17, SCH_TF32X3>(S, F, status, nullptr, st);
    return cudaErrorInvalidValue;
}

}  // namespace tck
}  // namespace lcg
