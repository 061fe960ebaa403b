// Tensor-core sweep, scheme SCH_EXACT: convolution (16, 29 taps) and
// wavelet decompose / recompose (8, 16 polyphase taps) instantiations, and
// the batched convolution forms.
#include "tc_kernel.cuh"

namespace lcg {
namespace tck {

cudaError_t launch_exact(const Sweep &S, const TcFilter &F, int *status, const int *lineE,
                          cudaStream_t st) {
    if (S.kind == KCONV && S.ntaps == 16) return launch<KCONV, 16, SCH_EXACT>(S, F, status, lineE, st);
    if (S.kind == KCONV && S.ntaps == 17) return launch_fd(S, F, SCH_EXACT, status, lineE, st);
    if (S.kind == KCONV && S.ntaps == 29) return launch<KCONV, 29, SCH_EXACT>(S, F, status, lineE, st);
    if (S.kind == KDEC && S.ntaps == 8) return launch<KDEC, 8, SCH_EXACT>(S, F, status, lineE, st);
    if (S.kind == KDEC && S.ntaps == 16) return launch<KDEC, 16, SCH_EXACT>(S, F, status, lineE, st);
    if (S.kind == KREC && S.ntaps == 8) return launch<KREC, 8, SCH_EXACT>(S, F, status, lineE, st);
    if (S.kind == KREC && S.ntaps == 16) return launch<KREC, 16, SCH_EXACT>(S, F, status, lineE, st);
    return cudaErrorInvalidValue;
}

int exact_conv_window(int ntaps) {
    if (ntaps == 16) return Geom<KCONV, 16, SCH_EXACT>::KT;
    if (ntaps == 17) return Geom<KCONV, 17, SCH_EXACT>::KT;
    if (ntaps == 29) return Geom<KCONV, 29, SCH_EXACT>::KT;
    return 1 << 30;
}

cudaError_t launch_exact_batch(int kind, int ntaps, const Sweep *descs, const long long *prefix,
                               int nsweeps, const TcFilter &F, int *status, const int *lineE,
                               cudaStream_t st) {
    if (kind == KCONV && ntaps == 16)
        return launch_batch<KCONV, 16, SCH_EXACT>(descs, prefix, nsweeps, F, status, lineE, st);
    if (kind == KCONV && ntaps == 29)
        return launch_batch<KCONV, 29, SCH_EXACT>(descs, prefix, nsweeps, F, status, lineE, st);
    return cudaErrorInvalidValue;
}

}  // namespace tck
}  // namespace lcg
