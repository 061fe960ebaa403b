// Allocation-free form of the 1D kinetic sweep with its energy term
// (d_s0s0_1d_sym8_d2_dotin_dev).
//
// The sweep kernel writes one partial sum of dot_in per thread block and a
// second kernel reduces them; in the regular entry point that scratch buffer
// is allocated by the library.  Here it is a file-scope device array of fixed
// size, so the call performs no device allocation at all: the caller passes
// x, y and dot_in (all device memory) and a stream.
#include <cuda_runtime.h>
#include <mutex>

#include "../../include/libconv_gb300.h"
#include "lcg_sweep.cuh"

namespace lcg {
int kinetic_dotin_sweep(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                        int narr, double a, double a_x, double a_y, Sweep &S);
int report(int code, const char *msg);
int report_cuda(cudaError_t e, const char *what);
}  // namespace lcg

namespace {

// Largest number of per-block partial sums the array holds: 65536 doubles
// (512 KB of device memory, held by every GPU that loads the library).
constexpr long long kMaxPartials = 65536;
__device__ __align__(256) double g_partials[kMaxPartials];

// Device address of g_partials for each device, looked up once per device.
double *g_addr[64] = {nullptr};
std::mutex g_mu;

int partials_address(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lcg::report_cuda(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return lcg::report(LIBCONV_ECUDA, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_partials);
        if (e != cudaSuccess) return lcg::report_cuda(e, "cudaGetSymbolAddress(partials)");
        g_addr[dev] = static_cast<double *>(p);
    }
    *out = g_addr[dev];
    return LIBCONV_OK;
}

}  // namespace

extern "C" int d_s0s0_1d_sym8_d2_dotin_noalloc(int d, int idim, const int *n, int bc,
                                               const int *nx, const int *ny, int narr,
                                               const double *x, double *y, double a,
                                               double a_x, double a_y, double *dot_in,
                                               void *stream) {
    if (!x || !y || !dot_in) return lcg::report(LIBCONV_EARG, "x, y and dot_in must not be null");
    lcg::Sweep S;
    int rc = lcg::kinetic_dotin_sweep(d, idim, n, bc, nx, ny, narr, a, a_x, a_y, S);
    if (rc) return rc;
    const long long nb = lcg::sweep_fp64_blocks(S);
    if (nb > kMaxPartials)
        return lcg::report(LIBCONV_ESIZE,
                           "d_s0s0_1d_sym8_d2_dotin_noalloc: the sweep needs more than 65536 "
                           "partial sums (lines/32 * ceil(outputs/64) * narr); use "
                           "d_s0s0_1d_sym8_d2_dotin_dev");
    double *part = nullptr;
    if ((rc = partials_address(&part))) return rc;
    S.x = x;
    S.y = y;
    S.dot_part = part;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = lcg::launch_sweep_fp64(S, st);
    if (e != cudaSuccess) return lcg::report_cuda(e, "sweep launch");
    e = lcg::launch_dot_reduce(part, nb, dot_in, 0, st);
    if (e != cudaSuccess) return lcg::report_cuda(e, "dot reduction launch");
    return LIBCONV_OK;
}
