// Potential step of the local Hamiltonian (BigDFT/libconv.f90:268-273):
// on the real-space grid psir (the MagicFilter of the orbital),
//   rho  += psir^2            (when rho is given)
//   epot  = sum pot * psir^2  (per-block partial sums, reduced afterwards)
//   psir  = pot * psir
// One pass over psir, pot and rho: an HBM-bound element-wise kernel
// (24 bytes per point, 40 with rho), grid-stride over a grid sized to the
// SM count.  The partial sums are summed in a fixed order (block, then
// launch_dot_reduce), so epot is the same on every run.
#include "lcg_sweep.cuh"

namespace lcg {
namespace {

constexpr int POT_THREADS = 256;

__global__ void __launch_bounds__(POT_THREADS)
potential_kernel(double *__restrict__ psir, const double *__restrict__ pot,
                 double *__restrict__ rho, long long count, double *__restrict__ part) {
    double acc = 0.0;
    const long long stride = (long long)gridDim.x * POT_THREADS;
    for (long long i = (long long)blockIdx.x * POT_THREADS + threadIdx.x; i < count; i += stride) {
        const double p = psir[i];
        const double hp = pot[i] * p;
        if (rho) rho[i] += p * p;
        acc = fma(p, hp, acc);
        psir[i] = hp;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[POT_THREADS / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < POT_THREADS / 32; ++w) s += ws[w];
        part[blockIdx.x] = s;
    }
}

}  // namespace

int potential_blocks(long long count, int sms) {
    long long want = (count + POT_THREADS - 1) / POT_THREADS;
    long long cap = (long long)sms * 8;
    if (want > cap) want = cap;
    return want < 1 ? 1 : (int)want;
}

cudaError_t launch_potential(double *psir, const double *pot, double *rho, long long count,
                             double *part, int nblocks, double *epot, cudaStream_t st) {
    potential_kernel<<<nblocks, POT_THREADS, 0, st>>>(psir, pot, rho, count, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_dot_reduce(part, nblocks, epot, 0, st);
}

}  // namespace lcg
