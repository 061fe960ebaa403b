// Potential step of the local Hamiltonian (BigDFT/libconv.f90:268-273) over
// norb orbitals laid back to back, on the real-space grid psir (the
// MagicFilter of each orbital):
//   rho  += sum_j psir_j^2        (when rho is given; j in order)
//   epot_j = sum pot * psir_j^2   (per-block partial sums, reduced afterwards)
//   psir_j = pot * psir_j
// One pass: pot and rho are read once for all orbitals, every psir_j is
// read and written once -- an HBM-bound element-wise kernel (16 bytes per
// point per orbital, plus 8 + 16 per point for pot and rho).  Each block
// owns POT_CHUNK consecutive points; consecutive threads touch consecutive
// points.  The density is summed with explicit round-to-nearest products
// and sums (no contraction), orbital after orbital, so rho is the same
// number the per-orbital form rho = rho + psir*psir gives.  The partial
// sums are reduced in a fixed order (block, then launch_dot_reduce_seg):
// the energies are the same on every run.
#include "lcg_sweep.cuh"

namespace lcg {
namespace {

constexpr int POT_THREADS = 256;
constexpr int POT_PER_THREAD = 4;
constexpr int POT_CHUNK = POT_THREADS * POT_PER_THREAD;

__global__ void __launch_bounds__(POT_THREADS)
potential_kernel(double *__restrict__ psir, const double *__restrict__ pot,
                 double *__restrict__ rho, long long count, int norb, double *__restrict__ part) {
    __shared__ double ws[POT_THREADS / 32];
    const long long base = (long long)blockIdx.x * POT_CHUNK + threadIdx.x;
    double v[POT_PER_THREAD], r[POT_PER_THREAD];
#pragma unroll
    for (int e = 0; e < POT_PER_THREAD; ++e) {
        const long long k = base + (long long)e * POT_THREADS;
        v[e] = k < count ? pot[k] : 0.0;
        r[e] = (rho && k < count) ? rho[k] : 0.0;
    }
    for (int j = 0; j < norb; ++j) {
        double *__restrict__ ps = psir + (long long)j * count;
        double acc = 0.0;
#pragma unroll
        for (int e = 0; e < POT_PER_THREAD; ++e) {
            const long long k = base + (long long)e * POT_THREADS;
            if (k < count) {
                const double p = ps[k];
                const double hp = v[e] * p;
                r[e] = __dadd_rn(r[e], __dmul_rn(p, p));
                acc = fma(p, hp, acc);
                ps[k] = hp;
            }
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < POT_THREADS / 32; ++w) s += ws[w];
            part[(long long)j * gridDim.x + blockIdx.x] = s;
        }
        __syncthreads();
    }
    if (rho) {
#pragma unroll
        for (int e = 0; e < POT_PER_THREAD; ++e) {
            const long long k = base + (long long)e * POT_THREADS;
            if (k < count) rho[k] = r[e];
        }
    }
}

}  // namespace

long long potential_blocks(long long count) {
    const long long b = (count + POT_CHUNK - 1) / POT_CHUNK;
    return b < 1 ? 1 : b;
}

cudaError_t launch_potential(double *psir, const double *pot, double *rho, long long count,
                             int norb, double *part, double *epot, long long epot_stride,
                             cudaStream_t st) {
    const long long nb = potential_blocks(count);
    if (nb > 0x7FFFFFFFLL || norb < 1) return cudaErrorInvalidValue;
    potential_kernel<<<(unsigned)nb, POT_THREADS, 0, st>>>(psir, pot, rho, count, norb, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_dot_reduce_seg(part, nb, norb, epot, epot_stride, st);
}

}  // namespace lcg
