// Potential step of the local Hamiltonian (BigDFT/libconv.f90:268-273) over
// norb orbitals laid back to back, on the real-space grid psir (the
// MagicFilter of each orbital):
//   rho  += sum_j psir_j^2        (when rho is given; j in order, one FMA each)
//   epot_j = sum pot * psir_j^2   (per-block partial sums, reduced afterwards)
//   psir_j = pot * psir_j
// One pass: pot and rho are read once for all orbitals, every psir_j is
// read and written once (16 bytes per point per orbital, plus 8 + 16 per
// point for pot and rho).  Each block owns POT_CHUNK consecutive points;
// consecutive threads touch consecutive points.  On GB300 the three FP64
// instructions per point and orbital (multiply, two FMAs) on the narrow
// FP64 pipe, not HBM, bound this kernel.  Orbitals are accumulated in
// order, so rho is the same whether the orbitals come in one call or one
// call each.  The partial sums are reduced in a fixed order (warp, block,
// then launch_dot_reduce_seg): the energies are the same on every run.
#include "lcg_sweep.cuh"

namespace lcg {
namespace {

constexpr int POT_THREADS = 256;
constexpr int POT_WARPS = POT_THREADS / 32;
constexpr int POT_PER_THREAD = 4;
constexpr int POT_CHUNK = POT_THREADS * POT_PER_THREAD;
constexpr int POT_OCHUNK = 32;     // orbitals per block synchronisation

__global__ void __launch_bounds__(POT_THREADS)
potential_kernel(double *__restrict__ psir, const double *__restrict__ pot,
                 double *__restrict__ rho, long long count, int norb, double *__restrict__ part) {
    __shared__ double ws[POT_OCHUNK][POT_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long base = (long long)blockIdx.x * POT_CHUNK + threadIdx.x;
    double v[POT_PER_THREAD], r[POT_PER_THREAD];
#pragma unroll
    for (int e = 0; e < POT_PER_THREAD; ++e) {
        const long long k = base + (long long)e * POT_THREADS;
        v[e] = k < count ? pot[k] : 0.0;
        r[e] = (rho && k < count) ? rho[k] : 0.0;
    }
    for (int j0 = 0; j0 < norb; j0 += POT_OCHUNK) {
        const int jn = norb - j0 < POT_OCHUNK ? norb - j0 : POT_OCHUNK;
        // warps run through the chunk's orbitals independently (shuffle
        // reductions only), so loads of later orbitals overlap earlier ones
#pragma unroll 4
        for (int jj = 0; jj < jn; ++jj) {
            double *__restrict__ ps = psir + (long long)(j0 + jj) * count;
            double acc = 0.0;
#pragma unroll
            for (int e = 0; e < POT_PER_THREAD; ++e) {
                const long long k = base + (long long)e * POT_THREADS;
                if (k < count) {
                    const double p = ps[k];
                    const double hp = v[e] * p;
                    r[e] = fma(p, p, r[e]);
                    acc = fma(p, hp, acc);
                    ps[k] = hp;
                }
            }
            for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) ws[jj][warp] = acc;
        }
        __syncthreads();
        if (threadIdx.x < jn) {
            double s = 0.0;
            for (int w = 0; w < POT_WARPS; ++w) s += ws[threadIdx.x][w];
            part[(long long)(j0 + threadIdx.x) * gridDim.x + blockIdx.x] = s;
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
