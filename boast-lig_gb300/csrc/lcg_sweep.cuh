// One 1D sweep of a separable convolution over a batch of lines: the unit of
// work every entry point of the library is decomposed into.  Semantics are
// those of one generated ConvolutionOperator1d call
// (BigDFT/GenericConvolution2.rb:1036-1442), applied to `narr` arrays.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lcg {

enum Kind { KCONV = 0, KDEC = 1, KREC = 2 };
enum Bc { BC_SHRINK = -1, BC_PERIODIC = 0, BC_GROW = 1, BC_FREE = 2 };

struct Sweep {
    int kind;            // KCONV (1 channel), KDEC (s0s1), KREC (s1s0)
    int ntaps;           // taps (polyphase taps for wavelets)
    int lowfil;          // first tap offset
    int bc;
    int ftab;            // offset of the filter in the device filter table
    int nL, n, nR;       // lines = nL*nR; n = processed size (pairs for wavelets)
    int in_lo, in_ext;   // input processed-dim index range [in_lo, in_lo+in_ext)
    int out_lo, out_ext; // output processed-dim index range
    int qlo, qhi;        // outputs computed: q in [qlo, qhi]
    int transpose;       // 1: y(line, q) (rotated), only with nL == 1
    int narr;
    long long x_arr, y_arr;   // element stride between the narr arrays
    const double *x;
    const double *x2;         // kinetic partial sum added to the output (or null)
    double *y;
    int has_a, has_ax, ay_mode, has_dot;   // ay_mode: 0 write, 1 a_y*y+out, 2 y+out
    double a, a_x, a_y;
    double *dot_part;         // one partial per block (device), when has_dot
    long long le_off = 0;     // first entry of this sweep's lines in a batched line-exponent array
    // tensor-core sweeps: the divisors of the tile index (output chunks per
    // line block, line blocks per array, nL) with their multiplicative
    // inverses, q = (n * m) >> s for every n < 2^31 (filled by tc_prepare)
    unsigned int tdiv_d[3] = {1, 1, 1}, tdiv_m[3] = {0, 0, 0}, tdiv_s[3] = {0, 0, 0};
    // tensor-core convolution sweeps: the tile's input window starts woff
    // elements before the first input position, so that along contiguous
    // lines its 8-element groups start on 32-byte boundaries (0 otherwise)
    int woff = 0;
    // per array: 0 = skip the array's lines (its output is left as it is); null:
    // every array (sweeps without a dot product only)
    const int *active = nullptr;
    // exact tensor-core transposed convolution sweeps whose tiles hold whole
    // lines of the next sweep (run_plan decides): the epilogue writes the
    // largest exponent field of each of the next sweep's lines,
    // le_next[a le_next_lines + i2 + le_n2 (q - out_lo)], for this sweep's line
    // i1 + le_n1 i2 and output q (le_n1 = the next sweep's line length: 32, 64
    // or 128, so that every tile column covers whole lines)
    int *le_next = nullptr;
    long long le_next_lines = 0;
    int le_n1 = 0, le_n2 = 0;
};

// Number of dot partials the FP64 sweep writes for S (grid size).
long long sweep_fp64_blocks(const Sweep &S);
// Enqueue the FP64 SIMT sweep on `st`.
cudaError_t launch_sweep_fp64(const Sweep &S, cudaStream_t st);
// Blocks of S in the batched FP64 sweep with output chunk qc (64 or 32;
// halved for the two-channel wavelet sweeps).
long long sweep_fp64_batch_blocks(const Sweep &S, int qc);
// Persistent grid of the batched FP64 sweep (SMs x resident CTAs per SM).
int sweep_fp64_batch_grid(int kind, int ntaps, int qc);
// One persistent launch over nsweeps sweeps (device descriptors, block
// prefix sums with prefix[nsweeps] = total) of one kind and filter; no dot.
cudaError_t launch_sweep_fp64_batch(int kind, int ntaps, int qc, const Sweep *descs,
                                    const long long *prefix, int nsweeps, int grid,
                                    cudaStream_t st);
// Deterministic sum of `count` partials into *out (device), on `st`.
cudaError_t launch_dot_reduce(const double *part, long long count, double *out, int accumulate,
                              cudaStream_t st);
// Segmented form: out[j * out_stride] = sum of part[j*seg_len .. (j+1)*seg_len)
// for j < nseg (fixed order), on `st`.
cudaError_t launch_dot_reduce_seg(const double *part, long long seg_len, int nseg, double *out,
                                  long long out_stride, cudaStream_t st);
// The m = nord/2 one-sided outputs at each end of every line of a
// non-periodic Poisson sweep (c1D(:, i-m) on the first nord+1 points, c1D(:,
// i-n+m+1) on the last), y = a * sum (or y += when accumulate).
cudaError_t launch_poisson_edges(const double *x, double *y, long long nL, int n, long long nR,
                                 int nord, double a, int accumulate, cudaStream_t st);
// Potential step of the local Hamiltonian over norb orbitals of `count`
// real-space points each (psir back to back): rho += sum_j psir_j^2 (rho may
// be null), epot[j * epot_stride] = sum pot psir_j^2, psir_j = pot psir_j.
// part holds potential_blocks(count) * norb partial sums.
long long potential_blocks(long long count);
cudaError_t launch_potential(double *psir, const double *pot, double *rho, long long count,
                             int norb, double *part, double *epot, long long epot_stride,
                             cudaStream_t st);

}  // namespace lcg
