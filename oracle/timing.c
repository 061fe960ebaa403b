/* CPU baseline timing build of the oracle restatement -- TEST AND BENCHMARK
 * INFRASTRUCTURE ONLY (the CUDA library never links it).
 *
 * liblibconv_timing.so is libconv_oracle.c compiled a second time for speed
 * (-O3, OpenMP, the compiler's default floating-point contraction), plus the
 * drivers below that run one benchmark step over a batch of grids with an
 * OpenMP team, one grid per thread at a time (the generated reference code
 * parallelises with OpenMP inside each operator, GenericConvolution2.rb
 * :1338; over independent grids the team needs no reduction).  Results equal
 * the parity build's to rounding (the contraction may differ).  Each driver
 * returns the wall time of the step in seconds. */
#include <omp.h>
#include <stdlib.h>

#include "libconv_oracle.h"

/* MagicFilter3D (oracle_d_sfrf_ld_narr) and Kinetic3D (oracle_d_kin) of each
 * of ngrids n[0] x n[1] x n[2] periodic grids x (back to back) into mf and
 * kin, with `threads` OpenMP threads. */
double timing_mfkin_step(int ngrids, const int *n, const double *x, double *mf, double *kin,
                         const double *a, int threads) {
    const long long N = (long long)n[0] * n[1] * n[2];
    const int bc[3] = {0, 0, 0};
    double *work = (double *)malloc(sizeof(double) * 2 * N * (size_t)threads);
    if (!work) return -1.0;
    const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int g = 0; g < ngrids; ++g) {
        double *w1 = work + 2 * N * (long long)omp_get_thread_num(), *w2 = w1 + N;
        oracle_d_sfrf_ld_narr(3, n, bc, n, n, 1, x + g * N, mf + g * N, w1, w2);
        oracle_d_kin(3, n, bc, x + g * N, kin + g * N, w1, w2, a, 0.0, 0.0);
    }
    const double t = omp_get_wtime() - t0;
    free(work);
    return t;
}

/* Wavelet synthesis (oracle_d_idwt_sym8: 8 subbands of n^3 -> (2n)^3) then
 * analysis back, for each of ngrids periodic grids. */
double timing_wavelet_step(int ngrids, const int *n, const double *x, double *y, double *back,
                           int threads) {
    const long long N = 8LL * n[0] * n[1] * n[2];
    const int bc[3] = {0, 0, 0};
    double *work = (double *)malloc(sizeof(double) * 2 * N * (size_t)threads);
    if (!work) return -1.0;
    const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int g = 0; g < ngrids; ++g) {
        double *w1 = work + 2 * N * (long long)omp_get_thread_num(), *w2 = w1 + N;
        oracle_d_idwt_sym8(3, n, bc, x + g * N, y + g * N, w1, w2);
        oracle_d_dwt_sym8(3, n, bc, y + g * N, back + g * N, w1, w2);
    }
    const double t = omp_get_wtime() - t0;
    free(work);
    return t;
}

int timing_max_threads(void) { return omp_get_max_threads(); }
