/* libconv-gb300: GB300 (sm_103a) implementation of BigDFT's separable
 * Daubechies-16 convolutions (MagicFilter, Kinetic, wavelet analysis and
 * synthesis) behind the procedure signatures that BOAST generates for them
 * in Nanosim-LIG/boast-lig (BigDFT/GenericConvolution2.rb).
 *
 * Conventions (same as the generated code):
 *   - arrays are Fortran-ordered (first index fastest), FP64;
 *   - n[], nx[], ny[], bc[] are small host int arrays of length d;
 *   - for wavelet operators n/nx/ny count coefficient pairs (the array extent
 *     along a dimension is twice the value);
 *   - bc: LIBCONV_BC_PERIODIC (0), LIBCONV_BC_GROW (1), LIBCONV_BC_SHRINK (-1),
 *     LIBCONV_BC_FREE (2, free boundary without growth);
 *   - narr independent arrays lie back to back in x and y.
 *
 * Every entry point returns LIBCONV_OK (0) or a negative status; the
 * generated reference procedures return nothing, and a caller that declares
 * them void may call these functions unchanged.
 *
 * Plain entry points take HOST pointers: inputs are copied to the GPU, the
 * operator runs, the outputs are copied back, and the call returns when the
 * result is in host memory.  The workspaces w1/w2 of the host-pointer 3D
 * entry points are accepted for signature compatibility and left untouched.
 * The *_dev entry points take DEVICE pointers and a cudaStream_t (passed as
 * void*, NULL = legacy default stream); they only enqueue work, and a
 * dot_in output of a *_dev entry point is a device pointer.
 *
 * Streams: the scratch a *_dev call needs besides the caller's buffers (dot
 * partial sums, per-line exponents of the exact tensor-core sweeps, energy
 * partials, the CG apply workspace) is leased to that call alone from a
 * per-device pool: calls on different streams, from one thread or several,
 * may be in flight at the same time and never share scratch (when more than
 * 16 streams are in flight at once, a new call is ordered after the oldest).
 * Calls on one stream reuse one lease in stream order.  The only state the
 * calls share is the device status word of the bounded waits (an error
 * flag) and, for d_s0s0_1d_sym8_d2_dotin_noalloc alone, its fixed array.
 */
#ifndef LIBCONV_GB300_H
#define LIBCONV_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define LIBCONV_OK        0
#define LIBCONV_EARG     -1   /* bad argument (null pointer, d/idim/n/narr out of range) */
#define LIBCONV_EBC      -2   /* boundary condition not supported by this operator */
#define LIBCONV_ESIZE    -3   /* nx/ny leading sizes too small for n and bc */
#define LIBCONV_ECUDA    -4   /* CUDA runtime error (message in libconv_gb300_last_error) */
#define LIBCONV_ENOMEM   -5   /* device allocation failed */
#define LIBCONV_EMODE    -6   /* unknown compute mode */
#define LIBCONV_ETIMEOUT -7   /* a bounded device-side wait gave up (status word set) */
#define LIBCONV_ENUMERIC -8   /* a solve produced a non-finite residual */

#define LIBCONV_BC_SHRINK   -1
#define LIBCONV_BC_PERIODIC  0
#define LIBCONV_BC_GROW      1
#define LIBCONV_BC_FREE      2
#define LIBCONV_BC_NPERIODIC -2   /* non-periodic: one-sided stencils (Poisson operators) */

/* Compute modes for libconv_gb300_set_mode (per calling thread).  The
 * tensor-core modes cover every sweep (MagicFilter, kinetic, derivative,
 * wavelet and combined wavelet-MagicFilter filters).  A thread starts in the
 * mode named by the environment variable LIBCONV_GB300_MODE (fp64, tc_exact,
 * tc_bf16x3, tc_tf32x3 or its number, read once per process), so callers of
 * the generated procedures can select a mode without a code change; in FP64
 * when the variable is unset or names no mode.
 *   FP64:      plain FP64 FMA kernels on the CUDA cores (default).
 *   TC_EXACT:  tcgen05 tensor cores with exact integer digit arithmetic (FP16
 *              byte digits, FP32 accumulation kept exact); FP64-class accuracy.
 *   TC_BF16X3: split precision, 3 bfloat16 terms per operand, 6 products,
 *              FP32 accumulation; relative error near 1e-7.
 *   TC_TF32X3: split precision, 2 tf32 terms per operand, 3 products, FP32
 *              accumulation; relative error near 1e-7. */
#define LIBCONV_MODE_FP64       0
#define LIBCONV_MODE_TC_EXACT   1
#define LIBCONV_MODE_TC_BF16X3  2
#define LIBCONV_MODE_TC_TF32X3  3

const char *libconv_gb300_version(void);
const char *libconv_gb300_strerror(int status);
/* Detailed message of the last failing call on this thread ("" if none). */
const char *libconv_gb300_last_error(void);
int libconv_gb300_set_mode(int mode);
int libconv_gb300_get_mode(void);
/* Synchronise `stream` (void* cudaStream_t) and report LIBCONV_ETIMEOUT if a
 * device-side wait of an earlier *_dev call on this device gave up; clears
 * the device status word. */
int libconv_gb300_check(void *stream);
/* Self-test of the bounded device-side waits: enqueues on `stream` one wait on
 * a barrier that nothing arrives at, limited to wait_us microseconds (1 to
 * 1e6) of the GPU's global timer; it gives up, sets the device status word
 * and returns, so the next libconv_gb300_check reports LIBCONV_ETIMEOUT (and
 * clears the word).  (The kernels' own waits give up after 4e9 SM clock
 * cycles, about 2 s at the maximum clock, longer at lower clocks.) */
int libconv_gb300_selftest_wait(int wait_us, void *stream);
/* Diagnostic, no counterpart in the reference: measured FP64 FMA throughput
 * of this GPU (the roof of the plain FP64 sweeps).  Runs 8 independent FMA
 * chains of `iters` steps in 8 x SMs blocks of 256 threads on `stream`, times
 * the launch with CUDA events and synchronises; *tflops = 2 x FMAs / time. */
int libconv_gb300_fp64_peak(int iters, double *tflops, void *stream);

/* ---------------------------------------------------------------------
 * 1D sweeps: GenericConvolutionOperator1d#procedure
 * (BigDFT/GenericConvolution2.rb:1560-1764), the ld + narr variants that
 * MagicFilter1d/Kinetic1d/Wavelet1d generate.  Shapes [1,0] / [0,1] /
 * [2,0,1] are selected from idim as the reference does (:1701-1761).
 *   y = a * fil (x)_idim x + a_x * x + a_y * y
 * ------------------------------------------------------------------- */

/* MagicFilter, filter 'sym8_md' = reverse(SYM8_MF), lowfil -8
 * (BigDFT/LibconvBase.rb:238-242; BigDFT/MagicFilter1d2.rb:5-24). */
int d_s0s0_1d_sym8_md(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                      int narr, const double *x, double *y, double a, double a_x, double a_y);
/* Inverse MagicFilter, filter 'sym8_imd' = SYM8_MF, lowfil -7
 * (BigDFT/LibconvBase.rb:244-248). */
int d_s0s0_1d_sym8_imd(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                       int narr, const double *x, double *y, double a, double a_x, double a_y);
/* First-derivative filter SYM8_D1 (29 taps) through the same generic
 * operator (BigDFT/WaveletFilters.rb:43-72; libconv.f90:412-413). */
int d_s0s0_1d_sym8_d1(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                      int narr, const double *x, double *y, double a, double a_x, double a_y);
/* Kinetic second derivative SYM8_D2 (29 taps) with the energy term
 * dot_in = sum x * (a * D2 x), taken before a_x is added
 * (BigDFT/Kinetic1d.rb:6-25; GenericConvolution2.rb:179-181).
 * dot_in sums over all narr arrays. */
int d_s0s0_1d_sym8_d2_dotin(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                            int narr, const double *x, double *y, double a, double a_x,
                            double a_y, double *dot_in);
/* Wavelet analysis (dwt), WaveletFilterDecompose of SYM8_LP:
 * x(0:1, p) interleaved -> y(q, 0:1) low block then high block
 * (BigDFT/LibconvBase.rb:226-230; GenericConvolution2.rb:505-587). */
int d_s0s1_1d_sym8(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                   int narr, const double *x, double *y, double a, double a_y);
/* Wavelet synthesis (idwt), WaveletFilterRecompose of SYM8_LP
 * (BigDFT/LibconvBase.rb:232-236; GenericConvolution2.rb:589-671). */
int d_s1s0_1d_sym8(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                   int narr, const double *x, double *y, double a, double a_y);
/* s1tor: synthesis fused with the MagicFilter (combined filters of
 * GenericConvolution2.rb:336-384; BigDFT/LibconvBase.rb:250-255). */
int d_s1s0_1d_symicomb8(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                        int narr, const double *x, double *y, double a, double a_y);
/* rtos1: analysis fused with the MagicFilter (BigDFT/LibconvBase.rb:257-262). */
int d_s0s1_1d_symicomb8(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                        int narr, const double *x, double *y, double a, double a_y);

int d_s0s0_1d_sym8_md_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                          int narr, const double *x, double *y, double a, double a_x, double a_y,
                          void *stream);
int d_s0s0_1d_sym8_imd_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                           int narr, const double *x, double *y, double a, double a_x,
                           double a_y, void *stream);
int d_s0s0_1d_sym8_d1_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                          int narr, const double *x, double *y, double a, double a_x, double a_y,
                          void *stream);
int d_s0s0_1d_sym8_d2_dotin_dev(int d, int idim, const int *n, int bc, const int *nx,
                                const int *ny, int narr, const double *x, double *y, double a,
                                double a_x, double a_y, double *dot_in, void *stream);
int d_s0s1_1d_sym8_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                       int narr, const double *x, double *y, double a, double a_y, void *stream);
int d_s1s0_1d_sym8_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                       int narr, const double *x, double *y, double a, double a_y, void *stream);
int d_s1s0_1d_symicomb8_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                            int narr, const double *x, double *y, double a, double a_y,
                            void *stream);
int d_s0s1_1d_symicomb8_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                            int narr, const double *x, double *y, double a, double a_y,
                            void *stream);

/* No counterpart in the reference.  Allocation-free form of
 * d_s0s0_1d_sym8_d2_dotin_dev, for callers that must not allocate device
 * memory: applications whose device memory is wholly owned by their own
 * allocator or memory budget, and latency-sensitive inner loops where a
 * cudaMalloc/cudaFree (which can synchronise the device) is not acceptable.
 * x, y and dot_in are caller-owned device memory; the per-block partial sums
 * of dot_in live in a fixed device array inside the library (65536 doubles,
 * 512 KB, held on every GPU that loads the library until exit), so a sweep
 * needing more than 65536 partial sums (number of lines / 32, times
 * ceil(outputs / 64), times narr) is rejected with LIBCONV_ESIZE.
 * The first call on a device looks up that array's device address (a CUDA
 * runtime query, done once per device, with the device current); make the
 * first call before any stream capture; cudaDeviceReset between calls is not
 * supported (the address looked up before it would be stale).  Calls share
 * the array: calls that overlap on the GPU (different streams, concurrently)
 * race, and what they corrupt is dot_in (y does not use the array).  Always
 * runs the FP64 sweep kernel, whatever the compute mode. */
int d_s0s0_1d_sym8_d2_dotin_noalloc(int d, int idim, const int *n, int bc, const int *nx,
                                    const int *ny, int narr, const double *x, double *y,
                                    double a, double a_x, double a_y, double *dot_in,
                                    void *stream);

/* ---------------------------------------------------------------------
 * Multi-dimensional operators: GenericConvolutionOperator#procedure
 * (BigDFT/GenericConvolution2.rb:1934-2243).
 * ------------------------------------------------------------------- */

/* 3D MagicFilter (transpose = 1, ld, narr, work): MagicFilter() of
 * BigDFT/MagicFilter2.rb:46-70 built on the filter named 'sfrf' in
 * BigDFT/MagicFilter_test2.rb:60 (reverse(SYM8_MF) centre 8). */
int d_sfrf_ld_narr(int d, const int *n, const int *bc, const int *nx, const int *ny, int narr,
                   const double *x, double *y, double *w1, double *w2);
/* Same with the inverse filter 'rfsf' (BigDFT/MagicFilter_test2.rb:152). */
int d_rfsf_ld_narr(int d, const int *n, const int *bc, const int *nx, const int *ny, int narr,
                   const double *x, double *y, double *w1, double *w2);
/* 3D kinetic (transpose = 0, a[d], a_x, a_y, kinetic, zero_out_work):
 * Kinetic() of BigDFT/Kinetic2.rb:1068-1090 on the filter 'kin'
 * (BigDFT/Kinetic_test2.rb:33):  y = sum_i a[i] D2_i x + a_x x + a_y y.
 * Periodic and free (no-grow) boundaries. */
int d_kin(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
          double *w2, const double *a, double a_x, double a_y);
/* 3D kinetic with the kinetic energy of every direction:
 * kinetic_per_ref_optim_ekin (BigDFT/Kinetic2.rb:21-112), generalised to the
 * d_kin options.  y = sum_i a_i D2_i x + a_x x + a_y y as d_kin, and
 * kstrten[i] = x . (a_i D2_i x) for each of the d directions (the reference's
 * kstrten(1:3); with a_i = -0.5/h_i^2, a_x = 0, a_y = 1 it is that routine).
 * kstrten: d doubles (host pointer here, device pointer for _dev). */
int d_kin_ekin(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
               double *w2, const double *a, double a_x, double a_y, double *kstrten);
/* Extension (no counterpart in the generated code, which has no narr for
 * Kinetic()): the same 3D kinetic over narr grids laid back to back in x, y,
 * w1 and w2, in one launch per sweep. */
int d_kin_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y,
               double *w1, double *w2, const double *a, double a_x, double a_y);
/* 3D wavelet analysis / synthesis (transpose = 1, work): Wavelet() of
 * BigDFT/Wavelet2.rb:2-21 (BigDFT/Wavelet_test2.rb:86-154). */
int d_dwt_sym8(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
               double *w2);
int d_idwt_sym8(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
                double *w2);
/* Extension (no counterpart in the generated code): the same 3D wavelet
 * analysis / synthesis over narr grids laid back to back, one launch per
 * sweep. */
int d_dwt_sym8_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y,
                    double *w1, double *w2);
int d_idwt_sym8_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y,
                     double *w1, double *w2);

/* Device-pointer forms; w1/w2 are device workspaces sized like the
 * reference's (the largest intermediate grid, times narr). */
int d_sfrf_ld_narr_dev(int d, const int *n, const int *bc, const int *nx, const int *ny,
                       int narr, const double *x, double *y, double *w1, double *w2,
                       void *stream);
int d_rfsf_ld_narr_dev(int d, const int *n, const int *bc, const int *nx, const int *ny,
                       int narr, const double *x, double *y, double *w1, double *w2,
                       void *stream);
int d_kin_dev(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
              double *w2, const double *a, double a_x, double a_y, void *stream);
int d_kin_ekin_dev(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
                   double *w2, const double *a, double a_x, double a_y, double *kstrten,
                   void *stream);
int d_kin_narr_dev(int d, const int *n, const int *bc, int narr, const double *x, double *y,
                   double *w1, double *w2, const double *a, double a_x, double a_y, void *stream);
int d_dwt_sym8_dev(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
                   double *w2, void *stream);
int d_dwt_sym8_narr_dev(int d, const int *n, const int *bc, int narr, const double *x,
                        double *y, double *w1, double *w2, void *stream);
int d_idwt_sym8_narr_dev(int d, const int *n, const int *bc, int narr, const double *x,
                         double *y, double *w1, double *w2, void *stream);
int d_idwt_sym8_dev(int d, const int *n, const int *bc, const double *x, double *y,
                    double *w1, double *w2, void *stream);

/* ---------------------------------------------------------------------
 * Local Hamiltonian of one orbital: the pipeline of the libconvw module
 * (BigDFT/libconv.f90:248-294; the reference leaves it as an unfinished
 * subroutine body), composed of the operators above on one stream:
 *   psi_fscf = idwt(psig)            s1s0_md     SYM8_LP   grow
 *   psir     = MF(psi_fscf)          s0s0_md     SYM8_MD   grow
 *   rho     += psir^2                (skipped when rho is NULL)
 *   epot     = sum pot * psir^2
 *   psir     = pot * psir
 *   hpsi     = MI(psir)              s0s0_md     SYM8_MI   shrink
 *   hpsi    += sum_i a_kin[i] D2_i psi_fscf, and per direction
 *   ekin[i]  = psi_fscf . (a_kin[i] D2_i psi_fscf)
 *                                    s0s0_1ds_dot SYM8_D2  no-grow, a_y = 1
 *   hpsig    = dwt(hpsi)             s0s1_md     SYM8_LP   shrink
 * Along an axis with bc[i] = LIBCONV_BC_FREE the steps use the grow/shrink
 * boundaries shown; along an axis with LIBCONV_BC_PERIODIC every step is
 * periodic.  n[3]: coarse points (wavelet pairs) per axis; psig and hpsig
 * hold 2n[0] x 2n[1] x 2n[2] values laid out as d_idwt_sym8's input.  The
 * fine grid of psi_fscf has 2n[i] + 14 points along a free axis (2n[i]
 * periodic), and the real-space grid of psir, pot and rho 15 more along a
 * free axis.  a_kin[i]: scale of the kinetic filter along axis i, as a[] of
 * d_kin (-0.5/h_i^2 for BigDFT's kinetic energy on spacing h_i).  The
 * calling thread's compute mode applies to every sweep.
 * Extension: no generated procedure of the reference does this in one call.
 * ------------------------------------------------------------------- */
/* Element counts: psig/hpsig, the real-space grid (pot, rho), and the
 * device workspace of libconv_hamiltonian_dev.  Any output may be NULL. */
int libconv_hamiltonian_sizes(const int *n, const int *bc, long long *nsig, long long *nreal,
                              long long *nwork);
/* Host pointers; ekin: 3 doubles, epot: 1 double; rho is read and updated
 * when not NULL. */
int libconv_hamiltonian(const int *n, const int *bc, const double *a_kin, const double *psig,
                        const double *pot, double *rho, double *hpsig, double *ekin,
                        double *epot);
/* Device pointers, enqueued on `stream`; energies: 4 doubles on the device
 * (ekin[0..2], epot); work: nwork doubles. */
int libconv_hamiltonian_dev(const int *n, const int *bc, const double *a_kin, const double *psig,
                            const double *pot, double *rho, double *hpsig, double *energies,
                            double *work, void *stream);
/* norb orbitals at once (psig and hpsig: norb arrays of nsig back to back),
 * sharing one potential; every step is one launch over all orbitals.  rho
 * (when not NULL) accumulates psir_j^2 for j = 0..norb-1 in order, giving
 * the same numbers as norb single-orbital calls.  energies: norb x 4
 * doubles, [ekin_x, ekin_y, ekin_z, epot] of each orbital (host pointer for
 * libconv_hamiltonian_narr, device pointer for the _dev form).  nwork of
 * libconv_hamiltonian_narr_sizes grows with norb (about 10 nsig per
 * orbital). */
int libconv_hamiltonian_narr_sizes(const int *n, const int *bc, int norb, long long *nsig,
                                   long long *nreal, long long *nwork);
int libconv_hamiltonian_narr(const int *n, const int *bc, const double *a_kin, int norb,
                             const double *psig, const double *pot, double *rho, double *hpsig,
                             double *energies);
int libconv_hamiltonian_narr_dev(const int *n, const int *bc, const double *a_kin, int norb,
                                 const double *psig, const double *pot, double *rho,
                                 double *hpsig, double *energies, double *work, void *stream);

/* ---------------------------------------------------------------------
 * Poisson finite-difference operators (BigDFT/Poisson.rb): first
 * derivatives of order nord in {2, 4, 6, 8, 16} (the c1D table of
 * Poisson.rb:20-166), periodic or non-periodic (LIBCONV_BC_NPERIODIC:
 * one-sided stencils on the nord/2 first and last points of a line, which
 * needs at least nord + 1 points).  Grids are n01 x n02 x n03, Fortran
 * order; hgrids[3] (host) are the spacings, each derivative scaled by
 * 1/hgrids[i] as the generated drivers do.  geocode selects the axes:
 * 1 free (x, z non-periodic), 2 periodic, 3 surface (y non-periodic)
 * (Poisson.rb:2122-2128).  The calling thread's compute mode applies.
 * ------------------------------------------------------------------- */
/* Poisson_broker (Poisson.rb:1951-2043): du = a d/dx_idim u on the 3D grid
 * nn[3], idim 0..2, bc LIBCONV_BC_PERIODIC or LIBCONV_BC_NPERIODIC. */
int Poisson_broker(int nord, int idim, const int *nn, int bc, const double *u, double *du,
                   double a);
int Poisson_broker_dev(int nord, int idim, const int *nn, int bc, const double *u, double *du,
                       double a, void *stream);
/* div_u_i (Poisson.rb:2067-2194): u(n01,n02,n03,3) -> du = sum_i d_i u_i;
 * when cc is not NULL also cc = sum_i u_i^2 d_i u_i
 * + 2 (u0 u1 d0 u1 + u0 u2 d0 u2 + u1 u2 d1 u2).  _dev: work of
 * 5 n01 n02 n03 doubles when cc is given (unused otherwise). */
int div_u_i(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
            const double *hgrids, double *cc);
int div_u_i_dev(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                const double *hgrids, double *cc, double *work, void *stream);
/* nabla_u (Poisson.rb:2553-2620): du(n01,n02,n03,3) = grad u. */
int nabla_u(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
            const double *hgrids);
int nabla_u_dev(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                const double *hgrids, void *stream);
/* nabla_u_and_square (Poisson.rb:2197-2275): du = grad u, ddu = |grad u|^2. */
int nabla_u_and_square(int geocode, int n01, int n02, int n03, const double *u, double *du,
                       double *ddu, int nord, const double *hgrids);
int nabla_u_and_square_dev(int geocode, int n01, int n02, int n03, const double *u, double *du,
                           double *ddu, int nord, const double *hgrids, void *stream);
/* nabla_u_square (Poisson.rb:2278-2359): ddu = |grad u|^2.  _dev: work of
 * 3 n01 n02 n03 doubles. */
int nabla_u_square(int geocode, int n01, int n02, int n03, const double *u, double *ddu, int nord,
                   const double *hgrids);
int nabla_u_square_dev(int geocode, int n01, int n02, int n03, const double *u, double *ddu,
                       int nord, const double *hgrids, double *work, void *stream);
/* nabla_u_epsilon (Poisson.rb:2362-2443): du = eps grad u. */
int nabla_u_epsilon(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                    const double *hgrids, const double *eps);
int nabla_u_epsilon_dev(int geocode, int n01, int n02, int n03, const double *u, double *du,
                        int nord, const double *hgrids, const double *eps, void *stream);
/* update_rhopol (Poisson.rb:2446-2550): res = (dlogeps . grad u)/(4 pi),
 * res = eta (res - rhopol), rhopol += res, *rhores2 = sum res^2;
 * dlogeps(3,n01,n02,n03) component fastest.  _dev: rhores2 is a device
 * pointer, work of update_rhopol_work_size doubles. */
int update_rhopol(int geocode, int n01, int n02, int n03, const double *u, int nord,
                  const double *hgrids, double eta, const double *dlogeps, double *rhopol,
                  double *rhores2);
int update_rhopol_dev(int geocode, int n01, int n02, int n03, const double *u, int nord,
                      const double *hgrids, double eta, const double *dlogeps, double *rhopol,
                      double *rhores2, double *work, void *stream);
/* Extension: work size (doubles) of update_rhopol_dev. */
int update_rhopol_work_size(int n01, int n02, int n03, long long *nwork);

/* ---------------------------------------------------------------------
 * Cost model (ConvolutionOperator1d#cost / GenericConvolutionOperator#cost,
 * BigDFT/GenericConvolution2.rb:1269-1276, 1850-1932): the flop count the
 * reference uses for every GFlop/s it prints (n * filter.cost * ndat per
 * sweep; filter.cost = 2*taps for convolutions, 4*length for wavelets).
 * ------------------------------------------------------------------- */
int d_s0s0_1d_sym8_md_cost(int d, int idim, const int *n, int bc, int narr, long long *cost);
int d_s0s0_1d_sym8_d2_cost(int d, int idim, const int *n, int bc, int narr, long long *cost);
int d_s0s1_1d_sym8_cost(int d, int idim, const int *n, int bc, int narr, long long *cost);
int d_sfrf_cost(int d, const int *n, const int *bc, int narr, long long *cost);
int d_kin_cost(int d, const int *n, const int *bc, long long *cost);
int d_dwt_sym8_cost(int d, const int *n, const int *bc, long long *cost);

/* ---------------------------------------------------------------------
 * Batched 3D operators over many grids of different sizes (extension: no
 * counterpart in the generated code, which runs one grid per call), for the
 * orbitals of uneven localisation regions.  Grid g has dims[3g..3g+2]; the
 * grids are packed back to back (each in Fortran order) in x, y_mf and
 * y_kin, at the element offsets libconv_batch_offsets reports.
 *   - MagicFilter3D (mf_bc != NULL): sfrf_ld_narr of each grid, output sizes
 *     by mf_bc (grow: n + 15 per axis);
 *   - Kinetic3D (kin_bc != NULL; periodic or free): d_kin of each grid with
 *     kin_a[3], kin_ax (a_y = 0).
 * Each sweep stage of an operator is ONE persistent launch over the sweeps of
 * all grids; a run is a CUDA graph of those launches (captured on the first
 * run on a stream; the legacy default stream runs the launches uncaptured).
 * The batch keeps the compute mode of the thread that created it and owns
 * its device workspaces (allocated at creation).  libconv_batch_tune times
 * every engine and sweep order the mode allows on the caller's buffers and
 * keeps the fastest, recorded in the JSON file $LIBCONV_GB300_TUNE_CACHE
 * (default $HOME/.cache/libconv_gb300_tune.json) and reused by later
 * batches of the same shapes on the same GPU model and mode.
 * --------------------------------------------------------------------- */
typedef struct libconv_batch libconv_batch;
#define LIBCONV_BATCH_OP_MF   0
#define LIBCONV_BATCH_OP_KIN  1
/* engines: FP64 sweep with 64- or 32-output chunks, or the tensor-core sweep
 * of the batch's mode (not in LIBCONV_MODE_FP64) */
#define LIBCONV_ENGINE_FP64_Q64  0
#define LIBCONV_ENGINE_FP64_Q32  1
#define LIBCONV_ENGINE_TC        2
int libconv_batch_create(libconv_batch **b, int ngrids, const int *dims, const int *mf_bc,
                         const int *kin_bc, const double *kin_a, double kin_ax);
int libconv_batch_sizes(const libconv_batch *b, long long *in_elems, long long *mf_elems,
                        long long *kin_elems);
/* ngrids + 1 offsets each (last = total); NULL arrays are skipped */
int libconv_batch_offsets(const libconv_batch *b, long long *in_off, long long *mf_off,
                          long long *kin_off);
/* order: the three axes in sweep order; for the MagicFilter order[0] = -1
 * selects the reference's rotating sweeps (transpose = 1) */
int libconv_batch_set_config(libconv_batch *b, int op, int engine, const int *order);
int libconv_batch_get_config(const libconv_batch *b, int op, int *engine, int *order, int *tuned);
int libconv_batch_tune(libconv_batch *b, const double *x, double *y_mf, double *y_kin,
                       void *stream);
/* device pointers; enqueues only (check with libconv_gb300_check) */
int libconv_batch_run(libconv_batch *b, const double *x, double *y_mf, double *y_kin,
                      void *stream);
int libconv_batch_destroy(libconv_batch *b);

/* ---------------------------------------------------------------------
 * Shifted kinetic solves (extension: no counterpart in the generated code).
 * nsys systems (T - eps_s) x_s = b_s on periodic n^3 grids (n a multiple of
 * 8) with grid spacings h[3], T the 3D kinetic operator (kinetic sweeps of
 * the thread's compute mode), eps_s < 0; vectors are device float64 arrays
 * of nsys * n^3 values, eps a device array of nsys values.
 * --------------------------------------------------------------------- */
/* Weights of the learned preconditioner (device pointers): four 3x3x3
 * convolutions, wt[l] bfloat16 [27][16 cout][16 cin] (tap t = (dx+1) +
 * 3(dy+1) + 9(dz+1)), bias[l] float [16]; input channels (r / s, eps),
 * output channel 0; s = rms(r) per system; ReLU after layers 0-2. */
typedef struct {
    const void *wt[4];
    const float *bias[4];
} libconv_cnn_weights;
/* y = (T - eps) x for every system. */
int libconv_cg_apply(int n, int nsys, const double *h, const double *eps, const double *x,
                     double *y, void *stream);
/* x = solution from x0 = 0 by Jacobi-preconditioned CG (w == NULL) or by
 * flexible CG preconditioned with z = s M(r / s, eps) (w != NULL); a system
 * stops at ||r|| <= tol ||b||, or with LIBCONV_ENUMERIC when its residual
 * becomes non-finite.  iters (host, nsys or NULL): iteration of
 * convergence (maxit + 1 if not reached); res (host, nsys or NULL): the
 * true residual norm ||b - (T - eps) x|| recomputed with the FP64 operator;
 * fell_back (host, nsys or NULL): the iteration at which a system left the
 * learned preconditioner for the plain one, 0 if it never did.  Returns
 * LIBCONV_ETIMEOUT if a bounded device-side wait of its kinetic sweeps or
 * network layers gave up (the device status word is read and cleared). */
/* Stagnation test of the learned phase (calling thread): a system whose
 * residual norm is above ratio times its value `window` iterations earlier
 * (tested every `window` iterations) continues with the plain preconditioner
 * (CG restarted from its current iterate).  Default 10 and 0.5. */
int libconv_cg_set_stall(int window, double ratio);
int libconv_cg_solve(int n, int nsys, const double *h, const double *eps, const double *b,
                     double *x, double tol, int maxit, const libconv_cnn_weights *w, int *iters,
                     double *res, int *fell_back, void *stream);
/* One 3x3x3 periodic convolution layer of the network over nsys n^3 grids.
 * src_kind 0: 16-channel bfloat16 activations [sys][z][y][x][16];
 *          1: float64 field times src_fac[s], with eps[s] as channel 1;
 *          2: float64 field times src_fac[s] (single channel).
 * dst_kind 0: bfloat16 activations relu(conv + bias);
 *          1: float64 field dst_fac[s] (conv channel 0 + bias[0]);
 *          2: bfloat16 activations conv, zeroed where mask (activations) <= 0.
 * cout: output channels computed (<= 8: channels 0-7 only); active (device,
 * nsys ints, or NULL): systems with 0 are skipped (their output untouched).
 * n >= 16 runs on the tensor cores (tcgen05); a bounded wait that gives up
 * sets the device status word (libconv_gb300_check reports it). */
int libconv_cnn_conv(int n, int nsys, int src_kind, int dst_kind, const void *src,
                     const double *src_fac, const double *eps, const void *wt, const float *bias,
                     void *dst, const double *dst_fac, const void *mask, int cout,
                     const int *active, void *stream);
/* Weight gradient of a layer: out[27*256 + 16] (float) = sum over points of
 * g[p][cout] x[p + d_t][cin] ([27][16 cout][16 cin]) and of g[p][cout]
 * (bias); g of kind 0 or 2, x of kind 0 or 1 (see libconv_cnn_conv); part:
 * device scratch of libconv_cnn_wgrad_parts() * (27*256 + 16) floats. */
int libconv_cnn_wgrad(int n, int nsys, int g_kind, const void *g, const double *g_fac, int x_kind,
                      const void *x, const double *x_fac, const double *eps, float *part,
                      float *out, void *stream);
int libconv_cnn_wgrad_parts(int n, int nsys);

#ifdef __cplusplus
}
#endif
#endif /* LIBCONV_GB300_H */
