/* CPU oracle for libconv-gb300 -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64, single-threaded restatement of the reference's arithmetic:
 *   - the hand-written Fortran reference kernels (BigDFT/magicfilter_refs.f90,
 *     BigDFT/Kinetic2.rb:981-1061, BigDFT/old/Synthesis.rb:23-146,
 *     BigDFT/old/AnaRotPer-2.rb:22-64 and the periodic form at :258-296);
 *   - the generated 1D operator contract (BigDFT/GenericConvolution2.rb:
 *     ConvolutionOperator1d, 1036-1442, with the post-processing of 173-203
 *     and 440-462) and the 1D / multi-D dispatchers (1560-1764, 1934-2243).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the checker or the timed CPU baseline.
 * The GPU library never links or calls it.
 *
 * Parity pinning: the periodic MagicFilter restatement is checked bit-for-bit
 * against the reference's own C file benchmark/convolutions-c/MagicFilter.c
 * built from the reference sources into oracle/_ref/, and every routine is
 * checked against an independent numpy restatement and the algebraic
 * identities the reference's tests assert.
 */
#ifndef LIBCONV_ORACLE_H
#define LIBCONV_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* ---- Fortran reference kernels (same argument meaning, by value) ---- */
void oracle_magicfilter_per_ref(int n1, int ndat, const double *x, double *y);
void oracle_magicfilter_per_t_ref(int n1, int ndat, const double *x, double *y);
void oracle_magicfilter_free_ref(int n1, int ndat, const double *x, double *y);
void oracle_magicfilter_free_t_ref(int n1, int ndat, const double *x, double *y);
void oracle_kinetic_per_ref(int n1, int n2, int n3, const double *hgrid,
                            const double *x, double *y, double c);
void oracle_synthesis_per_ref(int n, int ndat, const double *x, double *y);
void oracle_synthesis_free_ref(int n, int ndat, const double *x, double *y);
void oracle_analysis_per_ref(int n, int ndat, const double *x, double *y);
void oracle_analysis_free_ref(int n, int ndat, const double *x, double *y);

/* ---- generated-libconv entry points (GenericConvolution2.rb dispatchers) ----
 * Same names as the GPU library with an "oracle_" prefix; return 0 or a
 * negative error code (same codes as the GPU library). */
int oracle_d_s0s0_1d_sym8_md(int d, int idim, const int *n, int bc, const int *nx,
                             const int *ny, int narr, const double *x, double *y,
                             double a, double a_x, double a_y);
int oracle_d_s0s0_1d_sym8_imd(int d, int idim, const int *n, int bc, const int *nx,
                              const int *ny, int narr, const double *x, double *y,
                              double a, double a_x, double a_y);
int oracle_d_s0s0_1d_sym8_d1(int d, int idim, const int *n, int bc, const int *nx,
                             const int *ny, int narr, const double *x, double *y,
                             double a, double a_x, double a_y);
int oracle_d_s0s0_1d_sym8_d2_dotin(int d, int idim, const int *n, int bc, const int *nx,
                                   const int *ny, int narr, const double *x, double *y,
                                   double a, double a_x, double a_y, double *dot_in);
int oracle_d_s0s1_1d_sym8(int d, int idim, const int *n, int bc, const int *nx,
                          const int *ny, int narr, const double *x, double *y,
                          double a, double a_y);
int oracle_d_s1s0_1d_sym8(int d, int idim, const int *n, int bc, const int *nx,
                          const int *ny, int narr, const double *x, double *y,
                          double a, double a_y);
int oracle_d_s0s1_1d_symicomb8(int d, int idim, const int *n, int bc, const int *nx,
                               const int *ny, int narr, const double *x, double *y,
                               double a, double a_y);
int oracle_d_s1s0_1d_symicomb8(int d, int idim, const int *n, int bc, const int *nx,
                               const int *ny, int narr, const double *x, double *y,
                               double a, double a_y);

int oracle_d_sfrf_ld_narr(int d, const int *n, const int *bc, const int *nx, const int *ny,
                          int narr, const double *x, double *y, double *w1, double *w2);
int oracle_d_rfsf_ld_narr(int d, const int *n, const int *bc, const int *nx, const int *ny,
                          int narr, const double *x, double *y, double *w1, double *w2);
/* kinetic_per_ref_optim_ekin: y += T x, kstrten[d] = x . (T_d x) */
void oracle_kinetic_per_ref_ekin(int n1, int n2, int n3, const double *hgrid, const double *x,
                                 double *y, double *kstrten);
int oracle_d_kin(int d, const int *n, const int *bc, const double *x, double *y,
                 double *w1, double *w2, const double *a, double a_x, double a_y);
int oracle_d_dwt_sym8(int d, const int *n, const int *bc, const double *x, double *y,
                      double *w1, double *w2);
int oracle_d_idwt_sym8(int d, const int *n, const int *bc, const double *x, double *y,
                       double *w1, double *w2);
/* Local Hamiltonian of one orbital (BigDFT/libconv.f90:248-294): idwt grow,
 * MagicFilter grow, rho += psir^2 (rho may be NULL), epot = sum v psir^2,
 * psir = v psir, inverse MagicFilter shrink, kinetic no-grow accumulated
 * with ekin[3] per direction, dwt shrink.  bc[i]: periodic (0) or free (2). */
/* Poisson finite-difference operators (BigDFT/Poisson.rb): the 1D broker
 * (bc 0 periodic, -2 non-periodic), the generated 3D drivers and the
 * Fortran div_u_i_ref. */
int oracle_poisson_broker(int nord, int idim, const int *nn, int bc, const double *u, double *du,
                          double a);
int oracle_div_u_i(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                   const double *hgrids, double *cc);
int oracle_nabla_u(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                   const double *hgrids);
int oracle_nabla_u_and_square(int geocode, int n01, int n02, int n03, const double *u, double *du,
                              double *ddu, int nord, const double *hgrids);
int oracle_nabla_u_square(int geocode, int n01, int n02, int n03, const double *u, double *ddu,
                          int nord, const double *hgrids);
int oracle_nabla_u_epsilon(int geocode, int n01, int n02, int n03, const double *u, double *du,
                           int nord, const double *hgrids, const double *eps);
int oracle_update_rhopol(int geocode, int n01, int n02, int n03, const double *u, int nord,
                         const double *hgrids, double eta, const double *dlogeps, double *rhopol,
                         double *rhores2);
int oracle_div_u_i_ref(int geocode, int n01, int n02, int n03, const double *u, double *du,
                       int nord, const double *hgrids);
int oracle_hamiltonian(const int *n, const int *bc, const double *a_kin, const double *psig,
                       const double *pot, double *rho, double *hpsig, double *ekin, double *epot);

#ifdef __cplusplus
}
#endif
#endif
