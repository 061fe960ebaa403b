/* Generated from libconv_gb300.h by boast-lig_gb300/build.py: the host-pointer
 * compute entry points with the void prototypes of the generated procedures
 * (scalars by value, arrays by pointer, no status), exported by
 * libconv_gb300_boast.so.  A failure is reported on stderr and aborts the
 * process; libconv_gb300.h gives the same procedures with an int status.
 * Include one of the two headers, not both. */
#ifndef LIBCONV_BOAST_H
#define LIBCONV_BOAST_H

#ifdef __cplusplus
extern "C" {
#endif

void d_s0s0_1d_sym8_md(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, const double *x, double *y, double a, double a_x, double a_y);
void d_s0s0_1d_sym8_imd(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, const double *x, double *y, double a, double a_x, double a_y);
void d_s0s0_1d_sym8_d1(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, const double *x, double *y, double a, double a_x, double a_y);
void d_s0s0_1d_sym8_d2_dotin(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, const double *x, double *y, double a, double a_x, double a_y, double *dot_in);
void d_s0s1_1d_sym8(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, const double *x, double *y, double a, double a_y);
void d_s1s0_1d_sym8(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, const double *x, double *y, double a, double a_y);
void d_s1s0_1d_symicomb8(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, const double *x, double *y, double a, double a_y);
void d_s0s1_1d_symicomb8(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, const double *x, double *y, double a, double a_y);
void d_sfrf_ld_narr(int d, const int *n, const int *bc, const int *nx, const int *ny, int narr, const double *x, double *y, double *w1, double *w2);
void d_rfsf_ld_narr(int d, const int *n, const int *bc, const int *nx, const int *ny, int narr, const double *x, double *y, double *w1, double *w2);
void d_kin(int d, const int *n, const int *bc, const double *x, double *y, double *w1, double *w2, const double *a, double a_x, double a_y);
void d_kin_ekin(int d, const int *n, const int *bc, const double *x, double *y, double *w1, double *w2, const double *a, double a_x, double a_y, double *kstrten);
void d_kin_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y, double *w1, double *w2, const double *a, double a_x, double a_y);
void d_dwt_sym8(int d, const int *n, const int *bc, const double *x, double *y, double *w1, double *w2);
void d_idwt_sym8(int d, const int *n, const int *bc, const double *x, double *y, double *w1, double *w2);
void d_dwt_sym8_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y, double *w1, double *w2);
void d_idwt_sym8_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y, double *w1, double *w2);
void Poisson_broker(int nord, int idim, const int *nn, int bc, const double *u, double *du, double a);
void div_u_i(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord, const double *hgrids, double *cc);
void nabla_u(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord, const double *hgrids);
void nabla_u_and_square(int geocode, int n01, int n02, int n03, const double *u, double *du, double *ddu, int nord, const double *hgrids);
void nabla_u_square(int geocode, int n01, int n02, int n03, const double *u, double *ddu, int nord, const double *hgrids);
void nabla_u_epsilon(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord, const double *hgrids, const double *eps);
void update_rhopol(int geocode, int n01, int n02, int n03, const double *u, int nord, const double *hgrids, double eta, const double *dlogeps, double *rhopol, double *rhores2);

#ifdef __cplusplus
}
#endif
#endif /* LIBCONV_BOAST_H */
