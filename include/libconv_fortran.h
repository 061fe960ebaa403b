/* libconv-gb300: Fortran-facing libconv procedures.
 *
 * The libconv module of BigDFT (BigDFT/libconv.f90) declares its procedures
 * as interfaces without bodies; this library gives them bodies on the GPU.
 * They are exported the way gfortran calls an external procedure: lower-case
 * name with a trailing underscore, every argument by reference, and one
 * hidden length (size_t) after the last argument for each CHARACTER
 * argument.  Fortran declares them as external subroutines, e.g.
 *     call s0s0_md(fil_id, 8, 3, n, bc, nx, ny, 1, 1.0d0, 0.0d0, 0.0d0, x, y, work)
 * Arrays are host arrays (Fortran order); the call returns when y holds the
 * result.  Work arrays are accepted and left untouched (the library stages
 * in its own device memory).
 *
 * Status: a Fortran subroutine returns nothing; every call records its
 * status for the calling thread (0 = ok, else a LIBCONV_E* code of
 * libconv_gb300.h), read with  call libconv_status(ierr).
 *
 * Ids: filters 1 SYM8_LP, 2 SYM8_MD, 3 SYM8_MI (alias SYM8_IMD), 4 SYM8_D1,
 * 5 SYM8_D2, 6 SYMICOMB8 (wavelet combined with the magic filter:
 * s1s0 = s1tor, s0s1 = rtos1); boundaries 'P' 0, 'G' 1, 'S' -1, 'F' 2 (also
 * the generator's 'FG', 'FS', 'FD').  tp (the real kind) must be 8.
 *
 * Semantics beyond the reference's interface comments:
 *   - wavelet extents n, nx, ny count coefficient pairs, as in
 *     libconv_gb300.h; idim is 1-based (a Fortran dimension index);
 *   - s0s1_md / s1s0_md / s0s0_md: y = a (F_d ... F_1 x) + a_y y, with a and
 *     a_y applied on the last sweep; a_x must be 0 unless d = 1 (the
 *     generated multi-dimensional dispatcher adds a_x x on its first sweep
 *     only, GenericConvolution2.rb:2040-2043, which is not a_x x of the
 *     product); the summed forms (s0s0_1ds*) take a_x for any d;
 *   - s0s0_1ds / s0s0_1ds_dot: y = sum_i a(i) F_i x + a_x x + a_y y with
 *     periodic or free (no-grow) boundaries and nx = ny = n; dot_in(i) =
 *     x . (a(i) F_i x), summed over the narr arrays.
 */
#ifndef LIBCONV_FORTRAN_H
#define LIBCONV_FORTRAN_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status of the calling thread's last libconv Fortran call (0 = ok).
 * Extension: no counterpart in the reference. */
void libconv_status_(int *status);

/* get_filter_id / get_filter_name / get_bc_id / get_bc_name
 * (libconv.f90:23-34). */
void get_filter_id_(const char *filt_name, int *filt_id, size_t filt_name_len);
void get_filter_name_(const int *filt_id, char *filt_name, size_t filt_name_len);
void get_bc_id_(const char *bc_name, int *bc_id, size_t bc_name_len);
void get_bc_name_(const int *bc_id, char *bc_name, size_t bc_name_len);

/* Size queries in the argument order of the pipeline's calls
 * (libconv.f90:248-256): (d, n(d), fil_id, bc(d), result).  Input/output
 * sizes are per-axis extents (pairs for the wavelet transforms); work sizes
 * are element counts.  The module's own get_s0s1_*_size interfaces
 * (libconv.f90:36-43) list four arguments; the pipeline calls them with five. */
void get_s0s1_input_size_(const int *d, const int *n, const int *fil_id, const int *bc, int *nx);
void get_s0s1_output_size_(const int *d, const int *n, const int *fil_id, const int *bc, int *ny);
void get_s0s1_work_size_(const int *d, const int *n, const int *fil_id, const int *bc, int *nwork);
void get_s1s0_input_size_(const int *d, const int *n, const int *fil_id, const int *bc, int *nx);
void get_s1s0_output_size_(const int *d, const int *n, const int *fil_id, const int *bc, int *ny);
void get_s1s0_work_size_(const int *d, const int *n, const int *fil_id, const int *bc, int *nwork);
void get_s0s0_md_output_size_(const int *d, const int *n, const int *fil_id, const int *bc,
                              int *ny);
void get_s0s0_md_work_size_(const int *d, const int *n, const int *fil_id, const int *bc,
                            int *nwork);
void get_s0s0_1ds_output_size_(const int *d, const int *n, const int *fil_id, const int *bc,
                               int *ny);
void get_s0s0_1ds_work_size_(const int *d, const int *n, const int *fil_id, const int *bc,
                             int *nwork);

/* s0s1_1d (libconv.f90:58-73): y = a dwt_i x + a_y y along dimension idim. */
void s0s1_1d_(const int *fil_id, const int *tp, const int *d, const int *idim, const int *n,
              const int *bc_id, const int *nx, const int *ny, const int *narr, const double *a,
              const double *a_y, const double *x, double *y);
/* s1s0_1d (libconv.f90:77-91, with the idim of s0s1_1d). */
void s1s0_1d_(const int *fil_id, const int *tp, const int *d, const int *idim, const int *n,
              const int *bc_id, const int *nx, const int *ny, const int *narr, const double *a,
              const double *a_y, const double *x, double *y);
/* s0s1_md / s1s0_md (libconv.f90:95-129). */
void s0s1_md_(const int *fil_id, const int *tp, const int *d, const int *n, const int *bc,
              const int *nx, const int *ny, const int *narr, const double *a, const double *a_y,
              const double *x, double *y, double *work);
void s1s0_md_(const int *fil_id, const int *tp, const int *d, const int *n, const int *bc,
              const int *nx, const int *ny, const int *narr, const double *a, const double *a_y,
              const double *x, double *y, double *work);
/* s0s0_1d (libconv.f90:137-153). */
void s0s0_1d_(const int *fil_id, const int *tp, const int *d, const int *idim, const int *n,
              const int *bc_id, const int *nx, const int *ny, const int *narr, const double *a,
              const double *a_x, const double *a_y, const double *x, double *y);
/* s0s0_1ds / s0s0_1ds_dot (libconv.f90:157-192); dot_in: d doubles. */
void s0s0_1ds_(const int *fil_id, const int *tp, const int *d, const int *n, const int *bc,
               const int *nx, const int *ny, const int *narr, const double *a, const double *a_x,
               const double *a_y, const double *x, double *y, double *work);
void s0s0_1ds_dot_(const int *fil_id, const int *tp, const int *d, const int *n, const int *bc,
                   const int *nx, const int *ny, const int *narr, const double *a,
                   const double *a_x, const double *a_y, const double *x, double *y,
                   double *dot_in, double *work);
/* s0s0_md (libconv.f90:201-217). */
void s0s0_md_(const int *fil_id, const int *tp, const int *d, const int *n, const int *bc,
              const int *nx, const int *ny, const int *narr, const double *a, const double *a_x,
              const double *a_y, const double *x, double *y, double *work);

/* Alpha-release names, real(kind=8) (libconv.f90:298-459). */
void s0s1_1d_sym8_lp_d_(const int *d, const int *idim, const int *n, const int *bc_id,
                        const int *nx, const int *ny, const int *narr, const double *a,
                        const double *a_y, const double *x, double *y);
void s1s0_1d_sym8_lp_d_(const int *d, const int *idim, const int *n, const int *bc_id,
                        const int *nx, const int *ny, const int *narr, const double *a,
                        const double *a_y, const double *x, double *y);
void s0s1_sym8_lp_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                     const int *narr, const double *a, const double *a_y, const double *x,
                     double *y, double *work);
void s1s0_sym8_lp_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                     const int *narr, const double *a, const double *a_y, const double *x,
                     double *y, double *work);
void s0s0_1d_sym8_md_d_(const int *d, const int *idim, const int *n, const int *bc_id,
                        const int *nx, const int *ny, const int *narr, const double *a,
                        const double *a_x, const double *a_y, const double *x, double *y);
/* Declared without arguments in the reference (:388-389); arguments as
 * s0s0_1d_sym8_md_d. */
void s0s0_1d_sym8_mi_d_(const int *d, const int *idim, const int *n, const int *bc_id,
                        const int *nx, const int *ny, const int *narr, const double *a,
                        const double *a_x, const double *a_y, const double *x, double *y);
void s0s0_1ds_sym8_d2_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                         const int *narr, const double *a, const double *a_x, const double *a_y,
                         const double *x, double *y, double *work);
/* Declared without arguments in the reference (:407-408); arguments as
 * s0s0_1ds_sym8_d2_d. */
void s0s0_1ds_sym8_d1_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                         const int *narr, const double *a, const double *a_x, const double *a_y,
                         const double *x, double *y, double *work);
void s0s0_1ds_dot_sym8_d2_d_(const int *d, const int *n, const int *bc, const int *nx,
                             const int *ny, const int *narr, const double *a, const double *a_x,
                             const double *a_y, const double *x, double *y, double *dot_in,
                             double *work);
void s0s0_sym8_md_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                     const int *narr, const double *a, const double *a_x, const double *a_y,
                     const double *x, double *y, double *work);
/* Declared without arguments in the reference (:455-456); arguments as
 * s0s0_sym8_md_d. */
void s0s0_sym8_mi_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                     const int *narr, const double *a, const double *a_x, const double *a_y,
                     const double *x, double *y, double *work);

#ifdef __cplusplus
}
#endif
#endif
