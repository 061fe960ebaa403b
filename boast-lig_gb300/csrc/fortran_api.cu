// Fortran-facing libconv layer: the procedures of the libconv module
// (BigDFT/libconv.f90:22-217), the size queries its pipeline sketch calls
// (:248-256) and the "alpha release" names (:298-459), exported the way
// gfortran calls an external procedure: lower-case name plus a trailing
// underscore, every argument by reference, and one hidden length (size_t)
// after the last argument for each CHARACTER argument.  The reference
// declares these procedures without bodies; the bodies here run the GPU
// library's plans (host arrays, staged through device memory).
//
// Fortran subroutines return nothing: each call records its status for the
// calling thread, read with libconv_status_(ierr) (0 = ok) and, as text,
// with libconv_gb300_last_error().
//
// Filter ids (get_filter_id): 1 SYM8_LP (wavelet low pass: s0s1 = dwt,
// s1s0 = idwt), 2 SYM8_MD (magic filter), 3 SYM8_MI (inverse magic filter),
// 4 SYM8_D1 (first derivative), 5 SYM8_D2 (second derivative, kinetic),
// 6 SYMICOMB8 (wavelet combined with the magic filter: s1s0 = s1tor,
// s0s1 = rtos1; LibconvBase.rb:250-262).  Boundary ids (get_bc_id) are the
// generator's (GenericConvolution2.rb:684-690): 'P' periodic 0, 'G' grow 1,
// 'S' shrink -1, 'F' free without growth 2.
#include <cctype>
#include <cstddef>
#include <cstring>

#include "../../include/libconv_gb300.h"
#include "../../include/libconv_fortran.h"
#include "lcg_plan.cuh"

using namespace lcg;

namespace {

thread_local int t_status = LIBCONV_OK;

enum FilId { FIL_LP = 1, FIL_MD = 2, FIL_MI = 3, FIL_D1 = 4, FIL_D2 = 5, FIL_COMB = 6 };

struct FilName { const char *name; int id; };
const FilName kFilters[] = {
    {"SYM8_LP", FIL_LP}, {"SYM8_MD", FIL_MD}, {"SYM8_MI", FIL_MI}, {"SYM8_IMD", FIL_MI},
    {"SYM8_D1", FIL_D1}, {"SYM8_D2", FIL_D2}, {"SYMICOMB8", FIL_COMB},
};
struct BcName { const char *name; int id; };
const BcName kBcs[] = {
    {"P", BC_PERIODIC}, {"G", BC_GROW}, {"S", BC_SHRINK}, {"F", BC_FREE},
    {"FG", BC_GROW}, {"FS", BC_SHRINK}, {"FD", BC_FREE},   // the generator's routine-name forms
};

int done(int st) {
    t_status = st;
    return st;
}

// Fortran CHARACTER argument (blank padded, length len) equals `want`,
// ignoring case and trailing blanks.
bool fstr_eq(const char *s, size_t len, const char *want) {
    while (len && s[len - 1] == ' ') --len;
    if (len != strlen(want)) return false;
    for (size_t i = 0; i < len; ++i)
        if (toupper((unsigned char)s[i]) != want[i]) return false;
    return true;
}

void fstr_set(char *s, size_t len, const char *v) {
    const size_t n = strlen(v);
    for (size_t i = 0; i < len; ++i) s[i] = i < n ? v[i] : ' ';
}

// Operator of a wavelet transform direction (s0s1: analysis, s1s0: synthesis).
int wavelet_op(int fil, bool s0s1) {
    if (fil == FIL_LP) return s0s1 ? OPID_DWT : OPID_IWT;
    if (fil == FIL_COMB) return s0s1 ? OPID_RTOS1 : OPID_S1TOR;
    return -1;
}
// Operator of a one-level (s0s0) convolution.
int conv_op(int fil) {
    switch (fil) {
    case FIL_MD: return OPID_MD;
    case FIL_MI: return OPID_IMD;
    case FIL_D1: return OPID_D1;
    case FIL_D2: return OPID_D2;
    default: return -1;
    }
}

int check_tp(const int *tp) {
    if (!tp) return report(LIBCONV_EARG, "tp must not be null");
    if (*tp != 8) return report(LIBCONV_EARG, "only tp = 8 (real(kind=8)) is built");
    return LIBCONV_OK;
}

int wav1d(int fil, bool s0s1, const int *d, const int *idim, const int *n, const int *bc,
          const int *nx, const int *ny, const int *narr, const double *a, const double *a_y,
          const double *x, double *y) {
    if (!d || !idim || !bc || !narr || !a || !a_y) return report(LIBCONV_EARG, "null argument");
    const int op = wavelet_op(fil, s0s1);
    if (op < 0) return report(LIBCONV_EARG, "filter is not a wavelet filter");
    // Fortran dimension index idim is 1-based
    auto f = op == OPID_DWT ? d_s0s1_1d_sym8 : op == OPID_IWT ? d_s1s0_1d_sym8
           : op == OPID_RTOS1 ? d_s0s1_1d_symicomb8 : d_s1s0_1d_symicomb8;
    return f(*d, *idim - 1, n, *bc, nx, ny, *narr, x, y, *a, *a_y);
}

int conv1d(int fil, const int *d, const int *idim, const int *n, const int *bc, const int *nx,
           const int *ny, const int *narr, const double *a, const double *a_x, const double *a_y,
           const double *x, double *y) {
    if (!d || !idim || !bc || !narr || !a || !a_x || !a_y) return report(LIBCONV_EARG, "null argument");
    const int op = conv_op(fil);
    if (op < 0) return report(LIBCONV_EARG, "filter is not a one-level convolution filter");
    if (op == OPID_D2) {
        double dot = 0.0;
        return d_s0s0_1d_sym8_d2_dotin(*d, *idim - 1, n, *bc, nx, ny, *narr, x, y, *a, *a_x, *a_y,
                                       &dot);
    }
    auto f = op == OPID_MD ? d_s0s0_1d_sym8_md : op == OPID_IMD ? d_s0s0_1d_sym8_imd
                                                                : d_s0s0_1d_sym8_d1;
    return f(*d, *idim - 1, n, *bc, nx, ny, *narr, x, y, *a, *a_x, *a_y);
}

int md(int op, const int *d, const int *n, const int *bc, const int *nx, const int *ny,
       const int *narr, const double *a, const double *a_x, const double *a_y, const double *x,
       double *y) {
    if (op < 0) return report(LIBCONV_EARG, "filter does not fit this procedure");
    if (!d || !narr || !a || !a_y) return report(LIBCONV_EARG, "null argument");
    return md_generic(op, *d, n, bc, nx, ny, *narr, *a, a_x ? *a_x : 0.0, *a_y, x, y);
}

int sum1d(int fil, const int *d, const int *n, const int *bc, const int *nx, const int *ny,
          const int *narr, const double *a, const double *a_x, const double *a_y, const double *x,
          double *y, double *dot) {
    if (!d || !narr || !a_x || !a_y) return report(LIBCONV_EARG, "null argument");
    const int op = conv_op(fil);
    if (op < 0) return report(LIBCONV_EARG, "filter is not a one-level convolution filter");
    return sum1d_generic(op, *d, n, bc, nx, ny, *narr, a, *a_x, *a_y, x, y, dot);
}

// Size queries: per-axis extents in the operator's units (pairs for the
// wavelet transforms), or the work size (elements: two ping-pong buffers of
// the largest intermediate).
int sizes(int op, const int *d, const int *n, const int *bc, int *in, int *out, int *work) {
    if (op < 0) return report(LIBCONV_EARG, "filter does not fit this procedure");
    if (!d) return report(LIBCONV_EARG, "null argument");
    long long inter = 0;
    int rc = extents(op, *d, n, bc, in, out, &inter);
    if (rc) return rc;
    if (work) {
        if (2 * inter > 0x7FFFFFFFLL) return report(LIBCONV_EARG, "work size exceeds a default integer");
        *work = (int)(2 * inter);
    }
    return LIBCONV_OK;
}

}  // namespace

extern "C" {

// ---- status ---------------------------------------------------------------------
void libconv_status_(int *status) {
    if (status) *status = t_status;
}

// ---- names and ids (libconv.f90:23-34) --------------------------------------------
void get_filter_id_(const char *name, int *id, size_t len) {
    if (!id) { done(report(LIBCONV_EARG, "null argument")); return; }
    *id = 0;
    for (const FilName &f : kFilters)
        if (name && fstr_eq(name, len, f.name)) { *id = f.id; done(LIBCONV_OK); return; }
    done(report(LIBCONV_EARG, "unknown filter name"));
}

void get_filter_name_(const int *id, char *name, size_t len) {
    if (!id || !name) { done(report(LIBCONV_EARG, "null argument")); return; }
    for (const FilName &f : kFilters)
        if (f.id == *id) { fstr_set(name, len, f.name); done(LIBCONV_OK); return; }
    fstr_set(name, len, "");
    done(report(LIBCONV_EARG, "unknown filter id"));
}

void get_bc_id_(const char *name, int *id, size_t len) {
    if (!id) { done(report(LIBCONV_EARG, "null argument")); return; }
    *id = 0;
    for (const BcName &b : kBcs)
        if (name && fstr_eq(name, len, b.name)) { *id = b.id; done(LIBCONV_OK); return; }
    done(report(LIBCONV_EBC, "unknown boundary condition name"));
}

void get_bc_name_(const int *id, char *name, size_t len) {
    if (!id || !name) { done(report(LIBCONV_EARG, "null argument")); return; }
    for (const BcName &b : kBcs)
        if (b.id == *id) { fstr_set(name, len, b.name); done(LIBCONV_OK); return; }
    fstr_set(name, len, "");
    done(report(LIBCONV_EBC, "unknown boundary condition id"));
}

// ---- size queries, in the argument order of the pipeline's calls
// (libconv.f90:248-256): (d, n, fil_id, bc, result) -----------------------------------
void get_s0s1_input_size_(const int *d, const int *n, const int *fil, const int *bc, int *nx) {
    done(fil ? sizes(wavelet_op(*fil, true), d, n, bc, nx, nullptr, nullptr)
             : report(LIBCONV_EARG, "null argument"));
}
void get_s0s1_output_size_(const int *d, const int *n, const int *fil, const int *bc, int *ny) {
    done(fil ? sizes(wavelet_op(*fil, true), d, n, bc, nullptr, ny, nullptr)
             : report(LIBCONV_EARG, "null argument"));
}
void get_s0s1_work_size_(const int *d, const int *n, const int *fil, const int *bc, int *nw) {
    done(fil ? sizes(wavelet_op(*fil, true), d, n, bc, nullptr, nullptr, nw)
             : report(LIBCONV_EARG, "null argument"));
}
void get_s1s0_input_size_(const int *d, const int *n, const int *fil, const int *bc, int *nx) {
    done(fil ? sizes(wavelet_op(*fil, false), d, n, bc, nx, nullptr, nullptr)
             : report(LIBCONV_EARG, "null argument"));
}
void get_s1s0_output_size_(const int *d, const int *n, const int *fil, const int *bc, int *ny) {
    done(fil ? sizes(wavelet_op(*fil, false), d, n, bc, nullptr, ny, nullptr)
             : report(LIBCONV_EARG, "null argument"));
}
void get_s1s0_work_size_(const int *d, const int *n, const int *fil, const int *bc, int *nw) {
    done(fil ? sizes(wavelet_op(*fil, false), d, n, bc, nullptr, nullptr, nw)
             : report(LIBCONV_EARG, "null argument"));
}
void get_s0s0_md_output_size_(const int *d, const int *n, const int *fil, const int *bc, int *ny) {
    done(fil ? sizes(conv_op(*fil), d, n, bc, nullptr, ny, nullptr)
             : report(LIBCONV_EARG, "null argument"));
}
void get_s0s0_md_work_size_(const int *d, const int *n, const int *fil, const int *bc, int *nw) {
    done(fil ? sizes(conv_op(*fil), d, n, bc, nullptr, nullptr, nw)
             : report(LIBCONV_EARG, "null argument"));
}
void get_s0s0_1ds_output_size_(const int *d, const int *n, const int *fil, const int *bc, int *ny) {
    if (!d || !n || !fil || !bc || !ny || *d < 1) { done(report(LIBCONV_EARG, "null argument")); return; }
    if (conv_op(*fil) < 0) { done(report(LIBCONV_EARG, "filter is not a one-level convolution filter")); return; }
    for (int i = 0; i < *d; ++i) ny[i] = n[i];   // summed sweeps keep the shape
    done(LIBCONV_OK);
}
void get_s0s0_1ds_work_size_(const int *d, const int *n, const int *fil, const int *bc, int *nw) {
    if (!d || !n || !fil || !bc || !nw || *d < 1) { done(report(LIBCONV_EARG, "null argument")); return; }
    long long t = 1;
    for (int i = 0; i < *d; ++i) t *= n[i];
    if (2 * t > 0x7FFFFFFFLL) { done(report(LIBCONV_EARG, "work size exceeds a default integer")); return; }
    *nw = (int)(2 * t);
    done(LIBCONV_OK);
}

// ---- generic procedures (libconv.f90:58-217) --------------------------------------------
void s0s1_1d_(const int *fil, const int *tp, const int *d, const int *idim, const int *n,
              const int *bc, const int *nx, const int *ny, const int *narr, const double *a,
              const double *a_y, const double *x, double *y) {
    int rc = check_tp(tp);
    done(rc ? rc : wav1d(fil ? *fil : 0, true, d, idim, n, bc, nx, ny, narr, a, a_y, x, y));
}
// The reference's interface of s1s0_1d omits idim (libconv.f90:77-91); the
// argument list here is that of s0s1_1d, as in its alpha form
// s1s0_1d_sym8_lp_d.
void s1s0_1d_(const int *fil, const int *tp, const int *d, const int *idim, const int *n,
              const int *bc, const int *nx, const int *ny, const int *narr, const double *a,
              const double *a_y, const double *x, double *y) {
    int rc = check_tp(tp);
    done(rc ? rc : wav1d(fil ? *fil : 0, false, d, idim, n, bc, nx, ny, narr, a, a_y, x, y));
}
void s0s1_md_(const int *fil, const int *tp, const int *d, const int *n, const int *bc,
              const int *nx, const int *ny, const int *narr, const double *a, const double *a_y,
              const double *x, double *y, double *work) {
    (void)work;
    int rc = check_tp(tp);
    done(rc ? rc : md(fil ? wavelet_op(*fil, true) : -1, d, n, bc, nx, ny, narr, a, nullptr, a_y, x, y));
}
void s1s0_md_(const int *fil, const int *tp, const int *d, const int *n, const int *bc,
              const int *nx, const int *ny, const int *narr, const double *a, const double *a_y,
              const double *x, double *y, double *work) {
    (void)work;
    int rc = check_tp(tp);
    done(rc ? rc : md(fil ? wavelet_op(*fil, false) : -1, d, n, bc, nx, ny, narr, a, nullptr, a_y, x, y));
}
void s0s0_1d_(const int *fil, const int *tp, const int *d, const int *idim, const int *n,
              const int *bc, const int *nx, const int *ny, const int *narr, const double *a,
              const double *a_x, const double *a_y, const double *x, double *y) {
    int rc = check_tp(tp);
    done(rc ? rc : conv1d(fil ? *fil : 0, d, idim, n, bc, nx, ny, narr, a, a_x, a_y, x, y));
}
void s0s0_1ds_(const int *fil, const int *tp, const int *d, const int *n, const int *bc,
               const int *nx, const int *ny, const int *narr, const double *a, const double *a_x,
               const double *a_y, const double *x, double *y, double *work) {
    (void)work;
    int rc = check_tp(tp);
    done(rc ? rc : sum1d(fil ? *fil : 0, d, n, bc, nx, ny, narr, a, a_x, a_y, x, y, nullptr));
}
void s0s0_1ds_dot_(const int *fil, const int *tp, const int *d, const int *n, const int *bc,
                   const int *nx, const int *ny, const int *narr, const double *a, const double *a_x,
                   const double *a_y, const double *x, double *y, double *dot_in, double *work) {
    (void)work;
    int rc = check_tp(tp);
    if (!rc && !dot_in) rc = report(LIBCONV_EARG, "dot_in must not be null");
    done(rc ? rc : sum1d(fil ? *fil : 0, d, n, bc, nx, ny, narr, a, a_x, a_y, x, y, dot_in));
}
void s0s0_md_(const int *fil, const int *tp, const int *d, const int *n, const int *bc,
              const int *nx, const int *ny, const int *narr, const double *a, const double *a_x,
              const double *a_y, const double *x, double *y, double *work) {
    (void)work;
    int rc = check_tp(tp);
    done(rc ? rc : md(fil ? conv_op(*fil) : -1, d, n, bc, nx, ny, narr, a, a_x, a_y, x, y));
}

// ---- alpha-release names (libconv.f90:298-459), real(kind=8) ---------------------------
void s0s1_1d_sym8_lp_d_(const int *d, const int *idim, const int *n, const int *bc, const int *nx,
                        const int *ny, const int *narr, const double *a, const double *a_y,
                        const double *x, double *y) {
    done(wav1d(FIL_LP, true, d, idim, n, bc, nx, ny, narr, a, a_y, x, y));
}
void s1s0_1d_sym8_lp_d_(const int *d, const int *idim, const int *n, const int *bc, const int *nx,
                        const int *ny, const int *narr, const double *a, const double *a_y,
                        const double *x, double *y) {
    done(wav1d(FIL_LP, false, d, idim, n, bc, nx, ny, narr, a, a_y, x, y));
}
void s0s1_sym8_lp_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                     const int *narr, const double *a, const double *a_y, const double *x,
                     double *y, double *work) {
    (void)work;
    done(md(OPID_DWT, d, n, bc, nx, ny, narr, a, nullptr, a_y, x, y));
}
void s1s0_sym8_lp_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                     const int *narr, const double *a, const double *a_y, const double *x,
                     double *y, double *work) {
    (void)work;
    done(md(OPID_IWT, d, n, bc, nx, ny, narr, a, nullptr, a_y, x, y));
}
void s0s0_1d_sym8_md_d_(const int *d, const int *idim, const int *n, const int *bc, const int *nx,
                        const int *ny, const int *narr, const double *a, const double *a_x,
                        const double *a_y, const double *x, double *y) {
    done(conv1d(FIL_MD, d, idim, n, bc, nx, ny, narr, a, a_x, a_y, x, y));
}
// Declared without arguments in the reference (libconv.f90:388-389); the
// arguments here are those of s0s0_1d_sym8_md_d.
void s0s0_1d_sym8_mi_d_(const int *d, const int *idim, const int *n, const int *bc, const int *nx,
                        const int *ny, const int *narr, const double *a, const double *a_x,
                        const double *a_y, const double *x, double *y) {
    done(conv1d(FIL_MI, d, idim, n, bc, nx, ny, narr, a, a_x, a_y, x, y));
}
void s0s0_1ds_sym8_d2_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                         const int *narr, const double *a, const double *a_x, const double *a_y,
                         const double *x, double *y, double *work) {
    (void)work;
    done(sum1d(FIL_D2, d, n, bc, nx, ny, narr, a, a_x, a_y, x, y, nullptr));
}
// Declared without arguments in the reference (libconv.f90:407-408).
void s0s0_1ds_sym8_d1_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                         const int *narr, const double *a, const double *a_x, const double *a_y,
                         const double *x, double *y, double *work) {
    (void)work;
    done(sum1d(FIL_D1, d, n, bc, nx, ny, narr, a, a_x, a_y, x, y, nullptr));
}
void s0s0_1ds_dot_sym8_d2_d_(const int *d, const int *n, const int *bc, const int *nx,
                             const int *ny, const int *narr, const double *a, const double *a_x,
                             const double *a_y, const double *x, double *y, double *dot_in,
                             double *work) {
    (void)work;
    done(dot_in ? sum1d(FIL_D2, d, n, bc, nx, ny, narr, a, a_x, a_y, x, y, dot_in)
                : report(LIBCONV_EARG, "dot_in must not be null"));
}
void s0s0_sym8_md_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                     const int *narr, const double *a, const double *a_x, const double *a_y,
                     const double *x, double *y, double *work) {
    (void)work;
    done(md(OPID_MD, d, n, bc, nx, ny, narr, a, a_x, a_y, x, y));
}
// Declared without arguments in the reference (libconv.f90:455-456).
void s0s0_sym8_mi_d_(const int *d, const int *n, const int *bc, const int *nx, const int *ny,
                     const int *narr, const double *a, const double *a_x, const double *a_y,
                     const double *x, double *y, double *work) {
    (void)work;
    done(md(OPID_IMD, d, n, bc, nx, ny, narr, a, a_x, a_y, x, y));
}

}  // extern "C"
