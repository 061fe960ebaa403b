/* CPU oracle for libconv-gb300 -- TEST INFRASTRUCTURE ONLY (see libconv_oracle.h).
 *
 * Plain C99, FP64, single-threaded, compiled with -ffp-contract=off so that
 * the x86 and aarch64 builds give the same bits.  Tap order and
 * post-processing order follow the reference line by line (citations inline).
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include "libconv_oracle.h"
#include "../boast-lig_gb300/csrc/libconv_filters.h"

/* Boundary-condition ids: GenericConvolution2.rb:684-689. */
enum { BC_SHRINK = -1, BC_PERIODIC = 0, BC_GROW = 1, BC_FREE = 2 };
/* Error codes shared with the GPU library (include/libconv_gb300.h). */
enum { OK = 0, E_ARG = -1, E_BC = -2, E_SIZE = -3 };
enum { K_CONV = 0, K_DEC = 1, K_REC = 2 };

static int imod(int a, int n) { int r = a % n; return r < 0 ? r + n : r; }

/* ======================================================================
 * Fortran reference kernels
 * ====================================================================== */

/* BigDFT/magicfilter_refs.f90:92-133.  x(0:n1-1,ndat) -> y(ndat,0:n1-1). */
void oracle_magicfilter_per_ref(int n1, int ndat, const double *x, double *y)
{
    for (int j = 0; j < ndat; ++j)
        for (int i = 0; i < n1; ++i) {
            double tt = 0.0;
            for (int l = -8; l <= 7; ++l)
                tt = tt + x[imod(i + l, n1) + (size_t)n1 * j] * LCG_MF_FORTRAN[l + 8];
            y[j + (size_t)ndat * i] = tt;
        }
}

/* BigDFT/magicfilter_refs.f90:135-181: reversed filter, lowfil=-7. */
void oracle_magicfilter_per_t_ref(int n1, int ndat, const double *x, double *y)
{
    for (int j = 0; j < ndat; ++j)
        for (int i = 0; i < n1; ++i) {
            double tt = 0.0;
            for (int l = -7; l <= 8; ++l)
                tt = tt + x[imod(i + l, n1) + (size_t)n1 * j] * LCG_MF_FORTRAN[15 - (l + 7)];
            y[j + (size_t)ndat * i] = tt;
        }
}

/* BigDFT/magicfilter_refs.f90:2-44: grow, y(ndat,-7:n1+7), clipped taps. */
void oracle_magicfilter_free_ref(int n1, int ndat, const double *x, double *y)
{
    for (int j = 0; j < ndat; ++j)
        for (int i = -7; i <= n1 - 1 + 8; ++i) {
            double tt = 0.0;
            int lo = -i > -8 ? -i : -8, hi = 7 < n1 - 1 - i ? 7 : n1 - 1 - i;
            for (int l = lo; l <= hi; ++l)
                tt = tt + x[(i + l) + (size_t)n1 * j] * LCG_MF_FORTRAN[l + 8];
            y[j + (size_t)ndat * (i + 7)] = tt;
        }
}

/* BigDFT/magicfilter_refs.f90:48-90: shrink, x(-7:n1+7,ndat) -> y(ndat,0:n1-1). */
void oracle_magicfilter_free_t_ref(int n1, int ndat, const double *x, double *y)
{
    const int ext = n1 + 15;
    for (int j = 0; j < ndat; ++j)
        for (int i = 0; i < n1; ++i) {
            double tt = 0.0;
            for (int l = -7; l <= 8; ++l)
                tt = tt + x[(i + l + 7) + (size_t)ext * j] * LCG_MF_FORTRAN[15 - (l + 7)];
            y[j + (size_t)ndat * i] = tt;
        }
}

/* BigDFT/Kinetic2.rb:981-1061 (kinetic_per_ref): y = c*x + sum_d scale_d*D2_d x,
 * scale_d = -0.5/h_d^2 folded into the filter as the Fortran does. */
void oracle_kinetic_per_ref(int n1, int n2, int n3, const double *hgrid,
                            const double *x, double *y, double c)
{
    double fil[3][29];
    for (int d = 0; d < 3; ++d) {
        double scale = -0.5 / (hgrid[d] * hgrid[d]);
        for (int i = 0; i <= 14; ++i) {
            fil[d][14 + i] = LCG_KIN_FORTRAN[i] * scale;
            fil[d][14 - i] = fil[d][14 + i];
        }
    }
#define X(a, b, c_) x[(a) + (size_t)n1 * ((b) + (size_t)n2 * (c_))]
#define Y(a, b, c_) y[(a) + (size_t)n1 * ((b) + (size_t)n2 * (c_))]
    for (int i3 = 0; i3 < n3; ++i3) {
        for (int i2 = 0; i2 < n2; ++i2)
            for (int i1 = 0; i1 < n1; ++i1) {
                double tt = X(i1, i2, i3) * c;
                for (int l = -14; l <= 14; ++l)
                    tt = tt + X(imod(i1 + l, n1), i2, i3) * fil[0][l + 14];
                Y(i1, i2, i3) = tt;
            }
        for (int i1 = 0; i1 < n1; ++i1)
            for (int i2 = 0; i2 < n2; ++i2) {
                double tt = 0.0;
                for (int l = -14; l <= 14; ++l)
                    tt = tt + X(i1, imod(i2 + l, n2), i3) * fil[1][l + 14];
                Y(i1, i2, i3) = Y(i1, i2, i3) + tt;
            }
    }
    for (int i2 = 0; i2 < n2; ++i2)
        for (int i1 = 0; i1 < n1; ++i1)
            for (int i3 = 0; i3 < n3; ++i3) {
                double tt = 0.0;
                for (int l = -14; l <= 14; ++l)
                    tt = tt + X(i1, i2, imod(i3 + l, n3)) * fil[2][l + 14];
                Y(i1, i2, i3) = Y(i1, i2, i3) + tt;
            }
#undef X
#undef Y
}

/* ch(-8:9), cg(-8:9) of old/Synthesis.rb:32-47: the 16 Daubechies taps
 * padded with one zero on each side. */
static double ch_s(int m) { return (m < -7 || m > 8) ? 0.0 : LCG_CH_FORTRAN[m + 7]; }
static double cg_s(int m) { return (m < -7 || m > 8) ? 0.0 : LCG_CG_FORTRAN[m + 7]; }

/* old/Synthesis.rb:100-146: x(0:2n-1,ndat) [s|d] -> y(ndat,0:2n-1) interleaved. */
void oracle_synthesis_per_ref(int n, int ndat, const double *x, double *y)
{
    for (int j = 0; j < ndat; ++j) {
        const double *xj = x + (size_t)2 * n * j;
        for (int i = 0; i < n; ++i) {
            double se = 0.0, so = 0.0;
            for (int l = -4; l <= 4; ++l) {
                int k = imod(i - l, n);
                se = se + ch_s(2 * l) * xj[k] + cg_s(2 * l) * xj[n + k];
                so = so + ch_s(2 * l + 1) * xj[k] + cg_s(2 * l + 1) * xj[n + k];
            }
            y[j + (size_t)ndat * (2 * i)] = se;
            y[j + (size_t)ndat * (2 * i + 1)] = so;
        }
    }
}

/* old/Synthesis.rb:23-82: free (grow), y(ndat,-7:2n+6). */
void oracle_synthesis_free_ref(int n, int ndat, const double *x, double *y)
{
#define YF(jj, m) y[(jj) + (size_t)ndat * ((m) + 7)]
    for (int j = 0; j < ndat; ++j) {
        const double *xj = x + (size_t)2 * n * j;
        int i = -4;
        double so = 0.0, se;
        for (int l = (i - n + 1 > -4 ? i - n + 1 : -4); l <= (i < 4 ? i : 4); ++l)
            so = so + ch_s(2 * l + 1) * xj[i - l] + cg_s(2 * l + 1) * xj[n + i - l];
        YF(j, 2 * i + 1) = so;
        for (i = -3; i <= n + 2; ++i) {
            se = 0.0; so = 0.0;
            for (int l = (i - n + 1 > -4 ? i - n + 1 : -4); l <= (i < 4 ? i : 4); ++l) {
                se = se + ch_s(2 * l) * xj[i - l] + cg_s(2 * l) * xj[n + i - l];
                so = so + ch_s(2 * l + 1) * xj[i - l] + cg_s(2 * l + 1) * xj[n + i - l];
            }
            YF(j, 2 * i) = se;
            YF(j, 2 * i + 1) = so;
        }
        i = n + 3;
        se = 0.0;
        for (int l = (i - n + 1 > -4 ? i - n + 1 : -4); l <= (i < 4 ? i : 4); ++l)
            se = se + ch_s(2 * l) * xj[i - l] + cg_s(2 * l) * xj[n + i - l];
        YF(j, 2 * i) = se;
    }
#undef YF
}

/* Periodic analysis.  The live reference (old/AnaRotPer-2.rb:86-221) is an
 * unrolled form sized 0:2n+1 with a modulo table; its plain form is kept in
 * the same file (:258-296): ci = sum_{l=-7..8} ch(l) x(mod(l+2i,2n)). */
void oracle_analysis_per_ref(int n, int ndat, const double *x, double *y)
{
    for (int j = 0; j < ndat; ++j) {
        const double *xj = x + (size_t)2 * n * j;
        for (int i = 0; i < n; ++i) {
            double ci = 0.0, di = 0.0;
            for (int l = -7; l <= 8; ++l) {
                int k = imod(l + 2 * i, 2 * n);
                ci = ci + LCG_CH_FORTRAN[l + 7] * xj[k];
                di = di + LCG_CG_FORTRAN[l + 7] * xj[k];
            }
            y[j + (size_t)ndat * i] = ci;
            y[j + (size_t)ndat * (n + i)] = di;
        }
    }
}

/* old/AnaRotPer-2.rb:22-64: free (shrink), x(-7:2n+6,ndat) -> y(ndat,0:2n-1). */
void oracle_analysis_free_ref(int n, int ndat, const double *x, double *y)
{
    for (int j = 0; j < ndat; ++j) {
        const double *xj = x + (size_t)(2 * n + 14) * j;
        for (int i = 0; i < n; ++i) {
            double ci = 0.0, di = 0.0;
            for (int l = -7; l <= 8; ++l) {
                ci = ci + LCG_CH_FORTRAN[l + 7] * xj[l + 2 * i + 7];
                di = di + LCG_CG_FORTRAN[l + 7] * xj[l + 2 * i + 7];
            }
            y[j + (size_t)ndat * i] = ci;
            y[j + (size_t)ndat * (n + i)] = di;
        }
    }
}

/* ======================================================================
 * Generated 1D operator (ConvolutionOperator1d, GenericConvolution2.rb)
 * ====================================================================== */

typedef struct {
    int kind;       /* K_CONV, K_DEC (s0s1) or K_REC (s1s0) */
    int lowfil;     /* first tap (polyphase taps for wavelets) */
    int ntaps;
    int length;     /* filter.length: taps (conv) or full low-pass length (wavelets) */
    const double *f;                    /* conv taps, index l - lowfil */
    const double *le, *lo, *he, *ho;    /* wavelet polyphase filters */
} ofilt;

typedef struct {
    int nL, n, nR;          /* ndat_left, processed size (pairs for wavelets), ndat_right */
    int ld, nx, ny;         /* processed-dim leading sizes (pairs for wavelets) */
    int transpose;          /* 1: output index rotated (only with nL == 1) */
    const double *x, *x2;
    double *y;
    int has_a;  double a;
    int has_ax; double a_x;
    int ay_mode; double a_y;  /* 0: y written, 1: y = a_y*y + out, 2: y = y + out */
    double *dot;              /* accumulated when non-NULL */
} ocall;

static int upfil_of(const ofilt *F) { return F->lowfil + F->ntaps - 1; }

/* Input bounds of the processed dim (GenericConvolution2.rb:61-72, 206-223). */
static void in_bounds(const ofilt *F, int bc, const ocall *c, int *lo, int *ext)
{
    if (bc == BC_SHRINK) { *lo = F->lowfil; *ext = c->ld ? c->nx : c->n + upfil_of(F) - F->lowfil; }
    else { *lo = 0; *ext = c->ld ? c->nx : c->n; }
}
/* Output bounds (GenericConvolution2.rb:74-85, 215-225). */
static void out_bounds(const ofilt *F, int bc, const ocall *c, int *lo, int *ext)
{
    if (bc == BC_GROW) { *lo = -upfil_of(F); *ext = c->ld ? c->ny : c->n + upfil_of(F) - F->lowfil; }
    else { *lo = 0; *ext = c->ld ? c->ny : c->n; }
}

/* Offset of (position pos, channel ch) inside one line of the processed dim. */
static size_t proc_off(int layout_interleaved, int pos, int ch, int ext)
{
    return layout_interleaved ? (size_t)ch + 2 * (size_t)pos : (size_t)pos + (size_t)ext * ch;
}

static void conv1d(const ofilt *F, int bc, const ocall *c)
{
    const int wav = F->kind != K_CONV;
    const int nch = wav ? 2 : 1;
    int ilo, iext, olo, oext;
    in_bounds(F, bc, c, &ilo, &iext);
    out_bounds(F, bc, c, &olo, &oext);
    const size_t ipext = (size_t)iext * nch, opext = (size_t)oext * nch;
    const int in_il = F->kind == K_DEC;   /* decompose input interleaved x(0:1, p) */
    const int out_il = F->kind == K_REC;  /* recompose output interleaved y(0:1, q) */
    const int up = upfil_of(F);
    const int qlo = bc == BC_GROW ? -up : 0;
    const int qhi = bc == BC_GROW ? c->n - F->lowfil - 1 : c->n - 1;
    const int clip = (bc == BC_GROW || bc == BC_FREE);

    for (int r = 0; r < c->nR; ++r)
        for (int l = 0; l < c->nL; ++l) {
#define XIN(pos, ch) c->x[(size_t)l + (size_t)c->nL * (proc_off(in_il, (pos), (ch), iext) + ipext * r)]
            for (int q = qlo; q <= qhi; ++q) {
                int lmin = F->lowfil, lmax = up;
                if (clip) {   /* GenericConvolution2.rb:91-104, clipped on both sides */
                    if (lmin < -q) lmin = -q;
                    if (lmax > c->n - 1 - q) lmax = c->n - 1 - q;
                }
                double o0 = 0.0, o1 = 0.0;
                for (int t = lmin; t <= lmax; ++t) {
                    int p = q + t;
                    if (bc == BC_PERIODIC) p = imod(p, c->n);
                    int pos = p - ilo;
                    int k = t - F->lowfil;
                    if (F->kind == K_CONV) {
                        o0 = o0 + XIN(pos, 0) * F->f[k];                /* :168-171 */
                    } else if (F->kind == K_DEC) {                      /* :453-462, 471-476 */
                        double x0 = XIN(pos, 0), x1 = XIN(pos, 1);
                        o0 = o0 + x0 * F->le[k];
                        o1 = o1 + x0 * F->he[k];
                        o0 = o0 + x1 * F->lo[k];
                        o1 = o1 + x1 * F->ho[k];
                    } else {                                            /* :453-462, 600-605 */
                        double s = XIN(pos, 0), dd = XIN(pos, 1);
                        o0 = o0 + s * F->lo[k];
                        o1 = o1 + s * F->le[k];
                        o0 = o0 + dd * F->ho[k];
                        o1 = o1 + dd * F->he[k];
                    }
                }
                double outv[2] = { o0, o1 };
                for (int ch = 0; ch < nch; ++ch) {
                    double out = outv[ch];
                    if (c->has_a) out = out * c->a;                     /* :177 / :469-472 */
                    size_t oo = proc_off(out_il, q - olo, ch, oext);
                    size_t yi = c->transpose ? (size_t)r + (size_t)c->nR * oo
                                             : (size_t)l + (size_t)c->nL * (oo + opext * r);
                    if (!wav) {
                        /* :179-190: dot_in before a_x; grow only inside the input */
                        if ((c->dot || c->has_ax) && (bc != BC_GROW || (q >= 0 && q < c->n))) {
                            double xq = XIN(q - ilo, 0);
                            if (c->dot) *c->dot = *c->dot + xq * out;
                            if (c->has_ax) out = xq * c->a_x + out;
                        }
                        if (c->x2) {                                    /* :193 */
                            size_t x2i = bc == BC_GROW ? yi
                                : (size_t)l + (size_t)c->nL * ((size_t)(q - ilo) + ipext * r);
                            out = out + c->x2[x2i];
                        }
                    }
                    if (c->ay_mode == 2) out = out + c->y[yi];          /* :195-199 */
                    else if (c->ay_mode == 1) out = c->a_y * c->y[yi] + out;
                    c->y[yi] = out;
                }
            }
#undef XIN
        }
}

/* ---- filter objects ---- */
static const ofilt F_MD = { K_CONV, LCG_CONV_SYM8_MD_LOWFIL, 16, 16, LCG_CONV_SYM8_MD, 0, 0, 0, 0 };
static const ofilt F_IMD = { K_CONV, LCG_CONV_SYM8_IMD_LOWFIL, 16, 16, LCG_CONV_SYM8_IMD, 0, 0, 0, 0 };
static const ofilt F_D2 = { K_CONV, LCG_CONV_SYM8_D2_LOWFIL, 29, 29, LCG_SYM8_D2, 0, 0, 0, 0 };
static const ofilt F_D1 = { K_CONV, LCG_CONV_SYM8_D1_LOWFIL, 29, 29, LCG_SYM8_D1, 0, 0, 0, 0 };
#define WT(TAG, KIND) { KIND, TAG##_LOWFIL, TAG##_NTAPS, TAG##_LENGTH, 0, TAG##_LE, TAG##_LO, TAG##_HE, TAG##_HO }
static const ofilt F_DWT_P = WT(LCG_WT_SYM8_DEC_P, K_DEC);
static const ofilt F_DWT_GS = WT(LCG_WT_SYM8_DEC_GS, K_DEC);
static const ofilt F_IWT_P = WT(LCG_WT_SYM8_REC_P, K_REC);
static const ofilt F_IWT_GS = WT(LCG_WT_SYM8_REC_GS, K_REC);
static const ofilt F_RTOS1_P = WT(LCG_WT_SYMICOMB8_DEC_P, K_DEC);
static const ofilt F_RTOS1_GS = WT(LCG_WT_SYMICOMB8_DEC_GS, K_DEC);
static const ofilt F_S1TOR_P = WT(LCG_WT_SYMICOMB8_REC_P, K_REC);
static const ofilt F_S1TOR_GS = WT(LCG_WT_SYMICOMB8_REC_GS, K_REC);

static int bc_ok(int bc) { return bc == BC_PERIODIC || bc == BC_GROW || bc == BC_SHRINK || bc == BC_FREE; }

/* Required extents of the processed dim (pairs for wavelets). */
static int need_in(const ofilt *F, int bc, int n) { return bc == BC_SHRINK ? n + F->ntaps - 1 : n; }
static int need_out(const ofilt *F, int bc, int n) { return bc == BC_GROW ? n + F->ntaps - 1 : n; }

/* ======================================================================
 * 1D dispatcher: GenericConvolutionOperator1d#procedure, GenericConvolution2.rb:1560-1764
 * d_<base>_1d_<fil>(d, idim, n[], bc, nx[], ny[], narr, x, y, a, [a_x,] a_y [, dot_in])
 * ====================================================================== */
static int disp1d(const ofilt *Fp, const ofilt *Fgs, int d, int idim, const int *n, int bc,
                  const int *nx, const int *ny, int narr, const double *x, double *y,
                  double a, int use_ax, double a_x, double a_y, double *dot_in)
{
    if (d < 1 || idim < 0 || idim >= d || narr < 1 || !n || !nx || !ny || !x || !y) return E_ARG;
    if (!bc_ok(bc)) return E_BC;
    const ofilt *F = (bc == BC_GROW || bc == BC_SHRINK) ? Fgs : Fp;
    const int mul = F->kind == K_CONV ? 1 : 2;
    for (int i = 0; i < d; ++i) if (n[i] < 1 || nx[i] < 1 || ny[i] < 1) return E_ARG;
    if (nx[idim] < need_in(F, bc, n[idim]) || ny[idim] < need_out(F, bc, n[idim])) return E_SIZE;
    long nL = 1, nR = 1;
    for (int i = 0; i < idim; ++i) nL *= (long)nx[i] * mul;       /* :1725-1733 */
    for (int i = idim + 1; i < d; ++i) nR *= (long)nx[i] * mul;
    size_t nti = (size_t)nx[idim] * mul * nL * nR, nto = (size_t)ny[idim] * mul * nL * nR;
    ocall c = { (int)nL, n[idim], (int)nR, 1, nx[idim], ny[idim], 0, 0, 0, 0,
                a != 1.0, a, use_ax && a_x != 0.0, a_x, a_y != 0.0 ? 1 : 0, a_y, 0 };
    double acc = 0.0;
    if (dot_in) c.dot = &acc;
    for (int j = 0; j < narr; ++j) {                                  /* :1611-1618 */
        c.x = x + nti * j;
        c.y = y + nto * j;
        conv1d(F, bc, &c);
    }
    if (dot_in) *dot_in = acc;   /* sum over the narr arrays */
    return OK;
}

int oracle_d_s0s0_1d_sym8_md(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                             int narr, const double *x, double *y, double a, double a_x, double a_y)
{ return disp1d(&F_MD, &F_MD, d, idim, n, bc, nx, ny, narr, x, y, a, 1, a_x, a_y, 0); }
int oracle_d_s0s0_1d_sym8_imd(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                              int narr, const double *x, double *y, double a, double a_x, double a_y)
{ return disp1d(&F_IMD, &F_IMD, d, idim, n, bc, nx, ny, narr, x, y, a, 1, a_x, a_y, 0); }
int oracle_d_s0s0_1d_sym8_d1(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                             int narr, const double *x, double *y, double a, double a_x, double a_y)
{ return disp1d(&F_D1, &F_D1, d, idim, n, bc, nx, ny, narr, x, y, a, 1, a_x, a_y, 0); }
int oracle_d_s0s0_1d_sym8_d2_dotin(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                                   int narr, const double *x, double *y, double a, double a_x,
                                   double a_y, double *dot_in)
{
    double dummy;
    return disp1d(&F_D2, &F_D2, d, idim, n, bc, nx, ny, narr, x, y, a, 1, a_x, a_y,
                  dot_in ? dot_in : &dummy);
}
int oracle_d_s0s1_1d_sym8(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                          int narr, const double *x, double *y, double a, double a_y)
{ return disp1d(&F_DWT_P, &F_DWT_GS, d, idim, n, bc, nx, ny, narr, x, y, a, 0, 0.0, a_y, 0); }
int oracle_d_s1s0_1d_sym8(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                          int narr, const double *x, double *y, double a, double a_y)
{ return disp1d(&F_IWT_P, &F_IWT_GS, d, idim, n, bc, nx, ny, narr, x, y, a, 0, 0.0, a_y, 0); }
int oracle_d_s0s1_1d_symicomb8(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                               int narr, const double *x, double *y, double a, double a_y)
{ return disp1d(&F_RTOS1_P, &F_RTOS1_GS, d, idim, n, bc, nx, ny, narr, x, y, a, 0, 0.0, a_y, 0); }
int oracle_d_s1s0_1d_symicomb8(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                               int narr, const double *x, double *y, double a, double a_y)
{ return disp1d(&F_S1TOR_P, &F_S1TOR_GS, d, idim, n, bc, nx, ny, narr, x, y, a, 0, 0.0, a_y, 0); }

/* ======================================================================
 * Multi-D transposed dispatcher (transpose = 1): GenericConvolution2.rb:1934-2243
 * used by MagicFilter() (ld, narr, work) and Wavelet() (work).
 * Each sweep is shape [1,0] with the output index rotated, so after d
 * sweeps the array is back in its original orientation.
 * ====================================================================== */
static int dispmd_t(const ofilt *Fp, const ofilt *Fgs, int d, const int *n, const int *bc,
                    const int *nx, const int *ny, int narr, const double *x, double *y,
                    double *w1, double *w2)
{
    if (d < 1 || d > 16 || narr < 1 || !n || !bc || !x || !y) return E_ARG;
    if (d > 1 && (!w1 || (d > 2 && !w2))) return E_ARG;
    const int ld = nx != 0;
    if (ld && !ny) return E_ARG;
    long dims[16];
    const int mul = Fp->kind == K_CONV ? 1 : 2;
    for (int i = 0; i < d; ++i) {
        if (n[i] < 1) return E_ARG;
        if (!bc_ok(bc[i])) return E_BC;
        const ofilt *F = (bc[i] == BC_GROW || bc[i] == BC_SHRINK) ? Fgs : Fp;
        if (ld) {
            if (nx[i] < need_in(F, bc[i], n[i]) || ny[i] < need_out(F, bc[i], n[i])) return E_SIZE;
            dims[i] = (long)nx[i] * mul;                                 /* :1966-1972 */
        } else {
            dims[i] = (long)need_in(F, bc[i], n[i]) * mul;                /* :1973-1984 */
        }
    }
    for (int i = 0; i < d; ++i) {
        const ofilt *F = (bc[i] == BC_GROW || bc[i] == BC_SHRINK) ? Fgs : Fp;
        long ndat = 1;
        for (int j = 0; j < d; ++j) if (j != i) ndat *= dims[j];
        const double *src;
        double *dst;
        if (d == 1) { src = x; dst = y; }
        else if (i == 0) { src = x; dst = w1; }
        else if (i == d - 1) { src = ((d - 1) % 2 == 1) ? w1 : w2; dst = y; }
        else { src = (i % 2 == 1) ? w1 : w2; dst = (i % 2 == 1) ? w2 : w1; }
        /* ping-pong of :2155-2240: w1->w2 on odd sweeps, w2->w1 on even ones,
         * the last sweep writes y */
        long out_ext = ld ? (long)ny[i] * mul : (long)need_out(F, bc[i], n[i]) * mul;
        ocall c = { 1, n[i], (int)ndat, ld, ld ? nx[i] : 0, ld ? ny[i] : 0, 1, 0, 0, 0,
                    0, 1.0, 0, 0.0, 0, 0.0, 0 };
        size_t nti = (size_t)ndat * dims[i], nto = (size_t)ndat * out_ext;
        for (int j = 0; j < narr; ++j) {
            c.x = src + nti * j;
            c.y = dst + nto * j;
            conv1d(F, bc[i], &c);
        }
        dims[i] = out_ext;
    }
    return OK;
}

int oracle_d_sfrf_ld_narr(int d, const int *n, const int *bc, const int *nx, const int *ny,
                          int narr, const double *x, double *y, double *w1, double *w2)
{ return dispmd_t(&F_MD, &F_MD, d, n, bc, nx, ny, narr, x, y, w1, w2); }
int oracle_d_rfsf_ld_narr(int d, const int *n, const int *bc, const int *nx, const int *ny,
                          int narr, const double *x, double *y, double *w1, double *w2)
{ return dispmd_t(&F_IMD, &F_IMD, d, n, bc, nx, ny, narr, x, y, w1, w2); }
int oracle_d_dwt_sym8(int d, const int *n, const int *bc, const double *x, double *y,
                      double *w1, double *w2)
{ return dispmd_t(&F_DWT_P, &F_DWT_GS, d, n, bc, 0, 0, 1, x, y, w1, w2); }
int oracle_d_idwt_sym8(int d, const int *n, const int *bc, const double *x, double *y,
                       double *w1, double *w2)
{ return dispmd_t(&F_IWT_P, &F_IWT_GS, d, n, bc, 0, 0, 1, x, y, w1, w2); }

/* ======================================================================
 * Multi-D kinetic dispatcher (transpose = 0, kinetic, zero_out_work):
 * Kinetic2.rb:1068-1090 with GenericConvolution2.rb:2155-2240.
 *   sweep 0 (shape [1,0]):     w1 = a[0] D x + a_x x
 *   middle  (shape [2,0,1]):   w' = a[i] D_i x + w
 *   last    (shape [0,1]):     y  = a[d-1] D x + w + a_y y
 * Only size-preserving BCs (periodic, free no-grow): every sweep re-reads
 * the original x, so grow/shrink shapes cannot be chained.
 * ====================================================================== */
/* kinetic_per_ref_optim_ekin (BigDFT/Kinetic2.rb:21-112, conv_kin_x/y/z
 * 115-372): y += sum_d tt_d with tt_d = sum_l fil_d(l) x(.. i_d + l ..)
 * (periodic, fil_d = -0.5/h_d^2 * D2), and kstrten[d] = sum tt_d * x, the
 * kinetic energy of direction d.  Arrays 0:n_d-1 (the reference is called
 * with n_d - 1 as its upper bound). */
void oracle_kinetic_per_ref_ekin(int n1, int n2, int n3, const double *hgrid, const double *x,
                                 double *y, double *kstrten)
{
    double fil[3][29];
    for (int d = 0; d < 3; ++d) {
        double scale = -0.5 / (hgrid[d] * hgrid[d]);
        for (int i = 0; i <= 14; ++i) {
            fil[d][14 + i] = LCG_KIN_FORTRAN[i] * scale;
            fil[d][14 - i] = fil[d][14 + i];
        }
    }
    const int n[3] = {n1, n2, n3};
    for (int d = 0; d < 3; ++d) {
        double ekin = 0.0;
        for (int i3 = 0; i3 < n3; ++i3)
            for (int i2 = 0; i2 < n2; ++i2)
                for (int i1 = 0; i1 < n1; ++i1) {
                    const int c[3] = {i1, i2, i3};
                    double tt = 0.0;
                    for (int l = -14; l <= 14; ++l) {
                        int s[3] = {i1, i2, i3};
                        s[d] = imod(c[d] + l, n[d]);
                        tt = tt + x[s[0] + (size_t)n1 * (s[1] + (size_t)n2 * s[2])] * fil[d][l + 14];
                    }
                    const size_t k = i1 + (size_t)n1 * (i2 + (size_t)n2 * i3);
                    y[k] = y[k] + tt;
                    ekin = ekin + tt * x[k];
                }
        kstrten[d] = ekin;
    }
}

int oracle_d_kin(int d, const int *n, const int *bc, const double *x, double *y,
                 double *w1, double *w2, const double *a, double a_x, double a_y)
{
    if (d < 1 || d > 16 || !n || !bc || !x || !y || !a) return E_ARG;
    if (d > 1 && (!w1 || (d > 2 && !w2))) return E_ARG;
    for (int i = 0; i < d; ++i) {
        if (n[i] < 1) return E_ARG;
        if (bc[i] != BC_PERIODIC && bc[i] != BC_FREE) return E_BC;
    }
    for (int i = 0; i < d; ++i) {
        long nL = 1, nR = 1;
        for (int j = 0; j < i; ++j) nL *= n[j];
        for (int j = i + 1; j < d; ++j) nR *= n[j];
        const double *x2;
        double *dst;
        if (d == 1) { x2 = 0; dst = y; }
        else if (i == 0) { x2 = 0; dst = w1; }
        else if (i == d - 1) { x2 = ((d - 1) % 2 == 1) ? w1 : w2; dst = y; }
        else { x2 = (i % 2 == 1) ? w1 : w2; dst = (i % 2 == 1) ? w2 : w1; }
        const int last = (i == d - 1);
        ocall c = { (int)nL, n[i], (int)nR, 0, 0, 0, 0, x, x2, dst,
                    1, a[i], i == 0, a_x, (last && a_y != 0.0) ? 1 : 0, a_y, 0 };
        conv1d(&F_D2, bc[i], &c);
    }
    return OK;
}

/* ======================================================================
 * Local Hamiltonian of one orbital: the libconvw pipeline of
 * BigDFT/libconv.f90:248-294, composed of the dispatchers above.
 *   idwt        s1s0_md(dwt_fil, 3*[grow])              :258-260
 *   MagicFilter s0s0_md(md_fil, 3*[grow])               :262-264
 *   rho = rho + psir**2 ; psir = v*psir                 :266-271
 *   inverse MF  s0s0_md(mi_fil, 3*[shrink])             :274-276
 *   kinetic     s0s0_1ds_dot(kin_fil, 3*[nogrow], a_y=1):278-280
 *   dwt         s0s1_md(dwt_fil, 3*[shrink])            :284-286
 * Free axes take these boundaries; periodic axes are periodic in every
 * step.  ekin[i] = psi_fscf . (a_kin[i] D2_i psi_fscf) is the 1D dot_in
 * of the kinetic sweep along axis i; epot = sum psir * (v psir).
 * ====================================================================== */
int oracle_hamiltonian(const int *n, const int *bc, const double *a_kin, const double *psig,
                       const double *pot, double *rho, double *hpsig, double *ekin, double *epot)
{
    if (!n || !bc || !a_kin || !psig || !pot || !hpsig || !ekin || !epot) return E_ARG;
    int bw[3], bi[3], bk[3], n0[3], nr[3];
    for (int i = 0; i < 3; ++i) {
        if (n[i] < 1) return E_ARG;
        if (bc[i] != BC_PERIODIC && bc[i] != BC_FREE) return E_BC;
        const int fr = bc[i] == BC_FREE;
        bw[i] = fr ? BC_GROW : BC_PERIODIC;
        bi[i] = fr ? BC_SHRINK : BC_PERIODIC;
        bk[i] = fr ? BC_FREE : BC_PERIODIC;
        n0[i] = 2 * need_out(fr ? &F_IWT_GS : &F_IWT_P, bw[i], n[i]);
        nr[i] = need_out(&F_MD, bw[i], n0[i]);
    }
    const size_t nf = (size_t)n0[0] * n0[1] * n0[2], nrl = (size_t)nr[0] * nr[1] * nr[2];
    double *fscf = malloc(nf * sizeof(double)), *hpsi = malloc(nf * sizeof(double));
    double *tmp = malloc(nf * sizeof(double)), *psir = malloc(nrl * sizeof(double));
    double *w1 = malloc(nrl * sizeof(double)), *w2 = malloc(nrl * sizeof(double));
    int rc = (fscf && hpsi && tmp && psir && w1 && w2) ? OK : E_ARG;
    if (rc == OK) rc = oracle_d_idwt_sym8(3, n, bw, psig, fscf, w1, w2);
    if (rc == OK) rc = oracle_d_sfrf_ld_narr(3, n0, bw, 0, 0, 1, fscf, psir, w1, w2);
    if (rc == OK) {
        double ep = 0.0;
        for (size_t k = 0; k < nrl; ++k) {
            const double p = psir[k], hp = pot[k] * p;
            if (rho) rho[k] = rho[k] + p * p;
            ep = ep + p * hp;
            psir[k] = hp;
        }
        *epot = ep;
        rc = oracle_d_rfsf_ld_narr(3, n0, bi, 0, 0, 1, psir, hpsi, w1, w2);
    }
    if (rc == OK) rc = oracle_d_kin(3, n0, bk, fscf, hpsi, w1, w2, a_kin, 0.0, 1.0);
    for (int i = 0; i < 3 && rc == OK; ++i)
        rc = oracle_d_s0s0_1d_sym8_d2_dotin(3, i, n0, bk[i], n0, n0, 1, fscf, tmp, a_kin[i], 0.0,
                                            0.0, &ekin[i]);
    if (rc == OK) rc = oracle_d_dwt_sym8(3, n, bi, hpsi, hpsig, w1, w2);
    free(fscf); free(hpsi); free(tmp); free(psir); free(w1); free(w2);
    return rc;
}

/* ======================================================================
 * Poisson finite-difference operators (BigDFT/Poisson.rb).
 * c1D(j, k), j, k = -m..m, m = nord/2: derivative weights of order nord on
 * nodes 0..nord at node m + k (Poisson.rb:20-166); LCG_FD_EDGE holds the
 * rows k in order, each row j = -m..m.
 * ====================================================================== */
enum { BC_NPERIODIC = -2 };
static const double FD_EDGE[LCG_FD_EDGE_N] = LCG_FD_EDGE_INIT;
static const double ONEO4PI = 0.07957747154594766788444188168625718101722982287022822437383367203;

static const double *fd_rows(int nord)
{
    switch (nord) {
    case 2: return FD_EDGE + LCG_FD_EDGE_OFF_2;
    case 4: return FD_EDGE + LCG_FD_EDGE_OFF_4;
    case 6: return FD_EDGE + LCG_FD_EDGE_OFF_6;
    case 8: return FD_EDGE + LCG_FD_EDGE_OFF_8;
    case 16: return FD_EDGE + LCG_FD_EDGE_OFF_16;
    default: return 0;
    }
}
#define C1D(t, m, j, k) ((t)[((k) + (m)) * (2 * (m) + 1) + (j) + (m)])

/* Poisson_broker (Poisson.rb:1951-2043) running the generated 1D operator
 * (GenericConvolution2.rb, PoissonFilter 237-294: transpose 0, option a):
 * du = a * (sum_j c1D(j, k) u(..)) along axis idim.  Periodic: the central
 * stencil with modulo wrap; NPERIODIC: the one-sided stencils for the m
 * first (c1D(:, i-m) on nodes 0..nord) and m last points (c1D(:, i-n+m+1)
 * on the last nord+1 nodes) of every line (set_filter_val :begin/:end,
 * 265-281, and input_filter_index, 283-293); taps in ascending j. */
int oracle_poisson_broker(int nord, int idim, const int *nn, int bc, const double *u, double *du,
                          double a)
{
    const double *t = fd_rows(nord);
    if (!t || !nn || !u || !du || idim < 0 || idim > 2) return E_ARG;
    if (bc != BC_PERIODIC && bc != BC_NPERIODIC) return E_BC;
    const int m = nord / 2, n = nn[idim];
    if (nn[0] < 1 || nn[1] < 1 || nn[2] < 1) return E_ARG;
    if (bc == BC_NPERIODIC && n < nord + 1) return E_SIZE;
    long nL = 1, nR = 1;
    for (int k = 0; k < idim; ++k) nL *= nn[k];
    for (int k = idim + 1; k < 3; ++k) nR *= nn[k];
    for (long r = 0; r < nR; ++r)
        for (long l = 0; l < nL; ++l) {
            const double *x = u + l + nL * n * r;
            double *y = du + l + nL * n * r;
            for (int i = 0; i < n; ++i) {
                double tt = 0.0;
                if (bc == BC_PERIODIC || (i >= m && i < n - m)) {
                    for (int j = -m; j <= m; ++j) {
                        const int p = bc == BC_PERIODIC ? imod(i + j, n) : i + j;
                        tt = tt + C1D(t, m, j, 0) * x[nL * p];
                    }
                } else if (i < m) {
                    for (int j = -m; j <= m; ++j) tt = tt + C1D(t, m, j, i - m) * x[nL * (j + m)];
                } else {
                    for (int j = -m; j <= m; ++j)
                        tt = tt + C1D(t, m, j, i - n + m + 1) * x[nL * (n - 1 + j - m)];
                }
                y[nL * i] = tt * a;
            }
        }
    return OK;
}

/* geocode 1 (free): x and z non-periodic; 2 (periodic); 3 (surface): y
 * non-periodic (Poisson.rb:2122-2128). */
static int geocode_bc(int geocode, int bc[3])
{
    if (geocode < 1 || geocode > 3) return E_ARG;
    bc[0] = bc[1] = bc[2] = BC_PERIODIC;
    if (geocode == 1) bc[0] = bc[2] = BC_NPERIODIC;
    if (geocode != 2) bc[1] = BC_NPERIODIC;
    return OK;
}

static int nabla3(int geocode, const int *nn, const double *u, double *du, int nord,
                  const double *hgrids)
{
    int bc[3], rc = geocode_bc(geocode, bc);
    const size_t N = (size_t)nn[0] * nn[1] * nn[2];
    for (int i = 0; i < 3 && rc == OK; ++i)
        rc = oracle_poisson_broker(nord, i, nn, bc[i], u, du + i * N, 1.0 / hgrids[i]);
    return rc;
}

/* div_u_i (Poisson.rb:2067-2194): du = d0 u0 + d1 u1 + d2 u2; with cc, also
 * cc = u0^2 d0u0 + u1^2 d1u1 + u2^2 d2u2 + 2 (u0 u1 d0u1 + u0 u2 d0u2 + u1 u2 d1u2). */
int oracle_div_u_i(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                   const double *hgrids, double *cc)
{
    const int nn[3] = {n01, n02, n03};
    int bc[3], rc = geocode_bc(geocode, bc);
    if (rc || !u || !du || !hgrids || n01 < 1 || n02 < 1 || n03 < 1) return rc ? rc : E_ARG;
    const size_t N = (size_t)n01 * n02 * n03;
    const double a0 = 1.0 / hgrids[0], a1 = 1.0 / hgrids[1], a2 = 1.0 / hgrids[2];
    double *t = malloc((cc ? 5 : 3) * N * sizeof(double));
    if (!t) return E_ARG;
    if (cc) {
        rc = oracle_poisson_broker(nord, 0, nn, bc[0], u, du, a0);
        if (!rc) rc = oracle_poisson_broker(nord, 1, nn, bc[1], u + N, t, a1);
        if (!rc) rc = oracle_poisson_broker(nord, 2, nn, bc[2], u + 2 * N, t + N, a2);
        if (!rc) rc = oracle_poisson_broker(nord, 0, nn, bc[0], u + N, t + 2 * N, a0);
        if (!rc) rc = oracle_poisson_broker(nord, 0, nn, bc[0], u + 2 * N, t + 3 * N, a0);
        if (!rc) rc = oracle_poisson_broker(nord, 1, nn, bc[1], u + 2 * N, t + 4 * N, a1);
        for (size_t k = 0; k < N && !rc; ++k) {
            const double u0 = u[k], u1 = u[N + k], u2 = u[2 * N + k];
            const double du0 = du[k], du1 = t[k], du2 = t[N + k];
            cc[k] = (u0 * u0) * du0 + (u1 * u1) * du1 + (u2 * u2) * du2 +
                    2.0 * (u0 * u1 * t[2 * N + k] + u0 * u2 * t[3 * N + k] + u1 * u2 * t[4 * N + k]);
            du[k] = du0 + du1 + du2;
        }
    } else {
        rc = oracle_poisson_broker(nord, 0, nn, bc[0], u, t, a0);
        if (!rc) rc = oracle_poisson_broker(nord, 1, nn, bc[1], u + N, t + N, a1);
        if (!rc) rc = oracle_poisson_broker(nord, 2, nn, bc[2], u + 2 * N, t + 2 * N, a2);
        for (size_t k = 0; k < N && !rc; ++k) du[k] = t[k] + t[N + k] + t[2 * N + k];
    }
    free(t);
    return rc;
}

/* nabla_u (Poisson.rb:2553-2620): du(:,:,:,i) = d_i u. */
int oracle_nabla_u(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                   const double *hgrids)
{
    const int nn[3] = {n01, n02, n03};
    if (!u || !du || !hgrids || n01 < 1 || n02 < 1 || n03 < 1) return E_ARG;
    return nabla3(geocode, nn, u, du, nord, hgrids);
}

/* nabla_u_and_square (Poisson.rb:2197-2275): du as nabla_u, ddu = |du|^2. */
int oracle_nabla_u_and_square(int geocode, int n01, int n02, int n03, const double *u, double *du,
                              double *ddu, int nord, const double *hgrids)
{
    int rc = oracle_nabla_u(geocode, n01, n02, n03, u, du, nord, hgrids);
    if (rc || !ddu) return rc ? rc : E_ARG;
    const size_t N = (size_t)n01 * n02 * n03;
    for (size_t k = 0; k < N; ++k)
        ddu[k] = (du[k] * du[k]) + (du[N + k] * du[N + k]) + (du[2 * N + k] * du[2 * N + k]);
    return OK;
}

/* nabla_u_square (Poisson.rb:2278-2359): ddu = |nabla u|^2. */
int oracle_nabla_u_square(int geocode, int n01, int n02, int n03, const double *u, double *ddu,
                          int nord, const double *hgrids)
{
    const size_t N = (size_t)n01 * n02 * n03;
    double *du = malloc(3 * (N ? N : 1) * sizeof(double));
    if (!du) return E_ARG;
    int rc = oracle_nabla_u_and_square(geocode, n01, n02, n03, u, du, ddu, nord, hgrids);
    free(du);
    return rc;
}

/* nabla_u_epsilon (Poisson.rb:2362-2443): du(:,:,:,i) = d_i u * eps. */
int oracle_nabla_u_epsilon(int geocode, int n01, int n02, int n03, const double *u, double *du,
                           int nord, const double *hgrids, const double *eps)
{
    int rc = oracle_nabla_u(geocode, n01, n02, n03, u, du, nord, hgrids);
    if (rc || !eps) return rc ? rc : E_ARG;
    const size_t N = (size_t)n01 * n02 * n03;
    for (size_t k = 0; k < N; ++k) {
        du[k] = du[k] * eps[k];
        du[N + k] = du[N + k] * eps[k];
        du[2 * N + k] = du[2 * N + k] * eps[k];
    }
    return OK;
}

/* update_rhopol (Poisson.rb:2446-2550): res = (dlogeps . nabla u) / (4 pi);
 * res = (res - rhopol) eta; rhores2 = sum res^2; rhopol = res + rhopol.
 * dlogeps(3, n01, n02, n03): component fastest. */
int oracle_update_rhopol(int geocode, int n01, int n02, int n03, const double *u, int nord,
                         const double *hgrids, double eta, const double *dlogeps, double *rhopol,
                         double *rhores2)
{
    const size_t N = (size_t)n01 * n02 * n03;
    if (!dlogeps || !rhopol || !rhores2) return E_ARG;
    double *du = malloc(3 * (N ? N : 1) * sizeof(double));
    if (!du) return E_ARG;
    int rc = oracle_nabla_u(geocode, n01, n02, n03, u, du, nord, hgrids);
    double acc = 0.0;
    for (size_t k = 0; k < N && !rc; ++k) {
        double res = dlogeps[3 * k] * du[k] + dlogeps[3 * k + 1] * du[N + k] +
                     dlogeps[3 * k + 2] * du[2 * N + k];
        res = res * ONEO4PI;
        const double rho = rhopol[k];
        res = (res - rho) * eta;
        acc = acc + res * res;
        rhopol[k] = res + rho;
    }
    if (!rc) *rhores2 = acc;
    free(du);
    return rc;
}

/* div_u_i_ref as written in Fortran (Poisson.rb:181-340): the same stencils,
 * each directional sum divided by h (not multiplied by 1/h). */
int oracle_div_u_i_ref(int geocode, int n01, int n02, int n03, const double *u, double *du,
                       int nord, const double *hgrids)
{
    const double *t = fd_rows(nord);
    int bc[3];
    if (!t || !u || !du || !hgrids || geocode_bc(geocode, bc)) return E_ARG;
    const int m = nord / 2, nn[3] = {n01, n02, n03};
    const size_t N = (size_t)n01 * n02 * n03;
    const long st[3] = {1, n01, (long)n01 * n02};
    for (int i3 = 0; i3 < n03; ++i3)
        for (int i2 = 0; i2 < n02; ++i2)
            for (int i1 = 0; i1 < n01; ++i1) {
                const int ii[3] = {i1, i2, i3};
                const long k0 = i1 + (long)n01 * (i2 + (long)n02 * i3);
                double d[3];
                for (int a = 0; a < 3; ++a) {
                    const int n = nn[a], i = ii[a];
                    const double *x = u + a * N + k0 - (long)i * st[a];   /* start of the line */
                    double s = 0.0;
                    if (bc[a] == BC_PERIODIC || (i >= m && i < n - m)) {
                        for (int j = -m; j <= m; ++j) {
                            const int p = bc[a] == BC_PERIODIC ? imod(i + j, n) : i + j;
                            s = s + C1D(t, m, j, 0) * x[st[a] * p];
                        }
                    } else if (i < m) {
                        for (int j = -m; j <= m; ++j) s = s + C1D(t, m, j, i - m) * x[st[a] * (j + m)];
                    } else {
                        for (int j = -m; j <= m; ++j)
                            s = s + C1D(t, m, j, i - n + m + 1) * x[st[a] * (n - 1 + j - m)];
                    }
                    d[a] = s / hgrids[a];
                }
                du[k0] = d[0] + d[1] + d[2];
            }
    return OK;
}
