// C-ABI of libconv-gb300: the generated libconv dispatchers restated as
// plans of 1D sweeps (lcg::Sweep) launched on the GPU.
//
//  - 1D entry points follow GenericConvolutionOperator1d#procedure
//    (BigDFT/GenericConvolution2.rb:1560-1764);
//  - multi-D entry points follow GenericConvolutionOperator#procedure
//    (BigDFT/GenericConvolution2.rb:1934-2243) for transpose = 1
//    (MagicFilter, wavelets) and transpose = 0 with the kinetic options.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/libconv_gb300.h"
#include "lcg_plan.cuh"
#include "lcg_pool.cuh"
#include "lcg_sweep.cuh"
#include "lcg_tc.cuh"
#include "libconv_filters.h"

using namespace lcg;

namespace {

bool valid_mode(int m) {
    return m == LIBCONV_MODE_FP64 || m == LIBCONV_MODE_TC_EXACT || m == LIBCONV_MODE_TC_BF16X3 ||
           m == LIBCONV_MODE_TC_TF32X3;
}

// The mode a thread starts in: $LIBCONV_GB300_MODE (fp64, tc_exact, tc_bf16x3,
// tc_tf32x3, or the number of one of them), read once per process, so callers
// of the generated procedures can select the tensor-core sweeps without a
// code change; FP64 when it is unset or names no mode.
int initial_mode() {
    static const int m = [] {
        const char *e = getenv("LIBCONV_GB300_MODE");
        if (!e) return LIBCONV_MODE_FP64;
        static const struct { const char *name; int mode; } names[] = {
            {"fp64", LIBCONV_MODE_FP64}, {"tc_exact", LIBCONV_MODE_TC_EXACT},
            {"tc_bf16x3", LIBCONV_MODE_TC_BF16X3}, {"tc_tf32x3", LIBCONV_MODE_TC_TF32X3}};
        for (const auto &n : names)
            if (strcmp(e, n.name) == 0) return n.mode;
        char *end = nullptr;
        const long v = strtol(e, &end, 10);
        return (end != e && *end == '\0' && valid_mode((int)v)) ? (int)v : LIBCONV_MODE_FP64;
    }();
    return m;
}

thread_local std::string t_err;
thread_local int t_mode = initial_mode();

int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(LIBCONV_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

// ---- operator definitions ---------------------------------------------------
struct OpDef {
    int kind;
    int ftab[2], ntaps[2], lowfil[2];   // [0]: periodic/free filters, [1]: grow/shrink
    int length;                         // filter.length (cost model, grow extents)
    int cost_per_out;                   // filter.cost (GenericConvolution2.rb:231-233, 499-501)
};

#define CONV_OP(TAB, NT, LOW) { KCONV, {TAB, TAB}, {NT, NT}, {LOW, LOW}, NT, 2 * NT }
#define WT_OP(KIND, P, GS) { KIND, {LCG_FTAB_##P, LCG_FTAB_##GS}, {LCG_##P##_NTAPS, LCG_##GS##_NTAPS}, \
        {LCG_##P##_LOWFIL, LCG_##GS##_LOWFIL}, LCG_##P##_LENGTH, 4 * LCG_##P##_LENGTH }

const double h_ftab[LCG_FTAB_N] = LCG_FTAB_INIT;

const OpDef OP_MD = CONV_OP(LCG_FTAB_MD, 16, LCG_CONV_SYM8_MD_LOWFIL);
const OpDef OP_IMD = CONV_OP(LCG_FTAB_IMD, 16, LCG_CONV_SYM8_IMD_LOWFIL);
const OpDef OP_D1 = CONV_OP(LCG_FTAB_D1, 29, LCG_CONV_SYM8_D1_LOWFIL);
const OpDef OP_D2 = CONV_OP(LCG_FTAB_D2, 29, LCG_CONV_SYM8_D2_LOWFIL);
const OpDef OP_DWT = WT_OP(KDEC, WT_SYM8_DEC_P, WT_SYM8_DEC_GS);
const OpDef OP_IWT = WT_OP(KREC, WT_SYM8_REC_P, WT_SYM8_REC_GS);
const OpDef OP_RTOS1 = WT_OP(KDEC, WT_SYMICOMB8_DEC_P, WT_SYMICOMB8_DEC_GS);
const OpDef OP_S1TOR = WT_OP(KREC, WT_SYMICOMB8_REC_P, WT_SYMICOMB8_REC_GS);

bool bc_valid(int bc) {
    return bc == BC_PERIODIC || bc == BC_GROW || bc == BC_SHRINK || bc == BC_FREE;
}
int fam(int bc) { return (bc == BC_GROW || bc == BC_SHRINK) ? 1 : 0; }
int nch(const OpDef &op) { return op.kind == KCONV ? 1 : 2; }
// processed-dim extents needed (positions; pairs for wavelets)
int need_in(const OpDef &op, int bc, int n) { return bc == BC_SHRINK ? n + op.ntaps[1] - 1 : n; }
int need_out(const OpDef &op, int bc, int n) { return bc == BC_GROW ? n + op.ntaps[1] - 1 : n; }

// Fill the geometry of a sweep (GenericConvolution2.rb:61-85, 206-225, 1009-1022).
void geometry(const OpDef &op, int bc, int nL, int n, int nR, int ld_in, int ld_out, Sweep &S) {
    const int f = fam(bc);
    S.kind = op.kind;
    S.ntaps = op.ntaps[f];
    S.lowfil = op.lowfil[f];
    S.ftab = op.ftab[f];
    S.bc = bc;
    S.nL = nL; S.n = n; S.nR = nR;
    const int up = S.lowfil + S.ntaps - 1;
    S.in_lo = bc == BC_SHRINK ? S.lowfil : 0;
    S.in_ext = ld_in;
    S.out_lo = bc == BC_GROW ? -up : 0;
    S.out_ext = ld_out;
    S.qlo = bc == BC_GROW ? -up : 0;
    S.qhi = bc == BC_GROW ? n - S.lowfil - 1 : n - 1;
    S.transpose = 0;
    S.narr = 1;
    S.x_arr = S.y_arr = 0;
    S.x = S.x2 = nullptr;
    S.y = nullptr;
    S.has_a = S.has_ax = S.ay_mode = S.has_dot = 0;
    S.a = 1.0; S.a_x = 0.0; S.a_y = 0.0;
    S.dot_part = nullptr;
}

// ---- per-device resources ------------------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

// One slot of the host-pointer copy/compute pipeline: its own stream and
// buffers, so chunks in different slots run concurrently.
struct PipeSlot {
    cudaStream_t stream = nullptr;
    DevBuf buf[4];                   // x, y, w1, w2 of one chunk
    DevBuf scratch, lineexp;
};
// Chunks per host-pointer call (at most; each at least 48 MB in and out) and
// streams they rotate over: 16 chunks on 8 streams keep both copy directions
// busy; the first chunk's copy-in and the last chunk's sweeps and copy-out run
// alone, so smaller chunks shorten them (32 x 128^3 MagicFilter3D + Kinetic3D
// from pinned buffers: 8 chunks on 3 streams 8.74 Gpts/s, 16 on 8 9.04; 4-5
// streams sometimes 7.9).
constexpr int kPipeChunks = 16;
constexpr int kPipeSlots = 8;

struct DevState {
    bool init = false;
    PipeSlot pipe[kPipeSlots];       // chunked host-pointer execution (exec_host)
    cudaStream_t stream = nullptr;   // stream of the host-pointer entry points
    DevBuf buf[6];                   // x, y, w1, w2, dot partials, dot scalar
    DevBuf scratch;                  // dot partials of the host-pointer entry points
    DevBuf lineexp;                  // their per-line exponents (exact tensor-core sweeps)
    StreamPool pool;                 // scratch of the *_dev entry points, per call (lcg_pool.cuh)
    DevBuf dscalar;
    DevBuf status;                   // device status word (bounded waits)
    DevBuf potpart;                  // partial sums of the potential energy
    DevBuf hbuf;                     // staging of the host-pointer local Hamiltonian
    DevBuf pbuf;                     // staging of the host-pointer Poisson operators
};

std::recursive_mutex g_mu;   // recursive: composed host entry points hold it across sweeps
DevState g_dev[64];

int current_device(int &dev) {
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return fail(LIBCONV_ECUDA, "device index %d out of range", dev);
    return LIBCONV_OK;
}

int ensure(DevBuf &b, size_t bytes) {
    if (b.cap >= bytes) return LIBCONV_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(LIBCONV_ENOMEM, "cudaMalloc(%zu bytes): %s", want, cudaGetErrorString(e));
    }
    b.cap = want;
    return LIBCONV_OK;
}

DevState *dev_state(int &rc) {
    int dev;
    rc = current_device(dev);
    if (rc) return nullptr;
    DevState &s = g_dev[dev];
    if (!s.init) {
        cudaError_t e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { rc = cuda_fail(e, "cudaStreamCreate"); return nullptr; }
        if ((rc = ensure(s.status, sizeof(int)))) return nullptr;
        e = cudaMemset(s.status.p, 0, sizeof(int));
        if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemset"); return nullptr; }
        s.init = true;
    }
    return &s;
}

// ---- plans -------------------------------------------------------------------
void need(Plan &P, int b, size_t e) { if (P.elems[b] < e) P.elems[b] = e; }

// 1D dispatcher (GenericConvolution2.rb:1560-1764).
int plan_1d(const OpDef &op, int d, int idim, const int *n, int bc, const int *nx, const int *ny,
            int narr, double a, int use_ax, double a_x, double a_y, int dot, Plan &P) {
    if (d < 1 || idim < 0 || idim >= d) return fail(LIBCONV_EARG, "d=%d idim=%d", d, idim);
    if (!n || !nx || !ny) return fail(LIBCONV_EARG, "n/nx/ny must not be null");
    if (narr < 1 || narr > 65535) return fail(LIBCONV_EARG, "narr=%d out of [1,65535]", narr);
    if (!bc_valid(bc)) return fail(LIBCONV_EBC, "unknown boundary condition %d", bc);
    for (int i = 0; i < d; ++i)
        if (n[i] < 1 || nx[i] < 1 || ny[i] < 1)
            return fail(LIBCONV_EARG, "n/nx/ny[%d] must be >= 1", i);
    if (nx[idim] < need_in(op, bc, n[idim]) || ny[idim] < need_out(op, bc, n[idim]))
        return fail(LIBCONV_ESIZE, "nx[%d]=%d / ny[%d]=%d too small for n=%d bc=%d", idim, nx[idim],
                    idim, ny[idim], n[idim], bc);
    const long long m = nch(op);
    long long nL = 1, nR = 1;
    for (int i = 0; i < idim; ++i) nL *= nx[i] * m;
    for (int i = idim + 1; i < d; ++i) nR *= nx[i] * m;
    if (nL * nR > (1LL << 31) - 1) return fail(LIBCONV_EARG, "too many lines");
    PlanStep st;
    geometry(op, bc, (int)nL, n[idim], (int)nR, nx[idim], ny[idim], st.S);
    st.S.narr = narr;
    st.S.x_arr = (long long)nx[idim] * m * nL * nR;
    st.S.y_arr = (long long)ny[idim] * m * nL * nR;
    st.S.has_a = a != 1.0;
    st.S.a = a;
    st.S.has_ax = use_ax && a_x != 0.0;
    st.S.a_x = a_x;
    st.S.ay_mode = a_y != 0.0 ? 1 : 0;
    st.S.a_y = a_y;
    st.S.has_dot = dot;
    st.src = B_X; st.dst = B_Y; st.src2 = -1;
    P.steps.push_back(st);
    need(P, B_X, st.S.x_arr * narr);
    need(P, B_Y, st.S.y_arr * narr);
    P.y_read = st.S.ay_mode ? st.S.y_arr * narr : 0;
    // ld padding past the computed outputs is left untouched, as the
    // generated loops do: host callers get their padding back unchanged
    if (ny[idim] > need_out(op, bc, n[idim])) P.y_read = st.S.y_arr * narr;
    P.has_dot = dot;
    return LIBCONV_OK;
}

// Ping-pong of the multi-D dispatcher (GenericConvolution2.rb:2155-2240):
// sweep 0 x->w1, odd middle sweeps w1->w2, even ones w2->w1, last ->y.
void pingpong(int d, int i, int &src, int &dst) {
    if (d == 1) { src = B_X; dst = B_Y; return; }
    if (i == 0) { src = B_X; dst = B_W1; return; }
    if (i == d - 1) { src = ((d - 1) % 2 == 1) ? B_W1 : B_W2; dst = B_Y; return; }
    src = (i % 2 == 1) ? B_W1 : B_W2;
    dst = (i % 2 == 1) ? B_W2 : B_W1;
}

// Multi-D, transpose = 1 (MagicFilter, wavelets).
int plan_md_t(const OpDef &op, int d, const int *n, const int *bc, const int *nx, const int *ny,
              int narr, Plan &P) {
    if (d < 1 || d > 16) return fail(LIBCONV_EARG, "d=%d out of [1,16]", d);
    if (!n || !bc) return fail(LIBCONV_EARG, "n/bc must not be null");
    if (narr < 1 || narr > 65535) return fail(LIBCONV_EARG, "narr=%d out of [1,65535]", narr);
    const bool ld = nx != nullptr;
    if (ld && !ny) return fail(LIBCONV_EARG, "ny must not be null when nx is given");
    const long long m = nch(op);
    long long dims[16];
    for (int i = 0; i < d; ++i) {
        if (n[i] < 1) return fail(LIBCONV_EARG, "n[%d]=%d", i, n[i]);
        if (!bc_valid(bc[i])) return fail(LIBCONV_EBC, "unknown boundary condition %d", bc[i]);
        if (ld) {
            if (nx[i] < need_in(op, bc[i], n[i]) || ny[i] < need_out(op, bc[i], n[i]))
                return fail(LIBCONV_ESIZE, "nx[%d]=%d / ny[%d]=%d too small for n=%d bc=%d", i,
                            nx[i], i, ny[i], n[i], bc[i]);
            dims[i] = nx[i] * m;
        } else {
            dims[i] = need_in(op, bc[i], n[i]) * m;
        }
    }
    for (int i = 0; i < d; ++i) {
        long long ndat = 1;
        for (int j = 0; j < d; ++j) if (j != i) ndat *= dims[j];
        if (ndat > (1LL << 31) - 1) return fail(LIBCONV_EARG, "too many lines");
        const int in_ext = (int)(dims[i] / m);
        const int out_ext = ld ? ny[i] : need_out(op, bc[i], n[i]);
        PlanStep st;
        geometry(op, bc[i], 1, n[i], (int)ndat, in_ext, out_ext, st.S);
        st.S.transpose = 1;
        st.S.narr = narr;
        st.S.x_arr = ndat * dims[i];
        st.S.y_arr = ndat * out_ext * m;
        pingpong(d, i, st.src, st.dst);
        st.src2 = -1;
        need(P, st.src, st.S.x_arr * narr);
        need(P, st.dst, st.S.y_arr * narr);
        P.steps.push_back(st);
        dims[i] = out_ext * m;
        if (i == d - 1 && out_ext > need_out(op, bc[i], n[i])) P.y_read = st.S.y_arr * narr;
    }
    return LIBCONV_OK;
}

// Multi-D, transpose = 0, sweeps along order[0..d-1]: the same operator as
// plan_md_t (each sweep maps one axis in place instead of rotating it to the
// end, so after d sweeps both give the natural axis order), other
// intermediate shapes.
int plan_md_n(const OpDef &op, int d, const int *n, const int *bc, const int *order, Plan &P) {
    if (d < 1 || d > 16) return fail(LIBCONV_EARG, "d=%d out of [1,16]", d);
    if (!n || !bc || !order) return fail(LIBCONV_EARG, "n/bc/order must not be null");
    const long long m = nch(op);
    long long dims[16];
    unsigned seen = 0;
    for (int i = 0; i < d; ++i) {
        if (n[i] < 1) return fail(LIBCONV_EARG, "n[%d]=%d", i, n[i]);
        if (!bc_valid(bc[i])) return fail(LIBCONV_EBC, "unknown boundary condition %d", bc[i]);
        if (order[i] < 0 || order[i] >= d || (seen >> order[i]) & 1u)
            return fail(LIBCONV_EARG, "sweep order is not a permutation of 0..%d", d - 1);
        seen |= 1u << order[i];
        dims[i] = need_in(op, bc[i], n[i]) * m;
    }
    for (int k = 0; k < d; ++k) {
        const int i = order[k];
        long long nL = 1, nR = 1;
        for (int j = 0; j < i; ++j) nL *= dims[j];
        for (int j = i + 1; j < d; ++j) nR *= dims[j];
        if (nL * nR > (1LL << 31) - 1) return fail(LIBCONV_EARG, "too many lines");
        const int in_ext = (int)(dims[i] / m);
        const int out_ext = need_out(op, bc[i], n[i]);
        PlanStep st;
        geometry(op, bc[i], (int)nL, n[i], (int)nR, in_ext, out_ext, st.S);
        st.S.x_arr = nL * nR * dims[i];
        st.S.y_arr = nL * nR * out_ext * m;
        pingpong(d, k, st.src, st.dst);
        st.src2 = -1;
        need(P, st.src, st.S.x_arr);
        need(P, st.dst, st.S.y_arr);
        P.steps.push_back(st);
        dims[i] = out_ext * m;
    }
    return LIBCONV_OK;
}

// Multi-D kinetic, transpose = 0 (Kinetic2.rb:1068-1090), over narr grids
// laid back to back (narr = 1 is the reference's Kinetic()).
int plan_kin(int d, const int *n, const int *bc, const double *a, double a_x, double a_y,
             Plan &P, int narr = 1, const int *order = nullptr, bool ekin = false,
             const OpDef &op = OP_D2) {
    if (narr < 1 || narr > 65535) return fail(LIBCONV_EARG, "narr=%d out of [1,65535]", narr);
    if (d < 1 || d > 16) return fail(LIBCONV_EARG, "d=%d out of [1,16]", d);
    if (!n || !bc || !a) return fail(LIBCONV_EARG, "n/bc/a must not be null");
    long long tot = 1;
    for (int i = 0; i < d; ++i) {
        if (n[i] < 1) return fail(LIBCONV_EARG, "n[%d]=%d", i, n[i]);
        if (bc[i] != BC_PERIODIC && bc[i] != BC_FREE)
            return fail(LIBCONV_EBC, "summed 1D sweeps support periodic and free (no-grow) only, "
                        "bc[%d]=%d", i, bc[i]);
        tot *= n[i];
    }
    if (tot > (1LL << 31) - 1) return fail(LIBCONV_EARG, "grid too large");
    if (order) {
        unsigned seen = 0;
        for (int k = 0; k < d; ++k) {
            if (order[k] < 0 || order[k] >= d || (seen >> order[k]) & 1u)
                return fail(LIBCONV_EARG, "sweep order is not a permutation of 0..%d", d - 1);
            seen |= 1u << order[k];
        }
    }
    for (int k = 0; k < d; ++k) {
        const int i = order ? order[k] : k;
        long long nL = 1, nR = 1;
        for (int j = 0; j < i; ++j) nL *= n[j];
        for (int j = i + 1; j < d; ++j) nR *= n[j];
        PlanStep st;
        geometry(op, bc[i], (int)nL, n[i], (int)nR, n[i], n[i], st.S);
        const bool last = k == d - 1;
        st.S.has_a = 1;
        st.S.a = a[i];
        st.S.has_ax = k == 0 && a_x != 0.0;   // as the 1D dispatcher: no a_x term when 0
        st.S.a_x = a_x;
        st.S.ay_mode = (last && a_y != 0.0) ? 1 : 0;
        st.S.a_y = a_y;
        int s, t;
        pingpong(d, k, s, t);
        st.src = B_X;
        st.dst = t;
        st.src2 = k == 0 ? -1 : s;
        st.S.has_dot = ekin ? 1 : 0;   // x . (a_i D2_i x), before a_x x and the partial sum
        st.dot_slot = i;
        if (d == 3) st.exp_axis = i;
        st.S.narr = narr;
        st.S.x_arr = st.S.y_arr = tot;
        need(P, B_X, tot * narr);
        need(P, t, tot * narr);
        if (st.src2 >= 0) need(P, st.src2, tot * narr);
        P.steps.push_back(st);
    }
    P.y_read = a_y != 0.0 ? tot * narr : 0;
    P.has_dot = ekin ? 1 : 0;
    P.ndot = ekin ? d : 1;
    if (d == 3) {                  // the three sweeps read x: one exponent pass for all
        P.exp3[0] = n[0]; P.exp3[1] = n[1]; P.exp3[2] = n[2]; P.exp3[3] = narr;
    }
    return LIBCONV_OK;
}

// ---- execution ------------------------------------------------------------------
// Device scratch one plan run uses: dot partials (doubles) and per-line
// exponents of the exact tensor-core sweeps (ints), sized by plan_scratch
// before anything is enqueued.
struct Scratch {
    double *dot = nullptr;
    size_t ndot = 0;
    int *le = nullptr;
    size_t nle = 0;
};

// Elements of dot partials and of line exponents that run_plan(P) needs in
// the calling thread's mode.
// Exact tensor-core step k hands its successor the line exponents of its
// output (the epilogue writes them, Sweep::le_next) instead of a pre-pass
// over that output: k is a periodic transposed convolution with the plain
// store path (no dot, a_x, a_y or x2) over whole tiles of valid lines, k + 1 a
// periodic convolution reading k's output along its fastest axis (length n1
// = 32, 64 or 128, so that every tile column holds whole lines of k + 1: k's
// line i1 + n1 i2 and output q are k + 1's line i2 + n2 q at position i1).
bool exp_handoff(const Plan &P, size_t k, int &n1, int &n2) {
    if (t_mode != LIBCONV_MODE_TC_EXACT || k + 1 >= P.steps.size()) return false;
    const PlanStep &a = P.steps[k], &b = P.steps[k + 1];
    const Sweep &A = a.S, &B = b.S;
    if (!(A.kind == KCONV && A.transpose && A.nL == 1 && A.bc == BC_PERIODIC && !A.has_dot &&
          !A.has_ax && A.ay_mode == 0 && a.src2 < 0 && sweep_tc_supported(A)))
        return false;
    if (!(B.kind == KCONV && B.nL == 1 && B.bc == BC_PERIODIC && b.src == a.dst && b.exp_axis < 0 &&
          B.narr == A.narr && B.x_arr == A.y_arr && sweep_tc_supported(B)))
        return false;
    const long long lines = (long long)A.nL * A.nR;
    if (!(B.n == 32 || B.n == 64 || B.n == 128) || lines % 128 || lines % B.n) return false;
    if ((A.qhi - A.qlo + 1) % 64 || A.out_lo != 0 || A.qlo != 0 || B.in_lo != 0 || B.in_ext != B.n)
        return false;
    if ((long long)B.nR != lines / B.n * A.out_ext) return false;
    n1 = B.n;
    n2 = (int)(lines / B.n);
    return true;
}

void plan_scratch(const Plan &P, size_t &ndot, size_t &nle) {
    ndot = nle = 0;
    const bool exact = t_mode == LIBCONV_MODE_TC_EXACT;
    if (exact && P.exp3[0] > 0) {
        const size_t n0 = P.exp3[0], n1 = P.exp3[1], n2 = P.exp3[2], na = P.exp3[3];
        nle = (n1 * n2 + n0 * n2 + n0 * n1) * na;
    }
    for (const PlanStep &ps : P.steps) {
        const Sweep &S = ps.S;
        const bool tc = t_mode != LIBCONV_MODE_FP64 && sweep_tc_supported(S);
        if (S.has_dot) {
            const size_t nb = tc ? (size_t)sweep_tc_blocks(S) * 8 * S.narr : (size_t)sweep_fp64_blocks(S);
            if (nb > ndot) ndot = nb;
        }
        const bool shared = exact && P.exp3[0] > 0 && ps.exp_axis >= 0 && ps.src == B_X;
        if (tc && exact && !shared && (size_t)sweep_tc_lines(S) > nle) nle = (size_t)sweep_tc_lines(S);
    }
    // a hand-off writes the next step's exponents beside the ones being read
    int n1, n2;
    for (size_t k = 0; k + 1 < P.steps.size(); ++k)
        if (!(P.exp3[0] > 0) && exp_handoff(P, k, n1, n2)) {
            nle *= 2;
            break;
        }
}

// The host-pointer paths' scratch: their own buffers, grown under the lock
// (the host call synchronises before it returns).
int host_scratch(const Plan &P, DevBuf &dot, DevBuf &le, Scratch &sc) {
    size_t nd, nl;
    plan_scratch(P, nd, nl);
    int rc;
    if (nd && (rc = ensure(dot, nd * sizeof(double)))) return rc;
    if (nl && (rc = ensure(le, nl * sizeof(int)))) return rc;
    sc.dot = (double *)dot.p;
    sc.ndot = dot.cap / sizeof(double);
    sc.le = (int *)le.p;
    sc.nle = le.cap / sizeof(int);
    return LIBCONV_OK;
}

// Launch the plan's sweeps with bound device pointers.  dot_dev receives the
// dot product (device) when the plan has one; the partials and line
// exponents live in sc (at least plan_scratch's sizes).
int run_plan(const Plan &P, double *const bufs[4], const Scratch &sc, double *dot_dev, int *status,
             cudaStream_t st) {
    if (!valid_mode(t_mode)) return fail(LIBCONV_EMODE, "unknown mode %d", t_mode);
    {
        size_t nd, nl;
        plan_scratch(P, nd, nl);
        if (nd > sc.ndot || nl > sc.nle || (nd && !sc.dot) || (nl && !sc.le))
            return fail(LIBCONV_EARG, "internal: plan scratch not sized");
    }
    // exact tensor-core sweeps of one grid along its three axes: the line
    // exponents of all three come from one read of x
    int *shared_exp = nullptr;
    long long exp_off[3] = {0, 0, 0};
    if (t_mode == LIBCONV_MODE_TC_EXACT && P.exp3[0] > 0) {
        const long long n0 = P.exp3[0], n1 = P.exp3[1], n2 = P.exp3[2], na = P.exp3[3];
        exp_off[1] = n1 * n2 * na;
        exp_off[2] = exp_off[1] + n0 * n2 * na;
        shared_exp = sc.le;
        cudaError_t e = launch_line_exp3(bufs[B_X], (int)n0, (int)n1, (int)n2, (int)na, shared_exp,
                                         shared_exp + exp_off[1], shared_exp + exp_off[2], st, P.active);
        if (e != cudaSuccess) return cuda_fail(e, "line exponent launch");
    }
    if (P.active && P.has_dot) return fail(LIBCONV_EARG, "internal: active arrays with a dot product");
    // exponents handed from step to step: the step reads le_cur (ready when the
    // previous step wrote it) and writes its successor's into the other half
    int *le_cur = sc.le, *le_other = nullptr;
    bool le_ready = false;
    if (!shared_exp) {
        size_t half = 0;
        for (const PlanStep &ps : P.steps)
            if ((size_t)sweep_tc_lines(ps.S) > half) half = (size_t)sweep_tc_lines(ps.S);
        if (sc.le && sc.nle >= 2 * half) le_other = sc.le + half;
    }
    for (size_t k = 0; k < P.steps.size(); ++k) {
        const PlanStep &ps = P.steps[k];
        Sweep S = ps.S;
        S.active = P.active;
        S.x = bufs[ps.src];
        S.y = bufs[ps.dst];
        S.x2 = ps.src2 >= 0 ? bufs[ps.src2] : nullptr;
        if (!S.x || !S.y || (ps.src2 >= 0 && !S.x2))
            return fail(LIBCONV_EARG, "null device buffer in plan");
        const bool tc = t_mode != LIBCONV_MODE_FP64 && sweep_tc_supported(S);
        long long nb = 0, seg = 0;   // dot partials: total, and per array (array-major)
        if (S.has_dot) {
            if (tc) {
                seg = sweep_tc_blocks(S) * 8;
                nb = seg * S.narr;
            } else {
                nb = sweep_fp64_blocks(S);
                seg = nb / S.narr;
            }
            S.dot_part = sc.dot;
            if (tc && S.narr > 1) {   // slots of arrays a CTA has no tile of stay 0
                cudaError_t e = cudaMemsetAsync(S.dot_part, 0, (size_t)nb * sizeof(double), st);
                if (e != cudaSuccess) return cuda_fail(e, "clear dot partials");
            }
        }
        cudaError_t e;
        if (tc) {
            TcFilter F;
            const int sch = t_mode == LIBCONV_MODE_TC_EXACT    ? SCH_EXACT
                            : t_mode == LIBCONV_MODE_TC_BF16X3 ? SCH_BF16X3
                                                               : SCH_TF32X3;
            const int flat = S.kind == KCONV ? S.ntaps : 4 * S.ntaps;   // LE|LO|HE|HO
            if (sch == SCH_EXACT) tc_filter_digits(h_ftab + S.ftab, flat, S.has_a ? S.a : 1.0, F);
            else tc_filter_split(h_ftab + S.ftab, flat, S.has_a ? S.a : 1.0, sch, F);
            S.has_a = 0;   // folded into the filter operands
            int *lineE = nullptr;
            const bool shared = sch == SCH_EXACT && shared_exp && ps.exp_axis >= 0 && ps.src == B_X;
            bool ready = shared, handed = false;
            if (shared) {
                lineE = shared_exp + exp_off[ps.exp_axis];
            } else if (sch == SCH_EXACT) {
                if (shared_exp) return fail(LIBCONV_EARG, "plan shares line exponents but a step does not");
                lineE = le_cur;
                ready = le_ready;
                int n1, n2;
                if (le_other && exp_handoff(P, k, n1, n2)) {
                    const Sweep &B = P.steps[k + 1].S;
                    S.le_next = le_other;
                    S.le_next_lines = (long long)B.nL * B.nR;
                    S.le_n1 = n1;
                    S.le_n2 = n2;
                    handed = true;
                }
            }
            e = launch_sweep_tc(S, F, sch, status, lineE, st, ready);
            if (handed) std::swap(le_cur, le_other);
            le_ready = handed;
        } else {
            e = launch_sweep_fp64(S, st);
            le_ready = false;
        }
        if (e != cudaSuccess) return cuda_fail(e, "sweep launch");
        if (S.has_dot) {
            e = ps.dot_stride > 0
                    ? launch_dot_reduce_seg(S.dot_part, seg, S.narr, dot_dev + ps.dot_slot,
                                            ps.dot_stride, st)
                    : launch_dot_reduce(S.dot_part, nb, dot_dev + ps.dot_slot, 0, st);
            if (e != cudaSuccess) return cuda_fail(e, "dot reduction launch");
        }
    }
    return LIBCONV_OK;
}

// A pool entry of the current device for one enqueue-only call on st: buffer
// 0 dot partials, 1 line exponents, 2 potential-energy partials (bytes).
// Released by ~Lease after the call's work is enqueued.  Caller holds g_mu.
struct Lease {
    DevState *s = nullptr;
    PoolEntry *e = nullptr;
    cudaStream_t st = nullptr;
    Lease() = default;
    Lease(const Lease &) = delete;
    Lease &operator=(const Lease &) = delete;
    ~Lease() { if (s && e) s->pool.release(e, st); }
    int take(DevState *ds, cudaStream_t stream, size_t dot_b, size_t le_b, size_t pot_b = 0) {
        const size_t bytes[3] = {dot_b, le_b, pot_b};
        cudaError_t err = ds->pool.acquire(stream, bytes, 3, e);
        if (err != cudaSuccess) {
            cudaGetLastError();
            return err == cudaErrorMemoryAllocation
                       ? fail(LIBCONV_ENOMEM, "scratch allocation (%zu + %zu + %zu bytes): %s", dot_b,
                              le_b, pot_b, cudaGetErrorString(err))
                       : cuda_fail(err, "scratch lease");
        }
        s = ds;
        st = stream;
        return LIBCONV_OK;
    }
    Scratch scratch() const {
        Scratch sc;
        sc.dot = (double *)e->p[0];
        sc.ndot = e->cap[0] / sizeof(double);
        sc.le = (int *)e->p[1];
        sc.nle = e->cap[1] / sizeof(int);
        return sc;
    }
};

// Device-pointer execution (caller-owned buffers, no host synchronisation).
int exec_dev(const Plan &P, const double *x, double *y, double *w1, double *w2, double *dot_dev,
             void *stream) {
    if (!x || !y) return fail(LIBCONV_EARG, "x/y must not be null");
    if (P.elems[B_W1] && !w1) return fail(LIBCONV_EARG, "w1 workspace required");
    if (P.elems[B_W2] && !w2) return fail(LIBCONV_EARG, "w2 workspace required");
    if (P.has_dot && !dot_dev) return fail(LIBCONV_EARG, "dot_in must not be null");
    double *bufs[4] = {const_cast<double *>(x), y, w1, w2};
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    int rc;
    DevState *s = dev_state(rc);
    if (!s) return rc;
    size_t nd, nl;
    plan_scratch(P, nd, nl);
    Lease L;
    if ((rc = L.take(s, (cudaStream_t)stream, nd * sizeof(double), nl * sizeof(int)))) return rc;
    return run_plan(P, bufs, L.scratch(), dot_dev, (int *)s->status.p, (cudaStream_t)stream);
}

// Read and clear the device status word (after the work was synchronised).
int read_status(DevState &s) {
    int v = 0;
    cudaError_t e = cudaMemcpy(&v, s.status.p, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read status");
    if (v) {
        cudaMemset(s.status.p, 0, sizeof(int));
        return fail(LIBCONV_ETIMEOUT, "a tensor-core wait timed out on the device (status %d)", v);
    }
    return LIBCONV_OK;
}

// Page-locked host memory (cudaHostAlloc / cudaHostRegister): asynchronous
// copies to and from it overlap kernels; pageable memory is staged by the
// driver, so chunked copies would only add overhead.
bool pinned(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// narr of a plan whose steps all work on the same narr independent arrays
// (0 otherwise).
int plan_narr(const Plan &P) {
    int n = 0;
    for (const PlanStep &ps : P.steps) {
        if (n == 0) n = ps.S.narr;
        else if (ps.S.narr != n) return 0;
    }
    return n;
}

// The same plan over narr_new of the arrays (every buffer extent is per-array
// extent times narr).
Plan with_narr(const Plan &P, int narr_old, int narr_new) {
    Plan Q = P;
    for (PlanStep &ps : Q.steps) ps.S.narr = narr_new;
    for (int b = 0; b < 4; ++b) Q.elems[b] = P.elems[b] / narr_old * narr_new;
    Q.y_read = P.y_read / narr_old * narr_new;
    if (Q.exp3[0]) Q.exp3[3] = narr_new;
    return Q;
}

// Host-pointer execution of a plan over narr independent arrays, in chunks
// of arrays on kPipeSlots streams: the copy-in of one chunk, the sweeps of
// another and the copy-out of a third overlap (H2D and D2H copy engines and
// the SMs).  Chunk k runs in slot k % kPipeSlots; a slot's stream orders the
// reuse of its buffers.
int exec_host_pipelined(const Plan &P, int narr, const double *x, double *y, DevState &s) {
    const size_t xs = P.elems[B_X] / narr, ys = P.elems[B_Y] / narr;
    const size_t per = (xs + ys) * sizeof(double);
    int c = (narr + kPipeChunks - 1) / kPipeChunks;
    // at least 48 MB in and out per chunk: smaller chunks leave the host's
    // per-chunk launches comparable to their copies
    while ((size_t)c * per < (48u << 20) && c < narr) ++c;
    const int nchunk = (narr + c - 1) / c, rem = narr - (nchunk - 1) * c;
    const Plan Qc = with_narr(P, narr, c), Qr = with_narr(P, narr, rem);
    int rc;
    for (int k = 0; k < kPipeSlots && k < nchunk; ++k) {
        PipeSlot &ps = s.pipe[k];
        if (!ps.stream) {
            cudaError_t e = cudaStreamCreateWithFlags(&ps.stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
        }
        for (int b = 0; b < 4; ++b)
            if (Qc.elems[b] && (rc = ensure(ps.buf[b], Qc.elems[b] * sizeof(double)))) return rc;
        Scratch unused;   // sized for the full chunk (the last chunk needs no more)
        if ((rc = host_scratch(Qc, ps.scratch, ps.lineexp, unused))) return rc;
    }
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < nchunk && e == cudaSuccess; ++k) {
        PipeSlot &ps = s.pipe[k % kPipeSlots];
        const Plan &Q = k == nchunk - 1 ? Qr : Qc;
        const size_t a0 = (size_t)k * c, ca = k == nchunk - 1 ? rem : c;
        double *bufs[4];
        for (int b = 0; b < 4; ++b) bufs[b] = Q.elems[b] ? (double *)ps.buf[b].p : nullptr;
        e = cudaMemcpyAsync(bufs[B_X], x + a0 * xs, ca * xs * sizeof(double), cudaMemcpyHostToDevice,
                            ps.stream);
        if (e == cudaSuccess && P.y_read)
            e = cudaMemcpyAsync(bufs[B_Y], y + a0 * ys, ca * ys * sizeof(double),
                                cudaMemcpyHostToDevice, ps.stream);
        if (e != cudaSuccess) break;
        Scratch sc;
        if ((rc = host_scratch(Q, ps.scratch, ps.lineexp, sc))) return rc;
        if ((rc = run_plan(Q, bufs, sc, nullptr, (int *)s.status.p, ps.stream))) return rc;
        e = cudaMemcpyAsync(y + a0 * ys, bufs[B_Y], ca * ys * sizeof(double), cudaMemcpyDeviceToHost,
                            ps.stream);
    }
    if (e != cudaSuccess) return cuda_fail(e, "pipelined copy");
    for (int k = 0; k < kPipeSlots && k < nchunk; ++k)
        if ((e = cudaStreamSynchronize(s.pipe[k].stream)) != cudaSuccess) return cuda_fail(e, "synchronize");
    return read_status(s);
}

// Host-pointer execution: stage in device buffers owned by the library.
int exec_host(const Plan &P, const double *x, double *y, double *dot_host) {
    if (!x || !y) return fail(LIBCONV_EARG, "x/y must not be null");
    if (P.has_dot && !dot_host) return fail(LIBCONV_EARG, "dot_in must not be null");
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    int rc;
    DevState *s = dev_state(rc);
    if (!s) return rc;
    // independent arrays, no dot, at least 4 MB of input: pipelined chunks
    const int narr = plan_narr(P);
    if (!P.has_dot && narr >= 2 && P.elems[B_X] % narr == 0 && P.elems[B_Y] % narr == 0 &&
        P.y_read % narr == 0 && P.elems[B_X] * sizeof(double) >= (4u << 20) && pinned(x) &&
        pinned(y))
        return exec_host_pipelined(P, narr, x, y, *s);
    for (int b = 0; b < 4; ++b)
        if (P.elems[b] && (rc = ensure(s->buf[b], P.elems[b] * sizeof(double)))) return rc;
    if (P.has_dot && (rc = ensure(s->dscalar, sizeof(double) * P.ndot))) return rc;
    double *bufs[4];
    for (int b = 0; b < 4; ++b) bufs[b] = P.elems[b] ? (double *)s->buf[b].p : nullptr;
    cudaStream_t st = s->stream;
    cudaError_t e = cudaMemcpyAsync(bufs[B_X], x, P.elems[B_X] * sizeof(double),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy x to device");
    if (P.y_read) {
        e = cudaMemcpyAsync(bufs[B_Y], y, P.y_read * sizeof(double), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "copy y to device");
    }
    Scratch sc;
    if ((rc = host_scratch(P, s->scratch, s->lineexp, sc))) return rc;
    rc = run_plan(P, bufs, sc, P.has_dot ? (double *)s->dscalar.p : nullptr, (int *)s->status.p, st);
    if (rc) return rc;
    e = cudaMemcpyAsync(y, bufs[B_Y], P.elems[B_Y] * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy y to host");
    if (P.has_dot) {
        e = cudaMemcpyAsync(dot_host, s->dscalar.p, sizeof(double) * P.ndot, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return cuda_fail(e, "copy dot_in to host");
    }
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "synchronize");
    return read_status(*s);
}

// ---- local Hamiltonian (BigDFT/libconv.f90:248-294) -------------------------------
// The reference's libconvw sketch composes the dispatchers on one orbital:
// idwt (grow) -> MagicFilter (grow) -> density and potential -> inverse
// MagicFilter (shrink) -> kinetic with dot, accumulated (no-grow, a_y = 1)
// -> dwt (shrink).  Free axes take that grow/shrink chain; periodic axes are
// periodic in every step.  norb orbitals lie back to back and every step is
// one launch over all of them (narr = norb), so a sweep covers norb grids'
// worth of tiles; the energies are kept per orbital (segmented dots).
struct Ham {
    Plan idwt, mf, imf, kin, dwt;
    int norb = 1;
    int n0[3], nr[3];      // fine-grid extents of psi_fscf / hpsi and of psir
    size_t nsig = 0;       // elements of psig and hpsig, per orbital
    size_t nfscf = 0;      // elements of psi_fscf and hpsi, per orbital
    size_t nreal = 0;      // elements of psir, pot and rho, per orbital
    size_t nw = 0;         // elements of each ping-pong workspace (w1, w2), all orbitals
    size_t nwork() const { return (size_t)norb * (2 * nfscf + nreal) + 2 * nw; }
};

int plan_ham(const int *n, const int *bc, const double *a_kin, int norb, Ham &H) {
    if (!n || !bc || !a_kin) return fail(LIBCONV_EARG, "n/bc/a_kin must not be null");
    if (norb < 1 || norb > 65535) return fail(LIBCONV_EARG, "norb=%d out of [1,65535]", norb);
    int bw[3], bi[3], bk[3];
    for (int i = 0; i < 3; ++i) {
        if (n[i] < 1) return fail(LIBCONV_EARG, "n[%d]=%d", i, n[i]);
        if (bc[i] != BC_PERIODIC && bc[i] != BC_FREE)
            return fail(LIBCONV_EBC, "local Hamiltonian: bc[%d]=%d is neither periodic nor free",
                        i, bc[i]);
        const bool fr = bc[i] == BC_FREE;
        bw[i] = fr ? BC_GROW : BC_PERIODIC;     // idwt and MagicFilter
        bi[i] = fr ? BC_SHRINK : BC_PERIODIC;   // inverse MagicFilter and dwt
        bk[i] = fr ? BC_FREE : BC_PERIODIC;     // kinetic (no growth)
        if (n[i] > (1 << 28)) return fail(LIBCONV_EARG, "n[%d]=%d too large", i, n[i]);
        H.n0[i] = 2 * need_out(OP_IWT, bw[i], n[i]);
        H.nr[i] = need_out(OP_MD, bw[i], H.n0[i]);
    }
    H.norb = norb;
    int rc;
    if ((rc = plan_md_t(OP_IWT, 3, n, bw, nullptr, nullptr, norb, H.idwt))) return rc;
    if ((rc = plan_md_t(OP_MD, 3, H.n0, bw, nullptr, nullptr, norb, H.mf))) return rc;
    if ((rc = plan_md_t(OP_IMD, 3, H.n0, bi, nullptr, nullptr, norb, H.imf))) return rc;
    if ((rc = plan_kin(3, H.n0, bk, a_kin, 0.0, 1.0, H.kin, norb, nullptr, true))) return rc;
    if ((rc = plan_md_t(OP_DWT, 3, n, bi, nullptr, nullptr, norb, H.dwt))) return rc;
    for (PlanStep &ps : H.kin.steps) ps.dot_stride = 4;   // energies[j][i], j = orbital
    H.nsig = 8ull * n[0] * n[1] * n[2];
    H.nfscf = (size_t)H.n0[0] * H.n0[1] * H.n0[2];
    H.nreal = (size_t)H.nr[0] * H.nr[1] * H.nr[2];
    if ((double)H.nreal * norb > 9.0e15) return fail(LIBCONV_EARG, "grid too large");
    for (const Plan *P : {&H.idwt, &H.mf, &H.imf, &H.kin, &H.dwt})
        for (int b : {B_W1, B_W2}) if (P->elems[b] > H.nw) H.nw = P->elems[b];
    return LIBCONV_OK;
}

// Scratch of one run_ham: the largest need of its five plans, and the
// potential-energy partials (doubles).
void ham_scratch(const Ham &H, size_t &ndot, size_t &nle, size_t &npot) {
    ndot = nle = 0;
    for (const Plan *P : {&H.idwt, &H.mf, &H.imf, &H.kin, &H.dwt}) {
        size_t a, b;
        plan_scratch(*P, a, b);
        if (a > ndot) ndot = a;
        if (b > nle) nle = b;
    }
    npot = (size_t)potential_blocks((long long)H.nreal) * (size_t)H.norb;
}

// Enqueue the pipeline on `st`.  work: H.nwork() doubles; energies: 4
// doubles per orbital (ekin of the three directions, then epot), device;
// sc and potpart at least ham_scratch's sizes.
int run_ham(const Ham &H, const double *psig, const double *pot, double *rho, double *hpsig,
            double *work, double *energies, const Scratch &sc, double *potpart, int *status,
            cudaStream_t st) {
    const size_t no = (size_t)H.norb;
    double *fscf = work, *hpsi = fscf + no * H.nfscf, *psir = hpsi + no * H.nfscf;
    double *w1 = psir + no * H.nreal, *w2 = w1 + H.nw;
    double *b_idwt[4] = {const_cast<double *>(psig), fscf, w1, w2};
    int rc = run_plan(H.idwt, b_idwt, sc, nullptr, status, st);
    if (rc) return rc;
    double *b_mf[4] = {fscf, psir, w1, w2};
    if ((rc = run_plan(H.mf, b_mf, sc, nullptr, status, st))) return rc;
    cudaError_t e = launch_potential(psir, pot, rho, (long long)H.nreal, H.norb, potpart,
                                     energies + 3, 4, st);
    if (e != cudaSuccess) return cuda_fail(e, "potential launch");
    double *b_imf[4] = {psir, hpsi, w1, w2};
    if ((rc = run_plan(H.imf, b_imf, sc, nullptr, status, st))) return rc;
    double *b_kin[4] = {fscf, hpsi, w1, w2};
    if ((rc = run_plan(H.kin, b_kin, sc, energies, status, st))) return rc;
    double *b_dwt[4] = {hpsi, hpsig, w1, w2};
    return run_plan(H.dwt, b_dwt, sc, nullptr, status, st);
}

// The host-pointer Hamiltonian's scratch: the library's own buffers.
int ham_host_scratch(const Ham &H, DevState &s, Scratch &sc) {
    size_t nd, nl, np;
    ham_scratch(H, nd, nl, np);
    int rc;
    if (nd && (rc = ensure(s.scratch, nd * sizeof(double)))) return rc;
    if (nl && (rc = ensure(s.lineexp, nl * sizeof(int)))) return rc;
    if ((rc = ensure(s.potpart, np * sizeof(double)))) return rc;
    sc.dot = (double *)s.scratch.p;
    sc.ndot = s.scratch.cap / sizeof(double);
    sc.le = (int *)s.lineexp.p;
    sc.nle = s.lineexp.cap / sizeof(int);
    return LIBCONV_OK;
}

// Host-pointer form over many orbitals: chunks of orbitals pipelined on three
// streams -- copy-in of psig (two staging buffers), the pipeline of each
// chunk in order on one compute stream (so rho accumulates the orbitals in
// order, as one call does), copy-out of hpsig -- chained by events.
int ham_host_pipelined(const Ham &H, const int *n, const int *bc, const double *a_kin,
                       const double *psig, const double *pot, double *rho, double *hpsig,
                       double *energies, DevState &s) {
    const int norb = H.norb;
    const int c = (norb + 7) / 8, nchunk = (norb + c - 1) / c, rem = norb - (nchunk - 1) * c;
    Ham Hc, Hr;
    int rc = plan_ham(n, bc, a_kin, c, Hc);
    if (!rc) rc = plan_ham(n, bc, a_kin, rem, Hr);
    if (rc) return rc;
    const size_t ns = H.nsig, nc = (size_t)c * ns;
    const size_t nd = (rho ? 2 : 1) * H.nreal + Hc.nwork() + 4 * nc + 4 * (size_t)norb;
    if ((rc = ensure(s.hbuf, nd * sizeof(double)))) return rc;
    Scratch sc;   // one compute stream: the chunks use it in turn
    if ((rc = ham_host_scratch(Hc, s, sc))) return rc;
    double *d_pot = (double *)s.hbuf.p, *d_rho = rho ? d_pot + H.nreal : nullptr;
    double *d_work = d_pot + (rho ? 2 : 1) * H.nreal;
    double *d_in[2] = {d_work + Hc.nwork(), d_work + Hc.nwork() + nc};
    double *d_out[2] = {d_in[1] + nc, d_in[1] + 2 * nc};
    double *d_en = d_out[1] + nc;
    for (int k = 0; k < 3; ++k)
        if (!s.pipe[k].stream) {
            cudaError_t e = cudaStreamCreateWithFlags(&s.pipe[k].stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
        }
    cudaStream_t sin = s.pipe[0].stream, scomp = s.pipe[1].stream, sout = s.pipe[2].stream;
    std::vector<cudaEvent_t> ev(3 * nchunk + 1, nullptr);   // in[k], done[k], out[k], pot
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; i < ev.size() && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
    auto cleanup = [&]() { for (cudaEvent_t x : ev) if (x) cudaEventDestroy(x); };
    if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "cudaEventCreate"); }
    cudaEvent_t *ev_in = ev.data(), *ev_done = ev_in + nchunk, *ev_out = ev_done + nchunk;
    cudaEvent_t ev_pot = ev[3 * nchunk];
    e = cudaMemcpyAsync(d_pot, pot, H.nreal * sizeof(double), cudaMemcpyHostToDevice, sin);
    if (e == cudaSuccess && rho)
        e = cudaMemcpyAsync(d_rho, rho, H.nreal * sizeof(double), cudaMemcpyHostToDevice, sin);
    if (e == cudaSuccess) e = cudaEventRecord(ev_pot, sin);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(scomp, ev_pot, 0);
    for (int k = 0; k < nchunk && e == cudaSuccess && !rc; ++k) {
        const Ham &Q = k == nchunk - 1 ? Hr : Hc;
        const size_t a0 = (size_t)k * c, ca = (size_t)Q.norb;
        const int b = k & 1;
        // staging buffer b: its previous chunk (k - 2) must have been consumed
        if (k >= 2) e = cudaStreamWaitEvent(sin, ev_done[k - 2], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_in[b], psig + a0 * ns, ca * ns * sizeof(double),
                                cudaMemcpyHostToDevice, sin);
        if (e == cudaSuccess) e = cudaEventRecord(ev_in[k], sin);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(scomp, ev_in[k], 0);
        if (e == cudaSuccess && k >= 2) e = cudaStreamWaitEvent(scomp, ev_out[k - 2], 0);
        if (e != cudaSuccess) break;
        rc = run_ham(Q, d_in[b], d_pot, d_rho, d_out[b], d_work, d_en + 4 * a0, sc, (double *)s.potpart.p,
                     (int *)s.status.p, scomp);
        if (rc) break;
        e = cudaEventRecord(ev_done[k], scomp);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sout, ev_done[k], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hpsig + a0 * ns, d_out[b], ca * ns * sizeof(double),
                                cudaMemcpyDeviceToHost, sout);
        if (e == cudaSuccess) e = cudaEventRecord(ev_out[k], sout);
    }
    if (e == cudaSuccess && !rc) {
        e = cudaStreamWaitEvent(sout, ev_done[nchunk - 1], 0);
        if (e == cudaSuccess && rho)
            e = cudaMemcpyAsync(rho, d_rho, H.nreal * sizeof(double), cudaMemcpyDeviceToHost, sout);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(energies, d_en, 4 * (size_t)norb * sizeof(double),
                                cudaMemcpyDeviceToHost, sout);
    }
    for (int k = 0; k < 3; ++k) cudaStreamSynchronize(s.pipe[k].stream);
    cleanup();
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "pipelined Hamiltonian");
    return read_status(s);
}

// Host-pointer form: stage in the library's device buffer, run, copy back.
// energies: 4 doubles per orbital (host).
int ham_host(const Ham &H, const double *psig, const double *pot, double *rho, double *hpsig,
             double *energies, const int *n = nullptr, const int *bc = nullptr,
             const double *a_kin = nullptr) {
    if (!psig || !pot || !hpsig || !energies)
        return fail(LIBCONV_EARG, "psig/pot/hpsig/energies must not be null");
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    int rc;
    DevState *s = dev_state(rc);
    if (!s) return rc;
    if (n && H.norb >= 4 && pinned(psig) && pinned(hpsig))
        return ham_host_pipelined(H, n, bc, a_kin, psig, pot, rho, hpsig, energies, *s);
    const size_t no = (size_t)H.norb, ns = no * H.nsig;
    const size_t nd = 2 * ns + (rho ? 2 : 1) * H.nreal + H.nwork() + 4 * no;
    if ((rc = ensure(s->hbuf, nd * sizeof(double)))) return rc;
    double *d_psig = (double *)s->hbuf.p, *d_hpsig = d_psig + ns, *d_pot = d_hpsig + ns;
    double *d_rho = rho ? d_pot + H.nreal : nullptr;
    double *d_work = d_pot + (rho ? 2 : 1) * H.nreal, *d_en = d_work + H.nwork();
    cudaStream_t st = s->stream;
    cudaError_t e = cudaMemcpyAsync(d_psig, psig, ns * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_pot, pot, H.nreal * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && rho)
        e = cudaMemcpyAsync(d_rho, rho, H.nreal * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "copy inputs to device");
    Scratch sc;
    if ((rc = ham_host_scratch(H, *s, sc))) return rc;
    if ((rc = run_ham(H, d_psig, d_pot, d_rho, d_hpsig, d_work, d_en, sc, (double *)s->potpart.p,
                      (int *)s->status.p, st)))
        return rc;
    e = cudaMemcpyAsync(hpsig, d_hpsig, ns * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && rho)
        e = cudaMemcpyAsync(rho, d_rho, H.nreal * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(energies, d_en, 4 * no * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "copy outputs to host");
    return read_status(*s);
}

// ---- cost model (GenericConvolution2.rb:1269-1276, 1525-1558, 1850-1932) ----
int cost_1d(const OpDef &op, int d, int idim, const int *n, int bc, int narr, long long *cost) {
    if (!cost || !n || d < 1 || idim < 0 || idim >= d || narr < 1)
        return fail(LIBCONV_EARG, "bad cost arguments");
    if (!bc_valid(bc)) return fail(LIBCONV_EBC, "unknown boundary condition %d", bc);
    long long ndat = 1;
    for (int i = 0; i < d; ++i) if (i != idim) ndat *= n[i];
    *cost = (long long)n[idim] * op.cost_per_out * ndat * narr;
    return LIBCONV_OK;
}

int cost_md(const OpDef &op, int d, const int *n, const int *bc, int narr, long long *cost) {
    if (!cost || !n || !bc || d < 1 || d > 16 || narr < 1) return fail(LIBCONV_EARG, "bad cost arguments");
    const int m = nch(op);
    const int L = op.length;
    long long dims[16];
    for (int i = 0; i < d; ++i) {
        if (!bc_valid(bc[i])) return fail(LIBCONV_EBC, "unknown boundary condition %d", bc[i]);
        if (bc[i] == BC_SHRINK) dims[i] = m == 2 ? 2LL * n[i] + L - 2 : n[i] + L - 1;
        else dims[i] = (long long)m * n[i];
    }
    long long c = 0;
    for (int i = 0; i < d; ++i) {
        long long ndat = 1;
        for (int j = 0; j < d; ++j) if (j != i) ndat *= dims[j];
        c += (long long)n[i] * op.cost_per_out * ndat;
        if (bc[i] == BC_GROW) dims[i] = m == 2 ? 2LL * n[i] + L - 2 : n[i] + L - 1;
        else dims[i] = (long long)m * n[i];
    }
    *cost = c * narr;
    return LIBCONV_OK;
}

}  // namespace

namespace lcg {
// Validation and geometry of one 1D kinetic sweep with dot_in (the plan_1d
// restatement for OP_D2), filled into S without any container or allocation;
// used by the allocation-free entry point.
int kinetic_dotin_sweep(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                        int narr, double a, double a_x, double a_y, Sweep &S) {
    if (d < 1 || idim < 0 || idim >= d) return fail(LIBCONV_EARG, "d=%d idim=%d", d, idim);
    if (!n || !nx || !ny) return fail(LIBCONV_EARG, "n/nx/ny must not be null");
    if (narr < 1 || narr > 65535) return fail(LIBCONV_EARG, "narr=%d out of [1,65535]", narr);
    if (!bc_valid(bc)) return fail(LIBCONV_EBC, "unknown boundary condition %d", bc);
    for (int i = 0; i < d; ++i)
        if (n[i] < 1 || nx[i] < 1 || ny[i] < 1)
            return fail(LIBCONV_EARG, "n/nx/ny[%d] must be >= 1", i);
    if (nx[idim] < need_in(OP_D2, bc, n[idim]) || ny[idim] < need_out(OP_D2, bc, n[idim]))
        return fail(LIBCONV_ESIZE, "nx[%d]=%d / ny[%d]=%d too small for n=%d bc=%d", idim, nx[idim],
                    idim, ny[idim], n[idim], bc);
    long long nL = 1, nR = 1;
    for (int i = 0; i < idim; ++i) nL *= nx[i];
    for (int i = idim + 1; i < d; ++i) nR *= nx[i];
    if (nL * nR > (1LL << 31) - 1) return fail(LIBCONV_EARG, "too many lines");
    geometry(OP_D2, bc, (int)nL, n[idim], (int)nR, nx[idim], ny[idim], S);
    S.narr = narr;
    S.x_arr = (long long)nx[idim] * nL * nR;
    S.y_arr = (long long)ny[idim] * nL * nR;
    S.has_a = a != 1.0;
    S.a = a;
    S.has_ax = a_x != 0.0;
    S.a_x = a_x;
    S.ay_mode = a_y != 0.0 ? 1 : 0;
    S.a_y = a_y;
    S.has_dot = 1;
    return LIBCONV_OK;
}

const OpDef *op_of(int id) {
    switch (id) {
    case OPID_MD: return &OP_MD;
    case OPID_IMD: return &OP_IMD;
    case OPID_D1: return &OP_D1;
    case OPID_D2: return &OP_D2;
    case OPID_DWT: return &OP_DWT;
    case OPID_IWT: return &OP_IWT;
    case OPID_RTOS1: return &OP_RTOS1;
    case OPID_S1TOR: return &OP_S1TOR;
    default: return nullptr;
    }
}

// Multi-D product of 1D sweeps (transpose = 1, the dispatcher of
// GenericConvolution2.rb:1934-2243) with ld, narr, and the scalar options of
// the Fortran-facing API: y = a (F_{d-1} ... F_0 x) + a_y y, a and a_y on the
// last sweep; a_x (first sweep in the generated dispatcher, :2040-2043) only
// for d = 1, where it is y = a F x + a_x x + a_y y.
int md_generic(int op_id, int d, const int *n, const int *bc, const int *nx, const int *ny,
               int narr, double a, double a_x, double a_y, const double *x, double *y) {
    const OpDef *op = op_of(op_id);
    if (!op) return fail(LIBCONV_EARG, "unknown operator %d", op_id);
    if (a_x != 0.0 && (d != 1 || op->kind != KCONV))
        return fail(LIBCONV_EARG, "a_x is defined for one-dimensional convolutions only");
    Plan P;
    int rc = plan_md_t(*op, d, n, bc, nx, ny, narr, P);
    if (rc) return rc;
    Sweep &S = P.steps.back().S;
    S.has_a = a != 1.0;
    S.a = a;
    S.has_ax = a_x != 0.0;
    S.a_x = a_x;
    S.ay_mode = a_y != 0.0 ? 1 : 0;
    S.a_y = a_y;
    if (a_y != 0.0) P.y_read = P.elems[B_Y];
    return exec_host(P, x, y, nullptr);
}

// Sum of 1D convolutions along every axis (the kinetic form, transpose = 0):
// y = sum_i a[i] F_i x + a_x x + a_y y, with dot[i] = x . (a[i] F_i x) when
// dot is not null (host pointers; dot sums over the narr arrays).
int sum1d_generic(int op_id, int d, const int *n, const int *bc, const int *nx, const int *ny,
                  int narr, const double *a, double a_x, double a_y, const double *x, double *y,
                  double *dot) {
    const OpDef *op = op_of(op_id);
    if (!op || op->kind != KCONV) return fail(LIBCONV_EARG, "operator %d is not a convolution", op_id);
    if (n && (nx || ny))
        for (int i = 0; i < d && i < 16; ++i)
            if ((nx && nx[i] != n[i]) || (ny && ny[i] != n[i]))
                return fail(LIBCONV_ESIZE, "summed 1D sweeps need nx = ny = n (axis %d)", i);
    Plan P;
    int rc = plan_kin(d, n, bc, a, a_x, a_y, P, narr, nullptr, dot != nullptr, *op);
    return rc ? rc : exec_host(P, x, y, dot);
}

// Extents (in the operator's units: pairs for wavelets) that a sweep of
// op_id with boundary bc reads and writes for n points, and the elements of
// the largest intermediate of the multi-D product.
int extents(int op_id, int d, const int *n, const int *bc, int *in, int *out, long long *inter) {
    const OpDef *op = op_of(op_id);
    if (!op) return fail(LIBCONV_EARG, "unknown operator %d", op_id);
    if (d < 1 || d > 16 || !n || !bc) return fail(LIBCONV_EARG, "bad extent arguments");
    const long long m = nch(*op);
    long long cur = 1, big = 0;
    int dims[16];
    for (int i = 0; i < d; ++i) {
        if (n[i] < 1) return fail(LIBCONV_EARG, "n[%d]=%d", i, n[i]);
        if (!bc_valid(bc[i])) return fail(LIBCONV_EBC, "unknown boundary condition %d", bc[i]);
        dims[i] = need_in(*op, bc[i], n[i]);
        if (in) in[i] = dims[i];
        if (out) out[i] = need_out(*op, bc[i], n[i]);
        cur *= dims[i] * m;
    }
    big = cur;
    for (int i = 0; i < d; ++i) {               // sizes after each sweep
        cur = cur / (dims[i] * m) * need_out(*op, bc[i], n[i]) * m;
        if (cur > big) big = cur;
    }
    if (inter) *inter = big;
    return LIBCONV_OK;
}

// One Poisson broker sweep (Poisson.rb:1951-2043 over the generated 1D
// operator with the PoissonFilter, GenericConvolution2.rb:237-294) on device
// pointers: y = a d/dx_idim x (accumulate: y += ...).  The central stencil
// (17 taps, zero padded below nord 16) runs as a convolution sweep: periodic,
// or, for the non-periodic boundary, only over the outputs m..n-m-1 whose
// stencil stays inside the line; the m one-sided outputs at each end are
// written by launch_poisson_edges.
int poisson_sweep(int nord, int idim, const int *nn, int bc, double a, bool accumulate,
                  const double *x, double *y, cudaStream_t st) {
    int ftab;
    switch (nord) {
    case 2: ftab = LCG_FTAB_FD2; break;
    case 4: ftab = LCG_FTAB_FD4; break;
    case 6: ftab = LCG_FTAB_FD6; break;
    case 8: ftab = LCG_FTAB_FD8; break;
    case 16: ftab = LCG_FTAB_FD16; break;
    default: return fail(LIBCONV_EARG, "nord=%d: only 2, 4, 6, 8 and 16", nord);
    }
    if (!nn || !x || !y) return fail(LIBCONV_EARG, "nn/u/du must not be null");
    if (idim < 0 || idim > 2) return fail(LIBCONV_EARG, "idim=%d out of [0,2]", idim);
    if (bc != BC_PERIODIC && bc != LIBCONV_BC_NPERIODIC)
        return fail(LIBCONV_EBC, "Poisson operators take periodic (0) or non-periodic (-2), bc=%d", bc);
    for (int i = 0; i < 3; ++i)
        if (nn[i] < 1) return fail(LIBCONV_EARG, "nn[%d]=%d", i, nn[i]);
    const int n = nn[idim], m = nord / 2;
    const bool nper = bc == LIBCONV_BC_NPERIODIC;
    if (nper && n < nord + 1)
        return fail(LIBCONV_ESIZE, "non-periodic axis of %d points shorter than the %d-point stencil",
                    n, nord + 1);
    long long nL = 1, nR = 1;
    for (int i = 0; i < idim; ++i) nL *= nn[i];
    for (int i = idim + 1; i < 3; ++i) nR *= nn[i];
    if (nL * nR > (1LL << 31) - 1 || nL * nR * n > (1LL << 40)) return fail(LIBCONV_EARG, "grid too large");
    const OpDef fd = {KCONV, {ftab, ftab}, {LCG_FD_NTAPS, LCG_FD_NTAPS}, {LCG_FD_LOWFIL, LCG_FD_LOWFIL},
                      LCG_FD_NTAPS, 2 * LCG_FD_NTAPS};
    Plan P;
    PlanStep ps;
    geometry(fd, nper ? BC_FREE : BC_PERIODIC, (int)nL, n, (int)nR, n, n, ps.S);
    ps.S.has_a = 1;
    ps.S.a = a;
    ps.S.ay_mode = accumulate ? 2 : 0;
    if (nper) { ps.S.qlo = m; ps.S.qhi = n - m - 1; }
    ps.S.x_arr = ps.S.y_arr = nL * n * nR;
    ps.src = B_X; ps.dst = B_Y; ps.src2 = -1;
    P.steps.push_back(ps);
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    int rc;
    DevState *s = dev_state(rc);
    if (!s) return rc;
    double *bufs[4] = {const_cast<double *>(x), y, nullptr, nullptr};
    size_t nd, nl;
    plan_scratch(P, nd, nl);
    Lease L;
    if ((rc = L.take(s, st, nd * sizeof(double), nl * sizeof(int)))) return rc;
    if ((rc = run_plan(P, bufs, L.scratch(), nullptr, (int *)s->status.p, st))) return rc;
    if (nper) {
        cudaError_t e = launch_poisson_edges(x, y, nL, n, nR, nord, a, accumulate ? 1 : 0, st);
        if (e != cudaSuccess) return cuda_fail(e, "Poisson boundary launch");
    }
    return LIBCONV_OK;
}

// Device staging for composed host-pointer entry points: `bytes` of the
// library's buffer and its stream.  The caller holds library_lock().
double *host_staging(size_t bytes, cudaStream_t &st, int &rc) {
    DevState *s = dev_state(rc);
    if (!s) return nullptr;
    if ((rc = ensure(s->pbuf, bytes))) return nullptr;
    st = s->stream;
    return (double *)s->pbuf.p;
}
std::unique_lock<std::recursive_mutex> library_lock() {
    return std::unique_lock<std::recursive_mutex>(g_mu);
}
// Synchronise the library stream and read the device status word.
int host_finish(cudaStream_t st) {
    int rc;
    DevState *s = dev_state(rc);
    if (!s) return rc;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "synchronize");
    return read_status(*s);
}

int report(int code, const char *msg) { return fail(code, "%s", msg); }
int report_cuda(cudaError_t e, const char *what) { return cuda_fail(e, what); }

int plan_magicfilter(int d, const int *n, const int *bc, const int *order, Plan &P) {
    return order ? plan_md_n(OP_MD, d, n, bc, order, P)
                 : plan_md_t(OP_MD, d, n, bc, nullptr, nullptr, 1, P);
}
int plan_kinetic(int d, const int *n, const int *bc, const double *a, double a_x,
                 const int *order, Plan &P) {
    return plan_kin(d, n, bc, a, a_x, 0.0, P, 1, order);
}
const double *filter_table() { return h_ftab; }
int current_mode() { return t_mode; }
int kin_narr_active_dev(int d, const int *n, const int *bc, int narr, const double *x, double *y,
                        double *w1, double *w2, const double *a, const int *active, cudaStream_t st) {
    Plan P;
    int rc = plan_kin(d, n, bc, a, 0.0, 0.0, P, narr);
    if (rc) return rc;
    P.active = active;
    return exec_dev(P, x, y, w1, w2, nullptr, st);
}
int *device_status(int &rc) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevState *s = dev_state(rc);
    return s ? (int *)s->status.p : nullptr;
}
}  // namespace lcg

namespace lcg {
namespace {
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Self-test of the bounded device waits: one thread waits on an mbarrier that
// nothing arrives at, with the same try_wait / sleep / limit loop as the
// tensor-core kernels, gives up after `limit_ns` nanoseconds of the GPU's
// global timer (independent of the SM clock) and sets the status word.
// Nothing faults and the wait always ends.
__global__ void selftest_wait_kernel(int *status, unsigned long long limit_ns) {
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x != 0) return;
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    const unsigned long long t0 = global_ns();
    uint32_t ok = 0;
    while (true) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(b)
            : "memory");
        if (ok || global_ns() - t0 > limit_ns) break;
        __nanosleep(128);
    }
    if (!ok) atomicExch(status, 1);
}

// FP64 pipe probe: every thread runs 8 independent FMA chains (no dependency
// between consecutive FMAs of a chain's neighbours), so the FP64 pipe, not
// latency, bounds the kernel.  The sink store happens only for a value the
// chains never reach, which keeps the compiler from removing them.
__device__ double g_fp64_sink;
__global__ void __launch_bounds__(256) fp64_peak_kernel(int iters, double a, double b) {
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = (double)(threadIdx.x + j);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = fma(v[j], a, b);
    }
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) t += v[j];
    if (t == -1.0) g_fp64_sink = t;
}
}  // namespace
}  // namespace lcg

// =============================== exported C ABI ===============================
extern "C" {

const char *libconv_gb300_version(void) { return "libconv-gb300 0.1 (sm_103a)"; }

const char *libconv_gb300_strerror(int s) {
    switch (s) {
    case LIBCONV_OK: return "ok";
    case LIBCONV_EARG: return "invalid argument";
    case LIBCONV_EBC: return "unsupported boundary condition";
    case LIBCONV_ESIZE: return "leading dimension too small";
    case LIBCONV_ECUDA: return "CUDA error";
    case LIBCONV_ENOMEM: return "device allocation failed";
    case LIBCONV_EMODE: return "unknown compute mode";
    case LIBCONV_ETIMEOUT: return "device-side wait timed out";
    case LIBCONV_ENUMERIC: return "non-finite result";
    default: return "unknown status";
    }
}

const char *libconv_gb300_last_error(void) { return t_err.c_str(); }

int libconv_gb300_check(void *stream) {
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    int rc;
    DevState *s = dev_state(rc);
    if (!s) return rc;
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "synchronize");
    return read_status(*s);
}

int libconv_gb300_selftest_wait(int wait_us, void *stream) {
    if (wait_us < 1 || wait_us > 1000000) return fail(LIBCONV_EARG, "wait_us must be in [1, 1e6]");
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    int rc;
    DevState *s = dev_state(rc);
    if (!s) return rc;
    lcg::selftest_wait_kernel<<<1, 32, 0, (cudaStream_t)stream>>>((int *)s->status.p,
                                                                  1000ull * (unsigned long long)wait_us);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LIBCONV_OK : cuda_fail(e, "self-test launch");
}

int libconv_gb300_fp64_peak(int iters, double *tflops, void *stream) {
    if (iters < 1 || iters > (1 << 24) || !tflops) return fail(LIBCONV_EARG, "iters in [1, 2^24], tflops not null");
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "device query");
    const int grid = 8 * sms;          // 8 blocks of 256 threads per SM
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.0f;
    if (e == cudaSuccess) {
        lcg::fp64_peak_kernel<<<grid, 256, 0, st>>>(iters / 8 + 1, 1.0000001, 1e-9);   // warm-up
        e = cudaEventRecord(e0, st);
        if (e == cudaSuccess) lcg::fp64_peak_kernel<<<grid, 256, 0, st>>>(iters, 1.0000001, 1e-9);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(e, "FP64 peak probe");
    const double flops = 2.0 * 8.0 * (double)iters * (double)grid * 256.0;
    *tflops = ms > 0.0f ? flops / (ms * 1e-3) / 1e12 : 0.0;
    return LIBCONV_OK;
}

int libconv_gb300_set_mode(int mode) {
    if (!valid_mode(mode)) return fail(LIBCONV_EMODE, "unknown mode %d", mode);
    t_mode = mode;
    return LIBCONV_OK;
}
int libconv_gb300_get_mode(void) { return t_mode; }

#define LCG_CONV1D(NAME, OP)                                                                     \
    int NAME(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr,     \
             const double *x, double *y, double a, double a_x, double a_y) {                    \
        Plan P;                                                                                 \
        int rc = plan_1d(OP, d, idim, n, bc, nx, ny, narr, a, 1, a_x, a_y, 0, P);               \
        return rc ? rc : exec_host(P, x, y, nullptr);                                           \
    }                                                                                           \
    int NAME##_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, \
                   const double *x, double *y, double a, double a_x, double a_y, void *stream) { \
        Plan P;                                                                                 \
        int rc = plan_1d(OP, d, idim, n, bc, nx, ny, narr, a, 1, a_x, a_y, 0, P);               \
        return rc ? rc : exec_dev(P, x, y, nullptr, nullptr, nullptr, stream);                  \
    }

LCG_CONV1D(d_s0s0_1d_sym8_md, OP_MD)
LCG_CONV1D(d_s0s0_1d_sym8_imd, OP_IMD)
LCG_CONV1D(d_s0s0_1d_sym8_d1, OP_D1)

int d_s0s0_1d_sym8_d2_dotin(int d, int idim, const int *n, int bc, const int *nx, const int *ny,
                            int narr, const double *x, double *y, double a, double a_x,
                            double a_y, double *dot_in) {
    Plan P;
    int rc = plan_1d(OP_D2, d, idim, n, bc, nx, ny, narr, a, 1, a_x, a_y, 1, P);
    return rc ? rc : exec_host(P, x, y, dot_in);
}
int d_s0s0_1d_sym8_d2_dotin_dev(int d, int idim, const int *n, int bc, const int *nx,
                                const int *ny, int narr, const double *x, double *y, double a,
                                double a_x, double a_y, double *dot_in, void *stream) {
    Plan P;
    int rc = plan_1d(OP_D2, d, idim, n, bc, nx, ny, narr, a, 1, a_x, a_y, 1, P);
    return rc ? rc : exec_dev(P, x, y, nullptr, nullptr, dot_in, stream);
}

#define LCG_WAV1D(NAME, OP)                                                                      \
    int NAME(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr,     \
             const double *x, double *y, double a, double a_y) {                                \
        Plan P;                                                                                 \
        int rc = plan_1d(OP, d, idim, n, bc, nx, ny, narr, a, 0, 0.0, a_y, 0, P);               \
        return rc ? rc : exec_host(P, x, y, nullptr);                                           \
    }                                                                                           \
    int NAME##_dev(int d, int idim, const int *n, int bc, const int *nx, const int *ny, int narr, \
                   const double *x, double *y, double a, double a_y, void *stream) {            \
        Plan P;                                                                                 \
        int rc = plan_1d(OP, d, idim, n, bc, nx, ny, narr, a, 0, 0.0, a_y, 0, P);               \
        return rc ? rc : exec_dev(P, x, y, nullptr, nullptr, nullptr, stream);                  \
    }

LCG_WAV1D(d_s0s1_1d_sym8, OP_DWT)
LCG_WAV1D(d_s1s0_1d_sym8, OP_IWT)
LCG_WAV1D(d_s0s1_1d_symicomb8, OP_RTOS1)
LCG_WAV1D(d_s1s0_1d_symicomb8, OP_S1TOR)

#define LCG_MDT(NAME, OP)                                                                        \
    int NAME(int d, const int *n, const int *bc, const int *nx, const int *ny, int narr,        \
             const double *x, double *y, double *w1, double *w2) {                              \
        (void)w1; (void)w2;                                                                     \
        Plan P;                                                                                 \
        int rc = plan_md_t(OP, d, n, bc, nx, ny, narr, P);                                      \
        return rc ? rc : exec_host(P, x, y, nullptr);                                           \
    }                                                                                           \
    int NAME##_dev(int d, const int *n, const int *bc, const int *nx, const int *ny, int narr,  \
                   const double *x, double *y, double *w1, double *w2, void *stream) {          \
        Plan P;                                                                                 \
        int rc = plan_md_t(OP, d, n, bc, nx, ny, narr, P);                                      \
        return rc ? rc : exec_dev(P, x, y, w1, w2, nullptr, stream);                            \
    }

LCG_MDT(d_sfrf_ld_narr, OP_MD)
LCG_MDT(d_rfsf_ld_narr, OP_IMD)

int d_dwt_sym8(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
               double *w2) {
    (void)w1; (void)w2;
    Plan P;
    int rc = plan_md_t(OP_DWT, d, n, bc, nullptr, nullptr, 1, P);
    return rc ? rc : exec_host(P, x, y, nullptr);
}
int d_idwt_sym8(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
                double *w2) {
    (void)w1; (void)w2;
    Plan P;
    int rc = plan_md_t(OP_IWT, d, n, bc, nullptr, nullptr, 1, P);
    return rc ? rc : exec_host(P, x, y, nullptr);
}
int d_dwt_sym8_dev(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
                   double *w2, void *stream) {
    Plan P;
    int rc = plan_md_t(OP_DWT, d, n, bc, nullptr, nullptr, 1, P);
    return rc ? rc : exec_dev(P, x, y, w1, w2, nullptr, stream);
}
int d_idwt_sym8_dev(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
                    double *w2, void *stream) {
    Plan P;
    int rc = plan_md_t(OP_IWT, d, n, bc, nullptr, nullptr, 1, P);
    return rc ? rc : exec_dev(P, x, y, w1, w2, nullptr, stream);
}

int d_dwt_sym8_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y,
                    double *w1, double *w2) {
    (void)w1; (void)w2;
    Plan P;
    int rc = plan_md_t(OP_DWT, d, n, bc, nullptr, nullptr, narr, P);
    return rc ? rc : exec_host(P, x, y, nullptr);
}
int d_idwt_sym8_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y,
                     double *w1, double *w2) {
    (void)w1; (void)w2;
    Plan P;
    int rc = plan_md_t(OP_IWT, d, n, bc, nullptr, nullptr, narr, P);
    return rc ? rc : exec_host(P, x, y, nullptr);
}
int d_dwt_sym8_narr_dev(int d, const int *n, const int *bc, int narr, const double *x,
                        double *y, double *w1, double *w2, void *stream) {
    Plan P;
    int rc = plan_md_t(OP_DWT, d, n, bc, nullptr, nullptr, narr, P);
    return rc ? rc : exec_dev(P, x, y, w1, w2, nullptr, stream);
}
int d_idwt_sym8_narr_dev(int d, const int *n, const int *bc, int narr, const double *x,
                         double *y, double *w1, double *w2, void *stream) {
    Plan P;
    int rc = plan_md_t(OP_IWT, d, n, bc, nullptr, nullptr, narr, P);
    return rc ? rc : exec_dev(P, x, y, w1, w2, nullptr, stream);
}

int d_kin(int d, const int *n, const int *bc, const double *x, double *y, double *w1, double *w2,
          const double *a, double a_x, double a_y) {
    (void)w1; (void)w2;
    Plan P;
    int rc = plan_kin(d, n, bc, a, a_x, a_y, P);
    return rc ? rc : exec_host(P, x, y, nullptr);
}
int d_kin_dev(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
              double *w2, const double *a, double a_x, double a_y, void *stream) {
    Plan P;
    int rc = plan_kin(d, n, bc, a, a_x, a_y, P);
    return rc ? rc : exec_dev(P, x, y, w1, w2, nullptr, stream);
}

int d_kin_ekin(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
               double *w2, const double *a, double a_x, double a_y, double *kstrten) {
    (void)w1; (void)w2;
    Plan P;
    int rc = plan_kin(d, n, bc, a, a_x, a_y, P, 1, nullptr, true);
    return rc ? rc : exec_host(P, x, y, kstrten);
}
int d_kin_ekin_dev(int d, const int *n, const int *bc, const double *x, double *y, double *w1,
                   double *w2, const double *a, double a_x, double a_y, double *kstrten,
                   void *stream) {
    Plan P;
    int rc = plan_kin(d, n, bc, a, a_x, a_y, P, 1, nullptr, true);
    return rc ? rc : exec_dev(P, x, y, w1, w2, kstrten, stream);
}

int d_kin_narr(int d, const int *n, const int *bc, int narr, const double *x, double *y,
               double *w1, double *w2, const double *a, double a_x, double a_y) {
    (void)w1; (void)w2;
    Plan P;
    int rc = plan_kin(d, n, bc, a, a_x, a_y, P, narr);
    return rc ? rc : exec_host(P, x, y, nullptr);
}
int d_kin_narr_dev(int d, const int *n, const int *bc, int narr, const double *x, double *y,
                   double *w1, double *w2, const double *a, double a_x, double a_y, void *stream) {
    Plan P;
    int rc = plan_kin(d, n, bc, a, a_x, a_y, P, narr);
    return rc ? rc : exec_dev(P, x, y, w1, w2, nullptr, stream);
}

int libconv_hamiltonian_sizes(const int *n, const int *bc, long long *nsig, long long *nreal,
                              long long *nwork) {
    return libconv_hamiltonian_narr_sizes(n, bc, 1, nsig, nreal, nwork);
}

int libconv_hamiltonian_narr_sizes(const int *n, const int *bc, int norb, long long *nsig,
                                   long long *nreal, long long *nwork) {
    Ham H;
    const double a1[3] = {1.0, 1.0, 1.0};
    int rc = plan_ham(n, bc, a1, norb, H);
    if (rc) return rc;
    if (nsig) *nsig = (long long)H.nsig;
    if (nreal) *nreal = (long long)H.nreal;
    if (nwork) *nwork = (long long)H.nwork();
    return LIBCONV_OK;
}

int libconv_hamiltonian(const int *n, const int *bc, const double *a_kin, const double *psig,
                        const double *pot, double *rho, double *hpsig, double *ekin, double *epot) {
    if (!ekin || !epot) return fail(LIBCONV_EARG, "ekin/epot must not be null");
    Ham H;
    int rc = plan_ham(n, bc, a_kin, 1, H);
    if (rc) return rc;
    double en[4];
    if ((rc = ham_host(H, psig, pot, rho, hpsig, en))) return rc;
    for (int i = 0; i < 3; ++i) ekin[i] = en[i];
    *epot = en[3];
    return LIBCONV_OK;
}

int libconv_hamiltonian_dev(const int *n, const int *bc, const double *a_kin, const double *psig,
                            const double *pot, double *rho, double *hpsig, double *energies,
                            double *work, void *stream) {
    return libconv_hamiltonian_narr_dev(n, bc, a_kin, 1, psig, pot, rho, hpsig, energies, work,
                                        stream);
}

int libconv_hamiltonian_narr(const int *n, const int *bc, const double *a_kin, int norb,
                             const double *psig, const double *pot, double *rho, double *hpsig,
                             double *energies) {
    Ham H;
    int rc = plan_ham(n, bc, a_kin, norb, H);
    return rc ? rc : ham_host(H, psig, pot, rho, hpsig, energies, n, bc, a_kin);
}

int libconv_hamiltonian_narr_dev(const int *n, const int *bc, const double *a_kin, int norb,
                                 const double *psig, const double *pot, double *rho,
                                 double *hpsig, double *energies, double *work, void *stream) {
    if (!psig || !pot || !hpsig || !energies || !work)
        return fail(LIBCONV_EARG, "psig/pot/hpsig/energies/work must not be null");
    Ham H;
    int rc = plan_ham(n, bc, a_kin, norb, H);
    if (rc) return rc;
    std::lock_guard<std::recursive_mutex> lk(g_mu);
    DevState *s = dev_state(rc);
    if (!s) return rc;
    size_t nd, nl, np;
    ham_scratch(H, nd, nl, np);
    Lease L;
    if ((rc = L.take(s, (cudaStream_t)stream, nd * sizeof(double), nl * sizeof(int),
                     np * sizeof(double))))
        return rc;
    return run_ham(H, psig, pot, rho, hpsig, work, energies, L.scratch(), (double *)L.e->p[2],
                   (int *)s->status.p, (cudaStream_t)stream);
}

int d_s0s0_1d_sym8_md_cost(int d, int idim, const int *n, int bc, int narr, long long *cost) {
    return cost_1d(OP_MD, d, idim, n, bc, narr, cost);
}
int d_s0s0_1d_sym8_d2_cost(int d, int idim, const int *n, int bc, int narr, long long *cost) {
    return cost_1d(OP_D2, d, idim, n, bc, narr, cost);
}
int d_s0s1_1d_sym8_cost(int d, int idim, const int *n, int bc, int narr, long long *cost) {
    return cost_1d(OP_DWT, d, idim, n, bc, narr, cost);
}
int d_sfrf_cost(int d, const int *n, const int *bc, int narr, long long *cost) {
    return cost_md(OP_MD, d, n, bc, narr, cost);
}
int d_kin_cost(int d, const int *n, const int *bc, long long *cost) {
    return cost_md(OP_D2, d, n, bc, 1, cost);
}
int d_dwt_sym8_cost(int d, const int *n, const int *bc, long long *cost) {
    return cost_md(OP_DWT, d, n, bc, 1, cost);
}

}  // extern "C"
