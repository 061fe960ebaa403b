// Batched conjugate-gradient solves of (T - eps_s) x_s = b_s on periodic n^3
// grids, T the 3D kinetic operator (the library's kinetic sweeps), one shift
// eps_s < 0 per system.  All vectors, inner products and scalars are FP64 and
// stay on the device; the host only checks convergence every few iterations.
//
//   plain:    Jacobi-preconditioned CG (the diagonal of T - eps is one number
//             per system, so this is CG on the scaled system);
//   learned:  flexible CG (Notay's FCG(1): exact line search along p and
//             A-orthogonal directions,
//               alpha_k = (p_k, r_k) / (p_k, A p_k),
//               beta_k = -(z_{k+1}, A p_k) / (p_k, A p_k),
//             so the A-norm of the error never grows whatever the
//             preconditioner returns) with z = s M(r / s, eps), s = rms(r),
//             M the 4-layer BF16 network of the conv kernels (cnn.cu).
// A system stops updating once ||r_s|| <= tol ||b_s||; its iteration count
// is the first iteration at which that held.
// Fallback: a system whose residual norm fails to fall below `ratio` times
// its value `window` iterations earlier (libconv_cg_set_stall; default 0.5
// and 10) switches to the plain (Jacobi)
// preconditioner for the rest of its solve: z = jac r inside the same
// recurrence, which is then exactly preconditioned CG (restarted with
// beta = 0 at the switch).
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/libconv_gb300.h"
#include "lcg_plan.cuh"
#include "lcg_pool.cuh"
#include "libconv_filters.h"

namespace {

constexpr int kBPS = 64;        // reduction blocks per system
constexpr int kThreads = 256;
// stagnation test of the learned phase (per calling thread)
thread_local int t_stall_window = 10;
thread_local double t_stall_ratio = 0.5;

// Per-system partial sums of up to two inner products over a system's N
// points; block (b, s) covers a contiguous chunk.
__device__ __forceinline__ void block_sum2(double v0, double v1, double *p0, double *p1, int s, int b) {
    __shared__ double red[2][kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_down_sync(0xffffffffu, v0, o);
        v1 += __shfl_down_sync(0xffffffffu, v1, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { red[0][w] = v0; red[1][w] = v1; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int i = 0; i < kThreads / 32; ++i) { a += red[0][i]; c += red[1][i]; }
        p0[s * kBPS + b] = a;
        if (p1) p1[s * kBPS + b] = c;
    }
}

// Ap = Tp - eps p; partials (p, Ap) and, when r is given, (p, r)
__global__ void k_shift(const double *__restrict__ Tp, const double *__restrict__ p,
                        const double *__restrict__ eps, double *__restrict__ Ap,
                        const double *__restrict__ r, double *part, double *part_pr, long long N,
                        const int *active) {
    const int s = blockIdx.y, b = blockIdx.x;
    if (active && !active[s]) {                  // converged: nothing to update
        if (threadIdx.x == 0) { part[s * kBPS + b] = 0.0; if (r) part_pr[s * kBPS + b] = 0.0; }
        return;
    }
    const long long lo = N * b / kBPS, hi = N * (b + 1) / kBPS, off = (long long)s * N;
    const double e = eps[s];
    double acc = 0.0, pr = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += kThreads) {
        const double pv = p[off + i];
        const double a = Tp[off + i] - e * pv;
        Ap[off + i] = a;
        acc = fma(pv, a, acc);
        if (r) pr = fma(pv, r[off + i], pr);
    }
    block_sum2(acc, pr, part, r ? part_pr : nullptr, s, b);
}

// x += alpha p; r -= alpha Ap; partial (r, r)
__global__ void k_update(double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
                         const double *__restrict__ Ap, const double *__restrict__ alpha, double *part,
                         long long N, const int *active) {
    const int s = blockIdx.y, b = blockIdx.x;
    if (!active[s]) {                            // converged: x, r unchanged, (r, r) kept
        if (threadIdx.x == 0) part[s * kBPS + b] = -1.0;
        return;
    }
    const long long lo = N * b / kBPS, hi = N * (b + 1) / kBPS, off = (long long)s * N;
    const double al = alpha[s];
    double acc = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += kThreads) {
        x[off + i] = fma(al, p[off + i], x[off + i]);
        const double rv = fma(-al, Ap[off + i], r[off + i]);
        r[off + i] = rv;
        acc = fma(rv, rv, acc);
    }
    block_sum2(acc, 0.0, part, nullptr, s, b);
}

// partials (z, r) and (z, Ap)
__global__ void k_dot2(const double *__restrict__ z, const double *__restrict__ r,
                       const double *__restrict__ Ap, double *p0, double *p1, long long N,
                       const int *active = nullptr) {
    const int s = blockIdx.y, b = blockIdx.x;
    if (active && !active[s]) {
        if (threadIdx.x == 0) { p0[s * kBPS + b] = 0.0; p1[s * kBPS + b] = 0.0; }
        return;
    }
    const long long lo = N * b / kBPS, hi = N * (b + 1) / kBPS, off = (long long)s * N;
    double a = 0.0, c = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += kThreads) {
        const double zv = z[off + i];
        a = fma(zv, r[off + i], a);
        c = fma(zv, Ap[off + i], c);
    }
    block_sum2(a, c, p0, p1, s, b);
}

// p = coef_s v + beta_s p   (coef = null: 1)
__global__ void k_direction(double *__restrict__ p, const double *__restrict__ v,
                            const double *__restrict__ coef, const double *__restrict__ beta,
                            long long N, const int *active = nullptr) {
    const int s = blockIdx.y;
    if (active && !active[s]) return;
    const long long off = (long long)s * N;
    const double c = coef ? coef[s] : 1.0, be = beta[s];
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < N;
         i += (long long)gridDim.x * kThreads)
        p[off + i] = fma(be, p[off + i], c * v[off + i]);
}

// y = b - y (residual from y = A x)
__global__ void k_residual(const double *__restrict__ b, double *__restrict__ y, double *part,
                           long long N) {
    const int s = blockIdx.y, bl = blockIdx.x;
    const long long lo = N * bl / kBPS, hi = N * (bl + 1) / kBPS, off = (long long)s * N;
    double acc = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += kThreads) {
        const double v = b[off + i] - y[off + i];
        y[off + i] = v;
        acc = fma(v, v, acc);
    }
    block_sum2(acc, 0.0, part, nullptr, s, bl);
}

__device__ __forceinline__ double sum_parts(const double *part, int s) {
    double a = 0.0;
    for (int i = 0; i < kBPS; ++i) a += part[s * kBPS + i];
    return a;
}

struct Scalars {
    double *rz, *rr, *alpha, *beta, *jac, *scale, *inv_scale, *bnorm, *pAp, *rr_mark;
    int *active, *iters, *fallback;
};

// alpha = (z, r) / (p, Ap) (plain) or (p, r) / (p, Ap) (flexible) for active
// systems, else 0
__global__ void k_alpha(Scalars S, const double *pAp_part, const double *pr_part, int nsys) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const double pAp = sum_parts(pAp_part, s);
    const double num = pr_part ? sum_parts(pr_part, s) : S.rz[s];
    S.pAp[s] = pAp;
    S.alpha[s] = (S.active[s] && pAp > 0.0) ? num / pAp : 0.0;
}

// after the update: rr, convergence, the preconditioner scale; plain CG also
// forms beta (z = jac r, so (z, r) = jac rr)
__global__ void k_after_update(Scalars S, const double *rr_part, int nsys, long long N, double tol,
                               int it, int plain, int window, double ratio) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    if (!S.active[s]) return;                    // converged earlier: scalars frozen
    const double rr = sum_parts(rr_part, s);
    S.rr[s] = rr;
    if (!isfinite(rr)) {          // breakdown: stop, report -it
        S.active[s] = 0;
        S.iters[s] = -it;
    } else if (sqrt(rr) <= tol * S.bnorm[s]) {
        S.active[s] = 0;
        S.iters[s] = it;
    }
    const double sc = rr > 0.0 ? sqrt(rr / (double)N) : 1.0;
    S.scale[s] = sc;
    S.inv_scale[s] = 1.0 / sc;
    if (!plain && it % window == 0) {            // stagnation test of the learned phase
        if (S.active[s] && !S.fallback[s] && rr > ratio * ratio * S.rr_mark[s]) S.fallback[s] = it;
        S.rr_mark[s] = rr;
    }
    if (plain) {
        const double rz = S.jac[s] * rr;
        S.beta[s] = S.active[s] && S.rz[s] > 0.0 ? rz / S.rz[s] : 0.0;
        S.rz[s] = rz;
    }
}

// flexible CG: beta = -(z, Ap) / (p, Ap); (z, r) is kept as rz; beta = 0
// at the iteration a system switches to the fallback
__global__ void k_beta_fcg(Scalars S, const double *zr_part, const double *zAp_part, int nsys,
                           int it) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const double zr = sum_parts(zr_part, s), zAp = sum_parts(zAp_part, s);
    const bool restart = S.fallback[s] == it;
    S.beta[s] = (S.active[s] && S.pAp[s] > 0.0 && !restart) ? -zAp / S.pAp[s] : 0.0;
    S.rz[s] = zr;
}

// z = jac r for the systems on the fallback
__global__ void k_fallback_z(const Scalars S, double *__restrict__ z, const double *__restrict__ r,
                             long long N) {
    const int s = blockIdx.y;
    if (!S.fallback[s]) return;
    const long long off = (long long)s * N;
    const double j = S.jac[s];
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < N;
         i += (long long)gridDim.x * kThreads)
        z[off + i] = j * r[off + i];
}

// initial scalars from (b, b) (and (z0, r0) for the learned form)
__global__ void k_init(Scalars S, const double *rr_part, const double *eps, double dcoef, int nsys,
                       long long N) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const double rr = sum_parts(rr_part, s);
    S.rr[s] = rr;
    S.bnorm[s] = sqrt(rr);
    S.active[s] = rr > 0.0;
    S.iters[s] = 0;
    S.fallback[s] = 0;
    S.rr_mark[s] = rr;
    S.jac[s] = 1.0 / (dcoef - eps[s]);
    S.rz[s] = S.jac[s] * rr;
    S.beta[s] = 0.0;
    const double sc = rr > 0.0 ? sqrt(rr / (double)N) : 1.0;
    S.scale[s] = sc;
    S.inv_scale[s] = 1.0 / sc;
}

__global__ void k_set_rz(Scalars S, const double *zr_part, int nsys) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    S.rz[s] = sum_parts(zr_part, s);
}

__global__ void k_norms(const double *part, double *out, int nsys) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    out[s] = sqrt(sum_parts(part, s));
}

// ---- workspace -------------------------------------------------------------------
// Per device, a pool of workspaces leased per call (lcg_pool.cuh): an apply
// only enqueues on the caller's stream, so calls on different streams get
// different workspaces.
std::mutex g_mu;
lcg::StreamPool g_pool[64];

struct WorkLease {
    lcg::StreamPool *pool = nullptr;
    lcg::PoolEntry *e = nullptr;
    cudaStream_t st = nullptr;
    WorkLease() = default;
    WorkLease(const WorkLease &) = delete;
    WorkLease &operator=(const WorkLease &) = delete;
    ~WorkLease() { if (pool && e) pool->release(e, st); }
    void *p() const { return e->p[0]; }
};

int lease(WorkLease &w, size_t bytes, cudaStream_t st) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return lcg::report(LIBCONV_ECUDA, "no current device");
    const cudaError_t e = g_pool[dev].acquire(st, &bytes, 1, w.e);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return lcg::report(e == cudaErrorMemoryAllocation ? LIBCONV_ENOMEM : LIBCONV_ECUDA,
                           "CG workspace allocation failed");
    }
    w.pool = &g_pool[dev];
    w.st = st;
    return LIBCONV_OK;
}

// A x for all systems: y = T x - eps x; pAp partials of (x, y)
int apply_A(int n, int nsys, const double a[3], const double *eps, const double *x, double *y,
            double *w1, double *w2, double *Tx, double *part, cudaStream_t st,
            const double *r_for_pr = nullptr, double *part_pr = nullptr,
            const int *active = nullptr) {
    const int dims[3] = {n, n, n}, bc[3] = {0, 0, 0};
    // converged systems (active[s] == 0) are left out of the sweeps
    int rc = active ? lcg::kin_narr_active_dev(3, dims, bc, nsys, x, Tx, w1, w2, a, active, st)
                    : d_kin_narr_dev(3, dims, bc, nsys, x, Tx, w1, w2, a, 0.0, 0.0, st);
    if (rc) return rc;
    const long long N = (long long)n * n * n;
    k_shift<<<dim3(kBPS, nsys), kThreads, 0, st>>>(Tx, x, eps, y, r_for_pr, part, part_pr, N, active);
    return cudaGetLastError() == cudaSuccess ? LIBCONV_OK : lcg::report(LIBCONV_ECUDA, "k_shift launch");
}

// z = s M(r / s, eps): the four conv layers
int precondition(int n, int nsys, const libconv_cnn_weights *W, const double *r, const double *eps,
                 const double *scale, const double *inv_scale, void *act1, void *act2, double *z,
                 const int *active, cudaStream_t st) {
    int rc = libconv_cnn_conv(n, nsys, 1, 0, r, inv_scale, eps, W->wt[0], W->bias[0], act1, nullptr,
                              nullptr, 16, active, st);
    if (!rc) rc = libconv_cnn_conv(n, nsys, 0, 0, act1, nullptr, nullptr, W->wt[1], W->bias[1], act2,
                                   nullptr, nullptr, 16, active, st);
    if (!rc) rc = libconv_cnn_conv(n, nsys, 0, 0, act2, nullptr, nullptr, W->wt[2], W->bias[2], act1,
                                   nullptr, nullptr, 16, active, st);
    if (!rc) rc = libconv_cnn_conv(n, nsys, 0, 1, act1, nullptr, nullptr, W->wt[3], W->bias[3], z,
                                   scale, nullptr, 1, active, st);
    return rc ? lcg::report(rc, "preconditioner convolution failed") : LIBCONV_OK;
}

}  // namespace

extern "C" {

int libconv_cg_set_stall(int window, double ratio) {
    if (window < 1 || !(ratio > 0.0) || ratio > 1.0)
        return lcg::report(LIBCONV_EARG, "stall window must be >= 1 and ratio in (0, 1]");
    t_stall_window = window;
    t_stall_ratio = ratio;
    return LIBCONV_OK;
}

int libconv_cg_apply(int n, int nsys, const double *h, const double *eps, const double *x, double *y,
                     void *stream) {
    if (n < 1 || nsys < 1 || !h || !eps || !x || !y) return lcg::report(LIBCONV_EARG, "bad CG apply arguments");
    const long long N = (long long)n * n * n;
    std::lock_guard<std::mutex> lk(g_mu);
    const size_t need = sizeof(double) * (3 * N * nsys + (size_t)kBPS * nsys);
    WorkLease w;
    int rc = lease(w, need, (cudaStream_t)stream);
    if (rc) return rc;
    double *w1 = (double *)w.p(), *w2 = w1 + N * nsys, *Tx = w2 + N * nsys, *part = Tx + N * nsys;
    const double a[3] = {-0.5 / (h[0] * h[0]), -0.5 / (h[1] * h[1]), -0.5 / (h[2] * h[2])};
    return apply_A(n, nsys, a, eps, x, y, w1, w2, Tx, part, (cudaStream_t)stream);
}

int libconv_cg_solve(int n, int nsys, const double *h, const double *eps, const double *b, double *x,
                     double tol, int maxit, const libconv_cnn_weights *W, int *iters, double *res,
                     int *fell_back, void *stream) {
    if (n < 8 || n % 8 || nsys < 1 || !h || !eps || !b || !x || maxit < 0)
        return lcg::report(LIBCONV_EARG, "bad CG solve arguments (n must be a multiple of 8)");
    cudaStream_t st = (cudaStream_t)stream;
    const long long N = (long long)n * n * n, SN = N * nsys;
    std::lock_guard<std::mutex> lk(g_mu);
    // r, p, Ap, z, Tp, w1, w2 (FP64 vectors); two 16-channel BF16 activations;
    // partial sums; scalars
    const size_t vec = sizeof(double) * SN, act = sizeof(__nv_bfloat16) * 16 * SN;
    const size_t parts = sizeof(double) * kBPS * nsys;
    // 15 sub-buffers, each rounded up to 256 bytes
    const size_t need = 7 * vec + 2 * act + 5 * parts + sizeof(double) * 10 * nsys +
                        sizeof(int) * 3 * nsys + 17 * 256;
    WorkLease w;
    int rc = lease(w, need, st);
    if (rc) return rc;
    uint8_t *q = (uint8_t *)w.p();
    auto take = [&](size_t bytes) { uint8_t *r = q; q += (bytes + 255) & ~(size_t)255; return r; };
    double *r = (double *)take(vec), *p = (double *)take(vec), *Ap = (double *)take(vec),
           *z = (double *)take(vec), *Tp = (double *)take(vec), *w1 = (double *)take(vec),
           *w2 = (double *)take(vec);
    void *act1 = take(act), *act2 = take(act);
    double *pa = (double *)take(parts), *pb = (double *)take(parts), *pc = (double *)take(parts),
           *pd = (double *)take(parts), *pe = (double *)take(parts);
    Scalars S;
    double *sc = (double *)take(sizeof(double) * 10 * nsys);
    S.rz = sc; S.rr = sc + nsys; S.alpha = sc + 2 * nsys; S.beta = sc + 3 * nsys;
    S.jac = sc + 4 * nsys; S.scale = sc + 5 * nsys; S.inv_scale = sc + 6 * nsys; S.bnorm = sc + 7 * nsys;
    S.pAp = sc + 8 * nsys; S.rr_mark = sc + 9 * nsys;
    int *ic = (int *)take(sizeof(int) * 3 * nsys);
    S.active = ic; S.iters = ic + nsys; S.fallback = ic + 2 * nsys;

    const double a[3] = {-0.5 / (h[0] * h[0]), -0.5 / (h[1] * h[1]), -0.5 / (h[2] * h[2])};
    // diagonal of T: sum_d a_d D2(0) (the centre tap of the second derivative)
    const double d2c = lcg::filter_table()[LCG_FTAB_D2 - LCG_CONV_SYM8_D2_LOWFIL];
    const double dcoef = (a[0] + a[1] + a[2]) * d2c;
    const dim3 vgrid(kBPS, nsys), sgrid((nsys + 127) / 128);
    const bool learned = W != nullptr;

    cudaError_t e = cudaMemsetAsync(x, 0, vec, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, vec, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r, b, vec, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return lcg::report_cuda(e, "CG initialisation");
    k_dot2<<<vgrid, kThreads, 0, st>>>(r, r, r, pa, pb, N);   // (b, b)
    k_init<<<sgrid, 128, 0, st>>>(S, pa, eps, dcoef, nsys, N);
    if (learned) {
        if ((rc = precondition(n, nsys, W, r, eps, S.scale, S.inv_scale, act1, act2, z, nullptr, st)))
            return rc;
        k_dot2<<<vgrid, kThreads, 0, st>>>(z, r, r, pa, pb, N);
        k_set_rz<<<sgrid, 128, 0, st>>>(S, pa, nsys);
        e = cudaMemcpyAsync(p, z, vec, cudaMemcpyDeviceToDevice, st);
    } else {
        k_direction<<<dim3(kBPS, nsys), kThreads, 0, st>>>(p, r, S.jac, S.beta, N);   // p = jac r
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return lcg::report_cuda(e, "CG start");

    std::vector<int> h_active(nsys), h_fb(nsys);
    int it = 0;
    const int check_every = 8;
    bool use_net = learned;     // false once every active system is on the fallback
    while (it < maxit) {
        ++it;
        if ((rc = apply_A(n, nsys, a, eps, p, Ap, w1, w2, Tp, pa, st, learned ? r : nullptr,
                          learned ? pe : nullptr, S.active)))
            return rc;
        k_alpha<<<sgrid, 128, 0, st>>>(S, pa, learned ? pe : nullptr, nsys);
        k_update<<<vgrid, kThreads, 0, st>>>(x, r, p, Ap, S.alpha, pb, N, S.active);
        k_after_update<<<sgrid, 128, 0, st>>>(S, pb, nsys, N, tol, it, learned ? 0 : 1,
                                              t_stall_window, t_stall_ratio);
        if (learned) {
            if (use_net &&
                (rc = precondition(n, nsys, W, r, eps, S.scale, S.inv_scale, act1, act2, z, S.active,
                                   st)))
                return rc;
            k_fallback_z<<<dim3(kBPS, nsys), kThreads, 0, st>>>(S, z, r, N);
            k_dot2<<<vgrid, kThreads, 0, st>>>(z, r, Ap, pc, pd, N, S.active);
            k_beta_fcg<<<sgrid, 128, 0, st>>>(S, pc, pd, nsys, it);
            k_direction<<<dim3(kBPS, nsys), kThreads, 0, st>>>(p, z, nullptr, S.beta, N, S.active);
        } else {
            k_direction<<<dim3(kBPS, nsys), kThreads, 0, st>>>(p, r, S.jac, S.beta, N, S.active);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return lcg::report_cuda(e, "CG iteration launch");
        if (it % check_every == 0 || it == maxit) {
            e = cudaMemcpyAsync(h_active.data(), S.active, sizeof(int) * nsys, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return lcg::report_cuda(e, "CG convergence check");
            bool any = false;
            for (int v : h_active) any |= v != 0;
            if (!any) break;
            if (use_net) {   // the network is still needed by some active system?
                e = cudaMemcpy(h_fb.data(), S.fallback, sizeof(int) * nsys, cudaMemcpyDeviceToHost);
                if (e != cudaSuccess) return lcg::report_cuda(e, "CG fallback check");
                bool need = false;
                for (int s2 = 0; s2 < nsys; ++s2) need |= h_active[s2] && !h_fb[s2];
                use_net = need;
            }
        }
    }
    // iteration counts (maxit + 1 for systems that did not converge) and the
    // true residual norms ||b - A x|| recomputed with the FP64 operator
    if (iters) {
        std::vector<int> act_h(nsys), it_h(nsys);
        e = cudaMemcpyAsync(act_h.data(), S.active, sizeof(int) * nsys, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(it_h.data(), S.iters, sizeof(int) * nsys, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return lcg::report_cuda(e, "CG iteration counts");
        for (int s = 0; s < nsys; ++s) iters[s] = act_h[s] ? maxit + 1 : it_h[s];
        for (int s = 0; s < nsys; ++s)
            if (iters[s] < 0) return lcg::report(LIBCONV_ENUMERIC, "CG breakdown: non-finite residual");
    }
    if (fell_back) {
        e = cudaMemcpyAsync(fell_back, S.fallback, sizeof(int) * nsys, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return lcg::report_cuda(e, "CG fallback flags");
    }
    if (res) {
        if ((rc = apply_A(n, nsys, a, eps, x, Ap, w1, w2, Tp, pa, st))) return rc;
        k_residual<<<vgrid, kThreads, 0, st>>>(b, Ap, pa, N);
        k_norms<<<sgrid, 128, 0, st>>>(pa, S.rr, nsys);
        e = cudaMemcpyAsync(res, S.rr, sizeof(double) * nsys, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return lcg::report_cuda(e, "CG residual");
    }
    auto lib = lcg::library_lock();
    return lcg::host_finish(st);   // device status word of the bounded tensor-core waits
}

}  // extern "C"
