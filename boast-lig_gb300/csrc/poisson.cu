// Poisson finite-difference operators (BigDFT/Poisson.rb): the 1D broker
// (Poisson_broker, :1951-2043) and the generated 3D drivers div_u_i,
// nabla_u, nabla_u_and_square, nabla_u_square, nabla_u_epsilon and
// update_rhopol (:2067-2620), on GB300.
//
// Each derivative is one sweep of the central stencil through the library's
// sweep engines (lcg::poisson_sweep: FP64 or tensor-core, per the calling
// thread's mode) plus, along non-periodic axes, the one-sided boundary
// outputs from poisson_edge_kernel.  div_u_i accumulates its three
// derivatives in du (the second and third sweeps add into it), which is the
// generated code's (d0 + d1) + d2 without the three temporaries; the other
// drivers finish with one element-wise kernel.  Element-wise kernels are
// grid-stride loops over the points, consecutive threads on consecutive
// points.
#include <cstring>

#include "../../include/libconv_gb300.h"
#include "lcg_plan.cuh"
#include "lcg_sweep.cuh"
#include "libconv_filters.h"

namespace lcg {
namespace {

__constant__ double c_fd_edge[LCG_FD_EDGE_N] = LCG_FD_EDGE_INIT;

constexpr int kThreads = 256;
constexpr double kOneO4Pi = 0.07957747154594766788444188168625718101722982287022822437383367203;

int edge_offset(int nord) {
    switch (nord) {
    case 2: return LCG_FD_EDGE_OFF_2;
    case 4: return LCG_FD_EDGE_OFF_4;
    case 6: return LCG_FD_EDGE_OFF_6;
    case 8: return LCG_FD_EDGE_OFF_8;
    case 16: return LCG_FD_EDGE_OFF_16;
    default: return -1;
    }
}

int grid_for(long long count) {
    long long b = (count + kThreads - 1) / kThreads;
    if (b > 152LL * 16) b = 152LL * 16;
    return b < 1 ? 1 : (int)b;
}

// One thread per (line, boundary output); l fastest so strided lines read
// coalesced.  Output e < m is point e (stencil row e, nodes 0..2m); e >= m is
// point n-2m+e (row e+1, nodes n-1-2m..n-1).  Taps in node order.
__global__ void poisson_edge_kernel(const double *__restrict__ x, double *__restrict__ y,
                                    long long nL, int n, long long nR, int m, int off, double a,
                                    int accumulate) {
    const long long total = nL * nR * 2 * m;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long l = t % nL, rest = t / nL;
        const int e = (int)(rest % (2 * m));
        const long long r = rest / (2 * m);
        const int i = e < m ? e : n - 2 * m + e;
        const int w0 = e < m ? 0 : n - 1 - 2 * m;
        const double *c = c_fd_edge + off + (e < m ? e : e + 1) * (2 * m + 1);
        const double *xl = x + l + nL * (long long)n * r;
        double tt = 0.0;
        for (int j = 0; j <= 2 * m; ++j) tt = fma(c[j], xl[nL * (w0 + j)], tt);
        double out = tt * a;
        double *yp = y + l + nL * ((long long)n * r + i);
        if (accumulate) out += *yp;
        *yp = out;
    }
}

// div_u_i with cc (Poisson.rb:2132-2160): du holds d0 u0, t the five other
// derivatives (d1 u1, d2 u2, d0 u1, d0 u2, d1 u2).
__global__ void div_cc_kernel(const double *__restrict__ u, double *__restrict__ du,
                              const double *__restrict__ t, double *__restrict__ cc, long long N) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < N;
         k += (long long)gridDim.x * blockDim.x) {
        const double u0 = u[k], u1 = u[N + k], u2 = u[2 * N + k];
        const double du0 = du[k], du1 = t[k], du2 = t[N + k];
        cc[k] = (u0 * u0) * du0 + (u1 * u1) * du1 + (u2 * u2) * du2 +
                2.0 * (u0 * u1 * t[2 * N + k] + u0 * u2 * t[3 * N + k] + u1 * u2 * t[4 * N + k]);
        du[k] = du0 + du1 + du2;
    }
}

__global__ void square_kernel(const double *__restrict__ du, double *__restrict__ ddu, long long N) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < N;
         k += (long long)gridDim.x * blockDim.x) {
        const double a = du[k], b = du[N + k], c = du[2 * N + k];
        ddu[k] = (a * a) + (b * b) + (c * c);
    }
}

__global__ void epsilon_kernel(double *__restrict__ du, const double *__restrict__ eps, long long N) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < N;
         k += (long long)gridDim.x * blockDim.x) {
        const double e = eps[k];
        du[k] *= e;
        du[N + k] *= e;
        du[2 * N + k] *= e;
    }
}

// update_rhopol's point update (Poisson.rb:2496-2509); one partial of
// rhores2 per block (fixed-order warp, then block sum).
__global__ void rhopol_kernel(const double *__restrict__ du, const double *__restrict__ dlogeps,
                              double *__restrict__ rhopol, long long N, double eta,
                              double *__restrict__ part) {
    __shared__ double ws[kThreads / 32];
    double acc = 0.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < N;
         k += (long long)gridDim.x * blockDim.x) {
        double res = dlogeps[3 * k] * du[k] + dlogeps[3 * k + 1] * du[N + k] +
                     dlogeps[3 * k + 2] * du[2 * N + k];
        res = res * kOneO4Pi;
        const double rho = rhopol[k];
        res = (res - rho) * eta;
        acc = fma(res, res, acc);
        rhopol[k] = res + rho;
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += ws[w];
        part[blockIdx.x] = s;
    }
}

int geocode_bc(int geocode, int bc[3]) {
    if (geocode < 1 || geocode > 3) return report(LIBCONV_EARG, "geocode must be 1 (free), 2 (periodic) or 3 (surface)");
    bc[0] = bc[1] = bc[2] = LIBCONV_BC_PERIODIC;
    if (geocode == 1) bc[0] = bc[2] = LIBCONV_BC_NPERIODIC;
    if (geocode != 2) bc[1] = LIBCONV_BC_NPERIODIC;
    return LIBCONV_OK;
}

int check3(int n01, int n02, int n03, const double *hgrids) {
    if (n01 < 1 || n02 < 1 || n03 < 1) return report(LIBCONV_EARG, "grid extents must be >= 1");
    if (!hgrids) return report(LIBCONV_EARG, "hgrids must not be null");
    return LIBCONV_OK;
}

cudaError_t last(void) { return cudaGetLastError(); }

int cuda_rc(cudaError_t e, const char *what) {
    return e == cudaSuccess ? LIBCONV_OK : report_cuda(e, what);
}

// du[i] = d_i u for i = 0, 1, 2 (three arrays of N back to back).
int nabla3(int geocode, const int nn[3], const double *u, double *du, int nord,
           const double *hgrids, cudaStream_t st) {
    int bc[3], rc = geocode_bc(geocode, bc);
    const long long N = (long long)nn[0] * nn[1] * nn[2];
    for (int i = 0; i < 3 && !rc; ++i)
        rc = poisson_sweep(nord, i, nn, bc[i], 1.0 / hgrids[i], false, u, du + i * N, st);
    return rc;
}

// ---- device implementations -------------------------------------------------------
int div_u_i_impl(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                 const double *hgrids, double *cc, double *work, cudaStream_t st) {
    int rc = check3(n01, n02, n03, hgrids), bc[3];
    if (rc || (rc = geocode_bc(geocode, bc))) return rc;
    if (!u || !du) return report(LIBCONV_EARG, "u/du must not be null");
    const int nn[3] = {n01, n02, n03};
    const long long N = (long long)n01 * n02 * n03;
    const double a[3] = {1.0 / hgrids[0], 1.0 / hgrids[1], 1.0 / hgrids[2]};
    if (!cc) {
        for (int i = 0; i < 3 && !rc; ++i)
            rc = poisson_sweep(nord, i, nn, bc[i], a[i], i > 0, u + i * N, du, st);
        return rc;
    }
    if (!work) return report(LIBCONV_EARG, "div_u_i with cc needs a work array of 5 n01 n02 n03");
    // (component, axis) of du and of the five temporaries
    const int comp[6] = {0, 1, 2, 1, 2, 2}, axis[6] = {0, 1, 2, 0, 0, 1};
    for (int k = 0; k < 6 && !rc; ++k)
        rc = poisson_sweep(nord, axis[k], nn, bc[axis[k]], a[axis[k]], false, u + comp[k] * N,
                           k == 0 ? du : work + (k - 1) * N, st);
    if (rc) return rc;
    div_cc_kernel<<<grid_for(N), kThreads, 0, st>>>(u, du, work, cc, N);
    return cuda_rc(last(), "div_u_i cc launch");
}

int nabla_u_impl(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                 const double *hgrids, cudaStream_t st) {
    int rc = check3(n01, n02, n03, hgrids);
    if (rc) return rc;
    if (!u || !du) return report(LIBCONV_EARG, "u/du must not be null");
    const int nn[3] = {n01, n02, n03};
    return nabla3(geocode, nn, u, du, nord, hgrids, st);
}

int nabla_u_and_square_impl(int geocode, int n01, int n02, int n03, const double *u, double *du,
                            double *ddu, int nord, const double *hgrids, cudaStream_t st) {
    if (!ddu) return report(LIBCONV_EARG, "ddu must not be null");
    int rc = nabla_u_impl(geocode, n01, n02, n03, u, du, nord, hgrids, st);
    if (rc) return rc;
    const long long N = (long long)n01 * n02 * n03;
    square_kernel<<<grid_for(N), kThreads, 0, st>>>(du, ddu, N);
    return cuda_rc(last(), "square launch");
}

int nabla_u_epsilon_impl(int geocode, int n01, int n02, int n03, const double *u, double *du,
                         int nord, const double *hgrids, const double *eps, cudaStream_t st) {
    if (!eps) return report(LIBCONV_EARG, "eps must not be null");
    int rc = nabla_u_impl(geocode, n01, n02, n03, u, du, nord, hgrids, st);
    if (rc) return rc;
    const long long N = (long long)n01 * n02 * n03;
    epsilon_kernel<<<grid_for(N), kThreads, 0, st>>>(du, eps, N);
    return cuda_rc(last(), "epsilon launch");
}

long long rhopol_parts(long long N) { return grid_for(N); }

int update_rhopol_impl(int geocode, int n01, int n02, int n03, const double *u, int nord,
                       const double *hgrids, double eta, const double *dlogeps, double *rhopol,
                       double *rhores2, double *work, cudaStream_t st) {
    if (!dlogeps || !rhopol || !rhores2 || !work)
        return report(LIBCONV_EARG, "dlogeps/rhopol/rhores2/work must not be null");
    const long long N = (long long)n01 * n02 * n03;
    int rc = nabla_u_impl(geocode, n01, n02, n03, u, work, nord, hgrids, st);
    if (rc) return rc;
    const int nb = grid_for(N);
    rhopol_kernel<<<nb, kThreads, 0, st>>>(work, dlogeps, rhopol, N, eta, work + 3 * N);
    cudaError_t e = last();
    if (e == cudaSuccess) e = launch_dot_reduce(work + 3 * N, nb, rhores2, 0, st);
    return cuda_rc(e, "update_rhopol launch");
}

// ---- host staging --------------------------------------------------------------------
struct Stage {
    double *base = nullptr;
    size_t used = 0;
    double *take(size_t n) { double *p = base + used; used += n; return p; }
};

int to_dev(double *d, const double *h, size_t n, cudaStream_t st) {
    return cuda_rc(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, st), "copy to device");
}
int to_host(double *h, const double *d, size_t n, cudaStream_t st) {
    return cuda_rc(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, st), "copy to host");
}

}  // namespace

cudaError_t launch_poisson_edges(const double *x, double *y, long long nL, int n, long long nR,
                                 int nord, double a, int accumulate, cudaStream_t st) {
    const int off = edge_offset(nord);
    if (off < 0) return cudaErrorInvalidValue;
    const int m = nord / 2;
    poisson_edge_kernel<<<grid_for(nL * nR * 2 * m), kThreads, 0, st>>>(x, y, nL, n, nR, m, off, a,
                                                                        accumulate);
    return cudaGetLastError();
}

}  // namespace lcg

using namespace lcg;

extern "C" {

int Poisson_broker(int nord, int idim, const int *nn, int bc, const double *u, double *du,
                   double a) {
    if (!nn || !u || !du) return report(LIBCONV_EARG, "nn/u/du must not be null");
    if (nn[0] < 1 || nn[1] < 1 || nn[2] < 1) return report(LIBCONV_EARG, "nn must be >= 1");
    const size_t N = (size_t)nn[0] * nn[1] * nn[2];
    auto lk = library_lock();
    cudaStream_t st;
    int rc;
    Stage S;
    S.base = host_staging(2 * N * sizeof(double), st, rc);
    if (!S.base) return rc;
    double *dx = S.take(N), *dy = S.take(N);
    if ((rc = to_dev(dx, u, N, st))) return rc;
    if ((rc = poisson_sweep(nord, idim, nn, bc, a, false, dx, dy, st))) return rc;
    if ((rc = to_host(du, dy, N, st))) return rc;
    return host_finish(st);
}

int Poisson_broker_dev(int nord, int idim, const int *nn, int bc, const double *u, double *du,
                       double a, void *stream) {
    return poisson_sweep(nord, idim, nn, bc, a, false, u, du, (cudaStream_t)stream);
}

int div_u_i(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
            const double *hgrids, double *cc) {
    int rc = check3(n01, n02, n03, hgrids);
    if (rc) return rc;
    if (!u || !du) return report(LIBCONV_EARG, "u/du must not be null");
    const size_t N = (size_t)n01 * n02 * n03;
    auto lk = library_lock();
    cudaStream_t st;
    Stage S;
    S.base = host_staging((cc ? 10 : 4) * N * sizeof(double), st, rc);
    if (!S.base) return rc;
    double *du_ = S.take(3 * N), *dd = S.take(N);
    double *dcc = cc ? S.take(N) : nullptr, *w = cc ? S.take(5 * N) : nullptr;
    if ((rc = to_dev(du_, u, 3 * N, st))) return rc;
    if ((rc = div_u_i_impl(geocode, n01, n02, n03, du_, dd, nord, hgrids, dcc, w, st))) return rc;
    if ((rc = to_host(du, dd, N, st))) return rc;
    if (cc && (rc = to_host(cc, dcc, N, st))) return rc;
    return host_finish(st);
}

int div_u_i_dev(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                const double *hgrids, double *cc, double *work, void *stream) {
    return div_u_i_impl(geocode, n01, n02, n03, u, du, nord, hgrids, cc, work, (cudaStream_t)stream);
}

int nabla_u(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
            const double *hgrids) {
    int rc = check3(n01, n02, n03, hgrids);
    if (rc) return rc;
    if (!u || !du) return report(LIBCONV_EARG, "u/du must not be null");
    const size_t N = (size_t)n01 * n02 * n03;
    auto lk = library_lock();
    cudaStream_t st;
    Stage S;
    S.base = host_staging(4 * N * sizeof(double), st, rc);
    if (!S.base) return rc;
    double *du_ = S.take(N), *dd = S.take(3 * N);
    if ((rc = to_dev(du_, u, N, st))) return rc;
    if ((rc = nabla_u_impl(geocode, n01, n02, n03, du_, dd, nord, hgrids, st))) return rc;
    if ((rc = to_host(du, dd, 3 * N, st))) return rc;
    return host_finish(st);
}

int nabla_u_dev(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                const double *hgrids, void *stream) {
    return nabla_u_impl(geocode, n01, n02, n03, u, du, nord, hgrids, (cudaStream_t)stream);
}

int nabla_u_and_square(int geocode, int n01, int n02, int n03, const double *u, double *du,
                       double *ddu, int nord, const double *hgrids) {
    int rc = check3(n01, n02, n03, hgrids);
    if (rc) return rc;
    if (!u || !du || !ddu) return report(LIBCONV_EARG, "u/du/ddu must not be null");
    const size_t N = (size_t)n01 * n02 * n03;
    auto lk = library_lock();
    cudaStream_t st;
    Stage S;
    S.base = host_staging(5 * N * sizeof(double), st, rc);
    if (!S.base) return rc;
    double *du_ = S.take(N), *dd = S.take(3 * N), *d2 = S.take(N);
    if ((rc = to_dev(du_, u, N, st))) return rc;
    if ((rc = nabla_u_and_square_impl(geocode, n01, n02, n03, du_, dd, d2, nord, hgrids, st)))
        return rc;
    if ((rc = to_host(du, dd, 3 * N, st)) || (rc = to_host(ddu, d2, N, st))) return rc;
    return host_finish(st);
}

int nabla_u_and_square_dev(int geocode, int n01, int n02, int n03, const double *u, double *du,
                           double *ddu, int nord, const double *hgrids, void *stream) {
    return nabla_u_and_square_impl(geocode, n01, n02, n03, u, du, ddu, nord, hgrids,
                                   (cudaStream_t)stream);
}

int nabla_u_square(int geocode, int n01, int n02, int n03, const double *u, double *ddu, int nord,
                   const double *hgrids) {
    int rc = check3(n01, n02, n03, hgrids);
    if (rc) return rc;
    if (!u || !ddu) return report(LIBCONV_EARG, "u/ddu must not be null");
    const size_t N = (size_t)n01 * n02 * n03;
    auto lk = library_lock();
    cudaStream_t st;
    Stage S;
    S.base = host_staging(5 * N * sizeof(double), st, rc);
    if (!S.base) return rc;
    double *du_ = S.take(N), *dd = S.take(3 * N), *d2 = S.take(N);
    if ((rc = to_dev(du_, u, N, st))) return rc;
    if ((rc = nabla_u_and_square_impl(geocode, n01, n02, n03, du_, dd, d2, nord, hgrids, st)))
        return rc;
    if ((rc = to_host(ddu, d2, N, st))) return rc;
    return host_finish(st);
}

int nabla_u_square_dev(int geocode, int n01, int n02, int n03, const double *u, double *ddu,
                       int nord, const double *hgrids, double *work, void *stream) {
    if (!work) return report(LIBCONV_EARG, "work (3 n01 n02 n03) must not be null");
    return nabla_u_and_square_impl(geocode, n01, n02, n03, u, work, ddu, nord, hgrids,
                                   (cudaStream_t)stream);
}

int nabla_u_epsilon(int geocode, int n01, int n02, int n03, const double *u, double *du, int nord,
                    const double *hgrids, const double *eps) {
    int rc = check3(n01, n02, n03, hgrids);
    if (rc) return rc;
    if (!u || !du || !eps) return report(LIBCONV_EARG, "u/du/eps must not be null");
    const size_t N = (size_t)n01 * n02 * n03;
    auto lk = library_lock();
    cudaStream_t st;
    Stage S;
    S.base = host_staging(5 * N * sizeof(double), st, rc);
    if (!S.base) return rc;
    double *du_ = S.take(N), *dd = S.take(3 * N), *de = S.take(N);
    if ((rc = to_dev(du_, u, N, st)) || (rc = to_dev(de, eps, N, st))) return rc;
    if ((rc = nabla_u_epsilon_impl(geocode, n01, n02, n03, du_, dd, nord, hgrids, de, st))) return rc;
    if ((rc = to_host(du, dd, 3 * N, st))) return rc;
    return host_finish(st);
}

int nabla_u_epsilon_dev(int geocode, int n01, int n02, int n03, const double *u, double *du,
                        int nord, const double *hgrids, const double *eps, void *stream) {
    return nabla_u_epsilon_impl(geocode, n01, n02, n03, u, du, nord, hgrids, eps,
                                (cudaStream_t)stream);
}

int update_rhopol(int geocode, int n01, int n02, int n03, const double *u, int nord,
                  const double *hgrids, double eta, const double *dlogeps, double *rhopol,
                  double *rhores2) {
    int rc = check3(n01, n02, n03, hgrids);
    if (rc) return rc;
    if (!u || !dlogeps || !rhopol || !rhores2)
        return report(LIBCONV_EARG, "u/dlogeps/rhopol/rhores2 must not be null");
    const size_t N = (size_t)n01 * n02 * n03;
    const size_t nw = 3 * N + (size_t)rhopol_parts((long long)N);
    auto lk = library_lock();
    cudaStream_t st;
    Stage S;
    S.base = host_staging((5 * N + 1 + nw) * sizeof(double), st, rc);
    if (!S.base) return rc;
    double *du_ = S.take(N), *dl = S.take(3 * N), *rp = S.take(N), *r2 = S.take(1), *w = S.take(nw);
    if ((rc = to_dev(du_, u, N, st)) || (rc = to_dev(dl, dlogeps, 3 * N, st)) ||
        (rc = to_dev(rp, rhopol, N, st)))
        return rc;
    if ((rc = update_rhopol_impl(geocode, n01, n02, n03, du_, nord, hgrids, eta, dl, rp, r2, w, st)))
        return rc;
    if ((rc = to_host(rhopol, rp, N, st)) || (rc = to_host(rhores2, r2, 1, st))) return rc;
    return host_finish(st);
}

int update_rhopol_dev(int geocode, int n01, int n02, int n03, const double *u, int nord,
                      const double *hgrids, double eta, const double *dlogeps, double *rhopol,
                      double *rhores2, double *work, void *stream) {
    return update_rhopol_impl(geocode, n01, n02, n03, u, nord, hgrids, eta, dlogeps, rhopol,
                              rhores2, work, (cudaStream_t)stream);
}

int update_rhopol_work_size(int n01, int n02, int n03, long long *nwork) {
    if (!nwork || n01 < 1 || n02 < 1 || n03 < 1) return report(LIBCONV_EARG, "bad arguments");
    const long long N = (long long)n01 * n02 * n03;
    *nwork = 3 * N + rhopol_parts(N);
    return LIBCONV_OK;
}

}  // extern "C"
