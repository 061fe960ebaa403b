// FP64 SIMT sweep: the plain double-precision path.
//
// One CTA owns 32 lines x one chunk of QC outputs.  The input segment the
// chunk needs (QC + taps - 1 positions, periodic wrap / free-boundary zero
// fill / shrink offset applied at load time) is staged once in shared memory
// with coalesced loads, then every output is a chain of FP64 FMAs in the
// reference's tap order (lowfil..upfil).  Lanes map to lines, so the shared
// reads are conflict-free and the stores of strided shapes and of the
// rotated (transpose = 1) layout are coalesced.
#include "lcg_sweep.cuh"
#include "libconv_filters.h"

namespace lcg {

__constant__ double c_ftab[LCG_FTAB_N] = LCG_FTAB_INIT;

namespace {

constexpr int kLines = 32;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kPad = kLines + 1;

template <int KIND> struct Chunk { static constexpr int QC = KIND == KCONV ? 64 : 32; };

__device__ __forceinline__ int imod(int a, int n) {
    int r = a % n;
    return r < 0 ? r + n : r;
}

// Input element of line g at logical processed index p (channel ch), with the
// boundary condition applied; 0 outside the data of a free boundary.
template <int KIND>
__device__ __forceinline__ double fetch(const Sweep &S, const double *__restrict__ x, long long g,
                                        int p, int ch, long long in_pext) {
    int pos;
    if (S.bc == BC_PERIODIC) {
        pos = imod(p, S.n);
    } else if (S.bc == BC_SHRINK) {
        pos = p - S.in_lo;
    } else {
        if (p < 0 || p >= S.n) return 0.0;
        pos = p;
    }
    const long long l = g % S.nL, r = g / S.nL;
    const long long off = KIND == KDEC ? (long long)ch + 2LL * pos
                                       : (long long)pos + (long long)S.in_ext * ch;
    return x[l + (long long)S.nL * (off + in_pext * r)];
}

// One block of the sweep: lines [bx*32, bx*32+32) x output chunk by of array
// bz.  `tile` and `red` are the block's shared staging buffers.
template <int KIND, int NT, int QC>
__device__ __forceinline__ void sweep_block(const Sweep &S, long long bx, int by, int bz,
                                            double *tile, double *red, long long dot_index) {
    constexpr int NCH = KIND == KCONV ? 1 : 2;
    constexpr int SPAN = QC + NT - 1;
    constexpr int NROW = SPAN * NCH;

    const int arr = bz;
    const long long nlines = (long long)S.nL * S.nR;
    const long long g0 = bx * kLines;
    const int qc0 = S.qlo + by * QC;
    const int upfil = S.lowfil + NT - 1;
    const int plast = S.qhi + upfil;  // last logical input index any output needs
    const long long in_pext = (long long)S.in_ext * NCH;
    const long long out_pext = (long long)S.out_ext * NCH;
    const double *__restrict__ x = S.x + (long long)arr * S.x_arr;
    double *__restrict__ y = S.y + (long long)arr * S.y_arr;
    const double *__restrict__ x2 = S.x2 ? S.x2 + (long long)arr * S.x_arr : nullptr;

    // ---- stage the input segment: row j*NCH+ch holds logical index qc0+lowfil+j
    if (S.nL == 1) {
        // positions fastest: consecutive threads read consecutive memory of one line
        for (int idx = threadIdx.x; idx < NROW * kLines; idx += kThreads) {
            int w, j, ch;
            if (KIND == KREC) {          // blocked input: one channel block at a time
                j = idx % SPAN; const int t = idx / SPAN; ch = t % NCH; w = t / NCH;
            } else {                     // conv / interleaved input
                const int k = idx % NROW; w = idx / NROW; j = k / NCH; ch = k % NCH;
            }
            const long long g = g0 + w;
            const int p = qc0 + S.lowfil + j;
            double v = 0.0;
            if (g < nlines && p <= plast) v = fetch<KIND>(S, x, g, p, ch, in_pext);
            tile[(j * NCH + ch) * kPad + w] = v;
        }
    } else {
        // lines fastest: consecutive threads read consecutive l of one position
        for (int idx = threadIdx.x; idx < NROW * kLines; idx += kThreads) {
            const int w = idx % kLines, k = idx / kLines;
            const int j = k / NCH, ch = k % NCH;
            const long long g = g0 + w;
            const int p = qc0 + S.lowfil + j;
            double v = 0.0;
            if (g < nlines && p <= plast) v = fetch<KIND>(S, x, g, p, ch, in_pext);
            tile[k * kPad + w] = v;
        }
    }
    __syncthreads();

    const int w = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const long long g = g0 + w;
    const long long l = g % S.nL, r = g / S.nL;
    const double *f = c_ftab + S.ftab;
    double dot = 0.0;
    if (g < nlines) {
        for (int qr = wi; qr < QC; qr += kWarps) {
            const int q = qc0 + qr;
            if (q > S.qhi) break;
            double o0 = 0.0, o1 = 0.0;
#pragma unroll
            for (int k = 0; k < NT; ++k) {
                const int row = (qr + k) * NCH;
                if (KIND == KCONV) {
                    o0 = fma(tile[row * kPad + w], f[k], o0);
                } else if (KIND == KDEC) {          // f = LE | LO | HE | HO
                    const double x0 = tile[row * kPad + w], x1 = tile[(row + 1) * kPad + w];
                    o0 = fma(x0, f[k], o0);
                    o1 = fma(x0, f[2 * NT + k], o1);
                    o0 = fma(x1, f[NT + k], o0);
                    o1 = fma(x1, f[3 * NT + k], o1);
                } else {
                    const double s = tile[row * kPad + w], d = tile[(row + 1) * kPad + w];
                    o0 = fma(s, f[NT + k], o0);
                    o1 = fma(s, f[k], o1);
                    o0 = fma(d, f[3 * NT + k], o0);
                    o1 = fma(d, f[2 * NT + k], o1);
                }
            }
#pragma unroll
            for (int ch = 0; ch < NCH; ++ch) {
                double out = ch ? o1 : o0;
                if (S.has_a) out *= S.a;
                const int pos = q - S.out_lo;
                const long long off = KIND == KREC ? (long long)ch + 2LL * pos
                                                   : (long long)pos + (long long)S.out_ext * ch;
                const long long yi = S.transpose ? r + (long long)S.nR * off
                                                 : l + (long long)S.nL * (off + out_pext * r);
                if (KIND == KCONV) {
                    if ((S.has_dot || S.has_ax) && (S.bc != BC_GROW || (q >= 0 && q < S.n))) {
                        const double xq = tile[(qr - S.lowfil) * kPad + w];
                        if (S.has_dot) dot = fma(xq, out, dot);
                        if (S.has_ax) out = fma(xq, S.a_x, out);
                    }
                    if (x2) {
                        const long long x2i = S.bc == BC_GROW
                            ? yi : l + (long long)S.nL * ((long long)(q - S.in_lo) + in_pext * r);
                        out += x2[x2i];
                    }
                }
                if (S.ay_mode == 2) out += y[yi];
                else if (S.ay_mode == 1) out = fma(S.a_y, y[yi], out);
                y[yi] = out;
            }
        }
    }
    if (S.has_dot) {
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if (w == 0) red[wi] = dot;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int i = 0; i < kWarps; ++i) s += red[i];
            S.dot_part[dot_index] = s;
        }
    }
}

template <int KIND, int NT, int QC>
__global__ void __launch_bounds__(kThreads) sweep_fp64_kernel(const __grid_constant__ Sweep S) {
    constexpr int NROW = (QC + NT - 1) * (KIND == KCONV ? 1 : 2);
    __shared__ double tile[NROW * kPad];
    __shared__ double red[kWarps];
    if (S.active && !S.active[blockIdx.z]) return;          // array skipped (no dot here)
    const long long b = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    sweep_block<KIND, NT, QC>(S, blockIdx.x, blockIdx.y, blockIdx.z, tile, red, b);
}

// Blocks of one sweep (all narr arrays).
__host__ __device__ __forceinline__ long long blocks_of(const Sweep &S, int qc) {
    const long long nlines = (long long)S.nL * S.nR;
    const long long nq = S.qhi - S.qlo + 1;
    return ((nlines + kLines - 1) / kLines) * ((nq + qc - 1) / qc) * S.narr;
}

// Persistent form over a list of sweeps of the same kind and filter (one
// per grid of a batch of uneven grids): the blocks of all sweeps are numbered
// consecutively (prefix[i] = first block of sweep i) and each CTA walks them
// with a grid stride, locating a block's sweep by binary search.
template <int KIND, int NT, int QC>
__global__ void __launch_bounds__(kThreads)
sweep_fp64_batch_kernel(const Sweep *__restrict__ descs, const long long *__restrict__ prefix,
                        int nsweeps) {
    constexpr int NROW = (QC + NT - 1) * (KIND == KCONV ? 1 : 2);
    __shared__ double tile[NROW * kPad];
    __shared__ double red[kWarps];
    const long long total = prefix[nsweeps];
    for (long long b = blockIdx.x; b < total; b += gridDim.x) {
        int lo = 0, hi = nsweeps - 1;                    // last i with prefix[i] <= b
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (prefix[mid] <= b) lo = mid;
            else hi = mid - 1;
        }
        const Sweep &S = descs[lo];
        const long long lb = b - prefix[lo];
        const long long gx = ((long long)S.nL * S.nR + kLines - 1) / kLines;
        const int gy = (S.qhi - S.qlo + QC) / QC;
        sweep_block<KIND, NT, QC>(S, lb % gx, (int)((lb / gx) % gy), (int)(lb / (gx * gy)), tile,
                                  red, 0);
        __syncthreads();                                 // tile reused by the next block
    }
}

// Block b sums part[b*count .. (b+1)*count) in a fixed order into
// out[b*out_stride] (one block per segment: per-array dot products).
__global__ void dot_reduce_kernel(const double *__restrict__ part, long long count, double *out,
                                  long long out_stride, int accumulate) {
    __shared__ double red[256];
    part += (long long)blockIdx.x * count;
    out += (long long)blockIdx.x * out_stride;
    double s = 0.0;
    for (long long i = threadIdx.x; i < count; i += blockDim.x) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = accumulate ? *out + red[0] : red[0];
}

template <int KIND, int NT, int QC = Chunk<KIND>::QC>
cudaError_t launch_t(const Sweep &S, cudaStream_t st) {
    const long long nlines = (long long)S.nL * S.nR;
    const int nq = S.qhi - S.qlo + 1;
    dim3 grid((unsigned)((nlines + kLines - 1) / kLines), (unsigned)((nq + QC - 1) / QC),
              (unsigned)S.narr);
    sweep_fp64_kernel<KIND, NT, QC><<<grid, kThreads, 0, st>>>(S);
    return cudaGetLastError();
}

template <int KIND, int NT, int QC>
cudaError_t launch_batch_t(const Sweep *descs, const long long *prefix, int nsweeps, int grid,
                           cudaStream_t st) {
    sweep_fp64_batch_kernel<KIND, NT, QC><<<grid, kThreads, 0, st>>>(descs, prefix, nsweeps);
    return cudaGetLastError();
}

template <int KIND, int NT, int QC>
int batch_grid_t() {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, sweep_fp64_batch_kernel<KIND, NT, QC>,
                                                  kThreads, 0);
    return (sms > 0 ? sms : 148) * (per > 0 ? per : 1);
}

template <int QC>
int batch_grid_qc(int kind, int ntaps) {
    if (kind == KCONV && ntaps == 16) return batch_grid_t<KCONV, 16, QC>();
    if (kind == KCONV && ntaps == 29) return batch_grid_t<KCONV, 29, QC>();
    if (kind == KDEC && ntaps == 8) return batch_grid_t<KDEC, 8, QC / 2>();
    if (kind == KDEC && ntaps == 16) return batch_grid_t<KDEC, 16, QC / 2>();
    if (kind == KREC && ntaps == 8) return batch_grid_t<KREC, 8, QC / 2>();
    if (kind == KREC && ntaps == 16) return batch_grid_t<KREC, 16, QC / 2>();
    return 0;
}

template <int QC>
cudaError_t launch_batch_qc(int kind, int ntaps, const Sweep *descs, const long long *prefix,
                            int nsweeps, int grid, cudaStream_t st) {
    if (kind == KCONV && ntaps == 16) return launch_batch_t<KCONV, 16, QC>(descs, prefix, nsweeps, grid, st);
    if (kind == KCONV && ntaps == 29) return launch_batch_t<KCONV, 29, QC>(descs, prefix, nsweeps, grid, st);
    if (kind == KDEC && ntaps == 8) return launch_batch_t<KDEC, 8, QC / 2>(descs, prefix, nsweeps, grid, st);
    if (kind == KDEC && ntaps == 16) return launch_batch_t<KDEC, 16, QC / 2>(descs, prefix, nsweeps, grid, st);
    if (kind == KREC && ntaps == 8) return launch_batch_t<KREC, 8, QC / 2>(descs, prefix, nsweeps, grid, st);
    if (kind == KREC && ntaps == 16) return launch_batch_t<KREC, 16, QC / 2>(descs, prefix, nsweeps, grid, st);
    return cudaErrorInvalidValue;
}

}  // namespace

long long sweep_fp64_blocks(const Sweep &S) {
    const long long nlines = (long long)S.nL * S.nR;
    const int qc = S.kind == KCONV ? Chunk<KCONV>::QC : Chunk<KDEC>::QC;
    const long long nq = S.qhi - S.qlo + 1;
    return ((nlines + kLines - 1) / kLines) * ((nq + qc - 1) / qc) * S.narr;
}

cudaError_t launch_sweep_fp64(const Sweep &S, cudaStream_t st) {
    if (S.kind == KCONV && S.ntaps == 16) return launch_t<KCONV, 16>(S, st);
    if (S.kind == KCONV && S.ntaps == 17) return launch_t<KCONV, 17>(S, st);
    if (S.kind == KCONV && S.ntaps == 29) return launch_t<KCONV, 29>(S, st);
    if (S.kind == KDEC && S.ntaps == 8) return launch_t<KDEC, 8>(S, st);
    if (S.kind == KDEC && S.ntaps == 16) return launch_t<KDEC, 16>(S, st);
    if (S.kind == KREC && S.ntaps == 8) return launch_t<KREC, 8>(S, st);
    if (S.kind == KREC && S.ntaps == 16) return launch_t<KREC, 16>(S, st);
    return cudaErrorInvalidValue;
}

long long sweep_fp64_batch_blocks(const Sweep &S, int qc) {
    return blocks_of(S, S.kind == KCONV ? qc : qc / 2);
}

int sweep_fp64_batch_grid(int kind, int ntaps, int qc) {
    return qc == 64 ? batch_grid_qc<64>(kind, ntaps) : batch_grid_qc<32>(kind, ntaps);
}

cudaError_t launch_sweep_fp64_batch(int kind, int ntaps, int qc, const Sweep *descs,
                                    const long long *prefix, int nsweeps, int grid,
                                    cudaStream_t st) {
    if (qc == 64) return launch_batch_qc<64>(kind, ntaps, descs, prefix, nsweeps, grid, st);
    if (qc == 32) return launch_batch_qc<32>(kind, ntaps, descs, prefix, nsweeps, grid, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_dot_reduce(const double *part, long long count, double *out, int accumulate,
                              cudaStream_t st) {
    dot_reduce_kernel<<<1, 256, 0, st>>>(part, count, out, 0, accumulate);
    return cudaGetLastError();
}

cudaError_t launch_dot_reduce_seg(const double *part, long long seg_len, int nseg, double *out,
                                  long long out_stride, cudaStream_t st) {
    if (nseg < 1 || nseg > 65535) return cudaErrorInvalidValue;
    dot_reduce_kernel<<<nseg, 256, 0, st>>>(part, seg_len, out, out_stride, 0);
    return cudaGetLastError();
}

}  // namespace lcg
