// Plans: the sequence of 1D sweeps one entry point runs, with the buffers
// (x, y, w1, w2) each sweep reads and writes.  Shared by the C-ABI entry
// points and the batched (many-grid) operators.
#pragma once
#include <mutex>
#include <vector>

#include "lcg_sweep.cuh"

namespace lcg {

enum BufId { B_X = 0, B_Y = 1, B_W1 = 2, B_W2 = 3 };

struct PlanStep {
    Sweep S;
    int src, dst, src2;   // buffer ids (src2 = -1 if no x2)
    int dot_slot = 0;     // entry of the dot output this step's dot product goes to
    int dot_stride = 0;   // > 0: one dot per array, array j at dot_slot + j * dot_stride
    int exp_axis = -1;    // >= 0: line exponents from the plan's shared pass over x (this axis)
};

struct Plan {
    std::vector<PlanStep> steps;
    size_t elems[4] = {0, 0, 0, 0};   // elements each buffer must hold
    size_t y_read = 0;                // y is read (a_y != 0)
    int has_dot = 0;
    int ndot = 1;                     // dot outputs (one per kinetic direction for ekin)
    int exp3[4] = {0, 0, 0, 0};       // n0, n1, n2, narr of the x grid whose line exponents
                                      // the exact tensor-core steps share (0: none)
    const int *active = nullptr;      // device flags per array: 0 = skip it (no dot plans)
};

// 3D MagicFilter (sfrf_ld_narr, one grid).  order == nullptr: the reference's
// rotating sweeps (transpose = 1); otherwise non-rotating sweeps along
// axes order[0], order[1], order[2] (same result, other intermediates).
int plan_magicfilter(int d, const int *n, const int *bc, const int *order, Plan &P);
// 3D kinetic (one grid), sweeps along order[] (nullptr: 0, 1, ..., d-1).
int plan_kinetic(int d, const int *n, const int *bc, const double *a, double a_x,
                 const int *order, Plan &P);
// Host copy of the flat filter table.
const double *filter_table();
// Calling thread's compute mode (LIBCONV_MODE_*).
int current_mode();
// Device status word of the current device (bounded tensor-core waits).
int *device_status(int &rc);
// Operators of the Fortran-facing layer.
enum OpId { OPID_MD, OPID_IMD, OPID_D1, OPID_D2, OPID_DWT, OPID_IWT, OPID_RTOS1, OPID_S1TOR };
// Multi-D product y = a F x + a_y y (a_x: d = 1 convolutions only), host pointers.
int md_generic(int op_id, int d, const int *n, const int *bc, const int *nx, const int *ny,
               int narr, double a, double a_x, double a_y, const double *x, double *y);
// Sum of 1D convolutions y = sum_i a[i] F_i x + a_x x + a_y y, dot[i] = x . (a[i] F_i x)
// when dot is not null; host pointers.
int sum1d_generic(int op_id, int d, const int *n, const int *bc, const int *nx, const int *ny,
                  int narr, const double *a, double a_x, double a_y, const double *x, double *y,
                  double *dot);
// Per-axis input/output extents of op_id's sweeps and the largest
// intermediate (elements) of the multi-D product; any output may be null.
int extents(int op_id, int d, const int *n, const int *bc, int *in, int *out, long long *inter);
// One Poisson finite-difference sweep on device pointers (bc 0 periodic or
// LIBCONV_BC_NPERIODIC), y = a d/dx_idim x, or y += ... when accumulate.
int poisson_sweep(int nord, int idim, const int *nn, int bc, double a, bool accumulate,
                  const double *x, double *y, cudaStream_t st);
// Host-pointer composition: hold library_lock(), stage in host_staging(),
// run on its stream, then host_finish() (synchronise + device status).
std::unique_lock<std::recursive_mutex> library_lock();
double *host_staging(size_t bytes, cudaStream_t &st, int &rc);
int host_finish(cudaStream_t st);
int report(int code, const char *msg);
int report_cuda(cudaError_t e, const char *what);
// d_kin_narr_dev over the arrays a with active[a] != 0 (device flags, read by
// the kernels on `st`): the other arrays' y is left as it is.
int kin_narr_active_dev(int d, const int *n, const int *bc, int narr, const double *x, double *y,
                        double *w1, double *w2, const double *a, const int *active, cudaStream_t st);

}  // namespace lcg
