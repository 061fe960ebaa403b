"""The allocation-free kinetic sweep (d_s0s0_1d_sym8_d2_dotin_noalloc).

Some callers cannot allocate device memory: an application whose device
memory is entirely managed by its own allocator or budget, or an inner loop
that cannot afford the device synchronisation a cudaMalloc/cudaFree may
cause.  This entry point takes only caller-owned device buffers and keeps its
scratch (the per-block partial sums of dot_in) in a fixed device array inside
the library.  The test calls it through the C-ABI twice in a row, with
different inputs, for every boundary condition, and checks both results
against the regular device entry point and the oracle at the tolerance of the
other parity tests; it also checks that a call leaves the device's free
memory unchanged, and that a sweep needing more partial sums than the array
holds is refused before any launch.
This file is collected last so that a failure here leaves the rest of the
suite already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _bind(pkg):
    L = pkg.lib()
    fn = L.d_s0s0_1d_sym8_d2_dotin_noalloc
    I = ctypes.POINTER(ctypes.c_int)
    fn.argtypes = [ctypes.c_int, ctypes.c_int, I, ctypes.c_int, I, I, ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                   ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _ints(v):
    return (ctypes.c_int * len(v))(*v)


def _ext(bc, n):
    """(nx, ny) along the swept axis: 28 extra inputs for shrink, 28 extra outputs for grow."""
    return (n + 28 if bc == -1 else n), (n + 28 if bc == 1 else n)


@pytest.mark.parametrize('bc', [0, -1, 1, 2])
def test_noalloc_matches_regular_entry_point_twice(pkg, O, bc):
    """Two calls in a row (other axis, scalars and inputs each time) against the
    regular device entry point and the oracle, for every boundary condition:
    shrink and grow change how many partial sums the sweep writes and which
    outputs take part in dot_in."""
    import torch
    from boast_lig_gb300 import inputs
    fn = _bind(pkg)
    dev = torch.device('cuda:0')
    n = [20, 24, 18]
    narr = 2
    for call, (idim, a, a_x, a_y, seed) in enumerate([(1, -2.47, 0.5, 0.0, 41), (2, -1.3, 0.0, 1.0, 42)]):
        nx, ny = list(n), list(n)
        nx[idim], ny[idim] = _ext(bc, n[idim])
        Nx, Ny = int(np.prod(nx)) * narr, int(np.prod(ny)) * narr
        xh = inputs.uniform(seed, Nx)
        yh = inputs.uniform(seed + 100, Ny)
        x = torch.from_numpy(xh).to(dev)
        y0 = torch.from_numpy(yh).to(dev)
        y_na, y_ref = y0.clone(), y0.clone()
        d_na = torch.zeros(1, dtype=torch.float64, device=dev)
        d_ref = torch.zeros(1, dtype=torch.float64, device=dev)
        st = fn(3, idim, _ints(n), bc, _ints(nx), _ints(ny), narr, x.data_ptr(), y_na.data_ptr(),
                a, a_x, a_y, d_na.data_ptr(), None)
        assert st == 0, pkg.last_error()
        with pkg.mode(pkg.MODE_FP64):
            pkg.Kernel('d_s0s0_1d_sym8_d2_dotin').run_dev(3, idim, n, bc, nx, ny, narr, x, y_ref,
                                                          a, a_x, a_y, d_ref)
        torch.cuda.synchronize()
        assert rel(y_na.cpu().numpy(), y_ref.cpu().numpy()) <= TOL, call
        assert abs(d_na.item() - d_ref.item()) <= TOL * abs(d_ref.item()), call
        yo, do = yh.copy(), ctypes.c_double(0.0)
        assert O.call('oracle_d_s0s0_1d_sym8_d2_dotin', 3, idim, n, bc, nx, ny, narr, xh, yo, a,
                      a_x, a_y, ctypes.pointer(do)) == 0
        assert rel(y_na.cpu().numpy(), yo) <= TOL, call
        assert abs(d_na.item() - do.value) <= 1e-12 * abs(do.value), call


def test_noalloc_call_allocates_no_device_memory(pkg):
    """After the first call on the device (which looks up the fixed array's
    address), a call leaves the device's free memory unchanged."""
    import torch
    fn = _bind(pkg)
    n = [32, 40, 24]
    N = int(np.prod(n))
    x = torch.rand(N, dtype=torch.float64, device='cuda:0')
    y = torch.zeros(N, dtype=torch.float64, device='cuda:0')
    d = torch.zeros(1, dtype=torch.float64, device='cuda:0')
    args = (3, 0, _ints(n), 0, _ints(n), _ints(n), 1, x.data_ptr(), y.data_ptr(), -2.0, 0.0, 0.0,
            d.data_ptr(), None)
    assert fn(*args) == 0, pkg.last_error()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert fn(*args) == 0, pkg.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_more_partials_than_the_array_holds(pkg):
    """A sweep needing more partial sums than the fixed array holds is refused
    before any pointer is used (so the buffers here are one element each)."""
    import torch
    fn = _bind(pkg)
    n = [32, 32, 32]                  # idim 1: 1024 lines -> 32 blocks per array
    narr = 2049                       # 32 * 2049 > 65536 partial sums
    x = torch.zeros(1, dtype=torch.float64, device='cuda:0')
    y = torch.zeros(1, dtype=torch.float64, device='cuda:0')
    d = torch.zeros(1, dtype=torch.float64, device='cuda:0')
    st = fn(3, 1, _ints(n), 0, _ints(n), _ints(n), narr, x.data_ptr(), y.data_ptr(),
            1.0, 0.0, 0.0, d.data_ptr(), None)
    assert st == -3
    assert 'noalloc' in pkg.last_error()
