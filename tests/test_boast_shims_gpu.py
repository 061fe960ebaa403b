"""The void shims of libconv_gb300_boast.so (the generated procedures'
prototypes, no status) give bit for bit the results of the int-status entry
points of libconv_gb300.so: 1D MagicFilter along an inner axis with a_x and
a_y, 3D kinetic and 3D wavelet analysis, host pointers."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

I, D, P = ctypes.c_int, ctypes.c_double, ctypes.c_void_p


def ptr(a):
    return a.ctypes.data_as(P)


def ivec(v):
    return (ctypes.c_int * len(v))(*v)


@pytest.fixture
def libs(pkg):
    S = ctypes.CDLL(os.path.join(os.path.dirname(pkg.LIB_PATH), 'libconv_gb300_boast.so'))
    return S, pkg.lib()


def both(libs, name, argtypes, make_args, out_index):
    """Call name through the shim and through the main library with the same
    inputs; return the two outputs (the argument at out_index)."""
    S, L = libs
    fs, fl = getattr(S, name), getattr(L, name)
    fs.argtypes, fs.restype = argtypes, None
    fl.argtypes, fl.restype = argtypes, ctypes.c_int
    a1, a2 = make_args(), make_args()
    fs(*[x if not isinstance(x, np.ndarray) else ptr(x) for x in a1])
    assert fl(*[x if not isinstance(x, np.ndarray) else ptr(x) for x in a2]) == 0
    return a1[out_index], a2[out_index]


def test_magicfilter_1d_inner_axis(libs):
    n = [20, 18, 22]
    rng = np.random.default_rng(3)
    x = rng.standard_normal(int(np.prod(n)))
    y0 = rng.standard_normal(int(np.prod(n)))
    args = [I, I, P, I, P, P, I, P, P, D, D, D]
    make = lambda: [3, 1, ivec(n), 0, ivec(n), ivec(n), 1, x.copy(), y0.copy(), 1.5, 0.25, -0.5]
    ys, yl = both(libs, 'd_s0s0_1d_sym8_md', args, make, 8)
    assert np.array_equal(ys, yl)


def test_kinetic_3d(libs):
    n = [24, 20, 28]
    rng = np.random.default_rng(4)
    x = rng.standard_normal(int(np.prod(n)))
    args = [I, P, P, P, P, P, P, P, D, D]
    make = lambda: [3, ivec(n), ivec([0, 0, 0]), x.copy(), np.zeros(x.size), np.zeros(1), np.zeros(1),
                    np.array([-1.2, -0.8, -2.0]), 0.3, 0.0]
    ys, yl = both(libs, 'd_kin', args, make, 4)
    assert np.array_equal(ys, yl) and np.abs(ys).max() > 0


def test_wavelet_analysis_3d(libs):
    n = [12, 10, 14]
    rng = np.random.default_rng(5)
    N = 8 * int(np.prod(n))
    x = rng.standard_normal(N)
    args = [I, P, P, P, P, P, P]
    make = lambda: [3, ivec(n), ivec([0, 0, 0]), x.copy(), np.zeros(N), np.zeros(1), np.zeros(1)]
    ys, yl = both(libs, 'd_dwt_sym8', args, make, 4)
    assert np.array_equal(ys, yl) and np.abs(ys).max() > 0
