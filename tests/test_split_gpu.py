"""Split-precision tensor-core sweeps (BF16x3: three bfloat16 terms, six
products; TF32x3: two tf32 terms, three products; FP32 accumulation) against
the FP64 oracle.  These modes cannot meet the FP64 bar; their error,
max|y - y_oracle| / max|y_oracle|, is printed per operator and bounded by
TOL_SPLIT[scheme]: 1e-5 for BF16x3 (an exact split of the FP32 value: FP32
input rounding and accumulation, about 2^-24 per product) and 4e-5 for TF32x3
(about 2^-22 per product from the split and the dropped lo.lo term).  The
bounds carry the conditioning of the operators: up to three sweeps, and the
kinetic's cancellation on smooth data (sum |a f| |x| >> |y|)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_SPLIT = {'tc_bf16x3': 1e-5, 'tc_tf32x3': 4e-5}
ERRORS = {}


@pytest.fixture(params=['tc_bf16x3', 'tc_tf32x3'])
def split(request, pkg):
    m = pkg.MODE_TC_BF16X3 if request.param == 'tc_bf16x3' else pkg.MODE_TC_TF32X3
    with pkg.mode(m):
        yield request.param


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def seeded(seed, size):
    from boast_lig_gb300 import inputs
    return inputs.uniform(seed, size)


def check(key, err):
    ERRORS[key] = err
    print(f'{key}: max rel error {err:.3e}')
    assert err <= TOL_SPLIT[key[0]], (key, err)
    assert np.isfinite(err)


TAPS = {'d_s0s0_1d_sym8_md': 16, 'd_s0s0_1d_sym8_imd': 16, 'd_s0s0_1d_sym8_d1': 29,
        'd_s0s1_1d_sym8': 8, 'd_s1s0_1d_sym8': 8, 'd_s0s1_1d_symicomb8': 16,
        'd_s1s0_1d_symicomb8': 16}


@pytest.mark.parametrize('op', list(TAPS))
@pytest.mark.parametrize('bc', [0, 1, -1, 2])
@pytest.mark.parametrize('idim', [0, 2])
def test_split_1d(pkg, O, split, op, bc, idim):
    wav = not op.startswith('d_s0s0')
    n = [9, 13, 40] if idim == 2 else [40, 13, 9]
    t = TAPS[op]
    nx, ny = list(n), list(n)
    nx[idim] = n[idim] + t - 1 if bc == -1 else n[idim]
    ny[idim] = n[idim] + t - 1 if bc == 1 else n[idim]
    mul = 8 if wav else 1
    narr = 2
    sx, sy = mul * int(np.prod(nx)) * narr, mul * int(np.prod(ny)) * narr
    x = seeded(700 + idim, sx)
    y0 = seeded(800 + idim, sy)
    scal = (-1.25, 0.5) if wav else (0.7, -0.3, 1.5)
    yg, yo = y0.copy(), y0.copy()
    pkg.Kernel(op).run(3, idim, n, bc, nx, ny, narr, x, yg, *scal)
    assert O.call('oracle_' + op, 3, idim, n, bc, nx, ny, narr, x, yo, *scal) == 0
    check((split, op, bc, idim), rel(yg, yo))


@pytest.mark.parametrize('bc', [0, 1, -1, 2])
def test_split_kinetic_dotin(pkg, O, split, bc):
    op = 'd_s0s0_1d_sym8_d2_dotin'
    n = [33, 8, 17]
    nx, ny = list(n), list(n)
    nx[1] = n[1] + 28 if bc == -1 else n[1]
    ny[1] = n[1] + 28 if bc == 1 else n[1]
    sx, sy = int(np.prod(nx)) * 3, int(np.prod(ny)) * 3
    x = seeded(900, sx)
    yg, yo = np.zeros(sy), np.zeros(sy)
    st = pkg.Kernel(op).run(3, 1, n, bc, nx, ny, 3, x, yg, -2.47, 0.0, 0.0, None)
    d = ctypes.c_double(0.0)
    assert O.call('oracle_' + op, 3, 1, n, bc, nx, ny, 3, x, yo, -2.47, 0.0, 0.0,
                  ctypes.pointer(d)) == 0
    check((split, op, bc), rel(yg, yo))
    dg = st['reference_return']['dot_in']
    assert abs(dg - d.value) <= TOL_SPLIT[split] * np.abs(x).max() * np.abs(yo).max() * x.size


def test_split_3d_operators_128(pkg, O, split):
    """MagicFilter 3D and kinetic 3D on a 128^3 periodic grid of
    Gaussian-filtered noise (h = 0.45): the errors of the split schemes."""
    from boast_lig_gb300 import inputs
    n = [128, 128, 128]
    x = inputs.gaussian_filtered_noise(21, tuple(n)).ravel(order='F')
    N = x.size
    y, w = np.zeros(N), np.zeros(N)
    pkg.Kernel('d_sfrf_ld_narr').run(3, n, [0, 0, 0], n, n, 1, x, y, w, w)
    yo = np.zeros(N)
    O.call('oracle_d_sfrf_ld_narr', 3, n, [0, 0, 0], n, n, 1, x, yo, np.zeros(N), np.zeros(N))
    check((split, 'mf3d'), rel(y, yo))
    a = [-0.5 / 0.45 ** 2] * 3
    pkg.Kernel('d_kin').run(3, n, [0, 0, 0], x, y, w, w, a, 0.0, 0.0)
    O.call('oracle_d_kin', 3, n, [0, 0, 0], x, yo, np.zeros(N), np.zeros(N), np.array(a), 0.0, 0.0)
    check((split, 'kin3d'), rel(y, yo))


def test_split_wavelet_round_trip_96(pkg, O, split):
    """8 subbands of 48^3 -> 96^3 -> back, each direction against the oracle."""
    from boast_lig_gb300 import inputs
    n = [48, 48, 48]
    N = 96 ** 3
    c = inputs.uniform(23, N).reshape(96, 96, 96)
    c[48:, :, :] *= 1e-3
    c[:, 48:, :] *= 1e-3
    c[:, :, 48:] *= 1e-3
    s = np.ascontiguousarray(c).ravel()
    r, back, w = np.zeros(N), np.zeros(N), np.zeros(N)
    pkg.Kernel('d_idwt_sym8').run(3, n, [0, 0, 0], s, r, w, w)
    ro = np.zeros(N)
    O.call('oracle_d_idwt_sym8', 3, n, [0, 0, 0], s, ro, np.zeros(N), np.zeros(N))
    check((split, 'idwt96'), rel(r, ro))
    pkg.Kernel('d_dwt_sym8').run(3, n, [0, 0, 0], r, back, w, w)
    bo = np.zeros(N)
    O.call('oracle_d_dwt_sym8', 3, n, [0, 0, 0], ro, bo, np.zeros(N), np.zeros(N))
    check((split, 'dwt96'), rel(back, bo))
    check((split, 'round_trip96'), rel(back, s))
