"""Tensor-core (tcgen05) exact-digit sweeps against the oracle and an exact
rational evaluation.  The digit scheme is exact in FP32 accumulation, so the
result must be at FP64 level: tolerance 1e-13 relative to max|y| (the FP64
bar), and within 2x of the FP64 kernel's own error against exact
arithmetic."""
import ctypes
from fractions import Fraction

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture
def tc(pkg):
    with pkg.mode(pkg.MODE_TC_EXACT):
        yield pkg


def test_tc_one_periodic_magicfilter_sweep(tc, O):
    from boast_lig_gb300 import inputs
    n, ndat = 32, 1024
    x = inputs.uniform(1, n * ndat)
    y = np.zeros_like(x)
    tc.Kernel('d_s0s0_1d_sym8_md').run(1, 0, [n], 0, [n], [n], ndat, x, y, 1.0, 0.0, 0.0)
    yo = np.zeros_like(x)
    O.call('oracle_d_s0s0_1d_sym8_md', 1, 0, [n], 0, [n], [n], ndat, x, yo, 1.0, 0.0, 0.0)
    assert rel(y, yo) <= 1e-13


def _exact(x, n, ndat, taps, lowfil, a):
    X = x.reshape(ndat, n)
    out = np.zeros((ndat, n))
    for r in range(ndat):
        for q in range(n):
            s = sum(Fraction(f) * Fraction(X[r, (q + j + lowfil) % n]) for j, f in enumerate(taps))
            out[r, q] = float(s * Fraction(a))
    return out.ravel()


@pytest.mark.parametrize('op,taps_name,lowfil,a', [
    ('d_s0s0_1d_sym8_md', 'MD', -8, 1.0),
    ('d_s0s0_1d_sym8_d2_dotin', 'D2', -14, -0.5 / 0.45 ** 2),
])
def test_tc_accuracy_vs_exact(tc, O, op, taps_name, lowfil, a):
    from boast_lig_gb300 import gen_filters as G, inputs
    taps = [float(v) for v in (G.SYM8_MF[::-1] if taps_name == 'MD' else G.SYM8_D2)]
    n, ndat = 40, 12
    x = inputs.gaussian_filtered_noise(5, (n, ndat, 1)).ravel(order='F')
    ex = _exact(x, n, ndat, taps, lowfil, a)
    y = np.zeros_like(x)
    args = [1, 0, [n], 0, [n], [n], ndat, x, y, a, 0.0, 0.0]
    if op.endswith('dotin'):
        args.append(None)
    tc.Kernel(op).run(*args)
    with tc.mode(tc.MODE_FP64):
        y64 = np.zeros_like(x)
        args[8] = y64
        tc.Kernel(op).run(*args)
    e_tc, e_64 = rel(y, ex), rel(y64, ex)
    assert e_tc <= 1e-13
    assert e_tc <= max(2 * e_64, 1e-15), (e_tc, e_64)


def test_tc_lines_do_not_share_a_scale(tc, O):
    """A line of huge values or a NaN in the same 128-line tile must not change
    the other lines' results (each line segment has its own power-of-two scale)."""
    from boast_lig_gb300 import inputs
    n, ndat = 48, 100
    x = inputs.uniform(9, n * ndat)
    x[3 * n:4 * n] *= 1e200          # line 3: huge
    x[7 * n + 5] = np.nan             # line 7: one NaN
    x[11 * n:12 * n] *= 1e-200        # line 11: tiny
    y = np.zeros_like(x)
    tc.Kernel('d_s0s0_1d_sym8_md').run(1, 0, [n], 0, [n], [n], ndat, x, y, 1.0, 0.0, 0.0)
    yo = np.zeros_like(x)
    O.call('oracle_d_s0s0_1d_sym8_md', 1, 0, [n], 0, [n], [n], ndat, x, yo, 1.0, 0.0, 0.0)
    Y, R = y.reshape(ndat, n), yo.reshape(ndat, n)
    assert np.all(np.isnan(Y[7]))
    for r in range(ndat):
        if r == 7:
            continue
        assert rel(Y[r], R[r]) <= 1e-13, r
