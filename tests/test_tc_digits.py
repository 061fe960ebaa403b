"""CPU emulation of the tensor-core digit arithmetic (no GPU).

The exact tcgen05 sweep scales each line of FP64 data and the filter (a
folded in) to signed 62-bit integers (data truncated toward zero, filter
rounded), cuts each into 8 balanced byte digits in [-128, 127] held exactly
in FP16 (the bytes of X + 0x8080808080808080 minus 128), accumulates the
36 digit pairs of order k = s + t <= 7 in one FP32 accumulator per order
that starts at 1.5 * 2^23 (exact while every partial sum stays within
2^22: every value is then an integer in [2^23, 2^24], whose FP32 bits are
0x4B400000 plus the sum), and recombines
Y = sum_{k<=5} Acc_k 2^(46-8k) + round(Acc_6 / 4 + Acc_7 / 1024) in int64.
This test replays that arithmetic with exact integers on the kinetic and
MagicFilter filters, checks the 2^22 bound the exactness rests on and the
64-bit range of Y, and compares with an exact rational evaluation: the
error must be at FP64 level.
"""
from fractions import Fraction

import numpy as np
import pytest

S = 8                     # digits per operand


def filter_fixed(taps, a):
    """Signed 62-bit filter integers F = round(a f 2^(62 - ef)) and ef, as the
    host's tc_filter_digits (ef raised while sum |a f| >= 8 * 2^ef)."""
    af = [Fraction(a) * Fraction(float(t)) for t in taps]
    m = max(abs(v) for v in af)
    ef = int(np.frexp(float(m))[1])
    while Fraction(2) ** ef <= m:
        ef += 1
    while sum(abs(v) for v in af) >= 8 * Fraction(2) ** ef:
        ef += 1
    F = []
    for v in af:
        x = abs(v) * Fraction(2) ** (62 - ef)
        r = int(x + Fraction(1, 2))              # round half up on the magnitude
        F.append(-r if v < 0 else r)
    return np.array(F, dtype=object), ef


def data_fixed(row):
    """X = trunc(x 2^(62 - E)) per element, E from the row's largest
    exponent field (|x| < 2^E), as fixed_bal."""
    mx = max(((int(np.float64(v).view(np.int64)) >> 52) & 0x7FF) for v in row)
    E = max(mx, 1) - 1022
    X = []
    for v in row:
        q = Fraction(float(v)) * Fraction(2) ** (62 - E)
        X.append(int(q))                         # toward zero
    return np.array(X, dtype=object), E


def balanced_digits(X):
    """d_0 (top) .. d_7 with X = sum d_s 256^(7 - s), d in [-128, 127]."""
    out = []
    for v in X:
        assert -(2 ** 62) <= v <= 2 ** 62
        U = (int(v) + 0x8080808080808080) % 2 ** 64
        out.append([((U >> (8 * (7 - s))) & 0xFF) - 128 for s in range(S)])
    d = np.array(out, dtype=np.int64).T          # (S, len)
    for X_, col in zip(X, d.T):
        assert sum(int(c) * 256 ** (7 - s) for s, c in enumerate(col)) == X_
    return d


def emulate_periodic_sweep(x, n, ndat, taps, lowfil, a):
    """One periodic sweep along the contiguous axis, computed as the kernel does."""
    nt = len(taps)
    F, ef = filter_fixed(taps, a)
    e = balanced_digits(F)                                     # (S, nt)
    order_max = 7
    Xr = x.reshape(ndat, n)
    y = np.zeros((ndat, n))
    for r in range(ndat):
        X, E = data_fixed(Xr[r])
        d = balanced_digits(X)                                 # (S, n)
        acc = np.zeros((order_max + 1, n), dtype=np.int64)
        bound = np.zeros((order_max + 1, n), dtype=np.int64)
        for s in range(S):
            for t in range(S):
                k = s + t
                if k > order_max:
                    continue
                for j in range(nt):
                    xs = np.roll(d[s], -(j + lowfil))
                    acc[k] += e[t][j] * xs
                    bound[k] += abs(int(e[t][j])) * np.abs(xs)
        assert bound.max() <= 2 ** 22
        for q in range(n):
            Y = sum(int(acc[k, q]) * 2 ** (46 - 8 * k) for k in range(6))
            Y += (int(acc[6, q]) * 256 + int(acc[7, q]) + 512) >> 10
            assert abs(Y) < 2 ** 62
            # x f = X F 2^(E + ef - 124) and X F ~ Y 2^66
            y[r, q] = float(Fraction(Y) * Fraction(2) ** (E + ef - 58))
    return y.ravel()


def exact_periodic(x, n, ndat, taps, lowfil, a):
    X = x.reshape(ndat, n)
    out = np.zeros((ndat, n))
    fa = Fraction(a)
    for r in range(ndat):
        for q in range(n):
            acc = Fraction(0)
            for j, f in enumerate(taps):
                acc += Fraction(float(f)) * Fraction(float(X[r, (q + j + lowfil) % n]))
            out[r, q] = float(acc * fa)
    return out.ravel()


@pytest.mark.parametrize('which', ['md', 'd2'])
def test_digit_arithmetic_matches_oracle(O, pkg, which):
    import ctypes
    from boast_lig_gb300 import gen_filters as G, inputs
    n, ndat = 24, 6
    if which == 'md':
        taps = [float(v) for v in G.SYM8_MF[::-1]]
        lowfil, a = -8, 1.0
    else:
        taps = [float(v) for v in G.SYM8_D2]
        lowfil, a = -14, -0.5 / 0.45 ** 2
    x = inputs.gaussian_filtered_noise(3, (n, ndat, 1)).ravel(order='F')
    x[5] *= 1e-9                                   # a small element: truncation far below it
    y = emulate_periodic_sweep(x, n, ndat, taps, lowfil, a)
    ref = np.zeros_like(x)
    if which == 'md':
        assert O.call('oracle_d_s0s0_1d_sym8_md', 1, 0, [n], 0, [n], [n], ndat, x, ref, 1.0, 0.0, 0.0) == 0
    else:
        dd = ctypes.c_double(0)
        assert O.call('oracle_d_s0s0_1d_sym8_d2_dotin', 1, 0, [n], 0, [n], [n], ndat, x, ref,
                      a, 0.0, 0.0, ctypes.pointer(dd)) == 0
    ex = exact_periodic(x, n, ndat, taps, lowfil, a)
    err = np.abs(y - ex).max() / np.abs(ex).max()
    err64 = np.abs(ref - ex).max() / np.abs(ex).max()
    assert err <= max(2 * err64, 2e-16), (err, err64)     # FP64 level
    assert np.abs(y - ref).max() / np.abs(ref).max() < 1e-14


def test_accumulator_bound_is_tight_for_32_products():
    """The largest filter (32 products per output: the MagicFilter-combined
    wavelets) with every digit at -128 reaches exactly 2^22 in order 7,
    where the biased accumulator still holds: 1.5 * 2^23 + v is exact for
    |v| <= 2^22 and its bits are 0x4B400000 + v.  The start value comes from
    one MMA of a constant tile with 2048 (exact in FP16) at three K
    positions, as both operands: 3 * 2048^2 = 1.5 * 2^23."""
    v = 8 * 32 * 128 * 128
    assert v == 2 ** 22
    assert float(np.float16(2048.0)) == 2048.0
    assert int(np.array(2048.0, dtype=np.float16).view(np.uint16)) == 0x6800
    start = np.float32(0)
    for _ in range(3):
        start = np.float32(start + np.float32(2048.0) * np.float32(2048.0))
    assert float(start) == 1.5 * 2 ** 23
    for t in (-v, -v + 1, -1, 0, 1, v - 1, v):
        f = start + np.float32(t)
        assert float(f) == 1.5 * 2 ** 23 + t
        assert int(f.view(np.uint32)) == 0x4B400000 + t
