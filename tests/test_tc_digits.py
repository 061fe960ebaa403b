"""CPU emulation of the tensor-core digit arithmetic (no GPU).

The tcgen05 sweep scales FP64 data (per tile) and the filter to 62-bit
integers, splits each into 7 balanced base-512 digits held exactly in FP16,
accumulates the 21 digit pairs with s + t <= 5 plus order 6 (all 7 pairs for
the 29-tap filters, the leading (0,6) and (6,0) for the MagicFilter) per order k (exact in FP32 as long as every partial
sum is below 2^24), and recombines Y = sum_k Acc_k 512^(5-k).  This test
replays that arithmetic with exact integers on the kinetic and MagicFilter
filters, checks the 2^24 bound the exactness rests on, and compares with an
exact rational evaluation: the error must be at FP64 level.
"""
import numpy as np
import pytest

S = 7                     # digits per operand


def pairs(ntaps):
    """Digit pairs accumulated: every pair of order k = s + t <= 5, plus order 6
    in full for the 29-tap (cancelling) filters or its two leading pairs for
    the 16-tap MagicFilter."""
    base = [(s, k - s) for k in range(6) for s in range(k + 1)]
    return base + ([(s, 6 - s) for s in range(7)] if ntaps > 16 else [(0, 6), (6, 0)])


def to_fixed(v, E):
    """round(v * 2^(62 - E)) as exact int64 (|v| < 2^E)."""
    from fractions import Fraction
    return np.array([int(round(Fraction(float(t)) * 2 ** (62 - E))) for t in v], dtype=np.int64)


def balanced_digits(X):
    d = np.zeros((S,) + X.shape, dtype=np.int64)
    X = X.copy()
    for s in range(S - 1, 0, -1):
        u = X + 256
        d[s] = (u & 511) - 256
        X = u >> 9
    d[0] = X
    return d


def emulate_periodic_sweep(x, n, ndat, taps, lowfil, a):
    """One periodic sweep along the contiguous axis, computed as the kernel does."""
    f = np.asarray(taps)              # the operator scalar a multiplies the result
    ef = int(np.frexp(np.abs(f).max())[1])
    F = to_fixed(f, ef)
    e = balanced_digits(F)
    assert np.abs(e).max() <= 256
    X = x.reshape(ndat, n)
    E = int(np.frexp(np.abs(X).max())[1])
    Xi = np.array([to_fixed(row, E) for row in X])
    d = balanced_digits(Xi)                                    # (S, ndat, n)
    assert np.abs(d).max() <= 256
    nt = len(taps)
    acc = np.zeros((7, ndat, n), dtype=np.int64)
    bound = np.zeros((7, ndat, n), dtype=np.int64)
    for s, t in pairs(nt):
        for j in range(nt):
            xs = np.roll(d[s], -(j + lowfil), axis=1)
            acc[s + t] += e[t][j] * xs
            # every partial sum of products is bounded by the sum of |products|
            bound[s + t] += np.abs(e[t][j]) * np.abs(xs)
    assert bound.max() < 2 ** 24
    Y = sum(acc[k].astype(object) * (512 ** (5 - k)) for k in range(6))
    Y = Y + ((acc[6].astype(object) + 256) >> 9)
    # x*f = X F 2^(E+ef-124) and X F = 512^7 Y = 2^63 Y  ->  y = Y 2^(E+ef-61)
    y = np.array([[float(v) for v in row] for row in Y]) * (a * 2.0 ** (E + ef - 61))
    return y.ravel()


def exact_periodic(x, n, ndat, taps, lowfil, a):
    from fractions import Fraction
    X = x.reshape(ndat, n)
    out = np.zeros((ndat, n))
    fa = Fraction(a)
    for r in range(ndat):
        for q in range(n):
            acc = Fraction(0)
            for j, f in enumerate(taps):
                acc += Fraction(f) * Fraction(X[r, (q + j + lowfil) % n])
            out[r, q] = float(acc * fa)
    return out.ravel()


@pytest.mark.parametrize('which', ['md', 'd2'])
def test_digit_arithmetic_matches_oracle(O, pkg, which):
    from boast_lig_gb300 import gen_filters as G, inputs
    n, ndat = 24, 10
    if which == 'md':
        taps = [float(v) for v in G.SYM8_MF[::-1]]
        lowfil, a = -8, 1.0
        name = 'oracle_d_s0s0_1d_sym8_md'
    else:
        taps = [float(v) for v in G.SYM8_D2]
        lowfil, a = -14, -0.5 / 0.45 ** 2
        name = 'oracle_d_s0s0_1d_sym8_d1'  # placeholder, replaced below
    x = inputs.gaussian_filtered_noise(3, (n, ndat, 1)).ravel(order='F')
    y = emulate_periodic_sweep(x, n, ndat, taps, lowfil, a)
    ref = np.zeros_like(x)
    if which == 'md':
        assert O.call(name, 1, 0, [n], 0, [n], [n], ndat, x, ref, 1.0, 0.0, 0.0) == 0
    else:
        import ctypes
        dd = ctypes.c_double(0)
        assert O.call('oracle_d_s0s0_1d_sym8_d2_dotin', 1, 0, [n], 0, [n], [n], ndat, x, ref,
                      a, 0.0, 0.0, ctypes.pointer(dd)) == 0
    ex = exact_periodic(x, n, ndat, taps, lowfil, a)
    err = np.abs(y - ex).max() / np.abs(ex).max()
    err64 = np.abs(ref - ex).max() / np.abs(ex).max()
    assert err <= max(err64, 1e-15), (err, err64)       # at least as accurate as FP64
    assert np.abs(y - ref).max() / np.abs(ref).max() < 1e-14
