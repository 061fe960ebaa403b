"""Pin the CPU oracle (CPU only, no GPU).

1. Bit-for-bit against the reference's own C (benchmark/convolutions-c/
   MagicFilter.c) through the committed golden vectors, and live when
   oracle/_ref was built.
2. Against independent numpy restatements of the Fortran reference kernels.
3. The generated-operator restatement against the Fortran references, as the
   reference's tests do (MagicFilter_test2.rb, Kinetic_test2.rb,
   Kinetic1d-nb, Wavelet_test2.rb, TestOperations.ipynb), with their
   tolerances.
"""
import ctypes
import hashlib
import os

import numpy as np
import pytest

import numpy_ref as NR

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'magicfilter_ref_c.npz')
CASES = [
    ('mf_per_n32_ndat1024', 32, 1024, 1, False),
    ('mf_per_t_n32_ndat1024', 32, 1024, 1, True),
    ('mf_per_n8_ndat3', 8, 3, 5, False),
    ('mf_per_n16_ndat7', 16, 7, 6, True),
    ('mf_per_n64_ndat33', 64, 33, 7, False),
    ('mf_per_n128_ndat5', 128, 5, 8, True),
]


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize('name,n,ndat,seed,t', CASES)
def test_oracle_magicfilter_matches_reference_c_golden(O, pkg, name, n, ndat, seed, t):
    from boast_lig_gb300 import inputs
    g = np.load(GOLD)
    x = inputs.uniform(seed, n * ndat)
    assert hashlib.sha256(x.tobytes()).digest() == g[name + '__xsha'].tobytes()
    y = np.zeros(n * ndat)
    O.call('oracle_magicfilter_per_t_ref' if t else 'oracle_magicfilter_per_ref', n, ndat, x, y)
    assert np.array_equal(y, g[name])


def test_oracle_magicfilter_matches_reference_c_live(O, pkg):
    if O.ref_lib() is None:
        pytest.skip('oracle/_ref not built (reference tree absent)')
    from boast_lig_gb300 import inputs
    for n, ndat in [(8, 11), (24, 40), (100, 3), (256, 9)]:
        x = inputs.uniform(n + ndat, n * ndat)
        for t, fn in ((False, 'oracle_magicfilter_per_ref'), (True, 'oracle_magicfilter_per_t_ref')):
            y = np.zeros(n * ndat)
            O.call(fn, n, ndat, x, y)
            assert np.array_equal(y, O.ref_magicfilter(n, ndat, x, t))


def test_oracle_fortran_refs_vs_numpy(O, pkg):
    from boast_lig_gb300 import inputs
    n, ndat = 20, 13
    x = inputs.uniform(3, n * ndat)
    for inv, fn in ((False, 'oracle_magicfilter_per_ref'), (True, 'oracle_magicfilter_per_t_ref')):
        y = np.zeros(n * ndat)
        O.call(fn, n, ndat, x, y)
        assert rel(y, NR.mf_per(x, n, ndat, inv)) < 1e-15
    y = np.zeros((n + 15) * ndat)
    O.call('oracle_magicfilter_free_ref', n, ndat, x, y)
    assert rel(y, NR.mf_free(x, n, ndat)) < 1e-15
    shape = (9, 11, 14)
    xk = inputs.uniform(4, int(np.prod(shape)))
    yk = np.zeros_like(xk)
    h = np.array([0.5, 0.6, 0.7])
    O.call('oracle_kinetic_per_ref', *shape, h, xk, yk, 0.5)
    assert rel(yk, NR.kinetic_per(xk, shape, h, 0.5)) < 1e-14
    m = 10
    xs = inputs.uniform(5, 2 * m * ndat)
    ys = np.zeros_like(xs)
    O.call('oracle_synthesis_per_ref', m, ndat, xs, ys)
    assert rel(ys, NR.synthesis_per(xs, m, ndat)) < 1e-15
    ya = np.zeros_like(xs)
    O.call('oracle_analysis_per_ref', m, ndat, xs, ya)
    assert rel(ya, NR.analysis_per(xs, m, ndat)) < 1e-15


def test_filter_tables(pkg):
    from boast_lig_gb300 import gen_filters as G
    lp = np.array([float(v) for v in G.SYM8_LP])
    mf = np.array([float(v) for v in G.SYM8_MF])
    assert abs(lp.sum() - np.sqrt(2.0)) < 1e-15          # sum rule of the low-pass
    assert abs(mf.sum() - 1.0) < 1e-15                     # MagicFilter preserves constants
    assert abs(np.dot(lp, lp) - 1.0) < 1e-15               # orthonormality
    assert [float(v) for v in G.MF_FORTRAN] == [float(v) for v in G.SYM8_MF[::-1]]
    assert [float(v) for v in G.KIN_FORTRAN] == [float(v) for v in G.SYM8_D2[14:]]
    assert [float(v) for v in G.CH_FORTRAN] == [float(v) for v in G.SYM8_LP]
    assert [float(v) for v in G.CG_FORTRAN] == [float(v) for v in G.qmf_high(G.SYM8_LP)]
    d2 = np.array([float(v) for v in G.SYM8_D2])
    assert abs(d2.sum()) < 1e-14                            # second derivative kills constants
    t = np.arange(-14, 15)
    assert abs(np.dot(d2, t * t) - 2.0) < 1e-12             # and is exact on x^2


def test_combined_filters_match_decimal_derivation(pkg):
    """The s1tor/rtos1 filters equal MF (*) LP computed exactly then truncated
    to 30 decimals (GenericConvolution2.rb:336-384)."""
    from decimal import Decimal, ROUND_DOWN
    from boast_lig_gb300 import gen_filters as G
    c, lo, hi = G.combine(G.SYM8_LP, G.SYM8_MF, 8)
    assert c == 16 and len(lo) == 32 and len(hi) == 32
    lp = [Decimal(v) for v in G.SYM8_LP]
    mf = [Decimal(v) for v in G.SYM8_MF]
    # full linear convolution of lp and mf, indices aligned as in the reference
    full = [sum(lp[j] * mf[k - j] for j in range(16) if 0 <= k - j < 16) for k in range(31)]
    vals = [Decimal(v) for v in lo]
    # lp_cv(i) = sum_j lp[j+8] mf[i-j-1+8] -> full[i + 15] for i in -16..15
    for i in range(-16, 16):
        k = i + 15
        exp = full[k] if 0 <= k < 31 else Decimal(0)
        assert vals[i + 16] == exp.quantize(Decimal('1e-30'), rounding=ROUND_DOWN)


def dot_call(O, name, *args):
    d = ctypes.c_double(0.0)
    rc = O.call(name, *args, ctypes.pointer(d))
    return rc, d.value


def test_generated_mf_three_sweeps_equal_fortran_ref(O, pkg):
    """MagicFilter1d2.rb:49-80: three 1D sweeps == three magicfilter_per_ref."""
    from boast_lig_gb300 import inputs
    n = [14, 17, 19]
    N = int(np.prod(n))
    x = inputs.uniform(11, N)
    r, w = np.zeros(N), np.zeros(N)
    O.call('oracle_magicfilter_per_ref', n[0], n[1] * n[2], x, r)
    O.call('oracle_magicfilter_per_ref', n[1], n[0] * n[2], r, w)
    O.call('oracle_magicfilter_per_ref', n[2], n[0] * n[1], w, r)
    a, b, c = np.zeros(N), np.zeros(N), np.zeros(N)
    for idim, (src, dst) in enumerate(((x, a), (a, b), (b, c))):
        assert O.call('oracle_d_s0s0_1d_sym8_md', 3, idim, n, 0, n, n, 1, src, dst, 1.0, 0.0, 0.0) == 0
    assert np.array_equal(c, r)
    y3, w1, w2 = np.zeros(N), np.zeros(N), np.zeros(N)
    assert O.call('oracle_d_sfrf_ld_narr', 3, n, [0, 0, 0], n, n, 1, x, y3, w1, w2) == 0
    assert np.array_equal(y3, r)


def test_generated_mf_grow_shrink_equal_fortran_ref(O, pkg):
    """MagicFilter_test2.rb:89-182: 3D grow vs magicfilter_free_ref x3, shrink
    (inverse filter) vs magicfilter_free_t_ref x3, with narr=2 and ld."""
    from boast_lig_gb300 import inputs
    n = [9, 12, 10]
    g = [v + 15 for v in n]
    N, G = int(np.prod(n)), int(np.prod(g))
    x = inputs.uniform(12, N)
    r1, r2, r3 = np.zeros(g[0] * n[1] * n[2]), np.zeros(g[0] * g[1] * n[2]), np.zeros(G)
    O.call('oracle_magicfilter_free_ref', n[0], n[1] * n[2], x, r1)
    O.call('oracle_magicfilter_free_ref', n[1], g[0] * n[2], r1, r2)
    O.call('oracle_magicfilter_free_ref', n[2], g[0] * g[1], r2, r3)
    xx = np.concatenate([x, x])
    y, w1, w2 = np.zeros(2 * G), np.zeros(2 * G), np.zeros(2 * G)
    assert O.call('oracle_d_sfrf_ld_narr', 3, n, [1, 1, 1], n, g, 2, xx, y, w1, w2) == 0
    assert np.array_equal(y[:G], r3) and np.array_equal(y[G:], r3)
    xs = inputs.uniform(13, G)
    s1, s2, s3 = np.zeros(n[0] * g[1] * g[2]), np.zeros(n[0] * n[1] * g[2]), np.zeros(N)
    O.call('oracle_magicfilter_free_t_ref', n[0], g[1] * g[2], xs, s1)
    O.call('oracle_magicfilter_free_t_ref', n[1], n[0] * g[2], s1, s2)
    O.call('oracle_magicfilter_free_t_ref', n[2], n[0] * n[1], s2, s3)
    ys = np.zeros(N)
    assert O.call('oracle_d_rfsf_ld_narr', 3, n, [-1, -1, -1], g, n, 1, xs, ys, w1, w2) == 0
    assert np.array_equal(ys, s3)


def test_generated_kinetic_equals_fortran_ref(O, pkg):
    """Kinetic_test2.rb:91-104 (3D) and Kinetic1d-nb cells 15-21 (1D x3 with
    a_y = 1 accumulation and dot_in), tolerance 1e-12 / 1e-13."""
    from boast_lig_gb300 import inputs
    n = [13, 16, 11]
    N = int(np.prod(n))
    x = inputs.uniform(14, N)
    h = [0.5, 0.6, 0.7]
    sc = [-0.5 / t ** 2 for t in h]
    r = np.zeros(N)
    O.call('oracle_kinetic_per_ref', *n, np.array(h), x, r, 0.5)
    y, w1, w2 = np.zeros(N), np.zeros(N), np.zeros(N)
    assert O.call('oracle_d_kin', 3, n, [0, 0, 0], x, y, w1, w2, np.array(sc), 0.5, 0.0) == 0
    assert np.abs(y - r).max() < 1e-12
    y1 = np.zeros(N)
    rc, e0 = dot_call(O, 'oracle_d_s0s0_1d_sym8_d2_dotin', 3, 0, n, 0, n, n, 1, x, y1, sc[0], 0.5, 0.0)
    rc, e1 = dot_call(O, 'oracle_d_s0s0_1d_sym8_d2_dotin', 3, 1, n, 0, n, n, 1, x, y1, sc[1], 0.0, 1.0)
    rc, e2 = dot_call(O, 'oracle_d_s0s0_1d_sym8_d2_dotin', 3, 2, n, 0, n, n, 1, x, y1, sc[2], 0.0, 1.0)
    assert np.abs(y1 - r).max() < 1e-13
    assert abs((e0 + e1 + e2) - x @ (r - 0.5 * x)) < 1e-12 * abs(x @ (r - 0.5 * x))


def _shift(gen, n2, ndat):
    """Generated wavelet real-space index k holds the Fortran reference's k+1
    (LibconvBase.rb:92-96 shift_realspace)."""
    return np.roll(gen.reshape(ndat, n2), 1, axis=1).ravel()


def test_generated_wavelets_equal_fortran_refs_up_to_shift(O, pkg):
    from boast_lig_gb300 import inputs
    m, ndat = 9, 7
    s = inputs.uniform(15, 2 * m * ndat)
    ref = np.zeros_like(s)
    O.call('oracle_synthesis_per_ref', m, ndat, s, ref)           # y(ndat, 2m)
    gen = np.zeros_like(s)
    # one sweep, d=1, narr = ndat arrays of 2m values: y is 2m interleaved per array
    assert O.call('oracle_d_s1s0_1d_sym8', 1, 0, [m], 0, [m], [m], ndat, s, gen, 1.0, 0.0) == 0
    refT = ref.reshape(2 * m, ndat).T.ravel()                         # (ndat, 2m)
    assert rel(_shift(gen, 2 * m, ndat), refT) < 1e-14
    # analysis: dwt_gen(x) == dwt_ref(shift(x))
    xr = inputs.uniform(16, 2 * m * ndat)
    genA = np.zeros_like(xr)
    assert O.call('oracle_d_s0s1_1d_sym8', 1, 0, [m], 0, [m], [m], ndat, xr, genA, 1.0, 0.0) == 0
    xs = _shift(xr, 2 * m, ndat)
    refA = np.zeros_like(xr)
    O.call('oracle_analysis_per_ref', m, ndat, xs, refA)
    assert rel(genA, refA.reshape(2 * m, ndat).T.ravel()) < 1e-14


def test_wavelet_free_grow_equals_synthesis_free_ref(O, pkg):
    """Free-BC synthesis (grow, 2m -> 2m+14) vs synthesis_free_ref up to the
    same one-sample shift: generated index k <-> reference k+1."""
    from boast_lig_gb300 import inputs
    m, ndat = 11, 3
    s = inputs.uniform(17, 2 * m * ndat)
    ref = np.zeros((2 * m + 14) * ndat)
    O.call('oracle_synthesis_free_ref', m, ndat, s, ref)             # y(ndat, -7:2m+6)
    gen = np.zeros((2 * m + 14) * ndat)
    assert O.call('oracle_d_s1s0_1d_sym8', 1, 0, [m], 1, [m], [m + 7], ndat, s, gen, 1.0, 0.0) == 0
    # generated grow covers real-space -8..2m+5, reference -7..2m+6
    assert rel(gen.reshape(ndat, 2 * m + 14), ref.reshape(2 * m + 14, ndat).T) < 1e-14


def test_wavelet_identities(O, pkg):
    """Wavelet_test2.rb:126-254 and Wavelet1d-nb cells 6-8."""
    from boast_lig_gb300 import inputs
    n = [6, 7, 5]
    N = 8 * int(np.prod(n))
    x = inputs.uniform(18, N)
    t, u, w1, w2 = np.zeros(N), np.zeros(N), np.zeros(N), np.zeros(N)
    assert O.call('oracle_d_dwt_sym8', 3, n, [0, 0, 0], x, t, w1, w2) == 0
    assert O.call('oracle_d_idwt_sym8', 3, n, [0, 0, 0], t, u, w1, w2) == 0
    assert np.abs(u - x).max() < 1e-11
    # grow then shrink
    G = int(np.prod([2 * v + 14 for v in n]))
    g, w1, w2 = np.zeros(G), np.zeros(G), np.zeros(G)
    assert O.call('oracle_d_dwt_sym8', 3, n, [1, 1, 1], x, g, w1, w2) == 0
    back = np.zeros(N)
    assert O.call('oracle_d_idwt_sym8', 3, n, [-1, -1, -1], g, back, w1, w2) == 0
    assert np.abs(back - x).max() < 1e-11
    # 1D with scaling a and 1/a (Wavelet1d-nb cells 6-8)
    sc = [-0.5 / 0.25, -0.5 / 0.36, -0.5 / 0.49]
    a, b, c = np.zeros(N), np.zeros(N), np.zeros(N)
    for idim, (src, dst) in enumerate(((x, a), (a, b), (b, c))):
        assert O.call('oracle_d_s0s1_1d_sym8', 3, idim, n, 0, n, n, 1, src, dst, sc[idim], 0.0) == 0
    for idim, (src, dst) in enumerate(((c, a), (a, b), (b, c))):
        assert O.call('oracle_d_s1s0_1d_sym8', 3, idim, n, 0, n, n, 1, src, dst, 1 / sc[idim], 0.0) == 0
    assert np.abs(c - x).max() < 1e-11


def test_combined_operators(O, pkg):
    """TestOperations.ipynb cells 8-11: s1tor == mf o iwt, rtos1 == dwt o imf (periodic)."""
    from boast_lig_gb300 import inputs
    n = [6, 5, 7]
    nm = [2 * v for v in n]
    N = 8 * int(np.prod(n))
    x = inputs.uniform(19, N)
    w, d1, d2 = np.zeros(N), np.zeros(N), np.zeros(N)
    assert O.call('oracle_d_s1s0_1d_sym8', 3, 0, n, 0, n, n, 1, x, w, 1.0, 0.0) == 0
    assert O.call('oracle_d_s0s0_1d_sym8_md', 3, 0, nm, 0, nm, nm, 1, w, d1, 1.0, 0.0, 0.0) == 0
    assert O.call('oracle_d_s1s0_1d_symicomb8', 3, 0, n, 0, n, n, 1, x, d2, 1.0, 0.0) == 0
    assert np.abs(d1 - d2).max() < 1e-11
    assert O.call('oracle_d_s0s0_1d_sym8_imd', 3, 0, nm, 0, nm, nm, 1, x, w, 1.0, 0.0, 0.0) == 0
    assert O.call('oracle_d_s0s1_1d_sym8', 3, 0, n, 0, n, n, 1, w, d1, 1.0, 0.0) == 0
    assert O.call('oracle_d_s0s1_1d_symicomb8', 3, 0, n, 0, n, n, 1, x, d2, 1.0, 0.0) == 0
    assert np.abs(d1 - d2).max() < 1e-11


def test_analytic_known_answers(O, pkg):
    """MF of a constant is the constant; D2 of a constant is 0; D2 of a
    periodic cosine is its Fourier symbol times the cosine."""
    from boast_lig_gb300 import gen_filters as G
    n, ndat = 40, 3
    c = np.full(n * ndat, 0.75)
    y = np.zeros_like(c)
    assert O.call('oracle_d_s0s0_1d_sym8_md', 1, 0, [n], 0, [n], [n], ndat, c, y, 1.0, 0.0, 0.0) == 0
    assert np.abs(y - 0.75).max() < 1e-15
    assert O.call('oracle_d_s0s0_1d_sym8_d1', 1, 0, [n], 0, [n], [n], ndat, c, y, 1.0, 0.0, 0.0) == 0
    assert np.abs(y).max() < 1e-14
    k = 3
    i = np.arange(n)
    cs = np.tile(np.cos(2 * np.pi * k * i / n), ndat)
    rc, _ = dot_call(O, 'oracle_d_s0s0_1d_sym8_d2_dotin', 1, 0, [n], 0, [n], [n], ndat, cs, y, 1.0, 0.0, 0.0)
    d2 = np.array([float(v) for v in G.SYM8_D2])
    sym = sum(d2[j + 14] * np.cos(2 * np.pi * k * j / n) for j in range(-14, 15))
    assert np.abs(y - sym * cs).max() < 1e-13


def test_oracle_rejects_bad_arguments(O, pkg):
    x, y = np.zeros(64), np.zeros(64)
    assert O.call('oracle_d_s0s0_1d_sym8_md', 1, 0, [8], 7, [8], [8], 1, x, y, 1.0, 0.0, 0.0) == -2
    assert O.call('oracle_d_s0s0_1d_sym8_md', 1, 0, [8], 1, [8], [8], 1, x, y, 1.0, 0.0, 0.0) == -3
    assert O.call('oracle_d_s0s0_1d_sym8_md', 1, 2, [8], 0, [8], [8], 1, x, y, 1.0, 0.0, 0.0) == -1


def test_kinetic_ekin_restatement(O):
    """kinetic_per_ref_optim_ekin (Kinetic2.rb:21-112): y += T x, and
    kstrten(d) is the energy x . (T_d x) of direction d -- the same numbers as
    kinetic_per_ref for y and as the generated 1D kinetic sweep with dot_in
    for each direction."""
    n = [12, 10, 9]
    N = int(np.prod(n))
    h = np.array([0.45, 0.4, 0.5])
    rng = np.random.default_rng(0)
    x, y = rng.standard_normal(N), rng.standard_normal(N)
    y0 = y.copy()
    k = np.zeros(3)
    O.call('oracle_kinetic_per_ref_ekin', *n, h, x, y, k)
    r = np.zeros(N)
    O.call('oracle_kinetic_per_ref', *n, h, x, r, 0.0)
    assert np.abs(y - (y0 + r)).max() <= 1e-13 * np.abs(r).max()
    for d in range(3):
        yd, dd = np.zeros(N), ctypes.c_double(0.0)
        O.call('oracle_d_s0s0_1d_sym8_d2_dotin', 3, d, n, 0, n, n, 1, x, yd, -0.5 / h[d] ** 2,
               0.0, 0.0, ctypes.pointer(dd))
        assert abs(k[d] - dd.value) <= 1e-13 * abs(k[d])
    # the energies add up to x . (T x)
    assert abs(k.sum() - float(x @ r)) <= 1e-12 * abs(k.sum())


def _rot3(f, x, dims):
    """Apply a transposed 1D reference kernel f(x, n, ndat) along the three
    axes in turn (each call rotates the axes, so three give the original
    orientation); dims[i]: the input extent of axis i, f_out(i): its output."""
    d = list(dims)
    for _ in range(3):
        n = d[0]
        x = f(x, n, int(np.prod(d[1:])))
        d = d[1:] + [x.size // int(np.prod(d[1:]))]
    return x


def test_hamiltonian_restatement_periodic_numpy(O, pkg):
    """Local Hamiltonian (BigDFT/libconv.f90:248-294) with periodic axes: the
    oracle composition against an independent numpy one built from the
    Fortran reference kernels (synthesis, magic filter, its transpose,
    kinetic, analysis)."""
    n = [5, 6, 4]
    m = [2 * v for v in n]
    N = int(np.prod(m))
    h = np.array([0.45, 0.4, 0.5])
    a = -0.5 / h ** 2
    rng = np.random.default_rng(3)
    psig, pot = rng.standard_normal(N), rng.uniform(0.5, 1.5, N)
    rho0 = rng.uniform(0.0, 1.0, N)
    rho, hpsig, ek, ep = rho0.copy(), np.zeros(N), np.zeros(3), np.zeros(1)
    assert O.call('oracle_hamiltonian', n, [0, 0, 0], a, psig, pot, rho, hpsig, ek, ep) == 0
    def roll(x, s):
        # the generated wavelets' real-space index k is the Fortran
        # kernels' k+1 along every axis (LibconvBase.rb:92-96)
        return np.roll(x.reshape(m, order='F'), s, axis=(0, 1, 2)).ravel(order='F')

    fscf = roll(_rot3(lambda x, k, nd: NR.synthesis_per(x, k // 2, nd), psig, m), -1)
    psir = _rot3(lambda x, k, nd: NR.mf_per(x, k, nd), fscf, m)
    hpsi = _rot3(lambda x, k, nd: NR.mf_per(x, k, nd, inverse=True), pot * psir, m)
    kin = NR.kinetic_per(fscf, m, h, 0.0)
    want = _rot3(lambda x, k, nd: NR.analysis_per(x, k // 2, nd), roll(hpsi + kin, 1), m)
    assert rel(hpsig, want) < 1e-13
    assert rel(rho, rho0 + psir ** 2) < 1e-14
    assert abs(ep[0] - float(psir @ (pot * psir))) < 1e-13 * abs(ep[0])
    assert abs(ek.sum() - float(fscf @ kin)) < 1e-12 * abs(ek.sum())


@pytest.mark.parametrize('bc', [[2, 2, 2], [2, 0, 2], [0, 0, 0]])
def test_hamiltonian_restatement_symmetric(O, bc):
    """The composed operator is self-adjoint (dwt shrink is the transpose of
    idwt grow, the inverse magic filter shrink that of the grow one):
    <psig|H psig> = sum ekin + epot, <phi|H psi> = <H phi|psi>, and H is
    linear in psig."""
    n = [5, 4, 6]
    N = 8 * int(np.prod(n))
    nr = int(np.prod([(2 * v + 29) if b == 2 else 2 * v for v, b in zip(n, bc)]))
    rng = np.random.default_rng(4)
    a = np.array([-1.3, -2.1, -0.7])
    pot = rng.uniform(-1.0, 2.0, nr)
    phi, psi = rng.standard_normal(N), rng.standard_normal(N)

    def H(x):
        y, ek, ep = np.zeros(N), np.zeros(3), np.zeros(1)
        assert O.call('oracle_hamiltonian', n, bc, a, x, pot, None, y, ek, ep) == 0
        return y, ek.sum() + ep[0]

    hpsi, e = H(psi)
    hphi, _ = H(phi)
    assert abs(float(psi @ hpsi) - e) < 1e-13 * np.abs(psi).sum() * np.abs(hpsi).max()
    assert abs(float(phi @ hpsi) - float(hphi @ psi)) < 1e-12 * np.abs(phi).sum() * np.abs(hpsi).max()
    comb, _ = H(2.5 * psi - phi)
    assert np.abs(comb - (2.5 * hpsi - hphi)).max() < 1e-12 * np.abs(comb).max()


# ---- Poisson finite differences (BigDFT/Poisson.rb) ----------------------------------
POISSON_GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden',
                            'poisson_fd_c1d.npz')


def _fd_table(pkg, nord):
    import re
    h = open(os.path.join(os.path.dirname(pkg.LIB_PATH), 'csrc', 'libconv_filters.h')).read()
    edge = [float(v) for v in re.search(r'LCG_FD_EDGE_INIT \{(.*?)\}', h, re.S).group(1)
            .replace('\\', '').split(',')]
    off = int(re.search(rf'LCG_FD_EDGE_OFF_{nord} (\d+)', h).group(1))
    n = nord + 1
    return np.array(edge[off:off + n * n]).reshape(n, n)


@pytest.mark.parametrize('nord', [2, 4, 6, 8, 16])
def test_poisson_table_equals_reference_bits(pkg, nord):
    """The FD table computed by Fornberg's algorithm (plus the reference's
    one sign deviation at nord = 8) equals, bit for bit, the reference's
    table (fixture extracted from Poisson.rb:20-166 by
    tests/golden/make_poisson_golden.py)."""
    gold = np.load(POISSON_GOLD)[f'fd{nord}']
    assert np.array_equal(_fd_table(pkg, nord), gold)


def _numpy_fd_periodic(x, shape, axis, nord, a, pkg):
    t = _fd_table(pkg, nord)
    m = nord // 2
    X = x.reshape(shape, order='F')
    Y = sum(t[m, j + m] * np.roll(X, -j, axis=axis) for j in range(-m, m + 1))
    return (a * Y).ravel(order='F')


@pytest.mark.parametrize('nord', [2, 8, 16])
@pytest.mark.parametrize('idim', [0, 1, 2])
def test_poisson_broker_periodic_numpy(O, pkg, nord, idim):
    n = [19, 21, 18]
    x = np.random.default_rng(idim).uniform(0, 1, int(np.prod(n)))
    y = np.zeros_like(x)
    assert O.call('oracle_poisson_broker', nord, idim, n, 0, x, y, 2.5) == 0
    assert rel(y, _numpy_fd_periodic(x, n, idim, nord, 2.5, pkg)) < 1e-14


@pytest.mark.parametrize('nord', [2, 4, 6, 16])
def test_poisson_broker_nonperiodic_exact_on_polynomials(O, nord):
    """Every stencil of order nord differentiates polynomials of degree <=
    nord exactly, the one-sided ones at the boundaries included (nord = 8
    is left out: the reference's table has a sign slip in its first
    one-sided stencil, kept for parity)."""
    n = [nord + 9, 5, 4]
    s = np.arange(n[0], dtype=float) / n[0]
    rng = np.random.default_rng(nord)
    coef = rng.uniform(-1, 1, nord + 1)
    p = np.polynomial.polynomial.polyval(s, coef)
    dp = np.polynomial.polynomial.polyval(s, np.polynomial.polynomial.polyder(coef)) / n[0]
    x = np.tile(p, n[1] * n[2])
    y = np.zeros_like(x)
    assert O.call('oracle_poisson_broker', nord, 0, n, -2, x, y, 1.0) == 0
    assert np.abs(y.reshape(-1, n[0]) - dp).max() < 1e-10 * np.abs(dp).max()


def test_poisson_nord8_reference_slip_visible(O):
    """The kept sign deviation: at the first point of a non-periodic line the
    nord = 8 stencil is off by 35 u(4) (35/2 - (-35/2)) from the exact one."""
    n = [20, 1, 1]
    x = np.zeros(20)
    x[4] = 1.0
    y = np.zeros(20)
    assert O.call('oracle_poisson_broker', 8, 0, n, -2, x, y, 1.0) == 0
    assert y[0] == 35.0 / 2.0


@pytest.mark.parametrize('geocode', [1, 2, 3])
def test_poisson_div_u_i_generated_matches_fortran_ref(O, geocode):
    """Poisson_test.rb:86-93: the generated div_u_i against div_u_i_ref (the
    reference test's epsilon is 1e-10; the two differ only by x/h against
    x*(1/h))."""
    n01, n02, n03 = 20, 18, 22
    N = n01 * n02 * n03
    u = np.random.default_rng(geocode).uniform(0, 1, 3 * N)
    h = np.array([0.1, 0.12, 0.09])
    dg, dr = np.zeros(N), np.zeros(N)
    assert O.call('oracle_div_u_i', geocode, n01, n02, n03, u, dg, 16, h, None) == 0
    assert O.call('oracle_div_u_i_ref', geocode, n01, n02, n03, u, dr, 16, h) == 0
    assert rel(dg, dr) < 1e-13
    assert np.abs(dg - dr).max() < 1e-10
