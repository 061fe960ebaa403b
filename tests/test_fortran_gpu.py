"""GPU parity of the Fortran-facing libconv procedures (include/libconv_fortran.h,
the interfaces of BigDFT/libconv.f90), called the way gfortran calls them
(every argument by reference, 1-based idim), against the oracle on the same
seeded inputs.  Tolerance max|y - y_oracle| / max|y_oracle| <= 1e-13; dot
products relative 1e-12.  The last test replays the reference's pipeline
sketch (libconv.f90:258-290) call by call through these procedures and
checks it against libconv_hamiltonian."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


@pytest.fixture(autouse=True, params=['fp64', 'tc_exact'])
def compute_mode(request, pkg):
    m = pkg.MODE_FP64 if request.param == 'fp64' else pkg.MODE_TC_EXACT
    with pkg.mode(m):
        yield request.param


@pytest.fixture(scope='module')
def F(pkg):
    return pkg.Fortran()


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def rnd(seed, size):
    return np.random.default_rng(seed).uniform(-1.0, 1.0, size)


@pytest.mark.parametrize('fname,oname', [('SYM8_MD', 'md'), ('SYM8_MI', 'imd'), ('SYM8_D1', 'd1')])
@pytest.mark.parametrize('bc', [0, 1, 2])
def test_s0s0_1d(F, O, fname, oname, bc):
    n = [12, 9, 10]
    idim = 1                                     # 0-based axis 1: Fortran idim 2
    nx, ny = list(n), list(n)
    if bc == 1:
        ny[idim] += 28 if fname == 'SYM8_D1' else 15     # taps - 1
    x = rnd(1, int(np.prod(nx)))
    y0 = rnd(2, int(np.prod(ny)))
    yg, yo = y0.copy(), y0.copy()
    F.call('s0s0_1d', F.filter_id(fname), 8, 3, idim + 1, n, bc, nx, ny, 1, 1.7, 0.3, -0.6, x, yg)
    assert O.call(f'oracle_d_s0s0_1d_sym8_{oname}', 3, idim, n, bc, nx, ny, 1, x, yo, 1.7, 0.3,
                  -0.6) == 0
    assert rel(yg, yo) <= TOL


@pytest.mark.parametrize('comb', [False, True])
@pytest.mark.parametrize('bc', [0, 1, -1])
def test_wavelet_1d(F, O, comb, bc):
    """s0s1_1d / s1s0_1d (and the combined filter) along the last axis."""
    n = [5, 6, 7]
    fid = F.filter_id('SYMICOMB8' if comb else 'SYM8_LP')
    ntaps = 16 if comb else 8
    for fwd in (True, False):
        nx, ny = list(n), list(n)
        if bc == 1:
            ny[2] += ntaps - 1
        if bc == -1:
            nx[2] += ntaps - 1
        x = rnd(3, 8 * int(np.prod(nx)))
        y0 = rnd(4, 8 * int(np.prod(ny)))
        yg, yo = y0.copy(), y0.copy()
        F.call('s0s1_1d' if fwd else 's1s0_1d', fid, 8, 3, 3, n, bc, nx, ny, 1, 0.8, 0.25, x, yg)
        oname = ('oracle_d_s0s1_1d_' if fwd else 'oracle_d_s1s0_1d_') + ('symicomb8' if comb else 'sym8')
        assert O.call(oname, 3, 2, n, bc, nx, ny, 1, x, yo, 0.8, 0.25) == 0
        assert rel(yg, yo) <= TOL


@pytest.mark.parametrize('bc', [[0, 0, 0], [1, 1, 1], [1, 0, 1]])
def test_s0s0_md_magicfilter(F, O, bc):
    """s0s0_md with ld and narr = 2 against the 3D MagicFilter, then with a
    and a_y (y = a F x + a_y y)."""
    n = [10, 8, 9]
    nx = list(n)
    ny = [v + 15 if b == 1 else v for v, b in zip(n, bc)]
    ny[0] += 2                                    # ld padding on the output
    N, M = int(np.prod(nx)), int(np.prod(ny))
    x = rnd(5, 2 * N)
    yo, w1, w2 = np.zeros(2 * M), np.zeros(2 * M), np.zeros(2 * M)
    assert O.call('oracle_d_sfrf_ld_narr', 3, n, bc, nx, ny, 2, x, yo, w1, w2) == 0
    md = F.filter_id('SYM8_MD')
    yg = np.zeros(2 * M)
    F.call('s0s0_md', md, 8, 3, n, bc, nx, ny, 2, 1.0, 0.0, 0.0, x, yg, np.zeros(1))
    mask = yo != 0.0                              # padding stays untouched (zero here)
    assert rel(yg[mask], yo[mask]) <= TOL
    y0 = rnd(6, 2 * M)
    ya = y0.copy()
    F.call('s0s0_md', md, 8, 3, n, bc, nx, ny, 2, -2.5, 0.0, 0.75, x, ya, np.zeros(1))
    want = -2.5 * yo + 0.75 * y0
    assert rel(ya[mask], want[mask]) <= TOL
    # alpha name, same operator
    yb = np.zeros(2 * M)
    F.call('s0s0_sym8_md_d', 3, n, bc, nx, ny, 2, 1.0, 0.0, 0.0, x, yb, np.zeros(1))
    assert np.array_equal(yb, yg)
    # a_x is refused for d > 1 (not a term of the generated multi-D product)
    assert F.call('s0s0_md', md, 8, 3, n, bc, nx, ny, 2, 1.0, 0.5, 0.0, x, yb, np.zeros(1),
                  check=False) == -1


@pytest.mark.parametrize('bc', [[0, 0, 0], [1, 1, 1], [-1, -1, -1]])
def test_wavelet_md(F, O, bc):
    """s1s0_md / s0s1_md (and the alpha names) against the 3D transforms, with
    a and a_y on the last sweep."""
    n = [5, 4, 6]
    lp = F.filter_id('SYM8_LP')
    for fwd in (True, False):
        nx = [v + 7 if b == -1 else v for v, b in zip(n, bc)]
        ny = [v + 7 if b == 1 else v for v, b in zip(n, bc)]
        Nx, Ny = 8 * int(np.prod(nx)), 8 * int(np.prod(ny))
        x = rnd(7, Nx)
        yo, w1, w2 = np.zeros(Ny), np.zeros(max(Nx, Ny) * 2), np.zeros(max(Nx, Ny) * 2)
        oname = 'oracle_d_dwt_sym8' if fwd else 'oracle_d_idwt_sym8'
        assert O.call(oname, 3, n, bc, x, yo, w1, w2) == 0
        y0 = rnd(8, Ny)
        yg = y0.copy()
        F.call('s0s1_md' if fwd else 's1s0_md', lp, 8, 3, n, bc, nx, ny, 1, 1.5, -0.5, x, yg,
               np.zeros(1))
        assert rel(yg, 1.5 * yo - 0.5 * y0) <= TOL
        ya = np.zeros(Ny)
        F.call('s0s1_sym8_lp_d' if fwd else 's1s0_sym8_lp_d', 3, n, bc, nx, ny, 1, 1.0, 0.0, x, ya,
               np.zeros(1))
        assert rel(ya, yo) <= TOL


@pytest.mark.parametrize('fname,oname', [('SYM8_D2', 'd2_dotin'), ('SYM8_D1', 'd1'),
                                         ('SYM8_MD', 'md')])
@pytest.mark.parametrize('bc', [[0, 0, 0], [2, 2, 2], [0, 2, 0]])
def test_s0s0_1ds_and_dot(F, O, fname, oname, bc):
    """Sum of 1D convolutions y = sum_i a_i F_i x + a_x x + a_y y against the
    sum of the oracle's 1D sweeps, and dot_in(i) = x . (a_i F_i x)."""
    n = [11, 9, 13]
    N = int(np.prod(n))
    a = [-1.3, 0.7, -2.1]
    x, y0 = rnd(9, N), rnd(10, N)
    fid = F.filter_id(fname)
    want = 0.4 * x - 0.8 * y0
    dots, scale = [], []
    for i in range(3):
        t = np.zeros(N)
        args = [3, i, n, bc[i], n, n, 1, x, t, a[i], 0.0, 0.0]
        if oname == 'd2_dotin':
            dd = ctypes.c_double(0.0)
            assert O.call('oracle_d_s0s0_1d_sym8_d2_dotin', *args, ctypes.pointer(dd)) == 0
        else:
            assert O.call(f'oracle_d_s0s0_1d_sym8_{oname}', *args) == 0
        want = want + t
        dots.append(float(x @ t))
        scale.append(float(np.abs(x) @ np.abs(t)))   # the D1 dots cancel to rounding noise
    yg = y0.copy()
    F.call('s0s0_1ds', fid, 8, 3, n, bc, n, n, 1, np.array(a), 0.4, -0.8, x, yg, np.zeros(1))
    assert rel(yg, want) <= TOL
    yd, dg = y0.copy(), np.zeros(3)
    F.call('s0s0_1ds_dot', fid, 8, 3, n, bc, n, n, 1, np.array(a), 0.4, -0.8, x, yd, dg,
           np.zeros(1))
    assert rel(yd, want) <= TOL
    assert np.all(np.abs(dg - np.array(dots)) <= 1e-13 * np.array(scale)), (dg, dots)
    if fname == 'SYM8_D2':
        ye, de = y0.copy(), np.zeros(3)
        F.call('s0s0_1ds_dot_sym8_d2_d', 3, n, bc, n, n, 1, np.array(a), 0.4, -0.8, x, ye, de,
               np.zeros(1))
        assert np.array_equal(ye, yd) and np.array_equal(de, dg)


def test_pipeline_sketch_through_fortran_api(pkg, F):
    """libconv.f90:238-290 replayed through the Fortran procedures (ids and
    sizes from the get_* queries, the potential step done by the caller as
    the sketch leaves it) equals libconv_hamiltonian on the same inputs."""
    n = [7, 6, 8]
    dwt, kin = F.filter_id('SYM8_LP'), F.filter_id('SYM8_D2')
    mdf, mif = F.filter_id('SYM8_MD'), F.filter_id('SYM8_MI')
    grow, shrink, nogrow = F.bc_id('G'), F.bc_id('S'), F.bc_id('F')
    ns1 = F.sizes('get_s1s0_input_size', 3, n, dwt, [grow] * 3)
    ns0 = F.sizes('get_s1s0_output_size', 3, n, dwt, [grow] * 3)
    n0 = [2 * v for v in ns0]
    npsir = F.sizes('get_s0s0_md_output_size', 3, n0, mdf, [grow] * 3)
    nw = max(F.sizes('get_s1s0_work_size', 3, n, dwt, [grow] * 3, work=True),
             F.sizes('get_s0s0_md_work_size', 3, n0, mdf, [grow] * 3, work=True),
             F.sizes('get_s0s0_1ds_work_size', 3, n0, kin, [nogrow] * 3, work=True))
    work = np.zeros(nw)
    rng = np.random.default_rng(12)
    psig = rng.standard_normal(8 * int(np.prod(n)))
    pot = rng.uniform(-1.0, 2.0, int(np.prod(npsir)))
    h = [0.45, 0.4, 0.5]
    akin = np.array([-0.5 / v ** 2 for v in h])
    psi_fscf = np.zeros(int(np.prod(n0)))
    F.call('s1s0_md', dwt, 8, 3, n, [grow] * 3, ns1, ns0, 1, 1.0, 0.0, psig, psi_fscf, work)
    psir = np.zeros(int(np.prod(npsir)))
    F.call('s0s0_md', mdf, 8, 3, n0, [grow] * 3, n0, npsir, 1, 1.0, 0.0, 0.0, psi_fscf, psir, work)
    rho = psir ** 2
    epot = float(psir @ (pot * psir))
    psir = pot * psir
    hpsi = np.zeros(int(np.prod(n0)))
    F.call('s0s0_md', mif, 8, 3, n0, [shrink] * 3, npsir, n0, 1, 1.0, 0.0, 0.0, psir, hpsi, work)
    ekin = np.zeros(3)
    F.call('s0s0_1ds_dot', kin, 8, 3, n0, [nogrow] * 3, n0, n0, 1, akin, 0.0, 1.0, psi_fscf, hpsi,
           ekin, work)
    hpsig = np.zeros(psig.size)
    F.call('s0s1_md', dwt, 8, 3, n, [shrink] * 3, ns0, ns1, 1, 1.0, 0.0, hpsi, hpsig, work)
    rh = np.zeros(pot.size)
    hh, eh, ph = pkg.hamiltonian(n, [2, 2, 2], akin, psig, pot, rh)
    assert rel(hpsig, hh) <= TOL
    assert rel(rho, rh) <= TOL
    assert np.abs(ekin - eh).max() <= 1e-12 * np.abs(eh).max()
    assert abs(epot - ph) <= 1e-12 * float(np.abs(pot).max() * rho.sum())
