"""GPU parity: every C-ABI operator against the CPU oracle on the same seeded
inputs.  Tolerance: max|y - y_oracle| / max|y_oracle| <= 1e-13 (FP64; the
GPU uses fused multiply-adds, so results differ from the oracle only by
rounding of the same tap order), plus the reference tests' absolute
epsilons where they apply."""
import ctypes
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


@pytest.fixture(autouse=True, params=['fp64', 'tc_exact'])
def compute_mode(request, pkg):
    """Every parity case runs with the FP64 kernels and with the tensor-core
    exact-digit kernels (every sweep kind: convolution, wavelet, combined)."""
    m = pkg.MODE_FP64 if request.param == 'fp64' else pkg.MODE_TC_EXACT
    with pkg.mode(m):
        yield request.param


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def seeded(seed, size):
    import __graft_entry__ as ge
    ge.package()
    from boast_lig_gb300 import inputs
    return inputs.uniform(seed, size)


def run_both(pkg, O, name, args, y_len, dot=False):
    """Run the GPU library and the oracle on identical copies; returns (gpu, oracle[, dots])."""
    args = list(args)
    yi = 8 if name.startswith('d_s0s') or name.startswith('d_s1s0') else None
    y0 = args[yi]
    yg, yo = y0.copy(), y0.copy()
    ag, ao = list(args), list(args)
    ag[yi], ao[yi] = yg, yo
    if dot:
        st = pkg.Kernel(name).run(*ag, None)
        d = ctypes.c_double(0.0)
        assert O.call('oracle_' + name, *ao, ctypes.pointer(d)) == 0
        return yg, yo, st['reference_return']['dot_in'], d.value
    pkg.Kernel(name).run(*ag)
    assert O.call('oracle_' + name, *ao) == 0
    return yg, yo


CONV_OPS = ['d_s0s0_1d_sym8_md', 'd_s0s0_1d_sym8_imd', 'd_s0s0_1d_sym8_d1']
WAV_OPS = ['d_s0s1_1d_sym8', 'd_s1s0_1d_sym8', 'd_s0s1_1d_symicomb8', 'd_s1s0_1d_symicomb8']


def ext(op, bc, n):
    """(nx, ny) for the processed dim: taps-1 extra on the grown/shrunk side."""
    taps = {'d_s0s0_1d_sym8_md': 16, 'd_s0s0_1d_sym8_imd': 16, 'd_s0s0_1d_sym8_d1': 29,
            'd_s0s0_1d_sym8_d2_dotin': 29, 'd_s0s1_1d_sym8': 8, 'd_s1s0_1d_sym8': 8,
            'd_s0s1_1d_symicomb8': 16, 'd_s1s0_1d_symicomb8': 16}[op]
    return (n + taps - 1 if bc == -1 else n), (n + taps - 1 if bc == 1 else n)


@pytest.mark.parametrize('op', CONV_OPS)
@pytest.mark.parametrize('bc', [0, 1, -1, 2])
@pytest.mark.parametrize('idim', [0, 1, 2])
def test_conv1d_all_bcs_shapes(pkg, O, op, bc, idim):
    n = [7, 13, 20]
    nx, ny = list(n), list(n)
    nx[idim], ny[idim] = ext(op, bc, n[idim])
    narr = 2
    sx = int(np.prod(nx)) * narr
    sy = int(np.prod(ny)) * narr
    x = seeded(100 + idim, sx)
    for (a, ax, ay) in [(1.0, 0.0, 0.0), (0.7, -0.3, 1.5)]:
        y = seeded(200 + idim, sy)
        yg, yo = run_both(pkg, O, op, (3, idim, n, bc, nx, ny, narr, x, y, a, ax, ay), sy)
        assert rel(yg, yo) <= TOL, (op, bc, idim, a, ax, ay)


@pytest.mark.parametrize('op', WAV_OPS)
@pytest.mark.parametrize('bc', [0, 1, -1, 2])
@pytest.mark.parametrize('idim', [0, 1, 2])
def test_wavelet1d_all_bcs_shapes(pkg, O, op, bc, idim):
    n = [5, 9, 12]
    nx, ny = list(n), list(n)
    nx[idim], ny[idim] = ext(op, bc, n[idim])
    narr = 2
    sx = 8 * int(np.prod(nx)) * narr
    sy = 8 * int(np.prod(ny)) * narr
    x = seeded(300 + idim, sx)
    for (a, ay) in [(1.0, 0.0), (-1.25, 0.5)]:
        y = seeded(400 + idim, sy)
        yg, yo = run_both(pkg, O, op, (3, idim, n, bc, nx, ny, narr, x, y, a, ay), sy)
        assert rel(yg, yo) <= TOL, (op, bc, idim, a, ay)


@pytest.mark.parametrize('op', WAV_OPS)
@pytest.mark.parametrize('nproc', [41, 44, 46])
@pytest.mark.parametrize('idim', [0, 1, 2])
def test_wavelet1d_periodic_long_lines(pkg, O, op, nproc, idim):
    """Periodic lines of 41-46 positions (two channels each): a tile's window
    wraps once, and with lengths not a multiple of 4 the wrap falls inside
    the 4-position groups the sweeps load as runs."""
    n = [6, 5, 3]
    n[idim] = nproc
    narr = 2
    s = 8 * int(np.prod(n)) * narr
    x = seeded(500 + idim, s)
    y = seeded(600 + idim, s)
    yg, yo = run_both(pkg, O, op, (3, idim, n, 0, n, n, narr, x, y, 1.0, 0.0), s)
    assert rel(yg, yo) <= TOL, (op, nproc, idim)


@pytest.mark.parametrize('op', CONV_OPS)
@pytest.mark.parametrize('nproc', [80, 97, 130, 203])
@pytest.mark.parametrize('idim', [0, 1, 2])
def test_conv1d_periodic_long_lines(pkg, O, op, nproc, idim):
    """Periodic lines at least one tile window long (80 input elements for 16
    taps, 96 for 29), contiguous (idim 0) or strided: the exact sweep takes
    each tile window's largest exponent in its producers instead of a pass
    over the array (80 with 29 taps stays below the window and keeps the
    pass).  Lengths not a multiple of 4 put the wrap inside the 8-element
    groups.  Every line has its own magnitude (2^-40, 1, 2^40) and magnitudes
    also step by 2^20 along each line, so the tile windows of one line get
    different scales; each line must match the oracle to 1e-13 of its largest
    output."""
    n = [6, 5, 4]
    n[idim] = nproc
    narr = 2
    shape = (narr, n[2], n[1], n[0])
    ax = 3 - idim                                    # the line's axis in C order
    x = np.moveaxis(seeded(700 + nproc + 7 * idim, int(np.prod(shape))).reshape(shape), ax, -1)
    lines = x.shape[:-1]
    line_scale = 2.0 ** (40 * (np.arange(int(np.prod(lines))).reshape(lines) % 3 - 1))
    along = 2.0 ** (20 * ((np.arange(nproc) // 48) % 2))
    x = np.ascontiguousarray(np.moveaxis(x * line_scale[..., None] * along, -1, ax)).ravel()
    for (a, a_x, a_y) in [(1.0, 0.0, 0.0), (0.7, -0.3, 1.5)]:
        y = seeded(800 + nproc, x.size)
        yg, yo = run_both(pkg, O, op, (3, idim, n, 0, n, n, narr, x, y, a, a_x, a_y), x.size)
        g = np.moveaxis(yg.reshape(shape), ax, -1).reshape(-1, nproc)
        r = np.moveaxis(yo.reshape(shape), ax, -1).reshape(-1, nproc)
        err = np.abs(g - r).max(axis=1)
        assert np.all(err <= TOL * np.abs(r).max(axis=1)), (op, nproc, idim, a, a_x, a_y)


@pytest.mark.parametrize('bc', [0, 1, -1, 2])
@pytest.mark.parametrize('idim', [0, 1, 2])
def test_kinetic1d_dotin(pkg, O, bc, idim):
    op = 'd_s0s0_1d_sym8_d2_dotin'
    n = [33, 8, 17]
    nx, ny = list(n), list(n)
    nx[idim], ny[idim] = ext(op, bc, n[idim])
    sx, sy = int(np.prod(nx)) * 3, int(np.prod(ny)) * 3
    x = seeded(500 + idim, sx)
    y = seeded(600, sy)
    yg, yo, dg, do = run_both(pkg, O, op, (3, idim, n, bc, nx, ny, 3, x, y, -2.46, 0.5, 1.0), sy, dot=True)
    assert rel(yg, yo) <= TOL
    assert abs(dg - do) <= TOL * max(abs(do), 1e-300) * 10


def test_ld_padding_is_preserved(pkg, O):
    """Outputs past the computed range of a padded ld keep the caller's values."""
    n, ny = [10, 6], [14, 6]
    x = seeded(7, 60)
    y = np.full(84, 123.0)
    pkg.Kernel('d_s0s0_1d_sym8_md').run(2, 0, n, 0, n, ny, 1, x, y, 1.0, 0.0, 0.0)
    assert np.all(y.reshape(6, 14)[:, 10:] == 123.0)


@pytest.mark.parametrize('n', [[1, 1, 1], [1, 5, 2], [2, 3, 40], [64, 1, 3]])
def test_tiny_and_degenerate_grids(pkg, O, n):
    for bc in (0, 1, 2):
        for idim in range(3):
            nx, ny = list(n), list(n)
            nx[idim], ny[idim] = ext('d_s0s0_1d_sym8_md', bc, n[idim])
            x = seeded(8, int(np.prod(nx)))
            y = np.zeros(int(np.prod(ny)))
            yg, yo = run_both(pkg, O, 'd_s0s0_1d_sym8_md', (3, idim, n, bc, nx, ny, 1, x, y, 1.0, 0.0, 0.0), 0)
            assert rel(yg, yo) <= TOL


def test_c1_one_sweep_periodic_magicfilter(pkg, O):
    """The 1D workload: n=32, ndat=32*32, x uniform in [-1,1] from seed 1,
    a=1, a_x=a_y=0; against the oracle and the reference C's golden vector."""
    import os
    x = seeded(1, 32 * 1024)
    y = np.zeros_like(x)
    pkg.Kernel('d_s0s0_1d_sym8_md').run(1, 0, [32], 0, [32], [32], 1024, x, y, 1.0, 0.0, 0.0)
    yo = np.zeros_like(x)
    O.call('oracle_d_s0s0_1d_sym8_md', 1, 0, [32], 0, [32], [32], 1024, x, yo, 1.0, 0.0, 0.0)
    assert rel(y, yo) <= TOL
    # the reference routine writes y(ndat, n): compare through the transpose
    g = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'magicfilter_ref_c.npz'))
    ref = g['mf_per_n32_ndat1024'].reshape(32, 1024).T.ravel()
    assert rel(y, ref) <= TOL
    assert np.abs(y - ref).max() < 1e-14          # MagicFilter_test2.rb epsilon


@pytest.mark.parametrize('bcs', [[0, 0, 0], [1, 1, 1], [-1, -1, -1], [0, 1, 2], [2, 2, 2]])
def test_magicfilter3d(pkg, O, bcs):
    n = [11, 14, 9]
    op = 'd_sfrf_ld_narr' if -1 not in bcs else 'd_rfsf_ld_narr'
    nx = [v + 15 if b == -1 else v for v, b in zip(n, bcs)]
    ny = [v + 15 if b == 1 else v + 1 for v, b in zip(n, bcs)]   # padded outputs (ld)
    narr = 2
    X = int(np.prod(nx)) * narr
    big = max(int(np.prod([max(a, b) for a, b in zip(nx, ny)])), 1) * narr
    x = seeded(9, X)
    yg = np.zeros(int(np.prod(ny)) * narr)
    yo = yg.copy()
    w1, w2 = np.zeros(big), np.zeros(big)
    pkg.Kernel(op).run(3, n, bcs, nx, ny, narr, x, yg, w1, w2)
    assert O.call('oracle_' + op, 3, n, bcs, nx, ny, narr, x, yo, np.zeros(big), np.zeros(big)) == 0
    # compare the computed region (ld padding lines are computed from padding data)
    Y = yg.reshape(narr, ny[2], ny[1], ny[0])
    R = yo.reshape(narr, ny[2], ny[1], ny[0])
    qx = [v + 15 if b == 1 else v for v, b in zip(n, bcs)]
    sl = (slice(None), slice(0, qx[2]), slice(0, qx[1]), slice(0, qx[0]))
    assert rel(Y[sl], R[sl]) <= TOL


@pytest.mark.parametrize('bcs', [[0, 0, 0], [2, 2, 2], [0, 2, 0]])
def test_kinetic3d(pkg, O, bcs):
    n = [12, 19, 16]
    N = int(np.prod(n))
    x = seeded(10, N)
    a = [-0.5 / 0.5 ** 2, -0.5 / 0.6 ** 2, -0.5 / 0.7 ** 2]
    for ax, ay in [(0.0, 0.0), (0.5, 0.0), (0.3, -1.0)]:
        y0 = seeded(11, N)
        yg, yo = y0.copy(), y0.copy()
        w = np.zeros(N)
        pkg.Kernel('d_kin').run(3, n, bcs, x, yg, w, w, a, ax, ay)
        assert O.call('oracle_d_kin', 3, n, bcs, x, yo, np.zeros(N), np.zeros(N), np.array(a), ax, ay) == 0
        assert rel(yg, yo) <= TOL
        if bcs == [0, 0, 0] and ay == 0.0:
            r = np.zeros(N)
            O.call('oracle_kinetic_per_ref', *n, np.array([0.5, 0.6, 0.7]), x, r, ax)
            assert np.abs(yg - r).max() < 1e-12       # Kinetic_test2.rb epsilon


@pytest.mark.parametrize('bcs', [[0, 0, 0], [1, 1, 1], [-1, -1, -1], [2, 2, 2]])
def test_wavelet3d(pkg, O, bcs):
    n = [6, 9, 7]
    m = [2 * v + 14 if b == -1 else 2 * v for v, b in zip(n, bcs)]
    mo = [2 * v + 14 if b == 1 else 2 * v for v, b in zip(n, bcs)]
    x = seeded(12, int(np.prod(m)))
    big = int(np.prod([max(a, b) for a, b in zip(m, mo)]))
    for op in ('d_dwt_sym8', 'd_idwt_sym8'):
        yg, yo = np.zeros(int(np.prod(mo))), np.zeros(int(np.prod(mo)))
        w = np.zeros(big)
        pkg.Kernel(op).run(3, n, bcs, x, yg, w, w)
        assert O.call('oracle_' + op, 3, n, bcs, x, yo, np.zeros(big), np.zeros(big)) == 0
        assert rel(yg, yo) <= TOL, op


def test_device_entry_points_with_torch(pkg, O):
    import torch
    dev = torch.device('cuda:0')
    n = [16, 24, 20]
    N = int(np.prod(n))
    x = seeded(13, N)
    xd = torch.from_numpy(x).to(dev)
    yd = torch.zeros(N, dtype=torch.float64, device=dev)
    w1 = torch.zeros(N, dtype=torch.float64, device=dev)
    w2 = torch.zeros(N, dtype=torch.float64, device=dev)
    s = torch.cuda.Stream()
    pkg.Kernel('d_sfrf_ld_narr').run_dev(3, n, [0, 0, 0], n, n, 1, xd, yd, w1, w2, stream=s)
    s.synchronize()
    yo = np.zeros(N)
    O.call('oracle_d_sfrf_ld_narr', 3, n, [0, 0, 0], n, n, 1, x, yo, np.zeros(N), np.zeros(N))
    assert rel(yd.cpu().numpy(), yo) <= TOL
    dot = torch.zeros(1, dtype=torch.float64, device=dev)
    yd.zero_()
    pkg.Kernel('d_s0s0_1d_sym8_d2_dotin').run_dev(3, 1, n, 0, n, n, 1, xd, yd, -2.0, 0.0, 0.0, dot)
    torch.cuda.synchronize()
    yo = np.zeros(N)
    d = ctypes.c_double(0.0)
    O.call('oracle_d_s0s0_1d_sym8_d2_dotin', 3, 1, n, 0, n, n, 1, x, yo, -2.0, 0.0, 0.0, ctypes.pointer(d))
    assert rel(yd.cpu().numpy(), yo) <= TOL
    assert abs(dot.item() - d.value) <= 1e-12 * abs(d.value)


def test_full_size_magicfilter_kinetic_128(pkg, O):
    """The 3D workload at full size: MagicFilter and kinetic on a 128^3
    periodic grid of Gaussian-filtered noise (h = 0.45)."""
    from boast_lig_gb300 import inputs
    n = [128, 128, 128]
    x = inputs.gaussian_filtered_noise(21, tuple(n)).ravel(order='F')
    N = x.size
    y, w = np.zeros(N), np.zeros(N)
    pkg.Kernel('d_sfrf_ld_narr').run(3, n, [0, 0, 0], n, n, 1, x, y, w, w)
    yo = np.zeros(N)
    O.call('oracle_d_sfrf_ld_narr', 3, n, [0, 0, 0], n, n, 1, x, yo, np.zeros(N), np.zeros(N))
    assert rel(y, yo) <= TOL
    a = [-0.5 / 0.45 ** 2] * 3
    pkg.Kernel('d_kin').run(3, n, [0, 0, 0], x, y, w, w, a, 0.0, 0.0)
    O.call('oracle_d_kin', 3, n, [0, 0, 0], x, yo, np.zeros(N), np.zeros(N), np.array(a), 0.0, 0.0)
    assert rel(y, yo) <= TOL


def test_full_size_free_grow_magicfilter_64(pkg, O):
    from boast_lig_gb300 import inputs
    n = [64, 64, 64]
    g = [79, 79, 79]
    x = inputs.gaussian_filtered_noise(22, tuple(n)).ravel(order='F')
    G = 79 ** 3
    y = np.zeros(G)
    w = np.zeros(G)
    pkg.Kernel('d_sfrf_ld_narr').run(3, n, [1, 1, 1], n, g, 1, x, y, w, w)
    yo = np.zeros(G)
    O.call('oracle_d_sfrf_ld_narr', 3, n, [1, 1, 1], n, g, 1, x, yo, np.zeros(G), np.zeros(G))
    assert rel(y, yo) <= TOL


def test_full_size_wavelet_round_trip_96(pkg, O):
    """8 subbands of 48^3 synthesised into 96^3 and analysed back: coarse
    uniform [-1,1], details scaled by 1e-3; round trip to 1e-11
    (Wavelet_test2.rb epsilon) and each direction against the oracle."""
    from boast_lig_gb300 import inputs
    n = [48, 48, 48]
    N = 96 ** 3
    c = inputs.uniform(23, N).reshape(96, 96, 96)
    c[48:, :, :] *= 1e-3
    c[:, 48:, :] *= 1e-3
    c[:, :, 48:] *= 1e-3
    # the coarse (s,s,s) block is the first half of every axis
    s = np.ascontiguousarray(c).ravel()
    r, back, w = np.zeros(N), np.zeros(N), np.zeros(N)
    pkg.Kernel('d_idwt_sym8').run(3, n, [0, 0, 0], s, r, w, w)
    ro = np.zeros(N)
    O.call('oracle_d_idwt_sym8', 3, n, [0, 0, 0], s, ro, np.zeros(N), np.zeros(N))
    assert rel(r, ro) <= TOL
    pkg.Kernel('d_dwt_sym8').run(3, n, [0, 0, 0], r, back, w, w)
    assert np.abs(back - s).max() < 1e-11


def test_kinetic3d_narr_extension(pkg, O):
    """d_kin_narr: the 3D kinetic over narr grids in one call equals d_kin on each."""
    n = [10, 17, 12]
    N = int(np.prod(n))
    narr = 3
    x = seeded(30, N * narr)
    a = [-0.5 / 0.45 ** 2] * 3
    y0 = seeded(31, N * narr)
    yg = y0.copy()
    w = np.zeros(1)
    pkg.Kernel('d_kin_narr').run(3, n, [0, 0, 0], narr, x, yg, w, w, a, 0.25, 0.5)
    for j in range(narr):
        yo = y0[j * N:(j + 1) * N].copy()
        assert O.call('oracle_d_kin', 3, n, [0, 0, 0], x[j * N:(j + 1) * N].copy(), yo,
                      np.zeros(N), np.zeros(N), np.array(a), 0.25, 0.5) == 0
        assert rel(yg[j * N:(j + 1) * N], yo) <= TOL


@pytest.mark.parametrize('bcs', [[0, 0, 0], [1, 1, 1], [-1, -1, -1], [2, 2, 2]])
def test_wavelet3d_narr_extension(pkg, O, bcs):
    """d_dwt_sym8_narr / d_idwt_sym8_narr: narr grids in one call equal the
    oracle's d_dwt_sym8 / d_idwt_sym8 on each grid."""
    n = [6, 5, 7]
    m = [2 * v + 14 if b == -1 else 2 * v for v, b in zip(n, bcs)]
    mo = [2 * v + 14 if b == 1 else 2 * v for v, b in zip(n, bcs)]
    Ni, No = int(np.prod(m)), int(np.prod(mo))
    big = int(np.prod([max(a, b) for a, b in zip(m, mo)]))
    narr = 3
    x = seeded(32, Ni * narr)
    for op in ('d_dwt_sym8', 'd_idwt_sym8'):
        yg = np.zeros(No * narr)
        w = np.zeros(1)
        pkg.Kernel(op + '_narr').run(3, n, bcs, narr, x, yg, w, w)
        for j in range(narr):
            yo = np.zeros(No)
            assert O.call('oracle_' + op, 3, n, bcs, x[j * Ni:(j + 1) * Ni].copy(), yo,
                          np.zeros(big), np.zeros(big)) == 0
            assert rel(yg[j * No:(j + 1) * No], yo) <= TOL, (op, j)


def test_kinetic_ekin_matches_reference_form(pkg, O):
    """d_kin_ekin with a = -0.5/h^2, a_x = 0, a_y = 1 is
    kinetic_per_ref_optim_ekin: y += T x and kstrten per direction."""
    n = [24, 20, 18]
    N = int(np.prod(n))
    h = [0.45, 0.4, 0.5]
    x, y0 = seeded(40, N), seeded(41, N)
    yg, k = y0.copy(), np.zeros(3)
    pkg.Kernel('d_kin_ekin').run(3, n, [0, 0, 0], x, yg, np.zeros(1), np.zeros(1),
                                 [-0.5 / v ** 2 for v in h], 0.0, 1.0, k)
    yo, ko = y0.copy(), np.zeros(3)
    O.call('oracle_kinetic_per_ref_ekin', *n, np.array(h), x, yo, ko)
    assert rel(yg, yo) <= TOL
    assert np.abs(k - ko).max() <= TOL * np.abs(ko).max()


@pytest.mark.parametrize('bcs', [[2, 2, 2], [0, 2, 0]])
def test_kinetic_ekin_general_options(pkg, O, bcs):
    """Free / mixed BCs with a_x and a_y: y as d_kin, kstrten[i] as the 1D
    kinetic sweep with dot_in along axis i."""
    n = [17, 13, 11]
    N = int(np.prod(n))
    a = [-2.2, -1.7, -3.1]
    x, y0 = seeded(42, N), seeded(43, N)
    yg, k = y0.copy(), np.zeros(3)
    pkg.Kernel('d_kin_ekin').run(3, n, bcs, x, yg, np.zeros(1), np.zeros(1), a, 0.3, -0.7, k)
    yo = y0.copy()
    assert O.call('oracle_d_kin', 3, n, bcs, x, yo, np.zeros(N), np.zeros(N), np.array(a), 0.3,
                  -0.7) == 0
    assert rel(yg, yo) <= TOL
    for i in range(3):
        yd, dd = np.zeros(N), ctypes.c_double(0.0)
        assert O.call('oracle_d_s0s0_1d_sym8_d2_dotin', 3, i, n, bcs[i], n, n, 1, x, yd, a[i], 0.0,
                      0.0, ctypes.pointer(dd)) == 0
        assert abs(k[i] - dd.value) <= 1e-12 * abs(dd.value), (i, k[i], dd.value)


def test_kinetic_ekin_device_entry(pkg, O):
    import torch
    n = [16, 24, 20]
    N = int(np.prod(n))
    x = seeded(44, N)
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros(N, dtype=torch.float64, device='cuda')
    w1, w2 = torch.empty_like(yd), torch.empty_like(yd)
    kd = torch.zeros(3, dtype=torch.float64, device='cuda')
    h = [0.45] * 3
    pkg.Kernel('d_kin_ekin').run_dev(3, n, [0, 0, 0], xd, yd, w1, w2, [-0.5 / v ** 2 for v in h],
                                     0.0, 1.0, kd)
    torch.cuda.synchronize()
    yo, ko = np.zeros(N), np.zeros(3)
    O.call('oracle_kinetic_per_ref_ekin', *n, np.array(h), x, yo, ko)
    assert rel(yd.cpu().numpy(), yo) <= TOL
    assert np.abs(kd.cpu().numpy() - ko).max() <= TOL * np.abs(ko).max()
