"""The benchmark's own calls at full size, against the oracle grid by grid.

The headline step runs d_sfrf_ld_narr_dev and d_kin_narr_dev over a batch of
128^3 periodic grids in one call each (narr grids per launch, so tiles of
different grids share a launch and the line exponents of every grid sit in
one array), and its end-to-end form runs the host-pointer calls from pinned
buffers (pipelined chunks of grids on three streams).  Here 4 distinct grids
of seeded Gaussian-filtered noise go through exactly those calls in the
exact tensor-core mode the benchmark uses, and every grid is compared with
the oracle's d_sfrf_ld_narr / d_kin on that grid alone (1e-13 relative).
The reference tests the same operators at small sizes with narr = 2
(MagicFilter_test2.rb:60-87, Kinetic_test2.rb:91-104).

Also here: the 96^3 wavelet analysis direction against the oracle, and two
streams running the kinetic sweep with dot_in at the same time on different
inputs, each matching the oracle (the *_dev calls lease their scratch per
call).
"""
import concurrent.futures as cf
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13
N3 = [128, 128, 128]
NG = 4
A_KIN = [-0.5 / 0.45 ** 2] * 3


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope='module')
def grids(pkg):
    from boast_lig_gb300 import inputs
    return [inputs.gaussian_filtered_noise(1000 + i, tuple(N3)).ravel(order='F') * (1.0 + 1e-3 * i)
            for i in range(NG)]


@pytest.fixture(scope='module')
def oracle_out(O, grids):
    """(MagicFilter3D, Kinetic3D) of every grid by the oracle, one grid per thread."""
    N = grids[0].size

    def one(x):
        mf, kin = np.zeros(N), np.zeros(N)
        assert O.call('oracle_d_sfrf_ld_narr', 3, N3, [0, 0, 0], N3, N3, 1, x, mf, np.zeros(N),
                      np.zeros(N)) == 0
        assert O.call('oracle_d_kin', 3, N3, [0, 0, 0], x, kin, np.zeros(N), np.zeros(N),
                      np.array(A_KIN), 0.0, 0.0) == 0
        return mf, kin

    with cf.ThreadPoolExecutor(max_workers=NG) as ex:
        return list(ex.map(one, grids))


@pytest.mark.parametrize('mode', ['tc_exact', 'fp64'])
def test_headline_device_calls_every_grid(pkg, grids, oracle_out, mode):
    """d_sfrf_ld_narr_dev and d_kin_narr_dev with narr = 4 grids of 128^3 on a
    side stream, as the benchmark's timed step calls them."""
    import torch
    dev = torch.device('cuda:0')
    N = grids[0].size
    x = torch.from_numpy(np.concatenate(grids)).to(dev)
    o_mf = torch.empty(NG * N, dtype=torch.float64, device=dev)
    o_kin = torch.empty_like(o_mf)
    w1, w2 = torch.empty_like(o_mf), torch.empty_like(o_mf)
    s = torch.cuda.Stream()
    m = pkg.MODE_TC_EXACT if mode == 'tc_exact' else pkg.MODE_FP64
    with pkg.mode(m):
        pkg.Kernel('d_sfrf_ld_narr').run_dev(3, N3, [0, 0, 0], N3, N3, NG, x, o_mf, w1, w2, stream=s)
        pkg.Kernel('d_kin_narr').run_dev(3, N3, [0, 0, 0], NG, x, o_kin, w1, w2, A_KIN, 0.0, 0.0,
                                         stream=s)
    s.synchronize()
    pkg.check(s)
    mf, kin = o_mf.cpu().numpy(), o_kin.cpu().numpy()
    for j, (rmf, rkin) in enumerate(oracle_out):
        assert rel(mf[j * N:(j + 1) * N], rmf) <= TOL, ('magicfilter3d', mode, j)
        assert rel(kin[j * N:(j + 1) * N], rkin) <= TOL, ('kinetic3d', mode, j)


def test_headline_pipelined_host_calls_every_grid(pkg, grids, oracle_out):
    """The end-to-end form: host-pointer d_sfrf_ld_narr and d_kin_narr over the
    4 grids from page-locked buffers (the pipelined chunk path), tc_exact."""
    import torch
    N = grids[0].size
    keep = [torch.empty(NG * N, dtype=torch.float64, pin_memory=True) for _ in range(3)]
    hx, hmf, hkin = (t.numpy() for t in keep)
    hx[:] = np.concatenate(grids)
    w = np.zeros(1)
    with pkg.mode(pkg.MODE_TC_EXACT):
        pkg.Kernel('d_sfrf_ld_narr').run(3, N3, [0, 0, 0], N3, N3, NG, hx, hmf, w, w)
        pkg.Kernel('d_kin_narr').run(3, N3, [0, 0, 0], NG, hx, hkin, w, w, A_KIN, 0.0, 0.0)
    for j, (rmf, rkin) in enumerate(oracle_out):
        assert rel(hmf[j * N:(j + 1) * N], rmf) <= TOL, ('magicfilter3d', j)
        assert rel(hkin[j * N:(j + 1) * N], rkin) <= TOL, ('kinetic3d', j)


@pytest.mark.parametrize('mode', ['tc_exact', 'fp64'])
def test_full_size_wavelet_analysis_96(pkg, O, mode):
    """dwt of a 96^3 grid (into 8 subbands of 48^3) against the oracle's
    d_dwt_sym8; the input is the oracle's synthesis of the round-trip data."""
    from boast_lig_gb300 import inputs
    n = [48, 48, 48]
    N = 96 ** 3
    c = inputs.uniform(23, N).reshape(96, 96, 96)
    c[48:, :, :] *= 1e-3
    c[:, 48:, :] *= 1e-3
    c[:, :, 48:] *= 1e-3
    s = np.ascontiguousarray(c).ravel()
    r = np.zeros(N)
    assert O.call('oracle_d_idwt_sym8', 3, n, [0, 0, 0], s, r, np.zeros(N), np.zeros(N)) == 0
    back, w = np.zeros(N), np.zeros(N)
    m = pkg.MODE_TC_EXACT if mode == 'tc_exact' else pkg.MODE_FP64
    with pkg.mode(m):
        pkg.Kernel('d_dwt_sym8').run(3, n, [0, 0, 0], r, back, w, w)
    bo = np.zeros(N)
    assert O.call('oracle_d_dwt_sym8', 3, n, [0, 0, 0], r, bo, np.zeros(N), np.zeros(N)) == 0
    assert rel(back, bo) <= TOL
    assert np.abs(bo - s).max() < 1e-11


@pytest.mark.parametrize('mode', ['tc_exact', 'fp64'])
def test_two_streams_in_flight_keep_their_own_scratch(pkg, O, mode):
    """Two streams each run the 3D kinetic with its per-direction energies
    (d_kin_ekin_dev: dot partials and, in tc_exact, line exponents in scratch)
    and the 1D kinetic sweep with dot_in, interleaved call by call on
    different inputs without synchronising in between; every result and dot
    matches the oracle on its own input."""
    import torch
    from boast_lig_gb300 import inputs
    dev = torch.device('cuda:0')
    n = [96, 80, 72]
    N = int(np.prod(n))
    a = [-2.47, -1.9, -3.3]
    xs = [inputs.uniform(700 + k, N) for k in range(2)]
    xd = [torch.from_numpy(x).to(dev) for x in xs]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    ys = [torch.zeros(N, dtype=torch.float64, device=dev) for _ in range(2)]
    ks = [torch.zeros(3, dtype=torch.float64, device=dev) for _ in range(2)]
    y1 = [torch.zeros(N, dtype=torch.float64, device=dev) for _ in range(2)]
    d1 = [torch.zeros(1, dtype=torch.float64, device=dev) for _ in range(2)]
    ws = [(torch.empty(N, dtype=torch.float64, device=dev),
           torch.empty(N, dtype=torch.float64, device=dev)) for _ in range(2)]
    m = pkg.MODE_TC_EXACT if mode == 'tc_exact' else pkg.MODE_FP64
    kin, sw = pkg.Kernel('d_kin_ekin'), pkg.Kernel('d_s0s0_1d_sym8_d2_dotin')
    torch.cuda.synchronize()
    with pkg.mode(m):
        for rep in range(3):
            for k in range(2):
                kin.run_dev(3, n, [0, 0, 0], xd[k], ys[k], ws[k][0], ws[k][1], a, 0.0, 0.0, ks[k],
                            stream=streams[k])
                sw.run_dev(3, 1, n, 0, n, n, 1, xd[k], y1[k], a[1], 0.0, 0.0, d1[k],
                           stream=streams[k])
    for s in streams:
        s.synchronize()
        pkg.check(s)
    for k in range(2):
        yo, ko = np.zeros(N), np.zeros(3)
        assert O.call('oracle_d_kin', 3, n, [0, 0, 0], xs[k], yo, np.zeros(N), np.zeros(N),
                      np.array(a), 0.0, 0.0) == 0
        assert rel(ys[k].cpu().numpy(), yo) <= TOL, ('kinetic3d', k)
        for i in range(3):
            yd, dd = np.zeros(N), ctypes.c_double(0.0)
            assert O.call('oracle_d_s0s0_1d_sym8_d2_dotin', 3, i, n, 0, n, n, 1, xs[k], yd, a[i],
                          0.0, 0.0, ctypes.pointer(dd)) == 0
            ko[i] = dd.value
            if i == 1:
                assert rel(y1[k].cpu().numpy(), yd) <= TOL, ('sweep', k)
                assert abs(d1[k].item() - dd.value) <= 1e-12 * abs(dd.value), ('sweep dot', k)
        assert np.abs(ks[k].cpu().numpy() - ko).max() <= 1e-12 * np.abs(ko).max(), ('ekin', k)


def test_magicfilter3d_lines_keep_their_own_scale(pkg, O):
    """Every line of an exact tensor-core sweep is scaled by its own largest
    exponent.  Lines of the second MagicFilter3D sweep (along axis 1) get
    magnitudes 2^-40, 1 and 2^40 (the input scaled by its axis-2 index), so a
    line scaled by another line's exponent would lose up to 80 bits: the
    second sweep's output (left in w2) must match the oracle's to 1e-13 of
    each magnitude class, and y overall."""
    import torch
    from boast_lig_gb300 import inputs
    n = [64, 96, 32]
    narr = 2
    N = int(np.prod(n))
    x = inputs.uniform(801, N * narr).reshape(narr, n[2], n[1], n[0])
    scale = 2.0 ** (40 * (np.arange(n[2]) % 3 - 1))
    x = (x * scale[None, :, None, None]).ravel()
    dev = torch.device('cuda:0')
    xd = torch.from_numpy(x).to(dev)
    yd = torch.zeros(N * narr, dtype=torch.float64, device=dev)
    w1 = torch.zeros_like(yd)
    w2 = torch.zeros_like(yd)
    with pkg.mode(pkg.MODE_TC_EXACT):
        pkg.Kernel('d_sfrf_ld_narr').run_dev(3, n, [0, 0, 0], n, n, narr, xd, yd, w1, w2)
    torch.cuda.synchronize()
    yo, w1o, w2o = np.zeros(N * narr), np.zeros(N * narr), np.zeros(N * narr)
    assert O.call('oracle_d_sfrf_ld_narr', 3, n, [0, 0, 0], n, n, narr, x, yo, w1o, w2o) == 0
    # w2 (after the sweeps along axes 0 and 1) is laid out (i2, q0, q1): axis-2 index fastest
    g = w2.cpu().numpy().reshape(narr, n[1], n[0], n[2])
    r = w2o.reshape(narr, n[1], n[0], n[2])
    for cls in range(3):
        gc, rc = g[..., cls::3], r[..., cls::3]
        assert np.abs(gc - rc).max() <= TOL * np.abs(rc).max(), cls
    assert rel(yd.cpu().numpy(), yo) <= TOL


@pytest.mark.parametrize('narr', [1, 2])
def test_magicfilter3d_exponent_handoff_matches_separate_sweeps(pkg, narr):
    """On 128 x 64 x 32 grids each exact MagicFilter3D sweep hands the next one
    its line exponents from the epilogue (every tile column holds whole lines
    of the next sweep: 2 x 64 after the first sweep, 4 x 32 after the
    second).  The exact products depend only on each line's exponent, so the
    result must equal three 1D MagicFilter sweeps bit for bit: the first (128
    contiguous periodic points) takes its tile windows' exponents like the
    first MagicFilter3D sweep, the other two (64 and 32 points, shorter than a
    tile window) make their own line-exponent pass.  The input's magnitude
    steps by 2^40 along axis 2 (every line of the second sweep has its own
    scale).  The hand-off to 128-point lines runs in the full-size tests."""
    from boast_lig_gb300 import inputs
    n = [128, 64, 32]
    N = int(np.prod(n))
    x = inputs.uniform(907, N * narr).reshape(narr, n[2], n[1], n[0])
    x = (x * (2.0 ** (40 * (np.arange(n[2]) % 3 - 1)))[None, :, None, None]).ravel()
    y, w = np.zeros(N * narr), np.zeros(1)
    t1, t2, t3 = np.zeros(N * narr), np.zeros(N * narr), np.zeros(N * narr)
    with pkg.mode(pkg.MODE_TC_EXACT):
        pkg.Kernel('d_sfrf_ld_narr').run(3, n, [0, 0, 0], n, n, narr, x, y, w, w)
        k = pkg.Kernel('d_s0s0_1d_sym8_md')
        k.run(3, 0, n, 0, n, n, narr, x, t1, 1.0, 0.0, 0.0)
        k.run(3, 1, n, 0, n, n, narr, t1, t2, 1.0, 0.0, 0.0)
        k.run(3, 2, n, 0, n, n, narr, t2, t3, 1.0, 0.0, 0.0)
    assert np.array_equal(y, t3), float(np.abs(y - t3).max() / np.abs(t3).max())
