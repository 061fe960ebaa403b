"""Batched operators over uneven grids (libconv_batch_*): every engine and
sweep order the compute mode allows, per grid against the oracle's
single-grid operators (MagicFilter3D free grow, kinetic free no-grow and
periodic), graph replay, rebinding to new buffers, and the autotuner with its
persisted cache.  Tolerance 1e-13 relative to max|y| (FP64-accurate modes)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13
PERMS = [[0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]]


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def make_batch_inputs(seed, ngrids, lo, hi):
    from boast_lig_gb300 import inputs
    rng = np.random.default_rng(seed)
    dims = [[int(v) for v in rng.integers(lo, hi + 1, 3)] for _ in range(ngrids)]
    xs = [inputs.uniform(seed * 100 + g, int(np.prod(d))) for g, d in enumerate(dims)]
    return dims, xs


def oracle_outputs(O, dims, xs, mf_bc, kin_bc, a, ax):
    mf, kin = [], []
    for d, x in zip(dims, xs):
        if mf_bc is not None:
            ny = [v + 15 if b == 1 else v for v, b in zip(d, mf_bc)]
            big = int(np.prod([v + 15 for v in d]))
            y = np.zeros(int(np.prod(ny)))
            assert O.call('oracle_d_sfrf_ld_narr', 3, d, mf_bc, d, ny, 1, x, y,
                          np.zeros(big), np.zeros(big)) == 0
            mf.append(y)
        if kin_bc is not None:
            y = np.zeros(x.size)
            assert O.call('oracle_d_kin', 3, d, kin_bc, x, y, np.zeros(x.size), np.zeros(x.size),
                          np.array(a), ax, 0.0) == 0
            kin.append(y)
    return mf, kin


def check(B, outs, ref_mf, ref_kin):
    in_off, mf_off, kin_off = B.offsets()
    y_mf, y_kin = outs
    if ref_mf:
        h = y_mf.cpu().numpy()
        for g, r in enumerate(ref_mf):
            assert rel(h[mf_off[g]:mf_off[g + 1]], r) <= TOL, ('mf', g)
    if ref_kin:
        h = y_kin.cpu().numpy()
        for g, r in enumerate(ref_kin):
            assert rel(h[kin_off[g]:kin_off[g + 1]], r) <= TOL, ('kin', g)


def alloc(torch, B, xs):
    n_in, n_mf, n_kin = B.sizes()
    x = torch.from_numpy(np.concatenate(xs)).cuda()
    assert x.numel() == n_in
    y_mf = torch.zeros(max(n_mf, 1), dtype=torch.float64, device='cuda')
    y_kin = torch.zeros(max(n_kin, 1), dtype=torch.float64, device='cuda')
    return x, y_mf, y_kin


@pytest.mark.parametrize('mode', ['fp64', 'tc_exact'])
def test_batch_every_engine_and_order(pkg, O, mode, tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv('LIBCONV_GB300_TUNE_CACHE', str(tmp_path / 'tune.json'))
    m = pkg.MODE_FP64 if mode == 'fp64' else pkg.MODE_TC_EXACT
    dims, xs = make_batch_inputs(3, 6, 5, 21)
    a = [-0.5 / 0.45 ** 2, -0.5 / 0.4 ** 2, -0.5 / 0.5 ** 2]
    ref_mf, ref_kin = oracle_outputs(O, dims, xs, [1, 1, 1], [2, 2, 2], a, 0.3)
    with pkg.mode(m):
        B = pkg.Batch(dims, mf_bc=[1, 1, 1], kin_bc=[2, 2, 2], kin_a=a, kin_ax=0.3)
        x, y_mf, y_kin = alloc(torch, B, xs)
        s = torch.cuda.Stream()
        engines = [pkg.ENGINE_FP64_Q64, pkg.ENGINE_FP64_Q32]
        if mode != 'fp64':
            engines.append(pkg.ENGINE_TC)
        for e in engines:
            for order in [[-1, 0, 0]] + PERMS:
                B.set_config(pkg.BATCH_OP_MF, e, order)
                if order[0] >= 0:
                    B.set_config(pkg.BATCH_OP_KIN, e, order)
                y_mf.zero_()
                y_kin.zero_()
                B.run(x, y_mf, y_kin, stream=s)
                pkg.check(s)
                check(B, (y_mf, y_kin), ref_mf, ref_kin)
        B.close()


def test_batch_graph_replay_rebind_and_tuning_cache(pkg, O, tmp_path, monkeypatch):
    import torch
    cache = tmp_path / 'tune.json'
    monkeypatch.setenv('LIBCONV_GB300_TUNE_CACHE', str(cache))
    dims, xs = make_batch_inputs(4, 9, 6, 30)
    a = [-0.5 / 0.45 ** 2] * 3
    ref_mf, ref_kin = oracle_outputs(O, dims, xs, [1, 1, 1], [2, 2, 2], a, 0.0)
    with pkg.mode(pkg.MODE_TC_EXACT):
        B = pkg.Batch(dims, mf_bc=[1, 1, 1], kin_bc=[2, 2, 2], kin_a=a)
        assert B.get_config(pkg.BATCH_OP_MF)[2] is False
        x, y_mf, y_kin = alloc(torch, B, xs)
        s = torch.cuda.Stream()
        B.tune(x, y_mf, y_kin, stream=s)
        cfg_mf, cfg_kin = B.get_config(pkg.BATCH_OP_MF), B.get_config(pkg.BATCH_OP_KIN)
        assert cfg_mf[2] and cfg_kin[2]
        for _ in range(3):                          # graph captured once, replayed
            y_mf.zero_()
            y_kin.zero_()
            B.run(x, y_mf, y_kin, stream=s)
        pkg.check(s)
        check(B, (y_mf, y_kin), ref_mf, ref_kin)
        x2, y_mf2, y_kin2 = alloc(torch, B, xs)     # new buffers: descriptors rebound
        B.run(x2, y_mf2, y_kin2, stream=s)
        pkg.check(s)
        check(B, (y_mf2, y_kin2), ref_mf, ref_kin)
        B.close()
        saved = json.loads(cache.read_text())
        assert len(saved) == 2
        B2 = pkg.Batch(dims, mf_bc=[1, 1, 1], kin_bc=[2, 2, 2], kin_a=a)
        assert B2.get_config(pkg.BATCH_OP_MF) == cfg_mf
        assert B2.get_config(pkg.BATCH_OP_KIN) == cfg_kin
        B2.run(x, y_mf, y_kin, stream=s)
        pkg.check(s)
        check(B2, (y_mf, y_kin), ref_mf, ref_kin)
        B2.close()


def test_batch_periodic_kinetic_only_default_stream(pkg, O):
    import torch
    dims, xs = make_batch_inputs(5, 4, 8, 24)
    a = [-0.5 / 0.4 ** 2] * 3
    _, ref_kin = oracle_outputs(O, dims, xs, None, [0, 0, 0], a, 0.1)
    for m in (pkg.MODE_FP64, pkg.MODE_TC_EXACT):
        with pkg.mode(m):
            B = pkg.Batch(dims, kin_bc=[0, 0, 0], kin_a=a, kin_ax=0.1)
            x, _, y_kin = alloc(torch, B, xs)
            B.run(x, None, y_kin)                   # legacy stream: launches, no graph
            pkg.check(None)
            check(B, (None, y_kin), None, ref_kin)
            B.close()


@pytest.mark.parametrize('mode', ['tc_bf16x3', 'tc_tf32x3'])
def test_batch_split_precision(pkg, O, mode):
    import torch
    dims, xs = make_batch_inputs(6, 5, 8, 26)
    a = [-0.5 / 0.45 ** 2] * 3
    ref_mf, ref_kin = oracle_outputs(O, dims, xs, [1, 1, 1], [2, 2, 2], a, 0.0)
    m = pkg.MODE_TC_BF16X3 if mode == 'tc_bf16x3' else pkg.MODE_TC_TF32X3
    with pkg.mode(m):
        B = pkg.Batch(dims, mf_bc=[1, 1, 1], kin_bc=[2, 2, 2], kin_a=a)
        assert B.get_config(pkg.BATCH_OP_MF)[0] == pkg.ENGINE_TC
        x, y_mf, y_kin = alloc(torch, B, xs)
        s = torch.cuda.Stream()
        B.run(x, y_mf, y_kin, stream=s)
        pkg.check(s)
        _, mf_off, kin_off = B.offsets()
        hm, hk = y_mf.cpu().numpy(), y_kin.cpu().numpy()
        for g in range(len(dims)):
            assert rel(hm[mf_off[g]:mf_off[g + 1]], ref_mf[g]) <= 1e-5
            assert rel(hk[kin_off[g]:kin_off[g + 1]], ref_kin[g]) <= 4e-5
        B.close()


def test_batch_rejects_bad_arguments(pkg):
    with pytest.raises(pkg.LibconvError):
        pkg.Batch([[4, 4, 4]])                      # no operator
    with pytest.raises(pkg.LibconvError):
        pkg.Batch([[4, 0, 4]], kin_bc=[0, 0, 0], kin_a=[1, 1, 1])
    with pytest.raises(pkg.LibconvError):
        pkg.Batch([[8, 8, 8]], kin_bc=[1, 1, 1], kin_a=[1, 1, 1])   # kinetic grow
    with pkg.mode(pkg.MODE_FP64):
        B = pkg.Batch([[8, 8, 8]], kin_bc=[0, 0, 0], kin_a=[1, 1, 1])
        with pytest.raises(pkg.LibconvError):
            B.set_config(pkg.BATCH_OP_KIN, pkg.ENGINE_TC, [0, 1, 2])   # no TC in FP64 mode
        with pytest.raises(pkg.LibconvError):
            B.set_config(pkg.BATCH_OP_KIN, pkg.ENGINE_FP64_Q64, [0, 0, 2])
        B.close()
