"""Learned-preconditioner kernels and the batched shifted-kinetic solver.

* Convolution kernels (BF16 operands, FP32 accumulation) against a plain
  PyTorch FP32 conv3d with circular padding on the same BF16-rounded
  operands: FP32-accumulated outputs to 1e-4 relative (summation order over
  432 products); BF16-stored outputs to 1.6e-2 (two BF16 ulps).
* Input and weight gradients against torch autograd of the same reference.
* Plain CG against the exact solution of the circulant system by FFT (the
  kinetic symbol of the 29-tap second derivative), and its true residual.
* Flexible CG with a network equal to the identity on r (ReLU pairs)
  converges, within twice the plain CG iterations (BF16 rounding of r makes
  that preconditioner vary between iterations).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def P(pkg):
    from boast_lig_gb300 import precond
    return precond


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def _rnd(t):
    import torch
    return t.to(torch.bfloat16).float()


def _conv_ref(x, W, b=None):
    import torch.nn.functional as F
    return F.conv3d(F.pad(x, (1, 1, 1, 1, 1, 1), mode='circular'), W, b)


def _rand_act(torch, nsys, n, seed, relu=False):
    g = torch.Generator().manual_seed(seed)
    a = torch.randn(nsys, n, n, n, 16, generator=g)
    if relu:
        a = a.clamp(min=0)
    return a.to(torch.bfloat16).cuda()


def _rand_w(torch, seed, co=16, ci=16):
    g = torch.Generator().manual_seed(seed)
    W = torch.randn(co, ci, 3, 3, 3, generator=g) * 0.2
    full = torch.zeros(27, 16, 16)
    full[:, :co, :ci] = W.permute(2, 3, 4, 0, 1).reshape(27, co, ci)
    return _rnd(W).cuda(), full.to(torch.bfloat16).cuda()


def test_conv_forward_field_and_relu(pkg, P):
    import torch
    n, nsys = 16, 2
    L = P._bind()
    act = _rand_act(torch, nsys, n, 1)
    W, wt = _rand_w(torch, 2)
    bias = torch.linspace(-0.5, 0.5, 16).cuda()
    x = act.float().permute(0, 4, 1, 2, 3)
    ref = _conv_ref(x, W, bias)                                   # [nsys, 16, n, n, n]
    fac = torch.full((nsys,), 2.0, dtype=torch.float64, device='cuda')
    z = torch.empty(nsys * n ** 3, dtype=torch.float64, device='cuda')
    assert L.libconv_cnn_conv(n, nsys, 0, 1, P._p(act), None, None, P._p(wt), P._p(bias), P._p(z),
                              P._p(fac), None, 1, None, None) == 0
    torch.cuda.synchronize()
    assert rel(z, 2.0 * ref[:, 0].reshape(-1).double()) <= 1e-4
    out = torch.empty_like(act)
    assert L.libconv_cnn_conv(n, nsys, 0, 0, P._p(act), None, None, P._p(wt), P._p(bias), P._p(out),
                              None, None, 16, None, None) == 0
    torch.cuda.synchronize()
    want = torch.relu(ref).permute(0, 2, 3, 4, 1)
    assert rel(out.float(), want) <= 1.6e-2


@pytest.mark.parametrize('n', [8, 24])
def test_conv_field_input_with_eps_channel(pkg, P, n):
    import torch
    nsys = 3
    L = P._bind()
    g = torch.Generator().manual_seed(3)
    r = torch.randn(nsys * n ** 3, generator=g, dtype=torch.float64).cuda()
    fac = torch.tensor([0.5, 1.0, 2.0], dtype=torch.float64, device='cuda')
    eps = torch.tensor([-0.2, -0.5, -0.9], dtype=torch.float64, device='cuda')
    W, wt = _rand_w(torch, 4, co=16, ci=2)
    bias = torch.zeros(16, device='cuda')
    x = torch.stack([(r.view(nsys, n, n, n) * fac.view(-1, 1, 1, 1)).float(),
                     eps.view(-1, 1, 1, 1).expand(nsys, n, n, n).float()], 1)
    ref = torch.relu(_conv_ref(_rnd(x), W, bias)).permute(0, 2, 3, 4, 1)
    out = torch.empty(nsys * n ** 3 * 16, dtype=torch.bfloat16, device='cuda')
    assert L.libconv_cnn_conv(n, nsys, 1, 0, P._p(r), P._p(fac), P._p(eps), P._p(wt), P._p(bias),
                              P._p(out), None, None, 16, None, None) == 0
    torch.cuda.synchronize()
    assert rel(out.float().view(nsys, n, n, n, 16), ref) <= 1.6e-2


@pytest.mark.parametrize('n', [24, 48])
def test_conv_tensor_core_sizes_and_active(pkg, P, n):
    """The tensor-core kernel (n >= 16; 8 x 16 x 4 tiles, the last y tile of
    n = 24 overlapping the one before it) for every destination kind against
    the FP32 reference; systems marked inactive are left untouched."""
    import torch
    nsys = 3
    L = P._bind()
    act = _rand_act(torch, nsys, n, 11)
    W, wt = _rand_w(torch, 12)
    bias = torch.linspace(-0.3, 0.4, 16).cuda()
    ref = _conv_ref(act.float().permute(0, 4, 1, 2, 3), W, bias)
    active = torch.tensor([1, 0, 1], dtype=torch.int32, device='cuda')
    on = [0, 2]
    out = torch.full_like(act, 7.0)
    assert L.libconv_cnn_conv(n, nsys, 0, 0, P._p(act), None, None, P._p(wt), P._p(bias), P._p(out),
                              None, None, 16, P._p(active), None) == 0
    torch.cuda.synchronize()
    want = torch.relu(ref).permute(0, 2, 3, 4, 1)
    assert rel(out.float()[on], want[on]) <= 1.6e-2
    assert bool((out[1].float() == 7.0).all())
    fac = torch.tensor([0.5, 1.0, -2.0], dtype=torch.float64, device='cuda')
    z = torch.zeros(nsys * n ** 3, dtype=torch.float64, device='cuda')
    assert L.libconv_cnn_conv(n, nsys, 0, 1, P._p(act), None, None, P._p(wt), P._p(bias), P._p(z),
                              P._p(fac), None, 1, None, None) == 0
    torch.cuda.synchronize()
    assert rel(z, (fac.view(-1, 1, 1, 1) * ref[:, 0].double()).reshape(-1)) <= 1e-4
    # input-gradient kind: mask = a ReLU output
    mask = torch.relu(act.float()).to(torch.bfloat16)
    gin = torch.empty_like(act)
    assert L.libconv_cnn_conv(n, nsys, 0, 2, P._p(act), None, None, P._p(wt), None, P._p(gin),
                              None, P._p(mask), 16, None, None) == 0
    torch.cuda.synchronize()
    want = _conv_ref(act.float().permute(0, 4, 1, 2, 3), W).permute(0, 2, 3, 4, 1) * (mask.float() > 0)
    assert rel(gin.float(), want) <= 1.6e-2
    # single-channel field source with a mask (the last layer's input gradient)
    r = torch.randn(nsys * n ** 3, dtype=torch.float64, device='cuda')
    W1, wt1 = _rand_w(torch, 13, co=16, ci=1)
    g1 = torch.empty_like(act)
    assert L.libconv_cnn_conv(n, nsys, 2, 2, P._p(r), P._p(fac), None, P._p(wt1), None, P._p(g1),
                              None, P._p(mask), 16, None, None) == 0
    torch.cuda.synchronize()
    x1 = _rnd((r.view(nsys, n, n, n) * fac.view(-1, 1, 1, 1)).float()).unsqueeze(1)
    want = _conv_ref(x1, W1).permute(0, 2, 3, 4, 1) * (mask.float() > 0)
    assert rel(g1.float(), want) <= 1.6e-2
    assert L.libconv_gb300_check(None) == 0


def test_conv_tensor_core_many_tiles_per_cta(pkg, P):
    """16 systems of 48^3: 1728 tiles over at most 3 CTAs per SM, so every CTA
    runs several tiles (mbarrier phases alternating) and skips the tiles of
    inactive systems between active ones."""
    import torch
    n, nsys = 48, 16
    L = P._bind()
    act = _rand_act(torch, nsys, n, 21)
    W, wt = _rand_w(torch, 22)
    bias = torch.linspace(-0.2, 0.3, 16).cuda()
    active = torch.tensor([1, 1, 0, 1, 0, 0, 1, 1, 1, 0, 1, 1, 1, 1, 0, 1], dtype=torch.int32,
                          device='cuda')
    on = [s for s in range(nsys) if int(active[s]) != 0]
    out = torch.full_like(act, -3.0)
    assert L.libconv_cnn_conv(n, nsys, 0, 0, P._p(act), None, None, P._p(wt), P._p(bias), P._p(out),
                              None, None, 16, P._p(active), None) == 0
    torch.cuda.synchronize()
    assert L.libconv_gb300_check(None) == 0
    for s in range(nsys):
        if s in on:
            ref = _conv_ref(act[s:s + 1].float().permute(0, 4, 1, 2, 3), W, bias)
            assert rel(out[s:s + 1].float(), torch.relu(ref).permute(0, 2, 3, 4, 1)) <= 1.6e-2, s
        else:
            assert bool((out[s].float() == -3.0).all()), s


def test_input_and_weight_gradients(pkg, P):
    import torch
    n, nsys = 16, 2
    L = P._bind()
    act = _rand_act(torch, nsys, n, 5, relu=True)
    gout = _rand_act(torch, nsys, n, 6)
    W, wt = _rand_w(torch, 7)
    x = act.float().permute(0, 4, 1, 2, 3).clone().requires_grad_()
    Wr = W.clone().requires_grad_()
    y = _conv_ref(x, Wr)
    (y * gout.float().permute(0, 4, 1, 2, 3)).sum().backward()
    # input gradient: the kernel convolves with taps flipped and channels
    # swapped; mask = the input activations (ReLU outputs, > 0 where passed)
    full = wt.float()
    wtd = full.flip(0).transpose(1, 2).to(torch.bfloat16).contiguous()
    gin = torch.empty_like(act)
    assert L.libconv_cnn_conv(n, nsys, 0, 2, P._p(gout), None, None, P._p(wtd), None, P._p(gin),
                              None, P._p(act), 16, None, None) == 0
    torch.cuda.synchronize()
    want = x.grad.permute(0, 2, 3, 4, 1) * (act.float() > 0)
    assert rel(gin.float(), want) <= 1.6e-2
    # weight gradient
    parts = L.libconv_cnn_wgrad_parts(n, nsys)
    part = torch.empty(parts * (27 * 256 + 16), dtype=torch.float32, device='cuda')
    out = torch.empty(27 * 256 + 16, dtype=torch.float32, device='cuda')
    assert L.libconv_cnn_wgrad(n, nsys, 0, P._p(gout), None, 0, P._p(act), None, None, P._p(part),
                               P._p(out), None) == 0
    torch.cuda.synchronize()
    dW = out[:27 * 256].view(3, 3, 3, 16, 16).permute(3, 4, 0, 1, 2)
    assert rel(dW, Wr.grad) <= 1e-4
    db = out[27 * 256:]
    assert rel(db, gout.float().sum(dim=(0, 1, 2, 3))) <= 1e-4


def test_network_forward_and_backward(pkg, P):
    import torch
    n, nsys = 16, 2
    net = P.Net(seed=3)
    with torch.no_grad():
        for b in net.b:
            b.normal_(0, 0.1)
    g = torch.Generator().manual_seed(8)
    r = torch.randn(nsys * n ** 3, generator=g, dtype=torch.float64).cuda()
    eps = torch.tensor([-0.3, -0.8], dtype=torch.float64, device='cuda')
    fac = torch.tensor([1.0, 0.5], dtype=torch.float64, device='cuda')
    ws = net.workspace(n, nsys)
    net.pack()
    u = net.forward(n, r, eps, fac, ws).clone()
    ref = net.reference(n, r, eps, fac)
    torch.cuda.synchronize()
    assert rel(u, ref) <= 3e-2
    # gradients of sum(gz * u) against autograd of the reference
    gz = torch.randn(nsys * n ** 3, generator=g, dtype=torch.float64).cuda()
    net.backward(n, r, eps, fac, gz, ws)
    kgrads = [p.grad.clone() for p in net.params()]
    ref_net = P.Net(seed=3)
    with torch.no_grad():
        for a, b in zip(ref_net.params(), net.params()):
            a.copy_(b)
    import torch.nn.functional as F
    x = torch.stack([(r.view(nsys, n, n, n) * fac.view(-1, 1, 1, 1)).float(),
                     eps.view(-1, 1, 1, 1).expand(nsys, n, n, n).float()], 1)
    h = _rnd(x)
    for l in range(4):
        h = _conv_ref(h, _rnd(ref_net.W[l]), ref_net.b[l])
        if l < 3:
            h = _rnd(torch.relu(h))
    (h[:, 0].reshape(-1).double() * gz).sum().backward()
    for kg, p in zip(kgrads, ref_net.params()):
        assert rel(kg, p.grad) <= 6e-2


def _fft_solve(n, h, eps, b):
    """Exact solution of (T - eps) x = b on the periodic grid (circulant)."""
    import __graft_entry__ as ge
    ge.package()
    from boast_lig_gb300 import gen_filters as G
    d2 = np.array([float(v) for v in G.SYM8_D2])
    j = np.arange(-14, 15)
    k = np.arange(n)
    sym = (d2[None, :] * np.cos(2 * np.pi * k[:, None] * j[None, :] / n)).sum(1)
    lam = sum(-0.5 / h ** 2 * sym[tuple(slice(None) if a == ax else None for a in range(3))]
              for ax in range(3)) - eps
    B = np.fft.fftn(b.reshape(n, n, n))
    return np.real(np.fft.ifftn(B / lam)).ravel()


def test_plain_cg_against_fft_solution(pkg, P):
    import torch
    from boast_lig_gb300 import inputs
    n, nsys, h = 16, 3, 0.4
    bs = [inputs.gaussian_filtered_noise(40 + s, (n, n, n)).ravel(order='F') for s in range(nsys)]
    bs = [v / np.linalg.norm(v) for v in bs]
    eps_np = np.array([-0.1, -0.5, -1.0])
    b = torch.from_numpy(np.concatenate(bs)).cuda()
    eps = torch.from_numpy(eps_np).cuda()
    x = torch.empty_like(b)
    for mode in (pkg.MODE_FP64, pkg.MODE_TC_EXACT):
        with pkg.mode(mode):
            it, res = P.solve(n, eps, b, x, [h] * 3, tol=1e-10, maxit=2000)
        assert (it <= 2000).all() and (res <= 1.5e-10).all(), (it, res)
        xh = x.cpu().numpy()
        for s in range(nsys):
            # the operator is the same along every axis (equal spacings)
            xe = _fft_solve(n, h, eps_np[s], bs[s])
            assert np.abs(xh[s * n ** 3:(s + 1) * n ** 3] - xe).max() <= 1e-8 * np.abs(xe).max()
    # y = (T - eps) x equals b
    y = torch.empty_like(b)
    P.apply(n, eps, x, y, [h] * 3)
    assert float((y - b).abs().max()) <= 1e-9


def test_flexible_cg_with_identity_network(pkg, P):
    import torch
    from boast_lig_gb300 import inputs
    n, nsys, h = 16, 4, 0.4
    net = P.Net(seed=0)
    with torch.no_grad():
        for W in net.W:
            W.zero_()
        for b in net.b:
            b.zero_()
        c = (1, 1, 1)
        net.W[0][0, 0][c] = 1.0
        net.W[0][1, 0][c] = -1.0
        for l in (1, 2):
            net.W[l][0, 0][c] = 1.0
            net.W[l][1, 1][c] = 1.0
        net.W[3][0, 0][c] = 1.0
        net.W[3][0, 1][c] = -1.0
    net.pack()
    bs = [inputs.gaussian_filtered_noise(60 + s, (n, n, n)).ravel(order='F') for s in range(nsys)]
    b = torch.from_numpy(np.concatenate([v / np.linalg.norm(v) for v in bs])).cuda()
    eps = torch.tensor([-0.1, -0.3, -0.6, -1.0], dtype=torch.float64, device='cuda')
    x = torch.empty_like(b)
    it_plain, res_plain = P.solve(n, eps, b, x, [h] * 3, tol=1e-8, maxit=3000)
    it_flex, res_flex = P.solve(n, eps, b, x, [h] * 3, tol=1e-8, maxit=3000, net=net)
    assert (res_plain <= 1.5e-8).all() and (res_flex <= 1.5e-8).all(), (res_plain, res_flex)
    # the BF16 rounding of r / s makes this preconditioner vary from one
    # iteration to the next (about 2^-9 relative), which costs flexible CG(1)
    # part of CG's global orthogonality: bounded at twice the plain count
    assert (it_flex <= 2 * it_plain + 5).all(), (it_plain, it_flex)


def test_trained_checkpoint_reduces_iterations(pkg, P):
    """The committed checkpoint (48^3, h = 0.4) on held-out systems: flexible CG
    converges to 1e-8 in fewer iterations than plain CG."""
    import torch
    from boast_lig_gb300 import train_precond
    path = os.path.join(P.WEIGHTS_DIR, 'precond_n48_h0.40.npz')
    if not os.path.exists(path):
        pytest.skip('no trained checkpoint')
    net = P.Net.load(path)
    n, h = 48, [0.4] * 3
    b_np, eps_np = train_precond.test_systems(n, 8, seed=29)
    b = torch.from_numpy(b_np.reshape(-1)).cuda()
    eps = torch.from_numpy(eps_np).cuda()
    x = torch.empty_like(b)
    it_p, res_p = P.solve(n, eps, b, x, h, tol=1e-8, maxit=5000)
    it_l, res_l = P.solve(n, eps, b, x, h, tol=1e-8, maxit=5000, net=net)
    assert (res_p <= 1.5e-8).all() and (res_l <= 1.5e-8).all()
    assert it_l.mean() < it_p.mean(), (it_p, it_l)


def test_learned_preconditioner_doubles_solves_per_second(pkg, P):
    """The bar the learned preconditioner is built for, on 64 held-out 48^3
    systems (h = 0.4, eps uniform in [-1, -0.1], Gaussian-filtered noise
    right-hand sides), kinetic sweeps in the exact tensor-core mode as the
    benchmark runs them: flexible CG with the committed network brings every
    system's true FP64 residual ||b - (T - eps) x|| to 1e-8 or below, at two
    or more times the solves/s of plain CG on the same GPU (each timed with
    CUDA events on one stream after a warm-up solve)."""
    import torch
    from boast_lig_gb300 import train_precond
    path = os.path.join(P.WEIGHTS_DIR, 'precond_n48_h0.40.npz')
    if not os.path.exists(path):
        pytest.skip('no trained checkpoint')
    net = P.Net.load(path)
    n, h, nsys = 48, [0.4] * 3, 64
    b_np, eps_np = train_precond.test_systems(n, nsys, seed=31)
    b = torch.from_numpy(b_np.reshape(-1)).cuda()
    eps = torch.from_numpy(eps_np).cuda()
    x = torch.empty_like(b)
    s = torch.cuda.Stream()

    def timed(m):
        P.solve(n, eps, b, x, h, tol=1e-8, maxit=5000, net=m, stream=s)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        it, res = P.solve(n, eps, b, x, h, tol=1e-8, maxit=5000, net=m, stream=s)
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1), it, res

    with pkg.mode(pkg.MODE_TC_EXACT):
        ms_l, it_l, res_l = timed(net)
        ms_p, it_p, res_p = timed(None)
    print(f'learned {nsys / ms_l * 1e3:.0f} solves/s ({it_l.mean():.1f} it), plain '
          f'{nsys / ms_p * 1e3:.0f} solves/s ({it_p.mean():.1f} it), ratio {ms_p / ms_l:.2f}, '
          f'max residual {res_l.max():.3g} / {res_p.max():.3g}')
    assert (it_l <= 5000).all() and (it_p <= 5000).all()
    assert res_l.max() <= 1e-8 and res_p.max() <= 1e-8, (res_l.max(), res_p.max())
    assert ms_p / ms_l >= 2.0, (ms_p, ms_l)
