"""Train the learned preconditioner of the shifted kinetic solves and
compare flexible CG with it against plain (Jacobi) CG.

  python -m boast_lig_gb300.train_precond --n 48 --h 0.4 --pairs 20000 --out weights/precond_n48_h0.40.npz

(run through ``__graft_entry__.package()`` so the package imports as
``boast_lig_gb300``).  Steps:
 1. right-hand sides: Gaussian-filtered noise (sigma = 2 points, periodic,
    truncated at +-8), normalised to ||b|| = 1; eps uniform in [-1, -0.1];
 2. plain CG to ||r|| <= 1e-12 ||b|| gives x*; the same CG stopped after k
    iterations gives x_k, r_k = b - A x_k and e_k = x* - x_k; every
    (r_k, e_k, eps) divided by rms(r_k) is one training pair (pairs whose
    ||r_k|| fell below 1e-9 are dropped: their e_k is not known accurately);
 3. Adam on the relative A-norm error of M(r) against e, through the BF16
    convolution kernels;
 4. on-policy rounds: pairs from flexible CG with the current network
    stopped after k iterations (x* still from plain CG), appended to the
    set, and further training -- the network learns the residuals it leaves
    behind itself;
 5. checkpoint (npz) with the training metadata.
"""
import argparse
import json
import math
import time

import numpy as np

from . import inputs, precond


def gaussian_noise_torch(n, nsys, gen, device):
    """nsys periodic n^3 grids of Gaussian-filtered N(0,1) noise (the
    algorithm of inputs.gaussian_filtered_noise, on the GPU), unit RMS."""
    import torch
    g = torch.randn(nsys, n, n, n, generator=gen, dtype=torch.float64).to(device)
    k = torch.from_numpy(inputs.gaussian_kernel()).to(device)
    for ax in (1, 2, 3):
        acc = torch.zeros_like(g)
        for i in range(17):
            acc += k[i] * torch.roll(g, shifts=i - 8, dims=ax)
        g = acc
    g /= torch.sqrt((g * g).mean(dim=(1, 2, 3), keepdim=True))
    return g.reshape(nsys, -1)


def generate_pairs(n, h, npairs, seed, snaps=(0, 2, 4, 8, 16, 32, 48, 64, 96, 128), batch=256,
                   device='cuda', log=print, min_res=1e-9, net=None):
    """npairs (r, e, eps) pairs: x* by plain CG to 1e-12, x_k by plain CG
    (net None) or by flexible CG with `net` stopped after k iterations."""
    import torch
    gen = torch.Generator().manual_seed(seed)
    N = n ** 3
    per_sys = len(snaps)
    nsys_total = (npairs + per_sys - 1) // per_sys
    R = torch.empty(nsys_total * per_sys, N, dtype=torch.float32, device=device)
    E = torch.empty_like(R)
    EPS = torch.empty(nsys_total * per_sys, dtype=torch.float64, device=device)
    filled, t0, iters_12 = 0, time.time(), []
    while filled < nsys_total * per_sys:
        B = batch
        b = gaussian_noise_torch(n, B, gen, device)
        b /= b.norm(dim=1, keepdim=True)
        eps = (-1.0 + 0.9 * torch.rand(B, generator=gen, dtype=torch.float64)).to(device)
        xs = torch.empty_like(b)
        it, _ = precond.solve(n, eps, b, xs, h, tol=1e-12, maxit=20000)
        iters_12.append(it)
        xk = torch.empty_like(b)
        rk = torch.empty_like(b)
        for k in snaps:
            if k == 0:
                xk.zero_()
            else:
                precond.solve(n, eps, b, xk, h, tol=0.0, maxit=k, net=net)
            precond.apply(n, eps, xk, rk, h)
            rk = b - rk
            # pairs whose residual is still well above the 1e-12 of x*: the
            # error x* - x_k is then known to about 1e-3 relative or better
            ok = rk.norm(dim=1) >= min_res
            if not bool(ok.any()):
                continue
            rs, es, ep = rk[ok], (xs - xk)[ok], eps[ok]
            s = torch.sqrt((rs * rs).mean(dim=1, keepdim=True))
            m = min(rs.shape[0], R.shape[0] - filled)
            R[filled:filled + m] = (rs / s)[:m].float()
            E[filled:filled + m] = (es / s)[:m].float()
            EPS[filled:filled + m] = ep[:m]
            filled += m
            if filled >= R.shape[0]:
                break
        log(f'pairs {filled}/{R.shape[0]}  ({time.time() - t0:.1f} s)')
    its = np.concatenate(iters_12)
    return R[:npairs], E[:npairs], EPS[:npairs], {'cg_iters_1e-12_mean': float(its.mean()),
                                                  'cg_iters_1e-12_max': int(its.max())}


def train(n, h, R, E, EPS, steps=3000, batch=32, lr=2e-3, seed=1, device='cuda', log=print,
          net=None):
    import torch
    net = net or precond.Net(device=device, seed=seed)
    opt = torch.optim.Adam(net.params(), lr=lr)
    sched = torch.optim.lr_scheduler.LambdaLR(
        opt, lambda s: 0.5 * (1 + math.cos(math.pi * min(s, steps) / steps)))
    gen = torch.Generator(device=device).manual_seed(seed)
    ws = net.workspace(n, batch)
    ones = torch.ones(batch, dtype=torch.float64, device=device)
    Ad = torch.empty(batch * n ** 3, dtype=torch.float64, device=device)
    Ae = torch.empty_like(Ad)
    hist, t0 = [], time.time()
    for step in range(steps):
        idx = torch.randint(0, R.shape[0], (batch,), generator=gen, device=device)
        r = R[idx].double().reshape(-1)
        e = E[idx].double().reshape(-1)
        eps = EPS[idx].contiguous()
        net.pack()
        u = net.forward(n, r, eps, ones, ws)
        d = u - e
        precond.apply(n, eps, d, Ad, h)
        precond.apply(n, eps, e, Ae, h)
        num = (d.view(batch, -1) * Ad.view(batch, -1)).sum(1)
        den = (e.view(batch, -1) * Ae.view(batch, -1)).sum(1)
        loss = (num / den).mean()
        g = (2.0 / batch) * Ad.view(batch, -1) / den.view(-1, 1)
        opt.zero_grad(set_to_none=True)
        if not bool(torch.isfinite(loss)):
            sched.step()
            continue
        net.backward(n, r, eps, ones, g.reshape(-1).contiguous(), ws)
        torch.nn.utils.clip_grad_norm_(net.params(), 1.0)
        opt.step()
        sched.step()
        hist.append(float(loss))
        if step % 200 == 0 or step == steps - 1:
            log(f'step {step}  loss {np.mean(hist[-200:]):.4f}  ({time.time() - t0:.1f} s)')
    net.pack()
    return net, hist


def test_systems(n, nsys, seed=11):
    """The benchmark systems: seeded Gaussian-filtered noise right-hand sides
    (||b|| = 1) and eps uniform in [-1, -0.1]."""
    bs = []
    for s in range(nsys):
        g = inputs.gaussian_filtered_noise(seed * 1000 + s, (n, n, n)).ravel(order='F')
        bs.append(g / np.linalg.norm(g))
    eps = inputs.uniform(seed, nsys, -1.0, -0.1)
    return np.stack(bs), eps


def evaluate(n, h, net, nsys=256, seed=11, tol=1e-8, device='cuda', log=print, maxit=3000):
    import torch
    b_np, eps_np = test_systems(n, nsys, seed)
    b = torch.from_numpy(b_np.reshape(-1)).to(device)
    eps = torch.from_numpy(eps_np).to(device)
    out = {}
    for name, m in (('plain', None), ('learned', net)):
        x = torch.empty_like(b)
        precond.solve(n, eps, b, x, h, tol=tol, maxit=maxit, net=m)   # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        info = {}
        it, res = precond.solve(n, eps, b, x, h, tol=tol, maxit=maxit, net=m, info=info)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        fb = info['fell_back']
        out[name] = {'solves_per_s': nsys / t, 'seconds': t, 'iters_mean': float(it.mean()),
                     'iters_max': int(it.max()), 'max_true_residual': float(res.max()),
                     'fell_back': int((fb > 0).sum())}
        log(f'{name}: {nsys / t:.1f} solves/s, iterations mean {it.mean():.1f} max {it.max()}, '
            f'max ||b - Ax|| {res.max():.2e}, fell back {int((fb > 0).sum())}')
    return out


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument('--n', type=int, default=48)
    ap.add_argument('--h', type=float, default=0.4)
    ap.add_argument('--pairs', type=int, default=20000)
    ap.add_argument('--steps', type=int, default=3000)
    ap.add_argument('--batch', type=int, default=32)
    ap.add_argument('--lr', type=float, default=2e-3)
    ap.add_argument('--seed', type=int, default=5)
    ap.add_argument('--rounds', type=int, default=2, help='on-policy rounds')
    ap.add_argument('--round-pairs', type=int, default=4000)
    ap.add_argument('--round-steps', type=int, default=1500)
    ap.add_argument('--out', required=True)
    ap.add_argument('--report', default=None)
    ap.add_argument('--mode', default='tc_exact', choices=['tc_exact', 'fp64'],
                    help='kinetic sweeps inside the solves (both FP64-accurate)')
    args = ap.parse_args(argv)
    from . import set_mode, MODE_TC_EXACT, MODE_FP64
    set_mode(MODE_TC_EXACT if args.mode == 'tc_exact' else MODE_FP64)
    h = [args.h] * 3
    t0 = time.time()
    # round 0: plain-CG trajectories; rounds 1..: trajectories of flexible CG
    # with the current network (its own residuals), x* always from plain CG
    n0 = args.pairs - args.rounds * args.round_pairs
    R, E, EPS, gen_info = generate_pairs(args.n, h, n0, args.seed)
    t_gen = time.time() - t0
    net, hist = train(args.n, h, R, E, EPS, steps=args.steps, batch=args.batch, lr=args.lr)
    for rd in range(args.rounds):
        t1 = time.time()
        R2, E2, EPS2, _ = generate_pairs(args.n, h, args.round_pairs, args.seed + 100 + rd,
                                         snaps=(1, 2, 4, 6, 8, 10, 14, 20), net=net)
        R, E, EPS = torch.cat([R, R2]), torch.cat([E, E2]), torch.cat([EPS, EPS2])
        del R2, E2
        t_gen += time.time() - t1
        net, h2 = train(args.n, h, R, E, EPS, steps=args.round_steps, batch=args.batch,
                        lr=args.lr * 0.5, seed=2 + rd, net=net)
        hist += h2
    t_train = time.time() - t0 - t_gen
    del R, E
    torch.cuda.empty_cache()
    ev = evaluate(args.n, h, net)
    meta = {'n': args.n, 'h': args.h, 'pairs': args.pairs, 'steps': args.steps, 'batch': args.batch,
            'lr': args.lr, 'seed': args.seed, 'mode': args.mode, 'rounds': args.rounds,
            'round_pairs': args.round_pairs, 'round_steps': args.round_steps, 'final_loss': float(np.mean(hist[-100:]))}
    net.save(args.out, meta)
    rep = {'meta': meta, 'generation': gen_info, 'seconds_generate': t_gen,
           'seconds_train': t_train, 'loss_history_every_100': hist[::100], 'evaluation': ev}
    if args.report:
        json.dump(rep, open(args.report, 'w'), indent=1)
    print(json.dumps(rep['evaluation']))


if __name__ == '__main__':
    main()
