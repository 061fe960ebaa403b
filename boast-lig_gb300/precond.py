"""Learned preconditioner for the shifted kinetic solves (T - eps) x = r.

Network M (4 periodic 3x3x3 convolutions, 16 channels, ReLU after the first
three; inputs r / s and eps, s = rms(r); output channel 0) applied as
z = s M(r / s, eps) inside flexible CG (``libconv_cg_solve``).  Forward and
backward passes run the library's BF16 convolution kernels with FP32
accumulation (``libconv_cnn_conv`` / ``libconv_cnn_wgrad``); PyTorch holds the
FP32 master weights and runs the Adam optimiser.

Training pairs come from plain CG converged to 1e-12: for each system b the
solution x*, and for snapshot iterations k of the same CG run the residual
r_k = b - A x_k with its error e_k = x* - x_k (A e_k = r_k), both divided by
rms(r_k).  The loss is the relative A-norm error of M(r) against e,
sum_s (d_s, A d_s) / (e_s, A e_s) / B with d = M(r) - e.
"""
import ctypes
import os

import numpy as np

from . import _D, _dbl, _int, _vp, lib, LibconvError, last_error

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS_DIR = os.path.join(HERE, 'weights')
CIN = (2, 16, 16, 16)
COUT = (16, 16, 16, 1)


class _W(ctypes.Structure):
    _fields_ = [('wt', ctypes.c_void_p * 4), ('bias', ctypes.c_void_p * 4)]


def _bind():
    L = lib()
    if not getattr(L, '_cg_bound', False):
        P = ctypes.POINTER(ctypes.c_int)
        L.libconv_cg_apply.argtypes = [_int, _int, _D, _vp, _vp, _vp, _vp]
        L.libconv_cg_solve.argtypes = [_int, _int, _D, _vp, _vp, _vp, _dbl, _int,
                                       ctypes.POINTER(_W), P, _D, P, _vp]
        L.libconv_cnn_conv.argtypes = [_int, _int, _int, _int, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                       _vp, _int, _vp, _vp]
        L.libconv_cnn_wgrad.argtypes = [_int, _int, _int, _vp, _vp, _int, _vp, _vp, _vp, _vp, _vp,
                                        _vp]
        L.libconv_cnn_wgrad_parts.argtypes = [_int, _int]
        L.libconv_cg_set_stall.argtypes = [_int, _dbl]
        L.libconv_cg_set_stall.restype = _int
        for f in ('libconv_cg_apply', 'libconv_cg_solve', 'libconv_cnn_conv', 'libconv_cnn_wgrad',
                  'libconv_cnn_wgrad_parts'):
            getattr(L, f).restype = _int
        L._cg_bound = True
    return L


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _s(stream):
    if stream is None:
        return None
    return ctypes.c_void_p(stream.cuda_stream if hasattr(stream, 'cuda_stream') else int(stream))


def _h3(h):
    return ctypes.cast((ctypes.c_double * 3)(*[float(v) for v in h]), _D)


def _check(st, name):
    if st:
        raise LibconvError(st, name, last_error())


# ---- solver entry points ------------------------------------------------------------
def set_stall(window, ratio):
    """Stagnation test of the learned phase (libconv_cg_set_stall)."""
    _check(_bind().libconv_cg_set_stall(int(window), float(ratio)), 'libconv_cg_set_stall')


def apply(n, eps, x, y, h, stream=None):
    """y = (T - eps) x for every system (device float64 tensors)."""
    L = _bind()
    nsys = eps.numel()
    _check(L.libconv_cg_apply(n, nsys, _h3(h), _p(eps), _p(x), _p(y), _s(stream)), 'libconv_cg_apply')


def solve(n, eps, b, x, h, tol=1e-8, maxit=5000, net=None, stream=None, info=None):
    """Batched CG (net None: Jacobi) or flexible CG with the network; returns
    (iterations per system, true residual norms) as numpy arrays; info (dict)
    receives 'fell_back', the iteration each system switched to the plain
    preconditioner (0: never)."""
    L = _bind()
    nsys = eps.numel()
    it = (ctypes.c_int * nsys)()
    res = (ctypes.c_double * nsys)()
    fb = (ctypes.c_int * nsys)()
    w = net.struct() if net is not None else None
    IP = ctypes.POINTER(ctypes.c_int)
    _check(L.libconv_cg_solve(n, nsys, _h3(h), _p(eps), _p(b), _p(x), float(tol), int(maxit),
                              ctypes.byref(w) if w is not None else None, ctypes.cast(it, IP),
                              ctypes.cast(res, _D), ctypes.cast(fb, IP), _s(stream)),
           'libconv_cg_solve')
    if info is not None:
        info['fell_back'] = np.array(fb[:])
    return np.array(it[:]), np.array(res[:])


# ---- the network ----------------------------------------------------------------------
class Net:
    """FP32 master weights W[l] (torch, [cout, cin, 3, 3, 3]) and biases b[l]
    ([cout]); packed BF16 kernel layouts are refreshed by ``pack()``."""

    def __init__(self, device='cuda', seed=0):
        import torch
        g = torch.Generator().manual_seed(seed)
        self.device = torch.device(device)
        self.W, self.b = [], []
        for ci, co in zip(CIN, COUT):
            std = (2.0 / (27 * ci)) ** 0.5
            self.W.append((torch.randn(co, ci, 3, 3, 3, generator=g) * std).to(self.device).requires_grad_())
            self.b.append(torch.zeros(co, device=self.device).requires_grad_())
        with torch.no_grad():
            self.W[-1] *= 0.1
        self._packed = None

    def params(self):
        return self.W + self.b

    def pack(self):
        """Kernel layouts: wt [27][16 cout][16 cin] bf16, its dgrad form
        (taps flipped, cout/cin swapped), bias [16] float32."""
        import torch
        wt, wtd, bias = [], [], []
        with torch.no_grad():
            for W, b in zip(self.W, self.b):
                co, ci = W.shape[:2]
                full = torch.zeros(27, 16, 16, device=self.device)
                full[:, :co, :ci] = W.permute(2, 3, 4, 0, 1).reshape(27, co, ci)
                wt.append(full.to(torch.bfloat16).contiguous())
                wtd.append(full.flip(0).transpose(1, 2).to(torch.bfloat16).contiguous())
                bb = torch.zeros(16, device=self.device)
                bb[:co] = b
                bias.append(bb.contiguous())
        self._packed = (wt, wtd, bias)
        return self._packed

    def struct(self):
        wt, _, bias = self._packed or self.pack()
        s = _W()
        for l in range(4):
            s.wt[l] = wt[l].data_ptr()
            s.bias[l] = bias[l].data_ptr()
        return s

    # -- checkpoint
    def save(self, path, meta=None):
        arrs = {f'W{l}': self.W[l].detach().cpu().numpy() for l in range(4)}
        arrs.update({f'b{l}': self.b[l].detach().cpu().numpy() for l in range(4)})
        for k, v in (meta or {}).items():
            arrs['meta_' + k] = np.asarray(v)
        np.savez(path, **arrs)

    @classmethod
    def load(cls, path, device='cuda'):
        import torch
        z = np.load(path)
        net = cls(device=device)
        with torch.no_grad():
            for l in range(4):
                net.W[l].copy_(torch.from_numpy(z[f'W{l}']))
                net.b[l].copy_(torch.from_numpy(z[f'b{l}']))
        net.pack()
        net.meta = {k[5:]: z[k] for k in z.files if k.startswith('meta_')}
        return net

    # -- kernel forward / backward
    def forward(self, n, r, eps, fac, ws, stream=None):
        """u = M(r * fac, eps) (dst factor 1) with activations kept in ws for
        backward; r, u float64 [nsys * n^3]; ws: dict of buffers."""
        L = _bind()
        wt, _, bias = self._packed or self.pack()
        nsys = eps.numel()
        one = ws['one']
        a1, a2, a3, u = ws['a1'], ws['a2'], ws['a3'], ws['u']
        s = _s(stream)
        _check(L.libconv_cnn_conv(n, nsys, 1, 0, _p(r), _p(fac), _p(eps), _p(wt[0]), _p(bias[0]),
                                  _p(a1), None, None, 16, None, s), 'conv0')
        _check(L.libconv_cnn_conv(n, nsys, 0, 0, _p(a1), None, None, _p(wt[1]), _p(bias[1]), _p(a2),
                                  None, None, 16, None, s), 'conv1')
        _check(L.libconv_cnn_conv(n, nsys, 0, 0, _p(a2), None, None, _p(wt[2]), _p(bias[2]), _p(a3),
                                  None, None, 16, None, s), 'conv2')
        _check(L.libconv_cnn_conv(n, nsys, 0, 1, _p(a3), None, None, _p(wt[3]), _p(bias[3]), _p(u),
                                  _p(one), None, 1, None, s), 'conv3')
        return u

    def backward(self, n, r, eps, fac, g, ws, stream=None):
        """Gradients of sum(g * u) for the last forward; accumulates into
        W[l].grad / b[l].grad."""
        import torch
        L = _bind()
        _, wtd, _ = self._packed or self.pack()
        nsys = eps.numel()
        one = ws['one']
        a1, a2, a3, ga, gb = ws['a1'], ws['a2'], ws['a3'], ws['ga'], ws['gb']
        part, out = ws['part'], ws['out']
        s = _s(stream)
        grads = [None] * 4

        def wgrad(l, gk, G, gfac, xk, X, xfac, e):
            _check(L.libconv_cnn_wgrad(n, nsys, gk, _p(G), _p(gfac), xk, _p(X), _p(xfac), _p(e),
                                       _p(part), _p(out), s), f'wgrad{l}')
            grads[l] = out.clone()

        wgrad(3, 2, g, one, 0, a3, None, None)
        _check(L.libconv_cnn_conv(n, nsys, 2, 2, _p(g), _p(one), None, _p(wtd[3]), None, _p(ga),
                                  None, _p(a3), 16, None, s), 'dgrad3')
        wgrad(2, 0, ga, None, 0, a2, None, None)
        _check(L.libconv_cnn_conv(n, nsys, 0, 2, _p(ga), None, None, _p(wtd[2]), None, _p(gb),
                                  None, _p(a2), 16, None, s), 'dgrad2')
        wgrad(1, 0, gb, None, 0, a1, None, None)
        _check(L.libconv_cnn_conv(n, nsys, 0, 2, _p(gb), None, None, _p(wtd[1]), None, _p(ga),
                                  None, _p(a1), 16, None, s), 'dgrad1')
        wgrad(0, 0, ga, None, 1, r, fac, eps)
        with torch.no_grad():
            for l in range(4):
                co, ci = self.W[l].shape[:2]
                dW = grads[l][:27 * 256].view(27, 16, 16)[:, :co, :ci]
                dW = dW.reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2)
                db = grads[l][27 * 256:27 * 256 + co]
                self.W[l].grad = dW.clone() if self.W[l].grad is None else self.W[l].grad + dW
                self.b[l].grad = db.clone() if self.b[l].grad is None else self.b[l].grad + db

    def workspace(self, n, nsys):
        import torch
        L = _bind()
        N = nsys * n ** 3
        dev = self.device
        act = lambda: torch.empty(N * 16, dtype=torch.bfloat16, device=dev)
        return {'a1': act(), 'a2': act(), 'a3': act(), 'ga': act(), 'gb': act(),
                'u': torch.empty(N, dtype=torch.float64, device=dev),
                'one': torch.ones(nsys, dtype=torch.float64, device=dev),
                'part': torch.empty(L.libconv_cnn_wgrad_parts(n, nsys) * (27 * 256 + 16),
                                    dtype=torch.float32, device=dev),
                'out': torch.empty(27 * 256 + 16, dtype=torch.float32, device=dev)}

    # -- plain PyTorch FP32 reference of the same network (tests)
    def reference(self, n, r, eps, fac, bf16=True):
        """Torch FP32 forward with circular padding; bf16: round weights,
        inputs and hidden activations to bfloat16 as the kernels do."""
        import torch
        import torch.nn.functional as F
        nsys = eps.numel()
        rnd = (lambda t: t.to(torch.bfloat16).float()) if bf16 else (lambda t: t)
        x = torch.stack([(r.view(nsys, n, n, n) * fac.view(nsys, 1, 1, 1)).float(),
                         eps.view(nsys, 1, 1, 1).expand(nsys, n, n, n).float()], 1)
        h = rnd(x)
        for l in range(4):
            h = F.conv3d(F.pad(h, (1, 1, 1, 1, 1, 1), mode='circular'), rnd(self.W[l].detach()),
                         self.b[l].detach())
            if l < 3:
                h = rnd(torch.relu(h))
        return h[:, 0].reshape(-1).double()
