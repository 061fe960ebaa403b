"""Independent numpy restatements of the Fortran reference kernels, used to
pin the C oracle (vectorised with np.roll; different summation structure, so
agreement is to rounding, not bit-exact)."""
import numpy as np


def _f(name):
    import __graft_entry__ as ge
    ge.package()
    import importlib
    g = importlib.import_module('boast_lig_gb300.gen_filters')
    return np.array([float(v) for v in getattr(g, name)])


def mf_per(x, n, ndat, inverse=False):
    """magicfilter_per_ref / _per_t_ref (BigDFT/magicfilter_refs.f90:92-181)."""
    fil = _f('MF_FORTRAN')
    if inverse:
        fil, low = fil[::-1], -7
    else:
        low = -8
    X = x.reshape(ndat, n).T
    Y = sum(fil[k] * np.roll(X, -(k + low), axis=0) for k in range(16))
    return Y.T.copy().ravel(order='F')  # y(ndat, n) flat Fortran


def mf_free(x, n, ndat):
    """magicfilter_free_ref: grow to n+15 (BigDFT/magicfilter_refs.f90:2-44)."""
    fil = _f('MF_FORTRAN')
    X = x.reshape(ndat, n).T
    P = np.zeros((n + 30, ndat))
    P[15:15 + n] = X
    Y = np.zeros((n + 15, ndat))
    for i in range(-7, n + 8):
        for k in range(16):
            Y[i + 7] += fil[k] * P[15 + i + k - 8]
    return Y.ravel()  # rows are i: this is y(ndat, -7:n+7) in Fortran order


def kinetic_per(x, shape, hgrid, c):
    """kinetic_per_ref (BigDFT/Kinetic2.rb:981-1061)."""
    k = _f('KIN_FORTRAN')
    fil = np.concatenate([k[::-1], k[1:]])
    X = x.reshape(shape, order='F')
    Y = c * X
    for ax in range(3):
        s = -0.5 / hgrid[ax] ** 2
        Y = Y + sum(fil[j] * s * np.roll(X, -(j - 14), axis=ax) for j in range(29))
    return Y.ravel(order='F')


def synthesis_per(x, n, ndat):
    """synthesis_per_ref (BigDFT/old/Synthesis.rb:100-146)."""
    ch = np.concatenate([[0.0], _f('CH_FORTRAN'), [0.0]])   # -8..9
    cg = np.concatenate([[0.0], _f('CG_FORTRAN'), [0.0]])
    X = x.reshape(ndat, 2 * n).T
    s, d = X[:n], X[n:]
    Y = np.zeros((2 * n, ndat))
    for l in range(-4, 5):
        Y[0::2] += ch[2 * l + 8] * np.roll(s, l, axis=0) + cg[2 * l + 8] * np.roll(d, l, axis=0)
        Y[1::2] += ch[2 * l + 9] * np.roll(s, l, axis=0) + cg[2 * l + 9] * np.roll(d, l, axis=0)
    return Y.ravel()


def analysis_per(x, n, ndat):
    """analysis_per_ref, plain form (BigDFT/old/AnaRotPer-2.rb:258-296)."""
    ch, cg = _f('CH_FORTRAN'), _f('CG_FORTRAN')
    X = x.reshape(ndat, 2 * n).T
    Y = np.zeros((2 * n, ndat))
    for l in range(-7, 9):
        R = np.roll(X, -l, axis=0)[0::2]
        Y[:n] += ch[l + 7] * R
        Y[n:] += cg[l + 7] * R
    return Y.ravel()
