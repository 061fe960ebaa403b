"""Seeded synthetic inputs for the convolution workloads.

All streams come from SplitMix64 (Steele, Lea & Flood 2014), evaluated
vectorised in numpy so the same seed gives the same grid on any host.
No dataset is involved: the reference's own tests fill arrays with unseeded
uniform [0,1) numbers; here every workload is seeded and reproducible.
"""
import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, count, offset=0):
    """``count`` consecutive SplitMix64 outputs of stream ``seed``."""
    with np.errstate(over='ignore'):
        i = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed, count, lo=-1.0, hi=1.0, offset=0):
    """Uniform doubles in [lo, hi) with 53 random bits each."""
    u = (splitmix64(seed, count, offset) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return lo + (hi - lo) * u


def normal(seed, count):
    """Standard normal doubles by Box-Muller on two uniform streams."""
    m = (count + 1) // 2
    u1 = uniform(seed, m, 0.0, 1.0)
    u2 = uniform(seed, m, 0.0, 1.0, offset=m)
    r = np.sqrt(-2.0 * np.log1p(-u1))
    z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
    return z[:count]


def gaussian_kernel(sigma=2.0, half=8):
    t = np.arange(-half, half + 1, dtype=np.float64)
    k = np.exp(-0.5 * (t / sigma) ** 2)
    return k / k.sum()


def gaussian_filtered_noise(seed, shape, sigma=2.0):
    """N(0,1) white noise on a periodic grid of Fortran shape ``shape``,
    smoothed by a separable periodic Gaussian (sigma points, truncated at
    +-8 points, normalised to sum 1), rescaled to unit RMS.  Returned as a
    Fortran-ordered array of that shape."""
    g = normal(seed, int(np.prod(shape))).reshape(shape, order='F')
    k = gaussian_kernel(sigma)
    for ax in range(g.ndim):
        acc = np.zeros_like(g)
        for i, w in enumerate(k):
            acc += w * np.roll(g, i - 8, axis=ax)
        g = acc
    g /= np.sqrt(np.mean(g * g))
    return np.asfortranarray(g)


def orbital_dims(seed, count, lo=24, hi=72):
    """Per-orbital localisation-region sizes, each axis uniform in [lo, hi]."""
    z = splitmix64(seed, 3 * count)
    return (lo + (z % np.uint64(hi - lo + 1)).astype(np.int64)).reshape(count, 3)


def orbital(seed, dims, h=0.45, wlo=2.0, whi=6.0):
    """Centred Gaussian envelope exp(-r^2/2w^2) (w uniform in [wlo, whi] bohr,
    grid spacing h) times unit-RMS white noise, Fortran-ordered."""
    w = float(uniform(seed, 1, wlo, whi)[0])
    axes = [(np.arange(d) - (d - 1) / 2.0) * h for d in dims]
    r2 = axes[0][:, None, None] ** 2 + axes[1][None, :, None] ** 2 + axes[2][None, None, :] ** 2
    noise = normal(seed + 1, int(np.prod(dims))).reshape(dims, order='F')
    return np.asfortranarray(np.exp(-r2 / (2 * w * w)) * noise)
