"""GPU parity of the local Hamiltonian (libconv_hamiltonian, the pipeline of
BigDFT/libconv.f90:248-294) against the oracle composition on the same
seeded inputs, in the FP64 and the tensor-core exact modes.

Tolerances: hpsig and rho max|gpu - oracle| / max|oracle| <= 1e-13 (every
step is an FP64-accurate sweep; they differ from the oracle by rounding
only); the energies (sums over up to 10^6 products, summed in another
order) relative 1e-12.  At the full size the oracle is too slow, so the
size-independent properties of the operator are checked instead:
<psig|H psig> = sum ekin + epot, <phi|H psi> = <H phi|psi>, linearity."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13
ETOL = 1e-12


@pytest.fixture(autouse=True, params=['fp64', 'tc_exact'])
def compute_mode(request, pkg):
    m = pkg.MODE_FP64 if request.param == 'fp64' else pkg.MODE_TC_EXACT
    with pkg.mode(m):
        yield request.param


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def inputs_for(pkg, n, bc, seed):
    nsig, nreal, _ = pkg.hamiltonian_sizes(n, bc)
    rng = np.random.default_rng(seed)
    psig = rng.standard_normal(nsig)
    pot = rng.uniform(-1.0, 2.0, nreal)
    rho = rng.uniform(0.0, 1.0, nreal)
    return psig, pot, rho


def oracle_ham(O, n, bc, a, psig, pot, rho):
    hpsig, ek, ep = np.zeros(psig.size), np.zeros(3), np.zeros(1)
    assert O.call('oracle_hamiltonian', n, bc, np.array(a), psig, pot, rho, hpsig, ek, ep) == 0
    return hpsig, ek, ep[0]


@pytest.mark.parametrize('n,bc', [
    ([6, 5, 7], [2, 2, 2]),     # free: grow / shrink in every step
    ([8, 6, 5], [0, 0, 0]),     # periodic
    ([7, 6, 8], [2, 0, 2]),     # surface (periodic y)
    ([4, 9, 3], [0, 2, 0]),     # wire
])
def test_hamiltonian_matches_oracle(pkg, O, n, bc):
    a = [-0.5 / 0.45 ** 2, -0.5 / 0.4 ** 2, -0.5 / 0.5 ** 2]
    psig, pot, rho0 = inputs_for(pkg, n, bc, 7)
    rg = rho0.copy()
    hg, eg, pg = pkg.hamiltonian(n, bc, a, psig, pot, rg)
    ro = rho0.copy()
    ho, eo, po = oracle_ham(O, n, bc, a, psig, pot, ro)
    assert rel(hg, ho) <= TOL
    assert rel(rg, ro) <= TOL
    assert np.abs(eg - eo).max() <= ETOL * np.abs(eo).max(), (eg, eo)
    assert abs(pg - po) <= ETOL * np.abs(pot).max() * float(np.abs(rg - rho0).sum()), (pg, po)


def test_hamiltonian_without_density(pkg, O):
    n, bc = [5, 6, 5], [2, 2, 2]
    a = [-1.1, -0.9, -1.4]
    psig, pot, _ = inputs_for(pkg, n, bc, 8)
    hg, eg, pg = pkg.hamiltonian(n, bc, a, psig, pot)
    ho, eo, po = oracle_ham(O, n, bc, a, psig, pot, None)
    assert rel(hg, ho) <= TOL
    assert np.abs(eg - eo).max() <= ETOL * np.abs(eo).max()


def test_hamiltonian_device_entry(pkg, O):
    """libconv_hamiltonian_dev on a side stream with the workspace of
    libconv_hamiltonian_sizes: same results as the oracle, rho updated on
    the device, energies left on the device."""
    import torch
    n, bc = [6, 7, 5], [2, 0, 2]
    a = [-2.0, -1.5, -2.5]
    psig, pot, rho0 = inputs_for(pkg, n, bc, 9)
    H = pkg.Hamiltonian(n, bc, a)
    dpsig, dpot, drho = (torch.from_numpy(v).cuda() for v in (psig, pot, rho0))
    dh = torch.zeros_like(dpsig)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        en = H(dpsig, dpot, dh, drho, stream=s)
    s.synchronize()
    pkg.check(s)
    ro = rho0.copy()
    ho, eo, po = oracle_ham(O, n, bc, a, psig, pot, ro)
    assert rel(dh.cpu().numpy(), ho) <= TOL
    assert rel(drho.cpu().numpy(), ro) <= TOL
    e = en.cpu().numpy().ravel()
    assert np.abs(e[:3] - eo).max() <= ETOL * np.abs(eo).max()
    assert abs(e[3] - po) <= ETOL * np.abs(pot).max() * float(np.abs(ro - rho0).sum())


@pytest.mark.parametrize('n,bc,norb', [
    ([6, 5, 7], [2, 2, 2], 3),    # few tiles per orbital: CTAs skip orbitals
    ([8, 8, 6], [0, 0, 0], 4),
    ([7, 4, 9], [2, 0, 2], 2),
])
def test_hamiltonian_narr_matches_single_orbitals(pkg, O, n, bc, norb):
    """norb orbitals in one call: hpsig of every orbital bit-identical to the
    single-orbital call (same sweeps, only batched), rho bit-identical to
    the single-orbital calls made in order, per-orbital energies as the
    oracle's."""
    a = [-1.7, -2.2, -0.9]
    nsig, nreal, _ = pkg.hamiltonian_sizes(n, bc)
    rng = np.random.default_rng(21)
    psig = rng.standard_normal(norb * nsig) * np.repeat(1.0 + np.arange(norb), nsig)
    pot = rng.uniform(-1.0, 2.0, nreal)
    rho0 = rng.uniform(0.0, 1.0, nreal)
    rb = rho0.copy()
    hb, eb = pkg.hamiltonian_narr(n, bc, a, norb, psig, pot, rb)
    assert eb.shape == (norb, 4)
    rs, ro = rho0.copy(), rho0.copy()
    for j in range(norb):
        sl = slice(j * nsig, (j + 1) * nsig)
        hs, es, ps = pkg.hamiltonian(n, bc, a, psig[sl], pot, rs)
        assert np.array_equal(hb[sl], hs), j
        ho, eo, po = oracle_ham(O, n, bc, a, psig[sl].copy(), pot, ro)
        assert rel(hb[sl], ho) <= TOL
        assert np.abs(eb[j, :3] - eo).max() <= ETOL * np.abs(eo).max(), (j, eb[j], eo)
        assert abs(eb[j, 3] - po) <= ETOL * 2 * float(psig[sl] @ psig[sl]) * np.abs(pot).max()
    assert np.array_equal(rb, rs)
    assert rel(rb, ro) <= TOL


def test_hamiltonian_narr_device_entry(pkg, O):
    import torch
    n, bc, norb = [5, 6, 5], [2, 2, 2], 5
    a = [-1.0, -1.2, -1.4]
    nsig, nreal, _ = pkg.hamiltonian_sizes(n, bc)
    rng = np.random.default_rng(22)
    psig, pot = rng.standard_normal(norb * nsig), rng.uniform(0.1, 1.0, nreal)
    H = pkg.Hamiltonian(n, bc, a, norb=norb)
    dpsig, dpot = torch.from_numpy(psig).cuda(), torch.from_numpy(pot).cuda()
    dh = torch.zeros_like(dpsig)
    en = H(dpsig, dpot, dh)
    torch.cuda.synchronize()
    pkg.check()
    e = en.cpu().numpy()
    for j in range(norb):
        sl = slice(j * nsig, (j + 1) * nsig)
        ho, eo, po = oracle_ham(O, n, bc, a, psig[sl].copy(), pot, None)
        assert rel(dh[sl].cpu().numpy(), ho) <= TOL
        assert np.abs(e[j, :3] - eo).max() <= ETOL * np.abs(eo).max()
        assert abs(e[j, 3] - po) <= ETOL * abs(po)


def test_hamiltonian_repeated_calls_identical(pkg):
    """Two calls in a row give the same bits (deterministic reductions)."""
    n, bc = [7, 7, 7], [2, 2, 2]
    psig, pot, _ = inputs_for(pkg, n, bc, 10)
    h1, e1, p1 = pkg.hamiltonian(n, bc, [-1.0] * 3, psig, pot)
    h2, e2, p2 = pkg.hamiltonian(n, bc, [-1.0] * 3, psig, pot)
    assert np.array_equal(h1, h2) and np.array_equal(e1, e2) and p1 == p2


@pytest.mark.parametrize('bc', [[2, 2, 2], [0, 0, 0]])
def test_hamiltonian_full_size_properties(pkg, bc):
    """48^3 coarse points (96^3 wavelet coefficients; free: 110^3 fine and
    125^3 real-space points): self-adjointness, the energy identity and
    linearity, on the device."""
    import torch
    n = [48, 48, 48]
    a = [-0.5 / 0.4 ** 2] * 3
    nsig, nreal, _ = pkg.hamiltonian_sizes(n, bc)
    g = torch.Generator(device='cuda').manual_seed(11)
    psi = torch.randn(nsig, generator=g, device='cuda', dtype=torch.float64)
    phi = torch.randn(nsig, generator=g, device='cuda', dtype=torch.float64)
    pot = torch.rand(nreal, generator=g, device='cuda', dtype=torch.float64) * 3.0 - 1.0
    H = pkg.Hamiltonian(n, bc, a)

    def apply(x):
        y = torch.empty_like(x)
        e = H(x, pot, y).clone()
        return y, e

    hpsi, e = apply(psi)
    hphi, _ = apply(phi)
    torch.cuda.synchronize()
    pkg.check()
    scale = float(psi.abs().sum() * hpsi.abs().max())
    assert abs(float(psi @ hpsi) - float(e.sum())) <= 1e-13 * scale
    assert abs(float(phi @ hpsi) - float(hphi @ psi)) <= 1e-13 * scale
    comb, _ = apply(2.5 * psi - phi)
    torch.cuda.synchronize()
    assert float((comb - (2.5 * hpsi - hphi)).abs().max()) <= 1e-13 * float(comb.abs().max())


def test_hamiltonian_argument_errors(pkg):
    import torch
    with pytest.raises(pkg.LibconvError) as e:
        pkg.hamiltonian([4, 4, 4], [1, 1, 1], [-1.0] * 3, np.zeros(512), np.zeros(512))
    assert e.value.status == -2
    H = pkg.Hamiltonian([4, 4, 4], [0, 0, 0], [-1.0] * 3)
    x = torch.zeros(512, dtype=torch.float64, device='cuda')
    with pytest.raises(ValueError):
        H(x, torch.zeros(100, dtype=torch.float64, device='cuda'), x.clone())
    L = pkg._ham_lib()
    st = L.libconv_hamiltonian_dev(pkg._ints([4, 4, 4]), pkg._ints([0, 0, 0]),
                                   pkg._dbls([-1.0] * 3), None, None, None, None, None, None,
                                   None)
    assert st == -1
