"""GPU parity of the Poisson finite-difference operators (BigDFT/Poisson.rb)
against the oracle on the same seeded inputs, in the FP64 and tensor-core
exact modes.  Tolerance max|gpu - oracle| / max|oracle| <= 1e-13 (every
derivative is an FP64-accurate sweep), plus the reference test's absolute
epsilon 1e-10 (Poisson_test.rb:19) for div_u_i and cc at the reference's
own size, 256^3 with h = 0.1 and geocode 3.  rhores2 (a sum of squares over
the grid, summed in another order) relative 1e-12."""
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
def P(pkg):
    return pkg.Poisson()


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def rnd(seed, size):
    return np.random.default_rng(seed).uniform(0.0, 1.0, size)


H = np.array([0.1, 0.12, 0.09])


@pytest.mark.parametrize('nord', [2, 4, 6, 8, 16])
@pytest.mark.parametrize('bc', [0, -2])
@pytest.mark.parametrize('idim', [0, 1, 2])
def test_broker(P, O, nord, bc, idim):
    nn = [23, 19, 21]
    u = rnd(nord + idim, int(np.prod(nn)))
    du = P.broker(nord, idim, nn, bc, u, 7.5)
    do = np.zeros_like(u)
    assert O.call('oracle_poisson_broker', nord, idim, nn, bc, u, do, 7.5) == 0
    assert rel(du, do) <= TOL


def test_broker_short_periodic_line(P, O):
    """Periodic lines shorter than the 17-point stencil wrap (modulo)."""
    nn = [5, 7, 3]
    u = rnd(3, int(np.prod(nn)))
    for idim in range(3):
        du = P.broker(16, idim, nn, 0, u, 1.0)
        do = np.zeros_like(u)
        assert O.call('oracle_poisson_broker', 16, idim, nn, 0, u, do, 1.0) == 0
        assert rel(du, do) <= TOL


def test_broker_rejects(P, pkg):
    u = np.zeros(10 * 10 * 10)
    with pytest.raises(pkg.LibconvError) as e:
        P.broker(16, 0, [10, 10, 10], -2, u, 1.0)       # line shorter than 17 points
    assert e.value.status == -3
    with pytest.raises(pkg.LibconvError) as e:
        P.broker(10, 0, [10, 10, 10], 0, u, 1.0)        # no such order
    assert e.value.status == -1
    with pytest.raises(pkg.LibconvError) as e:
        P.broker(2, 0, [10, 10, 10], 1, u, 1.0)         # grow is not a Poisson boundary
    assert e.value.status == -2


@pytest.mark.parametrize('geocode', [1, 2, 3])
@pytest.mark.parametrize('nord', [4, 16])
def test_div_u_i(P, O, geocode, nord):
    n = [20, 18, 22]
    N = int(np.prod(n))
    u = rnd(geocode, 3 * N)
    du = P.div_u_i(geocode, n, u, nord, H)
    do = np.zeros(N)
    assert O.call('oracle_div_u_i', geocode, *n, u, do, nord, H, None) == 0
    assert rel(du, do) <= TOL
    du2, cc = P.div_u_i(geocode, n, u, nord, H, cc=True)
    do2, co = np.zeros(N), np.zeros(N)
    assert O.call('oracle_div_u_i', geocode, *n, u, do2, nord, H, co) == 0
    assert rel(du2, do2) <= TOL and rel(cc, co) <= TOL


@pytest.mark.parametrize('geocode', [1, 2, 3])
def test_nabla_family(P, O, geocode):
    n = [19, 20, 17]
    N = int(np.prod(n))
    u = rnd(10 + geocode, N)
    eps = rnd(20 + geocode, N) + 0.5
    du = P.nabla_u(geocode, n, u, 16, H)
    do = np.zeros(3 * N)
    assert O.call('oracle_nabla_u', geocode, *n, u, do, 16, H) == 0
    assert rel(du, do) <= TOL
    du2, ddu = P.nabla_u_and_square(geocode, n, u, 16, H)
    do2, ddo = np.zeros(3 * N), np.zeros(N)
    assert O.call('oracle_nabla_u_and_square', geocode, *n, u, do2, ddo, 16, H) == 0
    assert rel(du2, do2) <= TOL and rel(ddu, ddo) <= TOL
    assert rel(P.nabla_u_square(geocode, n, u, 16, H), ddo) <= TOL
    de = P.nabla_u_epsilon(geocode, n, u, 16, H, eps)
    deo = np.zeros(3 * N)
    assert O.call('oracle_nabla_u_epsilon', geocode, *n, u, deo, 16, H, eps) == 0
    assert rel(de, deo) <= TOL


@pytest.mark.parametrize('geocode', [1, 3])
def test_update_rhopol(P, O, geocode):
    """Poisson_test.rb:151-176 on a small grid: eta = 0.5, random dlogeps
    and u."""
    n = [18, 21, 19]
    N = int(np.prod(n))
    u = rnd(30, N)
    dl = rnd(31, 3 * N)
    rho0 = rnd(32, N)
    rg = rho0.copy()
    r2 = P.update_rhopol(geocode, n, u, 16, H, 0.5, dl, rg)
    ro = rho0.copy()
    r2o = np.zeros(1)
    assert O.call('oracle_update_rhopol', geocode, *n, u, 16, H, 0.5, dl, ro, r2o) == 0
    assert rel(rg, ro) <= TOL
    assert abs(r2 - r2o[0]) <= 1e-12 * r2o[0]


def test_div_u_i_reference_size(P, O):
    """The reference test's case (Poisson_test.rb:5-19, 79-112): 256^3,
    nord 16, h = 0.1, geocode 3 (y non-periodic), u random in [0, 1): du and
    cc against the oracle within the reference's epsilon 1e-10 and 1e-13
    relative."""
    n = [256, 256, 256]
    N = int(np.prod(n))
    h = np.array([0.1, 0.1, 0.1])
    u = rnd(256, 3 * N)
    du, cc = P.div_u_i(3, n, u, 16, h, cc=True)
    do, co = np.zeros(N), np.zeros(N)
    assert O.call('oracle_div_u_i', 3, *n, u, do, 16, h, co) == 0
    assert np.abs(du - do).max() <= 1e-10 and rel(du, do) <= TOL
    assert np.abs(cc - co).max() <= 1e-10 and rel(cc, co) <= TOL
