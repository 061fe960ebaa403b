"""Bounded device-side waits.  Every wait in the tensor-core kernels gives up
after a limit, sets the device status word and returns instead of hanging.
Here one wait on a barrier that nothing completes (libconv_gb300_selftest_wait,
about 2 ms) gives up: the next libconv_gb300_check reports LIBCONV_ETIMEOUT
with its message and clears the word, the check after it is clean, and the
same context still computes a 3D kinetic operator that matches the oracle.
No fault, trap or hang is involved."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ETIMEOUT = -7


def test_timed_out_wait_is_reported_and_the_context_keeps_working(pkg, O):
    L = pkg.lib()
    L.libconv_gb300_selftest_wait.argtypes = [ctypes.c_int, ctypes.c_void_p]
    L.libconv_gb300_check.argtypes = [ctypes.c_void_p]
    assert L.libconv_gb300_check(None) == 0
    assert L.libconv_gb300_selftest_wait(2000, None) == 0
    assert L.libconv_gb300_check(None) == ETIMEOUT
    assert 'timed out' in pkg.last_error()
    assert L.libconv_gb300_check(None) == 0
    assert L.libconv_gb300_selftest_wait(0, None) != 0          # argument checked on the host
    n = [20, 18, 22]
    N = int(np.prod(n))
    x = np.random.default_rng(3).uniform(-1.0, 1.0, N)
    a = [-1.1, -0.9, -1.3]
    yg, yo, w = np.zeros(N), np.zeros(N), np.zeros(N)
    with pkg.mode(pkg.MODE_TC_EXACT):
        pkg.Kernel('d_kin').run(3, n, [0, 0, 0], x, yg, w, w, a, 0.0, 0.0)
    assert O.call('oracle_d_kin', 3, n, [0, 0, 0], x, yo, np.zeros(N), np.zeros(N), np.array(a), 0.0, 0.0) == 0
    assert np.abs(yg - yo).max() <= 1e-13 * np.abs(yo).max()
    assert L.libconv_gb300_check(None) == 0
