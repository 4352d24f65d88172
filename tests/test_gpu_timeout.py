"""Failure detection on the device without a fault: a bounded wait that runs out.

Every barrier wait in the tcgen05 kernels gives up after a bound, records
DERR_TIMEOUT in the launch's error word, lets the MMAs already issued retire,
frees TMEM and returns; the entry point then returns EPHG_ERR_TIMEOUT.  The
hook ephg_debug_wait_timeout runs that give-up path on its own -- a barrier
nothing arrives on, a short limit, no TMA load or MMA issued -- and this test
checks the status it reports, that a wait that is satisfied reports none, and
that the context is still usable afterwards (a 3xTF32 GEMM against numpy).
"""
import ctypes as ct
import time

import numpy as np
import pytest

from elphbolt_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from elphbolt_gb300.build import build
    build()
    lib = _lib.load()
    lib.ephg_debug_wait_timeout.argtypes = [ct.c_int64, ct.c_int64, ct.POINTER(ct.c_int)]
    lib.ephg_debug_cgemm.argtypes = [ct.c_int64, ct.c_int64, ct.c_int64, _lib.c_dp, _lib.c_dp, _lib.c_dp]
    lib.ephg_debug_last_error.restype = ct.c_char_p
    return lib


def test_wait_that_runs_out_reports_timeout(L):
    err = ct.c_int(-1)
    t0 = time.time()
    rc = L.ephg_debug_wait_timeout(200_000, 0, ct.byref(err))    # ~0.1 ms at 2 GHz
    dt = time.time() - t0
    assert rc == _lib.EPHG_ERR_TIMEOUT
    assert err.value & 8                                          # DERR_TIMEOUT
    assert dt < 5.0


def test_wait_that_is_satisfied_reports_nothing(L):
    err = ct.c_int(-1)
    assert L.ephg_debug_wait_timeout(200_000, 1, ct.byref(err)) == _lib.EPHG_OK
    assert err.value == 0


def test_context_usable_after_timeout(L):
    err = ct.c_int(0)
    assert L.ephg_debug_wait_timeout(0, 0, ct.byref(err)) == _lib.EPHG_ERR_TIMEOUT
    rng = np.random.default_rng(5)
    M, N, K = 130, 70, 40
    A = rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K))
    B = rng.normal(size=(K, N)) + 1j * rng.normal(size=(K, N))
    C = np.zeros((M, N), dtype=np.complex128)
    dp = lambda a: a.ctypes.data_as(ct.POINTER(ct.c_double))
    assert L.ephg_debug_cgemm(M, N, K, dp(A), dp(B), dp(C)) == 0, L.ephg_debug_last_error()
    ref = A @ B
    assert np.max(np.abs(C - ref)) <= 1e-5 * np.abs(ref).max()


def test_limit_out_of_range_refused(L):
    assert L.ephg_debug_wait_timeout(-1, 0, None) == _lib.EPHG_ERR_ARG
