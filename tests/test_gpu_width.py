"""The generic split-form GEMM's two tile widths and its autotuner.

128-column tiles use one set of TMEM accumulators; 64-column tiles two, so
that a tile's MMAs overlap the previous tile's drain.  Every output element is
the same chain of MMAs at either width, so the results must agree bit for bit:
- the GEMM alone (ephg_debug_cgemm) at each forced width, and against numpy
  (the 3xTF32 bound of test_gpu_tc);
- a generic-shape rate request (nw 16, nb 6) at each width and autotuned;
- a small batch with grouped launches at each width.
The autotuner records a decision per problem class it timed.
"""
import ctypes as ct

import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from elphbolt_gb300.build import build
    build()
    lib = _lib.load()
    lib.ephg_debug_set_gemm_width.argtypes = [ct.c_int64]
    lib.ephg_debug_gemm_widths.argtypes = [ct.POINTER(ct.c_int64)] * 2 + [ct.POINTER(ct.c_double)] * 2
    lib.ephg_debug_cgemm.argtypes = [ct.c_int64, ct.c_int64, ct.c_int64, _lib.c_dp, _lib.c_dp, _lib.c_dp]
    lib.ephg_debug_last_error.restype = ct.c_char_p
    yield lib
    lib.ephg_debug_set_gemm_width(0)


def gemm(L, A, B):
    M, K = A.shape
    N = B.shape[1]
    a, b = np.ascontiguousarray(A), np.ascontiguousarray(B)
    c = np.zeros((M, N), dtype=np.complex128)
    dp = lambda x: x.ctypes.data_as(_lib.c_dp)
    assert L.ephg_debug_cgemm(M, N, K, dp(a), dp(b), dp(c)) == 0, L.ephg_debug_last_error()
    return c


@pytest.mark.parametrize("M,N,K", [(300, 200, 50), (130, 520, 279)])
def test_gemm_widths_bitwise(L, M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K))
    B = rng.normal(size=(K, N)) + 1j * rng.normal(size=(K, N))
    out = {}
    for w in (128, 64):
        assert L.ephg_debug_set_gemm_width(w) == 0
        out[w] = gemm(L, A, B)
    L.ephg_debug_set_gemm_width(0)
    assert np.array_equal(out[128], out[64])
    ref = A @ B
    scale = np.abs(A).max() * np.abs(B).max() * K
    assert np.max(np.abs(out[64] - ref)) <= 1e-6 * scale


def test_rates_widths_bitwise(L):
    from elphbolt_gb300.wannier import Wannier
    wd = S.make_wannier(S.make_crystal_si_like(), 16, supercell=(3, 3, 3), seed=41)
    req = S.si_like_request(wd, (6, 6, 6), window=0.5, shift=0.6)
    W = Wannier(wd)
    try:
        out = {}
        for w in (128, 64, 0):
            assert L.ephg_debug_set_gemm_width(w) == 0
            out[w] = W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)
        L.ephg_debug_set_gemm_width(0)
    finally:
        W.deallocate_wannier()
    assert out[128]["vertices"] > 0
    assert np.array_equal(out[128]["rates"], out[64]["rates"])
    assert np.array_equal(out[128]["rates"], out[0]["rates"])
    n128, n64 = ct.c_int64(), ct.c_int64()
    ms128, ms64 = ct.c_double(), ct.c_double()
    L.ephg_debug_gemm_widths(ct.byref(n128), ct.byref(n64), ct.byref(ms128), ct.byref(ms64))
    assert n128.value + n64.value >= 1 and ms128.value > 0 and ms64.value > 0


def test_batch_widths_bitwise(L):
    from elphbolt_gb300.wannier import Wannier, el_rates_batch
    specs = [(8, 4, (3, 3, 3)), (16, 2, (3, 3, 3))]
    wds, reqs = S.batch_workload(n_requests=6, mesh_range=(5, 7), crystals=specs)
    Ws = [Wannier(w) for w in wds]
    try:
        res = {}
        for w in (128, 64):
            assert L.ephg_debug_set_gemm_width(w) == 0
            res[w] = el_rates_batch([Ws[c] for c, _ in reqs], [r for _, r in reqs], nslots=3)[0]
        L.ephg_debug_set_gemm_width(0)
    finally:
        for W in Ws:
            W.deallocate_wannier()
    for a, b in zip(res[128], res[64]):
        assert np.array_equal(a["rates"], b["rates"])
