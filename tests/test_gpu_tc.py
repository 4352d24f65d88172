"""The 3xTF32 tcgen05 complex GEMM and the split-precision rate path.

Tolerances (split form): GEMM normwise relative error <= 1e-5 against the
complex128 product (FP32 accumulation over K ~ 300 complex terms dominates:
sqrt(6K) * 2^-24 ~ 2.5e-6 typical); |g|^2 per vertex |a-b| <= 1e-5 |b| + 1e-6 max|b|; RTA rates
<= 1e-6 relative per state (the split form's stated bound).
"""
import ctypes as ct

import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S
from tests.cases import case, CASES

pytestmark = pytest.mark.gpu


def cgemm(A, B):
    L = _lib.load()
    L.ephg_debug_cgemm.argtypes = [ct.c_int64, ct.c_int64, ct.c_int64, _lib.c_dp, _lib.c_dp, _lib.c_dp]
    L.ephg_debug_last_error.restype = ct.c_char_p
    M, K = A.shape
    N = B.shape[1]
    a = np.ascontiguousarray(A, dtype=np.complex128)
    b = np.ascontiguousarray(B, dtype=np.complex128)
    c = np.zeros((M, N), dtype=np.complex128)
    rc = L.ephg_debug_cgemm(M, N, K, a.ctypes.data_as(_lib.c_dp), b.ctypes.data_as(_lib.c_dp),
                            c.ctypes.data_as(_lib.c_dp))
    assert rc == 0, L.ephg_debug_last_error()
    return c


@pytest.fixture(scope="module", autouse=True)
def built():
    from elphbolt_gb300.build import build
    build()


@pytest.mark.parametrize("M,N,K", [(128, 128, 16), (200, 300, 279), (77, 1000, 5), (2048, 2304, 600)])
def test_cgemm_vs_fp64(M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))
    B = rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))
    ref = A @ B
    got = cgemm(A, B)
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err <= 1e-5, err
    # elementwise against the scale of each dot product
    scale = np.sqrt(np.abs(A) ** 2 @ np.abs(B) ** 2)
    assert np.max(np.abs(got - ref) / scale) <= 5e-5


def test_cgemm_phases():
    """Unit-modulus phase rows against decaying data: the shape of both contractions."""
    rng = np.random.default_rng(5)
    M, K, N = 300, 279, 384
    A = np.exp(2j * np.pi * rng.uniform(0, 1, (M, K)))
    B = (rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))) * np.exp(-rng.uniform(0, 5, (K, 1)))
    ref = A @ B
    got = cgemm(A, B)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-5


@pytest.mark.parametrize("name", CASES)
def test_el_rates_split_vs_oracle(oracle_lib, name):
    from elphbolt_gb300.wannier import Wannier
    wd, req = case(name)
    o = oracle_lib.Wannier(wd).el_rates(req, literal=True, vertices=True)
    W = Wannier(wd)
    g = W.el_rates(req, precision=_lib.PREC_SPLIT_TF32, vertices=True)
    W.deallocate_wannier()
    assert g["nwv"] == o["nwv"] and np.array_equal(g["indexlist"], o["indexlist"])
    assert g["vertices"] == o["vertices"]
    scale = np.abs(o["g2"]).max()
    assert np.all(np.abs(g["g2"] - o["g2"]) <= 1e-5 * np.abs(o["g2"]) + 1e-6 * scale)
    r, ro = g["rates"], o["rates"]
    mask = ro > 0
    rel = np.abs(r - ro)[mask] / ro[mask]
    assert rel.max() <= 1e-6, rel.max()
    assert np.all(r[~mask] == 0)


@pytest.mark.parametrize("delta", [1, 2])
def test_el_rates_split_simplex_deltas(oracle_lib, delta):
    from elphbolt_gb300.wannier import Wannier
    wd, req0 = case("si8")
    req = S.RateRequest(**{**req0.__dict__, "delta_kind": delta})
    o = oracle_lib.Wannier(wd).el_rates(req, literal=False)
    W = Wannier(wd)
    g = W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)
    W.deallocate_wannier()
    mask = o["rates"] > 1e-8 * o["rates"].max()
    rel = np.abs(g["rates"] - o["rates"])[mask] / o["rates"][mask]
    assert rel.max() <= 1e-6, rel.max()


def test_el_rates_split_many_window_bands(oracle_lib):
    """A window of +-3 eV holds 4 to 8 of the 8 bands at every k': the fused
    stage-B epilogue's path for more than two window bands per k' row."""
    from elphbolt_gb300.wannier import Wannier
    wd = S.make_wannier(S.make_crystal_si_like(), 8, supercell=(3, 3, 3), seed=12)
    req = S.si_like_request(wd, (4, 4, 4), window=3.0, shift=0.0)
    o = oracle_lib.Wannier(wd).el_rates(req, literal=True, vertices=True)
    W = Wannier(wd)
    g = W.el_rates(req, precision=_lib.PREC_SPLIT_TF32, vertices=True)
    W.deallocate_wannier()
    assert np.array_equal(g["indexlist"], o["indexlist"]) and g["vertices"] == o["vertices"]
    scale = np.abs(o["g2"]).max()
    assert np.all(np.abs(g["g2"] - o["g2"]) <= 1e-5 * np.abs(o["g2"]) + 1e-6 * scale)
    mask = o["rates"] > 0
    rel = np.abs(g["rates"] - o["rates"])[mask] / o["rates"][mask]
    assert rel.max() <= 1e-6, rel.max()


def test_el_rates_split_vs_fp64_multi_tile():
    """12^3 Si-like request (1,441 window k' rows: 12 row tiles, ~800 state-pair
    tiles): the split form against the library's FP64 form, which the oracle
    pins on the small cases; rates within 1e-6 relative."""
    from elphbolt_gb300.wannier import Wannier
    wd = S.si_like(nw=8)
    req = S.si_like_request(wd, (12, 12, 12))
    W = Wannier(wd)
    d = W.el_rates(req, precision=_lib.PREC_FP64)
    g = W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)
    W.deallocate_wannier()
    assert g["nwv"] > 1024 and np.array_equal(g["indexlist"], d["indexlist"])
    mask = d["rates"] > 0
    rel = np.abs(g["rates"] - d["rates"])[mask] / d["rates"][mask]
    assert rel.max() <= 1e-6, rel.max()
    assert np.all(g["rates"][~mask] == 0)


@pytest.mark.parametrize("nw,natoms", [(24, 2), (32, 2), (32, 4), (32, 6)])
def test_el_rates_wide_bands_vs_oracle(oracle_lib, nw, natoms):
    """Wide band sets (nw 24 and 32, nb 6, 12 and 18 -- the large instance's
    nw 32 / nb 18 shape) through the generic split
    path (stage-A rotation tiled over modes, the per-row epilogue of that nw)
    and the FP64 form, against the oracle: rates within 1e-6 (split) and 1e-10
    (FP64) relative."""
    from elphbolt_gb300.wannier import Wannier
    rng = np.random.default_rng(100 + nw + natoms)
    wd = S.make_wannier(S.make_crystal_multi(natoms, rng), nw, supercell=(2, 2, 2), seed=300 + nw + natoms)
    req = S.si_like_request(wd, (4, 4, 4), window=0.5, shift=0.6)
    o = oracle_lib.Wannier(wd).el_rates(req, nthreads=4, literal=False)
    W = Wannier(wd)
    try:
        outs = {p: W.el_rates(req, precision=p) for p in (_lib.PREC_SPLIT_TF32, _lib.PREC_FP64)}
    finally:
        W.deallocate_wannier()
    scale = np.abs(o["rates"]).max()
    for p, tol, floor in ((_lib.PREC_SPLIT_TF32, 1e-6, 1e-8), (_lib.PREC_FP64, 1e-10, 1e-14)):
        g = outs[p]
        assert np.array_equal(g["indexlist"], o["indexlist"]) and g["vertices"] == o["vertices"]
        err = np.abs(g["rates"] - o["rates"])
        assert np.all(err <= tol * np.abs(o["rates"]) + floor * scale), (p, float(err.max() / scale))
