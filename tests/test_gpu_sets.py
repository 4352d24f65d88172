"""Parameter sets that share one contraction (ephg_el_rates_sets) and the
serving loop's merged runs.

Requests that differ only in T, sigma and chempot have the same vertices and
|g|^2 (interactions.f90:2095-2400 reads neither); only the occupation and
delta factors of the rate sum (interactions.f90:2958-3063) change.  The library
runs the contractions once and the rate epilogue once per set, with the same
per-vertex factors as a lone request, so each set's rates must equal those of
its request run alone through ephg_el_rates: the bar is 1e-13 relative per
rate, bit-identical expected.  The FP64 and generic split paths run the same
epilogue kernels per set; the fused nw 8 / nb 6 kernel forms the other sets'
factors in its own loop from |g|^2 formed once, with every FP32 rounding of
the vertex factors explicit (no FMA contraction left to the compiler) and dn
formed the same way as for a lone request.  Covered: the fused nw 8 / nb 6 kernel
(non-polar and polar), the generic split path (nw 5 / nb 9 and nw 16), the
triangle delta, and FP64; the server merges queued requests of one crystal and
mesh and returns each its own rates.
"""
import numpy as np
import pytest

from elphbolt_gb300 import _lib
from elphbolt_gb300 import synthetic as S

from cases import case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    pytest.importorskip("torch")
    from elphbolt_gb300.build import build
    build()


def variants(req, n=3):
    """n requests equal to req but for T, sigma and chempot."""
    out = []
    for T, sig, dmu in [(300.0, 0.010, 0.0), (150.0, 0.020, 0.05), (600.0, 0.005, -0.10), (77.0, 0.015, 0.02)][:n]:
        out.append(S.RateRequest(mesh=req.mesh, enref=req.enref, fsthick=req.fsthick, chempot=req.chempot + dmu,
                                 T=T, delta_kind=req.delta_kind, sigma=sig))
    return out


def check_sets(W, reqs, precision, tol=1e-13):
    got = W.el_rates_sets(reqs, precision=precision)
    worst = 0.0
    for r, g in zip(reqs, got):
        ref = W.el_rates(r, precision=precision)
        assert np.array_equal(g["indexlist"], ref["indexlist"])
        a, b = g["rates"], ref["rates"]
        assert a.shape == b.shape
        nz = np.abs(b) > 0
        assert np.array_equal(a == 0, b == 0)
        rel = float(np.max(np.abs(a[nz] - b[nz]) / np.abs(b[nz]))) if nz.any() else 0.0
        worst = max(worst, rel)
    assert worst <= tol, worst
    # the sets really differ: set 1's rates are not set 0's
    assert not np.allclose(got[0]["rates"], got[1]["rates"], rtol=1e-3)


@pytest.mark.parametrize("name", ["si8", "sic", "odd"])
@pytest.mark.parametrize("precision", [_lib.PREC_SPLIT_TF32, _lib.PREC_FP64])
def test_sets_equal_lone_requests(name, precision):
    from elphbolt_gb300.wannier import Wannier
    wd, req = case(name)
    W = Wannier(wd)   # sic: a polar crystal, the long-range terms on
    try:
        check_sets(W, variants(req), precision)
    finally:
        W.deallocate_wannier()


def test_sets_fused_multi_tile_and_generic_nw16():
    """12^3 on the 6^3-WS bench crystal (many fused tiles, both m-bands of the
    walk at larger meshes use the same code) and an nw 16 crystal (generic GEMM
    + row epilogue), eight sets."""
    from elphbolt_gb300.wannier import Wannier
    for wd, mesh in [(S.si_like(), (12, 12, 12)),
                     (S.make_wannier(S.make_crystal_si_like(), 16, supercell=(3, 3, 3), seed=21), (8, 8, 8))]:
        W = Wannier(wd)
        try:
            base = S.si_like_request(wd, mesh)
            reqs = variants(base, 4)
            reqs += [S.RateRequest(mesh=base.mesh, enref=base.enref, fsthick=base.fsthick, chempot=base.chempot,
                                   T=T, delta_kind=0, sigma=0.010) for T in (50.0, 200.0, 400.0, 900.0)]
            check_sets(W, reqs, _lib.PREC_SPLIT_TF32)
        finally:
            W.deallocate_wannier()


def test_sets_triangle_delta():
    from elphbolt_gb300.wannier import Wannier
    wd, req = case("si8")
    W = Wannier(wd)
    try:
        tri = S.RateRequest(mesh=req.mesh, enref=req.enref, fsthick=req.fsthick, chempot=req.chempot, T=req.T,
                            delta_kind=1, sigma=req.sigma)
        check_sets(W, variants(tri), _lib.PREC_SPLIT_TF32)
    finally:
        W.deallocate_wannier()


def test_sets_refuse_mismatched_requests():
    from elphbolt_gb300.wannier import Wannier
    wd, req = case("si8")
    W = Wannier(wd)
    try:
        a, b = variants(req, 2)
        bad = S.RateRequest(mesh=(4, 4, 4), enref=b.enref, fsthick=b.fsthick, chempot=b.chempot, T=b.T,
                            delta_kind=0, sigma=b.sigma)
        with pytest.raises(_lib.EphgError) as e:
            W.el_rates_sets([a, bad])
        assert e.value.code == _lib.EPHG_ERR_ARG
        with pytest.raises(_lib.EphgError):
            W.el_rates_sets([a] * (_lib.MAX_SETS + 1))
    finally:
        W.deallocate_wannier()


def test_server_merges_queued_requests():
    """One slot: the first request starts alone, the others queue behind it and
    run as merged sets; every ticket gets the rates of its own request."""
    from elphbolt_gb300.serve import Server
    from elphbolt_gb300.wannier import Wannier
    wd = S.si_like()
    W = Wannier(wd)
    try:
        base = S.si_like_request(wd, (12, 12, 12))
        reqs = [base] + variants(base, 4)
        ref = [W.el_rates(r, precision=_lib.PREC_SPLIT_TF32)["rates"] for r in reqs]
        srv = Server([W], 64 << 30, nslots=1)
        try:
            tickets = [srv.submit(0, r) for r in reqs]
            outs = [srv.wait(t) for t in tickets]
            st = srv.stats()
        finally:
            srv.close()
        assert st["completed"] == len(reqs) and st["merged"] >= 2
        for o, r in zip(outs, ref):
            np.testing.assert_allclose(o["rates"], r, rtol=1e-13, atol=0)
    finally:
        W.deallocate_wannier()
