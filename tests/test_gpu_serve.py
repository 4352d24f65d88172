"""The serving loop on the GPU: each result is the same alone (ephg_el_rates)
and in the mix (requests on two crystals running concurrently on three
slots); requests that cannot fit the HBM budget are refused."""
import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S
from tests.cases import case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def crystals():
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    ws = []
    for name in ("tiny", "si8"):
        wd, req = case(name)
        ws.append((Wannier(wd), req))
    yield ws
    for W, _ in ws:
        W.deallocate_wannier()


def test_served_results_match_direct_calls(crystals):
    from elphbolt_gb300.serve import Server
    reqs = []
    for c, (W, req) in enumerate(crystals):
        for T, prec in ((300.0, _lib.PREC_SPLIT_TF32), (150.0, _lib.PREC_SPLIT_TF32), (300.0, _lib.PREC_FP64)):
            reqs.append((c, S.RateRequest(**{**req.__dict__, "T": T}), prec))
    direct = [crystals[c][0].el_rates(r, precision=p) for c, r, p in reqs]
    srv = Server([W for W, _ in crystals], hbm_budget_bytes=64 << 30, nslots=3)
    try:
        tickets = [srv.submit(c, r, precision=p) for c, r, p in reqs]
        outs = [srv.wait(t) for t in tickets]
        st = srv.stats()
    finally:
        srv.close()
    for o, d in zip(outs, direct):
        assert np.array_equal(o["indexlist"], d["indexlist"])
        np.testing.assert_allclose(o["rates"], d["rates"], rtol=1e-12, atol=0)
        assert o["stats"]["vertices"] == d["vertices"]
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["rejected"] == 0
    assert st["vertices"] == sum(d["vertices"] for d in direct)
    assert 0 < st["p50_ms"] <= st["p99_ms"]


def test_budget_refuses_requests_that_cannot_fit(crystals):
    from elphbolt_gb300.serve import Server
    W, req = crystals[1]
    # budget = resident data + 1 MB: a 12^3 request's set-up arrays alone need more
    srv = Server([W], hbm_budget_bytes=W_resident(W) + (1 << 20))
    try:
        big = S.RateRequest(**{**req.__dict__, "mesh": (12, 12, 12)})
        with pytest.raises(_lib.EphgError) as e:
            srv.submit(0, big)
        assert e.value.code == _lib.EPHG_ERR_NOMEM
        assert srv.stats()["rejected"] == 1
    finally:
        srv.close()


def W_resident(W):
    """Smallest budget the server accepts for W (probe by creation)."""
    from elphbolt_gb300.serve import Server
    lo, hi = 0, 64 << 30
    while hi - lo > (1 << 20):
        mid = (lo + hi) // 2
        try:
            Server([W], hbm_budget_bytes=mid).close()
            hi = mid
        except _lib.EphgError:
            lo = mid
    return hi
