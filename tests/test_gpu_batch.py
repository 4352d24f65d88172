"""The batched form on the GPU (ephg_el_rates_batch): many requests on random
crystals of different shapes in one call, the split form's generic GEMMs of
the running requests in grouped launches.

- every result equals the same request run alone (ephg_el_rates), bit for bit:
  the kernels and the per-element arithmetic are the same, only the launches
  that carry the GEMMs differ;
- grouped and ungrouped batches agree bit for bit, and the grouped one ran
  GEMMs of several requests in one launch;
- the split results stay within 1e-6 of the FP64 oracle;
- a budget too small for the requests side by side sends some to run alone
  afterwards, with the same results;
- a request that fails (empty window) fails alone: the others complete.
"""
import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S

pytestmark = pytest.mark.gpu

# (nw, natoms, WS supercell): the fused nw = 8, nb = 6 shape and three generic ones
SMALL = [(8, 2, (4, 4, 4)), (16, 2, (4, 4, 4)), (8, 4, (4, 4, 4)), (16, 4, (4, 4, 4))]


@pytest.fixture(scope="module")
def workload():
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    wds, reqs = S.batch_workload(n_requests=12, mesh_range=(6, 9), window_range=(0.4, 1.0), seed=777,
                                 crystals=SMALL)
    Ws = [Wannier(wd) for wd in wds]
    yield wds, Ws, reqs
    for W in Ws:
        W.deallocate_wannier()


def _batch(Ws, reqs, **kw):
    from elphbolt_gb300.wannier import el_rates_batch
    return el_rates_batch([Ws[c] for c, _ in reqs], [r for _, r in reqs], **kw)


@pytest.mark.parametrize("prec", [_lib.PREC_SPLIT_TF32, _lib.PREC_FP64])
def test_batch_equals_requests_alone(workload, prec):
    wds, Ws, reqs = workload
    outs, bs, status = _batch(Ws, reqs, precision=prec, nslots=4)
    assert status == [0] * len(reqs) and bs["failed"] == 0
    for (c, r), o in zip(reqs, outs):
        a = Ws[c].el_rates(r, precision=prec)
        assert o["nwv"] == a["nwv"] and np.array_equal(o["indexlist"], a["indexlist"])
        assert o["vertices"] == a["vertices"]
        assert np.array_equal(o["rates"], a["rates"])
    assert bs["vertices"] == sum(o["vertices"] for o in outs)
    if prec == _lib.PREC_SPLIT_TF32:
        # the generic shapes' GEMMs met in grouped launches
        assert bs["group_launches"] > 0 and bs["max_group"] >= 2
        assert bs["group_problems"] > bs["group_launches"]
    else:
        assert bs["group_launches"] == 0


def test_grouped_equals_ungrouped(workload):
    wds, Ws, reqs = workload
    g, bg, _ = _batch(Ws, reqs, nslots=6, grouped=True)
    u, bu, _ = _batch(Ws, reqs, nslots=6, grouped=False)
    assert bu["group_launches"] == 0 and bg["group_launches"] > 0
    for a, b in zip(g, u):
        assert np.array_equal(a["rates"], b["rates"]) and np.array_equal(a["indexlist"], b["indexlist"])


def test_batch_split_vs_oracle(workload, oracle_lib):
    """Split form within 1e-6 relative of the FP64 oracle (rates), on one
    request of each crystal shape."""
    wds, Ws, reqs = workload
    outs, _, _ = _batch(Ws, reqs, nslots=4)
    seen = set()
    for (c, r), o in zip(reqs, outs):
        if c in seen:
            continue
        seen.add(c)
        ref = oracle_lib.Wannier(wds[c]).el_rates(r, nthreads=4, literal=False)
        assert np.array_equal(o["indexlist"], ref["indexlist"])
        err = np.abs(o["rates"] - ref["rates"])
        scale = np.abs(ref["rates"]).max()
        assert np.all(err <= 1e-6 * np.abs(ref["rates"]) + 1e-8 * scale), float(
            np.max(err / (np.abs(ref["rates"]) + 1e-300)))
    assert len(seen) == len(SMALL)


def test_budget_sends_requests_to_run_alone(workload):
    """Budgets up to 3 GB chunk the GEMM outputs at the 64 MB floor, so each
    request's workspace is the same alone and in the batch: a budget just above
    the largest one fits every request alone but not six side by side."""
    wds, Ws, reqs = workload
    alone = []
    for c, r in reqs:
        o, b, _ = _batch(Ws, [(c, r)], nslots=1, budget=3 << 30)
        alone.append((o[0], b["peak_workspace_bytes"]))
    budget = int(1.05 * max(p for _, p in alone))
    outs, bs, status = _batch(Ws, reqs, nslots=6, budget=budget)
    assert status == [0] * len(reqs)
    assert bs["retried_alone"] > 0 and bs["peak_workspace_bytes"] <= budget
    for i, ((a, _), o) in enumerate(zip(alone, outs)):
        d = np.abs(o["rates"] - a["rates"])
        assert np.array_equal(o["rates"], a["rates"]), (i, reqs[i][0], float(d.max()), int((d > 0).sum()), bs)


def test_failing_request_fails_alone(workload):
    wds, Ws, reqs = workload
    bad = S.RateRequest(**{**reqs[1][1].__dict__, "enref": 1e3})   # nothing within the window
    mix = list(reqs[:4]) + [(reqs[1][0], bad)] + list(reqs[4:6])
    outs, bs, status = _batch(Ws, mix, nslots=3, raise_on_error=False)
    assert status[4] == _lib.EPHG_ERR_EMPTY_WINDOW and outs[4] is None
    assert all(s == 0 for i, s in enumerate(status) if i != 4) and bs["failed"] == 1
    for (c, r), o in zip(mix[:4], outs[:4]):
        assert np.array_equal(o["rates"], Ws[c].el_rates(r, precision=_lib.PREC_SPLIT_TF32)["rates"])
    with pytest.raises(_lib.EphgError) as ei:
        _batch(Ws, mix, nslots=3)
    assert ei.value.code == _lib.EPHG_ERR_EMPTY_WINDOW
