"""The batched workload (synthetic.batch_workload) on the CPU: seeded and
reproducible, the shapes it promises, and every request's window non-empty
(the oracle's el_wann over the request's mesh), so that a batch run fails on
nothing but the device."""
import numpy as np
import pytest

from elphbolt_gb300 import synthetic as S

SMALL = [(8, 2, (4, 4, 4)), (16, 2, (4, 4, 4)), (8, 4, (4, 4, 4)), (16, 4, (4, 4, 4))]


def test_batch_workload_is_seeded():
    a_w, a_r = S.batch_workload(n_requests=8, mesh_range=(6, 9), seed=5, crystals=SMALL)
    b_w, b_r = S.batch_workload(n_requests=8, mesh_range=(6, 9), seed=5, crystals=SMALL)
    for x, y in zip(a_w, b_w):
        assert np.array_equal(x.gwann, y.gwann) and np.array_equal(x.Hwann, y.Hwann)
    assert [(c, r.mesh, r.fsthick) for c, r in a_r] == [(c, r.mesh, r.fsthick) for c, r in b_r]


def test_batch_workload_shapes_and_windows(oracle_lib):
    wds, reqs = S.batch_workload(n_requests=8, mesh_range=(6, 9), window_range=(0.2, 1.0), seed=5, crystals=SMALL)
    assert [(w.numwannbands, w.numbranches) for w in wds] == [(nw, 3 * na) for nw, na, _ in SMALL]
    for c, r in reqs:
        assert 6 <= r.mesh[0] <= 9 and r.mesh[0] == r.mesh[1] == r.mesh[2]
        assert 0.1 <= r.fsthick <= 0.5
        e, _, _ = oracle_lib.Wannier(wds[c]).el_wann(S.mesh_kvecs(r.mesh), evecs=False)
        assert (np.abs(e - r.enref) <= r.fsthick).any()
