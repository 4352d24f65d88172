"""Host logic of the serving loop (slots, queue, admission by HBM budget with
workspace reservations, exclusive runs as a last resort, hand-over of the GPU
to the smallest running request, latency statistics), run against the
library's simulated executor: no GPU needed."""
import pytest

from elphbolt_gb300 import _lib, serve


@pytest.fixture(scope="module", autouse=True)
def built():
    from elphbolt_gb300.build import build
    build()


def test_all_requests_complete_on_one_slot():
    meshes = [8, 12, 16, 10] * 10
    rc, st, mc = serve.selftest(meshes, nslots=1, service_ms=0.5, budget=10 ** 9, per_request_bytes=1000)
    assert rc == _lib.EPHG_OK                      # every result reached its own ticket
    assert st["submitted"] == st["completed"] == len(meshes)
    assert st["failed"] == st["rejected"] == 0 and mc == 1
    assert st["vertices"] == sum(m ** 3 for m in meshes)
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    total = sum(0.5 * (m / 8) ** 3 for m in meshes)   # simulated device time
    assert st["max_ms"] >= 0.9 * total                 # the last request waited for all the others


def test_small_requests_overtake_a_large_one():
    # the large request starts first; the small ones take the GPU at its next yield point
    rc, st, mc = serve.selftest([16, 8, 8, 8, 8], nslots=3, service_ms=2.0)
    assert rc == _lib.EPHG_OK and st["completed"] == 5 and mc >= 2
    lat = st["latency_ms"]
    assert lat[1:].max() < lat[0]
    assert lat[1:].min() < 0.5 * lat[0]


def test_request_larger_than_budget_is_refused_at_submit():
    # two crystals of 1000 resident bytes; mesh 20 needs 8000 bytes > 6000 - 2000
    rc, st, _ = serve.selftest([8, 20, 8], nslots=2, service_ms=1.0, budget=6000, per_request_bytes=1000)
    assert rc == _lib.EPHG_OK
    assert (st["submitted"], st["completed"], st["rejected"], st["failed"]) == (3, 2, 1, 0)
    assert st["peak_device_bytes"] <= 6000


def test_request_that_cannot_reserve_runs_alone():
    # the budget leaves 1200 bytes; mesh 10 needs 1000 while the other slot holds 512: it waits and takes all
    rc, st, mc = serve.selftest([8, 10, 8, 10, 8, 8], nslots=2, service_ms=1.0, budget=3200)
    assert rc == _lib.EPHG_OK
    assert st["completed"] == 6 and st["failed"] == 0
    assert st["peak_device_bytes"] <= 3200


def test_several_exclusive_requests_do_not_deadlock():
    rc, st, mc = serve.selftest([10, 10, 10, 10], nslots=3, service_ms=1.0, budget=3200)
    assert rc == _lib.EPHG_OK and st["completed"] == 4 and mc == 1


def test_nearest_rank_percentiles():
    rc, st, _ = serve.selftest([4] * 100, nslots=1, service_ms=0.2, budget=10 ** 9, per_request_bytes=1)
    assert rc == _lib.EPHG_OK and st["completed"] == 100
    assert st["p99_ms"] >= st["p50_ms"] * 1.5         # all submitted at once: latency grows with queue position


def test_queued_requests_of_one_crystal_and_mesh_merge():
    # request 0 starts alone; the others queue behind it on one slot.  Requests
    # of one crystal and mesh that differ only in T share a run, and each gets
    # its own result (the fake writes crystal + 1000 T).
    meshes = [8] + [8, 8, 12, 8, 8, 12, 8, 8]
    temps = [100.0 + 10 * i for i in range(len(meshes))]
    rc, st, _ = serve.selftest(meshes, nslots=1, service_ms=2.0, temps=temps)
    assert rc == _lib.EPHG_OK                          # every result reached its own ticket
    assert st["completed"] == len(meshes) and st["failed"] == 0
    assert st["merged"] >= 4
    rc1, st1, _ = serve.selftest(meshes, nslots=1, service_ms=2.0, temps=temps, max_sets=1)
    assert rc1 == _lib.EPHG_OK and st1["completed"] == len(meshes) and st1["merged"] == 0
    assert st["max_ms"] < 0.7 * st1["max_ms"]          # merged runs take one request's time


def test_merge_respects_max_sets():
    meshes = [8] * 12
    temps = [100.0 + i for i in range(12)]
    rc, st, _ = serve.selftest(meshes, nslots=1, service_ms=1.0, temps=temps, max_sets=3)
    assert rc == _lib.EPHG_OK and st["completed"] == 12
    # request 0 alone, then 11 queued in runs of at most 3: at most 2 merged per run
    assert 0 < st["merged"] <= 2 * 4


def test_requests_without_a_valid_temperature_do_not_merge():
    rc, st, _ = serve.selftest([8] * 6, nslots=1, service_ms=0.5)   # T = 0
    assert rc == _lib.EPHG_OK and st["completed"] == 6 and st["merged"] == 0
