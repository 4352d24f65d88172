"""Serving loop: RTA-rate requests against resident crystals (``ephg_server_*``).

The reference answers one request per run, from files.  A ``Server`` keeps
several crystals' Wannier data resident on the GPU and answers requests from a
queue (see ``include/ephg.h``, "Serving loop"): worker threads start them in
arrival order on several execution slots whose work overlaps on the device
(continuous batching), admission is by an HBM budget, and the server reports
p50 / p99 latency (submit to completion) beside vertices/s.

    srv = Server([wann_a, wann_b], hbm_budget_bytes=64 << 30, nslots=3)
    t = srv.submit(0, req, precision=_lib.PREC_SPLIT_TF32)
    out = srv.wait(t)            # rates, indexlist, stats
    print(srv.stats())           # p50_ms, p99_ms, vertices_per_s, ...
    srv.close()
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib
from ._lib import c_dp, c_i64p, check


class Server:
    """Mirror of the C serving API; the Wannier objects must outlive the server
    and must not be used directly while it runs."""

    def __init__(self, crystals, hbm_budget_bytes: int, nslots: int = 3):
        self._L = _lib.load()
        self._crystals = list(crystals)
        arr = (ct.c_void_p * len(self._crystals))(*[c._h for c in self._crystals])
        self._s = ct.c_void_p()
        check(self._L.ephg_server_create(arr, len(self._crystals), int(hbm_budget_bytes), int(nslots),
                                         ct.byref(self._s)))
        self._req = {}

    def submit(self, crystal: int, req, precision=_lib.PREC_SPLIT_TF32) -> int:
        r = _lib.RateRequest()
        for i in range(3):
            r.mesh[i] = int(req.mesh[i])
        r.enref, r.fsthick, r.chempot, r.T = req.enref, req.fsthick, req.chempot, req.T
        r.delta_kind, r.sigma, r.precision = int(req.delta_kind), float(req.sigma), int(precision)
        t = ct.c_int64()
        check(self._L.ephg_submit(self._s, int(crystal), ct.byref(r), ct.byref(t)))
        self._req[t.value] = (int(np.prod(req.mesh)), self._crystals[crystal].numwannbands)
        return t.value

    def poll(self, ticket: int) -> int:
        st = ct.c_int()
        check(self._L.ephg_poll(self._s, int(ticket), ct.byref(st)))
        return st.value

    def wait(self, ticket: int):
        N, nw = self._req.pop(ticket)
        rates = np.zeros((N, nw), order="F")
        idx = np.zeros(N, dtype=np.int64)
        st = _lib.RateStats()
        lat = ct.c_double()
        check(self._L.ephg_wait(self._s, int(ticket), rates.ctypes.data_as(c_dp), idx.ctypes.data_as(c_i64p),
                                ct.byref(st), ct.byref(lat)))
        nwv = int(st.nwv)
        return dict(nwv=nwv, indexlist=idx[:nwv].copy(), rates=np.asfortranarray(rates[:nwv]), stats=st.as_dict(),
                    latency_ms=lat.value)

    def set_merge(self, max_sets: int):
        """Requests per merged run (``ephg_server_set_merge``); 1 turns merging off."""
        check(self._L.ephg_server_set_merge(self._s, int(max_sets)))

    def stats(self) -> dict:
        s = _lib.ServerStats()
        check(self._L.ephg_server_stats_get(self._s, ct.byref(s)))
        return s.as_dict()

    def close(self):
        if getattr(self, "_s", None) and self._s.value:
            self._L.ephg_server_destroy(self._s)
            self._s = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest(meshes, nslots=1, service_ms=1.0, budget=10 ** 9, per_request_bytes=1000, temps=None, max_sets=0):
    """Run the server's slots / queue / admission / GPU hand-over / merging /
    statistics against a simulated executor (no GPU;
    ``ephg_debug_server_selftest``).  ``temps``: per-request T, which makes
    requests mergeable.  Returns (status, statistics incl. per-request
    latency_ms, most requests in flight at once)."""
    L = _lib.load()
    L.ephg_debug_server_selftest.argtypes = [ct.c_int, ct.c_int, ct.c_double, ct.c_int64, ct.c_int64, c_i64p, c_dp,
                                             ct.c_int, ct.POINTER(_lib.ServerStats), ct.POINTER(ct.c_int), c_dp]
    m = np.ascontiguousarray(meshes, dtype=np.int64)
    tp = None if temps is None else np.ascontiguousarray(temps, dtype=np.float64)
    out = _lib.ServerStats()
    mc = ct.c_int()
    lat = np.zeros(len(m))
    rc = L.ephg_debug_server_selftest(len(m), int(nslots), float(service_ms), int(budget), int(per_request_bytes),
                                      m.ctypes.data_as(c_i64p), None if tp is None else tp.ctypes.data_as(c_dp),
                                      int(max_sets), ct.byref(out), ct.byref(mc), lat.ctypes.data_as(c_dp))
    d = out.as_dict()
    d["latency_ms"] = lat
    return rc, d, mc.value
