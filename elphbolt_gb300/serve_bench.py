"""Serving measurement: a Poisson stream of RTA-rate requests over resident crystals.

    python -m elphbolt_gb300.serve_bench --requests 400 --load 0.8 --slots 8 --budget-gb 160

Three synthetic Si-like crystals stay resident on the GPU: nw = 8 (the bench
crystal, 6^3 WS sets), nw = 16 and nw = 32 (4^3 WS sets, so that g(Re,Rp)
stays below 1 GB).  Each request picks a crystal at random and asks for RTA
rates on a cubic k = q mesh (8^3-24^3 for nw 8 and 16, 8^3-16^3 for nw 32),
T uniform in [100, 600] K and sigma uniform in [5, 20] meV, window +-0.5 eV
about mid-gap + 0.6 eV, split-FP32 form.  Each request is first run alone
(its isolated solve time), then all at once without merging (capacity of the
server's slots), then as a stream with Poisson arrivals at `load` times that
capacity, twice on the same arrival times: with the server's merging of queued
requests that differ only in T, sigma and chempot (one contraction, an
epilogue per request; the default) and without.  Reported: p50 / p99 / max
latency (submit to completion), the p99 of latency / isolated time, served
vertices/s, the requests that ran merged, the capacity with merging (all at
once), and the FP64 one-at-a-time vertices/s on a sample of the mix.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

MESH_RANGE = {0: (8, 24), 1: (8, 24), 2: (8, 16)}


def make_crystals(base=None):
    """The three resident crystals; `base` may supply the nw = 8 bench crystal already built."""
    from . import synthetic as S
    return [base if base is not None else S.si_like(nw=8),
            S.make_wannier(S.make_crystal_si_like(), 16, supercell=(4, 4, 4), seed=20260116),
            S.make_wannier(S.make_crystal_si_like(), 32, supercell=(4, 4, 4), seed=20260132)]


def request_mix(wds, n, rng):
    from . import synthetic as S
    out = []
    for _ in range(n):
        c = int(rng.integers(len(wds)))
        lo, hi = MESH_RANGE[c]
        m = int(rng.integers(lo, hi + 1))
        req = S.si_like_request(wds[c], (m, m, m), T=float(rng.uniform(100.0, 600.0)),
                                sigma=float(rng.uniform(0.005, 0.020)))
        out.append((c, req))
    return out


def measure(n_requests=400, load=0.8, seed=20260104, budget_bytes=160 << 30, nslots=8, fp64_sample=2, wds=None):
    """On one server: the isolated solve time of every request of a seeded stream
    (each run alone, which also trains the server's time models), capacity (the
    same requests submitted at once), then the stream with Poisson arrivals at
    `load` x capacity: p50 / p99 latency and the p99 of latency / isolated time."""
    from . import _lib
    from .serve import Server
    from .wannier import Wannier
    wds = wds or make_crystals()
    Ws = [Wannier(w) for w in wds]
    try:
        rng = np.random.default_rng(seed)
        reqs = request_mix(wds, n_requests, rng)
        srv = Server(Ws, budget_bytes, nslots=nslots)   # one server: its time models learn from the solo runs
        try:
            for c, w in enumerate(wds):   # warm-up: operand planes, workspaces
                srv.wait(srv.submit(c, request_mix([w], 1, np.random.default_rng(c))[0][1]))
            iso = []
            for c, r in reqs:             # alone
                iso.append(srv.wait(srv.submit(c, r))["latency_ms"])

            def saturated(max_sets):      # all at once
                srv.set_merge(max_sets)
                t0 = time.perf_counter()
                for t in [srv.submit(c, r) for c, r in reqs]:
                    srv.wait(t)
                return n_requests / (time.perf_counter() - t0)

            capacity = saturated(1)
            capacity_merged = saturated(_lib.MAX_SETS)
            arrivals = np.cumsum(rng.exponential(1.0 / (load * capacity), n_requests))

            def stream(max_sets):         # Poisson arrivals at load x capacity (without merging)
                srv.set_merge(max_sets)
                m0 = srv.stats()["merged"]
                tickets, t_sub = [], []
                t0 = time.perf_counter()
                for (c, r), at in zip(reqs, arrivals):
                    delay = t0 + at - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                    t_sub.append(time.perf_counter() - t0)
                    tickets.append(srv.submit(c, r))
                outs = [srv.wait(t) for t in tickets]
                lat = [o["latency_ms"] for o in outs]
                wall = max(ts + l * 1e-3 for ts, l in zip(t_sub, lat)) - t_sub[0]
                return outs, lat, wall, srv.stats()["merged"] - m0

            outs, lat, wall, merged = stream(_lib.MAX_SETS)
            _, lat1, wall1, _ = stream(1)
            peak = srv.stats()["peak_device_bytes"]
        finally:
            srv.close()
        vps = sum(o["stats"]["vertices"] for o in outs) / wall
        slow = np.asarray(lat) / np.asarray(iso)
        slow1 = np.asarray(lat1) / np.asarray(iso)
        q = lambda a, p: float(np.sort(a)[max(0, int(np.ceil(p * len(a))) - 1)])
        # plain FP64 one at a time vs split on the same (smallest) requests of the mix
        sample = sorted(reqs, key=lambda cr: int(np.prod(cr[1].mesh)))[:fp64_sample]
        v64 = t64 = vs = ts = 0.0
        for c, r in sample:
            o = Ws[c].el_rates(r, precision=_lib.PREC_FP64)["stats"]
            v64 += o["vertices"]
            t64 += o["ms_total"]
            o = Ws[c].el_rates(r, precision=_lib.PREC_SPLIT_TF32)["stats"]
            vs += o["vertices"]
            ts += o["ms_total"]
    finally:
        for W in Ws:
            W.deallocate_wannier()
    return {
        "requests": n_requests, "slots": nslots, "load": load, "completed": len(outs),
        "p50_ms": q(lat, 0.5), "p99_ms": q(lat, 0.99), "max_ms": float(np.max(lat)),
        "p50_slowdown": q(slow, 0.5), "p99_slowdown": q(slow, 0.99),
        "isolated_mean_ms": float(np.mean(iso)), "isolated_max_ms": float(np.max(iso)),
        "vertices_per_s": vps, "capacity_req_per_s": capacity,
        "merged": merged, "capacity_merged_req_per_s": capacity_merged,
        "no_merge": {"p50_ms": q(lat1, 0.5), "p99_ms": q(lat1, 0.99), "max_ms": float(np.max(lat1)),
                     "p50_slowdown": q(slow1, 0.5), "p99_slowdown": q(slow1, 0.99),
                     "vertices_per_s": sum(o["stats"]["vertices"] for o in outs) / wall1},
        "sequential_req_per_s": 1e3 / float(np.mean(iso)),
        "peak_device_bytes": peak, "hbm_budget_bytes": budget_bytes,
        "fp64_one_at_a_time_vertices_per_s": v64 / (t64 * 1e-3) if t64 else None,
        "split_same_sample_vertices_per_s": vs / (ts * 1e-3) if ts else None,
        "fp64_sample": "%d smallest requests of the stream" % len(sample),
        "mix": "3 resident Si-like crystals (nw 8 / 16 / 32, nb 6); cubic meshes 8^3-24^3 (8^3-16^3 for nw 32); "
               "T U[100,600] K; sigma U[5,20] meV; Poisson arrivals at %.0f%% of the capacity measured without "
               "merging; the same arrivals served with merging (main figures) and without (no_merge)" % (100 * load),
    }


def main(argv=None):
    ap = argparse.ArgumentParser(description="serving-loop latency / throughput on synthetic crystals")
    ap.add_argument("--requests", type=int, default=400)
    ap.add_argument("--load", type=float, default=0.8)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--budget-gb", type=float, default=160.0)
    ap.add_argument("--seed", type=int, default=20260104)
    a = ap.parse_args(argv)
    from . import build
    build.build()
    print(json.dumps(measure(a.requests, a.load, a.seed, budget_bytes=int(a.budget_gb * (1 << 30)), nslots=a.slots)),
          flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
