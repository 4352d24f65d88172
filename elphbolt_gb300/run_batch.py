"""Run the batched workload (ephg_el_rates_batch) and print its statistics as JSON lines.

    python -m elphbolt_gb300.run_batch --requests 64 --repeat 2

64 requests on 8 random crystals (nw 8/16/24, nb 6/12/18, WS sets of 93-279
vectors), cubic meshes 8^3-16^3, windows 0.2-1.0 eV, Gaussian delta 10 meV,
300 K, split form; --small uses 4 smaller crystals (WS 93) and meshes 6^3-9^3.
Useful for quick checks and for profiling the batched form.
"""
from __future__ import annotations

import argparse
import json
import sys


def main(argv=None):
    ap = argparse.ArgumentParser(description="batched e-ph RTA-rate requests on the GPU")
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--ungrouped", action="store_true")
    ap.add_argument("--small", action="store_true")
    a = ap.parse_args(argv)
    from . import build, synthetic as S
    from .wannier import Wannier, el_rates_batch
    build.build()
    if a.small:
        specs = [(8, 2, (4, 4, 4)), (16, 2, (4, 4, 4)), (8, 4, (4, 4, 4)), (16, 4, (4, 4, 4))]
        wds, reqs = S.batch_workload(n_requests=a.requests, mesh_range=(6, 9), crystals=specs)
    else:
        wds, reqs = S.batch_workload(n_requests=a.requests)
    Ws = [Wannier(wd) for wd in wds]
    crys, rq = [Ws[c] for c, _ in reqs], [r for _, r in reqs]
    for i in range(a.repeat):
        _, bs, _ = el_rates_batch(crys, rq, nslots=a.slots, grouped=not a.ungrouped)
        bs["repeat"] = i
        print(json.dumps(bs), flush=True)
    for W in Ws:
        W.deallocate_wannier()
    return 0


if __name__ == "__main__":
    sys.exit(main())
