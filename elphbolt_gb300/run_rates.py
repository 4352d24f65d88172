"""Run synthetic RTA-rate requests and print their statistics as JSON lines.

    python -m elphbolt_gb300.run_rates --mesh 12 --precision split --repeat 2
    python -m elphbolt_gb300.run_rates --mesh 12 --side ph --crystal sic
    python -m elphbolt_gb300.run_rates --mesh 40 --crystal large --window 0.1

The crystal is the Si-like synthetic one (fcc, 2 atoms, nw = 8, 6^3 WS
supercell), or with --crystal sic the polar zincblende SiC-like one (same
sizes, Born charges and dielectric tensor on), or with --crystal large the
large instance (6-atom cell, nw = 32, nb = 18, 279 + 279 WS cells, 23 GB of
g(Re,Rp)); the window is +-0.5 eV (--window) about mid-gap + 0.6 eV,
Gaussian delta 10 meV, 300 K.  --side el runs
ephg_el_rates (electron RTA rates), --side ph runs ephg_ph_rates with the
electron rates (both sides in one sweep); --sets K > 1 runs ephg_el_rates_sets
on K requests at temperatures spread over 100-600 K (one contraction, an
epilogue per temperature).  Useful for quick checks and for profiling a smaller
case of the same kernels as the benchmark.
"""
from __future__ import annotations

import argparse
import json
import sys


def main(argv=None):
    ap = argparse.ArgumentParser(description="synthetic e-ph RTA-rate requests on the GPU")
    ap.add_argument("--mesh", type=int, default=12)
    ap.add_argument("--precision", choices=["fp64", "split"], default="split")
    ap.add_argument("--delta", choices=["gaussian", "triangle", "tetra"], default="gaussian")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--nw", type=int, default=8)
    ap.add_argument("--side", choices=["el", "ph"], default="el")
    ap.add_argument("--crystal", choices=["si", "sic", "large"], default="si")
    ap.add_argument("--window", type=float, default=0.5, help="window half width, eV")
    ap.add_argument("--sets", type=int, default=1, help="temperatures sharing one contraction (electron side)")
    a = ap.parse_args(argv)
    from . import _lib, build, synthetic as S
    from .wannier import Wannier
    build.build()
    if a.crystal == "sic":
        wd = S.make_wannier(S.make_crystal_sic_like(), a.nw, supercell=(6, 6, 6), seed=20260105)
    elif a.crystal == "large":
        wd = S.large_instance()
    else:
        wd = S.si_like(nw=a.nw)
    req = S.si_like_request(wd, (a.mesh,) * 3, window=a.window,
                            delta_kind={"gaussian": 0, "triangle": 1, "tetra": 2}[a.delta])
    W = Wannier(wd)
    prec = _lib.PREC_SPLIT_TF32 if a.precision == "split" else _lib.PREC_FP64
    for i in range(a.repeat):
        sets = 1
        if a.side == "ph":
            out = W.ph_rates(req, precision=prec, electrons=True)
        elif a.sets > 1:
            reqs = [S.RateRequest(mesh=req.mesh, enref=req.enref, fsthick=req.fsthick, chempot=req.chempot, T=T,
                                  delta_kind=req.delta_kind, sigma=req.sigma)
                    for T in [100.0 + 500.0 * k / (a.sets - 1) for k in range(a.sets)]]
            out = W.el_rates_sets(reqs, precision=prec)[0]
            sets = a.sets
        else:
            out = W.el_rates(req, precision=prec)
        st = out["stats"]
        st["sets"] = sets
        st["vertices_per_s"] = sets * st["vertices"] / (st["ms_total"] * 1e-3)
        st["repeat"] = i
        print(json.dumps(st), flush=True)
    W.deallocate_wannier()
    return 0


if __name__ == "__main__":
    sys.exit(main())
