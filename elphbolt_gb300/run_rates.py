"""Run synthetic RTA-rate requests and print their statistics as JSON lines.

    python -m elphbolt_gb300.run_rates --mesh 12 --precision split --repeat 2

The crystal is the Si-like synthetic one (fcc, 2 atoms, nw = 8, 6^3 WS
supercell); the window is +-0.5 eV about mid-gap + 0.6 eV, Gaussian delta
10 meV, 300 K.  Useful for quick checks and for profiling a smaller case of
the same kernels as the benchmark.
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
    a = ap.parse_args(argv)
    from . import _lib, build, synthetic as S
    from .wannier import Wannier
    build.build()
    wd = S.si_like(nw=a.nw)
    req = S.si_like_request(wd, (a.mesh,) * 3, delta_kind={"gaussian": 0, "triangle": 1, "tetra": 2}[a.delta])
    W = Wannier(wd)
    prec = _lib.PREC_SPLIT_TF32 if a.precision == "split" else _lib.PREC_FP64
    for i in range(a.repeat):
        out = W.el_rates(req, precision=prec)
        st = out["stats"]
        st["vertices_per_s"] = st["vertices"] / (st["ms_total"] * 1e-3)
        st["repeat"] = i
        print(json.dumps(st), flush=True)
    W.deallocate_wannier()
    return 0


if __name__ == "__main__":
    sys.exit(main())
