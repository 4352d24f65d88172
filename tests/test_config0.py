"""The CPU-runnable benchmark configuration itself, pinned by the oracle.

Crystal: the seeded Si-like fcc cell (nw 8, nb 6, 279 Re / 279 Rp WS cells of
a 6x6x6 supercell); request: 12x12x12 k = q mesh, window +-0.5 eV about
mid-gap + 0.6 eV, Gaussian delta 10 meV, T = 300 K.  The fixture
tests/golden/golden_config0.npz (tests/golden/make_config0.py) holds the
oracle's RTA rates (interactions.f90:2958-3063) of 128 initial states spread
over the window, each a full sum over the 1,441 window k'.

- CPU: the oracle reproduces the fixture's first 8 states (1e-12 relative).
- GPU: both library forms over the whole request, through the C ABI, on the
  sampled states: FP64 1e-10 relative per rate, split-FP32 1e-6 relative per
  rate (the stated bound); the window k list is bit-exact.
"""
import os

import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load():
    z = np.load(os.path.join(HERE, "golden_config0.npz"))
    wd = S.si_like()
    req = S.RateRequest(mesh=tuple(int(x) for x in z["mesh"]), enref=float(z["enref"]), fsthick=float(z["fsthick"]),
                        chempot=float(z["chempot"]), T=float(z["T"]), delta_kind=0, sigma=float(z["sigma"]))
    return wd, req, z


def test_config0_oracle_reproduces_fixture(oracle_lib):
    wd, req, z = load()
    R = oracle_lib.RatesRun(oracle_lib.Wannier(wd), req, nthreads=os.cpu_count() or 1)
    try:
        out = R.run(0, 8, literal=False)
    finally:
        R.close()
    assert np.array_equal(out["indexlist"], z["indexlist"])
    assert out["nstates_inwindow"] > 0
    rows, bands, ref = z["rows"][:8], z["bands"][:8], z["rates"][:8]
    got = out["rates"][rows, bands]
    assert np.max(np.abs(got - ref) / ref) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(_lib.PREC_FP64, 1e-10), (_lib.PREC_SPLIT_TF32, 1e-6)])
def test_config0_gpu_vs_oracle(prec, tol):
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    wd, req, z = load()
    W = Wannier(wd)
    try:
        out = W.el_rates(req, precision=prec)
    finally:
        W.deallocate_wannier()
    assert np.array_equal(out["indexlist"], z["indexlist"])
    assert out["stats"]["nstates"] == int(z["nstates"])
    got = out["rates"][z["rows"], z["bands"]]
    rel = np.abs(got - z["rates"]) / z["rates"]
    assert np.max(rel) <= tol, (prec, float(np.max(rel)))
