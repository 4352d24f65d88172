"""The committed golden fixtures (tests/golden/make_golden.py).

They were produced by an independent numpy restatement of the path and
cross-checked against the C oracle before being written.  Here:
- the CPU test pins the oracle to them;
- the GPU tests pin the library's FP64 and split forms to them.

Tolerances: energies 1e-10 eV; |g|^2 and rates 1e-10 relative for FP64;
for the split form |g|^2 1e-5 relative + 1e-6 of the largest (vertices near
zero carry an FP32-level absolute error) and rates 1e-6 relative.
"""
import os

import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = {"tiny": dict(nw=4, supercell=(2, 2, 2), seed=11), "si8": dict(nw=8, supercell=(3, 3, 3), seed=12)}


def load(name):
    z = np.load(os.path.join(HERE, "golden_%s.npz" % name))
    c = CASES[name]
    wd = S.make_wannier(S.make_crystal_si_like(), c["nw"], supercell=c["supercell"], seed=c["seed"])
    req = S.RateRequest(mesh=tuple(int(x) for x in z["mesh"]), enref=float(z["enref"]), fsthick=float(z["fsthick"]),
                        chempot=float(z["chempot"]), T=float(z["T"]), delta_kind=0, sigma=float(z["sigma"]))
    return wd, req, z


def check(out, z, g2_rel, rate_rel, g2_absfrac=1e-12):
    assert np.array_equal(out["indexlist"], z["indexlist"])
    assert out["vertices"] == int(z["nvert"])
    r, rz = out["rates"], z["rates"]
    m = rz > 0
    assert np.all(np.abs(r[m] - rz[m]) <= rate_rel * rz[m]), np.max(np.abs(r[m] - rz[m]) / rz[m])
    assert np.all(r[~m] == 0)
    if g2_rel is not None:
        g = out["g2"][z["vsel"]]
        gz = z["g2"]
        assert np.all(np.abs(g - gz) <= g2_rel * np.abs(gz) + g2_absfrac * np.abs(gz).max())


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_reproduces_golden(oracle_lib, name):
    wd, req, z = load(name)
    out = oracle_lib.Wannier(wd).el_rates(req, literal=True, vertices=True)
    check(out, z, 1e-10, 1e-10)
    e, _, _ = oracle_lib.Wannier(wd).el_wann(S.mesh_kvecs(req.mesh)[z["indexlist"] - 1])
    assert np.max(np.abs(e - z["ens"])) < 1e-10
    om, _, _, _ = oracle_lib.Wannier(wd).ph_wann(S.mesh_kvecs(req.mesh))
    assert np.max(np.abs(om - z["om"])) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("prec", [_lib.PREC_FP64, _lib.PREC_SPLIT_TF32])
def test_library_reproduces_golden(name, prec):
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    wd, req, z = load(name)
    W = Wannier(wd)
    try:
        out = W.el_rates(req, precision=prec, vertices=True)
    finally:
        W.deallocate_wannier()
    if prec == _lib.PREC_FP64:
        check(out, z, 1e-10, 1e-10)
    else:
        check(out, z, 1e-5, 1e-6, g2_absfrac=1e-6)
