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
CASES = {"tiny": dict(nw=4, supercell=(2, 2, 2), seed=11), "si8": dict(nw=8, supercell=(3, 3, 3), seed=12),
         "sic": dict(nw=8, supercell=(3, 3, 3), seed=14, polar=True)}


def load(name):
    z = np.load(os.path.join(HERE, "golden_%s.npz" % name))
    c = CASES[name]
    crys = S.make_crystal_sic_like() if c.get("polar") else S.make_crystal_si_like()
    wd = S.make_wannier(crys, c["nw"], supercell=c["supercell"], seed=c["seed"])
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


def load_ph(name):
    return np.load(os.path.join(HERE, "golden_ph_%s.npz" % name))


def check_ph(rates_phe, g2, y, z, rel, absfrac, g2_rel, g2_absfrac):
    """Phonon side: ph-e rates per element within rel (plus absfrac of the
    largest, for the split form's FP32 floor), and the |g|^2 / Y vertex
    sample in the reference's phonon order."""
    rz = z["rates_phe"]
    assert np.all(np.abs(rates_phe - rz) <= rel * rz + absfrac * rz.max()), \
        np.max(np.abs(rates_phe - rz) / np.maximum(rz, 1e-300))
    if g2 is not None:
        s = z["vsel"]
        assert np.all(np.abs(g2[s] - z["g2"]) <= g2_rel * np.abs(z["g2"]) + g2_absfrac * np.abs(z["g2"]).max())
        assert np.all(np.abs(y[s] - z["y"]) <= g2_rel * np.abs(z["y"]) + g2_absfrac * np.abs(z["y"]).max())


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_reproduces_golden_ph(oracle_lib, name):
    """The oracle's ibzq 'g' + 'Y' + ph-e rates against the numpy restatement's fixtures."""
    wd, req, _ = load(name)
    z = load_ph(name)
    out = oracle_lib.Wannier(wd).ph_rates(req, spindeg=int(z["spindeg"]), nthreads=4, vertices=True)
    assert out["vertices"] == int(z["nvert"])
    check_ph(out["rates_phe"], out["g2"], out["y"], z, 1e-10, 0.0, 1e-10, 1e-12)


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


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("prec", [_lib.PREC_FP64, _lib.PREC_SPLIT_TF32])
def test_library_reproduces_golden_ph(name, prec):
    """ephg_ph_rates against the phonon-side fixtures: FP64 1e-10 relative; split
    1e-5 relative on every rate.  A phonon rate is one mode's sum over the k of
    the mesh; on these small meshes it sums a few hundred vertices, too few for
    the scatter of the split form's per-vertex |g|^2 error (FP32 accumulation,
    up to a few 1e-6) to average out, and up to 4e-6 is measured.  The electron
    rates, summed over all modes, keep 1e-6, as do all the rates of the 24^3
    bench workloads (test_gpu_ph.test_full_size_split_vs_fp64 and its polar
    twin)."""
    from elphbolt_gb300.build import build
    from elphbolt_gb300.interactions import ibzq_order
    from elphbolt_gb300.wannier import Wannier
    build()
    wd, req, zel = load(name)
    z = load_ph(name)
    W = Wannier(wd)
    try:
        out = W.ph_rates(req, precision=prec, spindeg=int(z["spindeg"]), electrons=True, vertices=True)
    finally:
        W.deallocate_wannier()
    assert out["vertices"] == int(z["nvert"])
    win = np.abs(zel["ens"] - req.enref) <= req.fsthick
    order, _, _, _ = ibzq_order(out["indexlist"], win, req.mesh, wd.numbranches)
    g2, y = out["g2"][order], out["y"][order]
    if prec == _lib.PREC_FP64:
        check_ph(out["rates_phe"], g2, y, z, 1e-10, 0.0, 1e-10, 1e-12)
    else:
        check_ph(out["rates_phe"], g2, y, z, 1e-5, 0.0, 1e-5, 1e-6)
