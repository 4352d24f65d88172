"""Phonon side on the GPU (ephg_ph_rates through the C ABI) against the CPU oracle.

The oracle walks the reference's ibzq loop (interactions.f90:1673-1930): per q,
g(Re,q) from gReq, then k, k + q, m, n with the 'el' g2; the library forms the
same vertices inside the electron-side sweep.  Tolerances:
- FP64 form: ph-e rates |a-b| <= 1e-10 |b| (+1e-300), |g|^2 and Y per vertex
  1e-10 relative + 1e-12 of the largest;
- split form: ph-e rates 1e-5 relative per rate, |g|^2 and Y per vertex 1e-5
  relative + 1e-6 of the largest.  The split form's per-vertex |g|^2 carries
  FP32 accumulation errors of up to a few 1e-6 (a bias of ~-2e-7 plus a
  scatter); a phonon rate is one mode's sum over the k of the mesh, and on
  these 4^3 / 5^3 meshes it sums a few hundred vertices, too few for the
  scatter to average out: up to 4e-6 measured.  On the 24^3 bench workloads
  every positive rate, electron and phonon, keeps 1e-6 relative with no floor
  (test_full_size_split_vs_fp64, test_full_size_polar_split_vs_fp64).
"""
import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S
from tests.cases import case, CASES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W_cache():
    from elphbolt_gb300.build import build
    build()
    cache = {}
    yield cache
    for w in cache.values():
        w.deallocate_wannier()


def gpu(W_cache, name):
    from elphbolt_gb300.wannier import Wannier
    if name not in W_cache:
        W_cache[name] = Wannier(case(name)[0])
    return W_cache[name]


def close(a, b, rel, absfrac, floor=0.0):
    a, b = np.asarray(a), np.asarray(b)
    tol = rel * np.abs(b) + absfrac * np.abs(b).max() + floor
    return bool(np.all(np.abs(a - b) <= tol)), float(np.max(np.abs(a - b) / (np.abs(b) + 1e-300)))


def window_of(oracle_lib, wd, req, indexlist):
    i = np.asarray(indexlist) - 1
    m = np.asarray(req.mesh)
    k = np.stack([i % m[0], (i // m[0]) % m[1], i // (m[0] * m[1])], 1) / m
    e, _, _ = oracle_lib.Wannier(wd).el_wann(k)
    return np.abs(e - req.enref) <= req.fsthick


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("delta", [0, 1, 2])
@pytest.mark.parametrize("prec", [_lib.PREC_FP64, _lib.PREC_SPLIT_TF32])
def test_ph_rates_vs_oracle(W_cache, oracle_lib, name, delta, prec):
    from elphbolt_gb300.interactions import ibzq_order
    wd, req0 = case(name)
    req = S.RateRequest(**{**req0.__dict__, "delta_kind": delta})
    o = oracle_lib.Wannier(wd).ph_rates(req, spindeg=2, nthreads=4, vertices=True)
    g = gpu(W_cache, name).ph_rates(req, precision=prec, spindeg=2, electrons=True, vertices=True)
    assert g["vertices"] == o["vertices"] > 0
    win = window_of(oracle_lib, wd, req, g["indexlist"])
    order, _, _, _ = ibzq_order(g["indexlist"], win, req.mesh, wd.numbranches)
    if prec == _lib.PREC_FP64:
        ok, worst = close(g["rates_phe"], o["rates_phe"], 1e-10, 0.0, 1e-300)
        assert ok, worst
        for key in ("g2", "y"):
            ok, worst = close(g[key][order], o[key], 1e-10, 1e-12)
            assert ok, (key, worst)
    else:
        ok, worst = close(g["rates_phe"], o["rates_phe"], 1e-5, 0.0, 1e-300)
        assert ok, worst
        for key in ("g2", "y"):
            ok, worst = close(g[key][order], o[key], 1e-5, 1e-6)
            assert ok, (key, worst)
    assert np.all(g["rates_phe"] >= 0)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("prec", [_lib.PREC_FP64, _lib.PREC_SPLIT_TF32])
def test_one_sweep_gives_el_rates(W_cache, name, prec):
    """The electron side of ephg_ph_rates is ephg_el_rates: the phonon terms
    only add atomics, the electron partials are untouched."""
    wd, req = case(name)
    W = gpu(W_cache, name)
    a = W.el_rates(req, precision=prec)
    b = W.ph_rates(req, precision=prec, electrons=True)
    assert np.array_equal(a["indexlist"], b["indexlist"])
    assert b["stats"]["vertices"] == a["stats"]["vertices"]
    if prec == _lib.PREC_FP64:
        assert np.array_equal(a["rates"], b["rates"])
    else:
        ok, worst = close(b["rates"], a["rates"], 1e-6, 0.0)
        assert ok, worst


def test_spindeg(W_cache):
    wd, req = case("si8")
    W = gpu(W_cache, "si8")
    one = W.ph_rates(req, precision=_lib.PREC_FP64, spindeg=1)["rates_phe"]
    two = W.ph_rates(req, precision=_lib.PREC_FP64, spindeg=2)["rates_phe"]
    ok, worst = close(two, 2 * one, 1e-12, 0.0, 1e-300)
    assert ok, worst
    for bad in (0, 3):
        with pytest.raises(_lib.EphgError) as ei:
            W.ph_rates(req, spindeg=bad)
        assert ei.value.code == _lib.EPHG_ERR_ARG


def test_ibzq_lists_reference_order(W_cache, oracle_lib):
    """calculate_eph_interaction_ibzq: the lists in the reference's phonon order
    with the istate1 / istate2 / phonon-state tags it writes to Y.istate*."""
    from elphbolt_gb300 import interactions as I
    wd, req = case("tiny")
    W = gpu(W_cache, "tiny")
    o = oracle_lib.Wannier(wd).ph_rates(req, spindeg=2, vertices=True)
    g2, iph = I.calculate_eph_interaction_ibzq(W, req, "g")
    y, i1, i2, iph2 = I.calculate_eph_interaction_ibzq(W, req, "Y")
    assert np.array_equal(iph, iph2)
    ok, worst = close(g2, o["g2"], 1e-10, 1e-12)
    assert ok, worst
    ok, worst = close(y, o["y"], 1e-10, 1e-12)
    assert ok, worst
    nw, nb = wd.numwannbands, wd.numbranches
    assert np.all(np.diff(iph) >= 0) and iph.min() >= 1 and iph.max() <= np.prod(req.mesh) * nb
    assert i1.min() >= 1 and i2.min() >= 1
    with pytest.raises(_lib.EphgError):
        I.calculate_eph_interaction_ibzq(W, req, "X")
    rates, st = I.calculate_ph_rta_rates(W, req)
    ok, worst = close(rates, o["rates_phe"], 1e-10, 0.0, 1e-300)
    assert ok, worst


def test_full_size_split_vs_fp64():
    """The bench workload (nw 8, 6^3 WS sets, 24^3 mesh): split-form ph-e rates
    against the FP64 form, 1e-6 relative on every positive rate; electron
    rates of the same sweep likewise."""
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    wd = S.si_like(nw=8)
    req = S.si_like_request(wd, (24, 24, 24))
    W = Wannier(wd)
    try:
        f = W.ph_rates(req, precision=_lib.PREC_FP64, electrons=True)
        s = W.ph_rates(req, precision=_lib.PREC_SPLIT_TF32, electrons=True)
    finally:
        W.deallocate_wannier()
    assert f["vertices"] == s["vertices"] > 10 ** 8
    mp = f["rates_phe"] > 0
    assert np.max(np.abs(s["rates_phe"][mp] - f["rates_phe"][mp]) / f["rates_phe"][mp]) < 1e-6
    m = f["rates"] > 0
    assert np.max(np.abs(s["rates"][m] - f["rates"][m]) / f["rates"][m]) < 1e-6
    assert mp.sum() > 0.5 * f["rates_phe"].size


def test_full_size_polar_split_vs_fp64():
    """The polar SiC-like crystal at the bench size (nw 8, 6^3 WS sets, 24^3
    mesh, Born charges and dielectric tensor on): both rate sets of one split
    sweep against the FP64 form, 1e-6 relative on every positive rate."""
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    wd = S.make_wannier(S.make_crystal_sic_like(), 8, supercell=(6, 6, 6), seed=20260105)
    req = S.si_like_request(wd, (24, 24, 24))
    W = Wannier(wd)
    try:
        f = W.ph_rates(req, precision=_lib.PREC_FP64, electrons=True)
        s = W.ph_rates(req, precision=_lib.PREC_SPLIT_TF32, electrons=True)
    finally:
        W.deallocate_wannier()
    mp, m = f["rates_phe"] > 0, f["rates"] > 0
    assert mp.sum() > 0.5 * f["rates_phe"].size
    assert np.max(np.abs(s["rates_phe"][mp] - f["rates_phe"][mp]) / f["rates_phe"][mp]) < 1e-6
    assert np.max(np.abs(s["rates"][m] - f["rates"][m]) / f["rates"][m]) < 1e-6
