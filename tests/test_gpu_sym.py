"""Crystal symmetry on the GPU: ephg_set_symmetry + ephg_el_rates over the
irreducible wedge against the oracle's restatement of the reference's
symmetric set-up (or_rates_setup_sym).

Tolerances: FP64 rates 1e-10 relative, split-form rates 1e-6 relative, per
band on the random crystals (no degeneracies); summed over degenerate bands on
the symmetric model, whose bands are degenerate at high-symmetry points (the
eigenvector gauge inside a degenerate subspace is the eigensolver's choice).
"""
import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S, symmetry as Y
from tests.cases import case
from tests.test_symmetry import degenerate_groups, symmetric_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W_cache():
    from elphbolt_gb300.build import build
    build()
    cache = {}
    yield cache
    for w in cache.values():
        w.deallocate_wannier()


def gpu(W_cache, name, wd=None):
    from elphbolt_gb300.wannier import Wannier
    if name not in W_cache:
        W_cache[name] = Wannier(wd if wd is not None else case(name)[0])
    return W_cache[name]


def close(a, b, rel, absfrac=0.0):
    a, b = np.asarray(a), np.asarray(b)
    return bool(np.all(np.abs(a - b) <= rel * np.abs(b) + absfrac * np.abs(b).max())), \
        float(np.max(np.abs(a - b) / (np.abs(b) + 1e-300)))


@pytest.mark.parametrize("name", ["tiny", "si8", "sic"])
@pytest.mark.parametrize("prec,delta", [(_lib.PREC_FP64, 0), (_lib.PREC_FP64, 1), (_lib.PREC_FP64, 2),
                                        (_lib.PREC_SPLIT_TF32, 0), (_lib.PREC_SPLIT_TF32, 2)])
def test_ibz_rates_vs_oracle(W_cache, oracle_lib, name, prec, delta):
    wd, req0 = case(name)
    req = S.RateRequest(**{**req0.__dict__, "delta_kind": delta})
    R, _ = Y.crystal_symmetry(wd.crystal)
    o = oracle_lib.Wannier(wd).el_rates_sym(req, R, nthreads=4, literal=False)
    W = gpu(W_cache, name)
    W.set_symmetry(R)
    try:
        g = W.el_rates(req, precision=prec)
    finally:
        W.set_symmetry(None)
    assert o["status"] == 0
    assert g["nwv"] == o["nwv"] and np.array_equal(g["indexlist"], o["indexlist"])
    assert g["vertices"] == o["vertices"] and g["nstates"] == o["nstates"]
    ok, worst = close(g["rates"], o["rates"], 1e-10 if prec == _lib.PREC_FP64 else 1e-6, 1e-14)
    assert ok, worst


@pytest.mark.parametrize("prec", [_lib.PREC_FP64, _lib.PREC_SPLIT_TF32])
def test_ibz_rows_equal_full_zone_on_symmetric_model(W_cache, oracle_lib, prec):
    """Symmetric model (nw 8, nb 6: the fused tcgen05 path in the split form):
    the IBZ rates are the full-zone rates of the irreducible points, and match
    the oracle's IBZ run (degenerate sums)."""
    wd, req = symmetric_case()
    R, _ = Y.crystal_symmetry(wd.crystal)
    W = gpu(W_cache, "symmetric", wd)
    f = W.el_rates(req, precision=prec)
    W.set_symmetry(R)
    try:
        a = W.el_rates(req, precision=prec)
    finally:
        W.set_symmetry(None)
    o = oracle_lib.Wannier(wd).el_rates_sym(req, R, nthreads=4, literal=False)
    assert a["nwv"] == 16 and f["nwv"] == 216 and np.array_equal(a["indexlist"], o["indexlist"])
    assert a["stats"]["vertices"] * 10 < f["stats"]["vertices"]
    e, _, _ = oracle_lib.Wannier(wd).el_wann(S.mesh_kvecs(req.mesh), evecs=False)
    pos = {int(k): i for i, k in enumerate(f["indexlist"])}
    scale = f["rates"].max()
    tol = 1e-10 if prec == _lib.PREC_FP64 else 1e-6
    # against the FP64 oracle the split form also carries its |g|^2 floor on
    # rates far below the largest (~2e-6 relative at 2e-3 of it): 1e-8 of the largest
    floor = 1e-13 if prec == _lib.PREC_FP64 else 1e-8
    for r, k in enumerate(a["indexlist"]):
        for grp in degenerate_groups(e[k - 1]):
            x, y, z = a["rates"][r, grp].sum(), f["rates"][pos[int(k)], grp].sum(), o["rates"][r, grp].sum()
            assert abs(x - y) <= tol * abs(y) + 1e-13 * scale, (k, grp, x, y)
            assert abs(x - z) <= tol * abs(z) + floor * scale, (k, grp, x, z)


def test_phonon_side_with_symmetry(W_cache):
    """With symmetry the phonon side keeps every window k (mapped energies) and
    returns every q: on the symmetric model it equals the run without symmetry."""
    wd, req = symmetric_case()
    R, _ = Y.crystal_symmetry(wd.crystal)
    W = gpu(W_cache, "symmetric", wd)
    a = W.ph_rates(req, precision=_lib.PREC_FP64, electrons=True)
    W.set_symmetry(R)
    try:
        b = W.ph_rates(req, precision=_lib.PREC_FP64, electrons=True)
    finally:
        W.set_symmetry(None)
    assert np.array_equal(a["indexlist"], b["indexlist"]) and a["vertices"] == b["vertices"]
    ok, worst = close(b["rates_phe"], a["rates_phe"], 1e-10, 1e-14)
    assert ok, worst


def test_set_symmetry_refuses_non_lattice_rotation(W_cache):
    W = gpu(W_cache, "si8")
    shear = np.array([[[1, 1, 0], [0, 1, 0], [0, 0, 1]]], dtype=np.int64)
    with pytest.raises(_lib.EphgError) as ei:
        W.set_symmetry(shear)
    assert ei.value.code == _lib.EPHG_ERR_ARG
    W.set_symmetry(None)
