"""Degenerate-subspace gauge fixing of |g|^2 (plot_along_path,
wannier.f90:1332-1384; test/check_interactions_symmetries.f90:330-384).

Individual |g|^2 inside a degenerate band or branch subspace depend on the
eigenvector gauge, which zheev (and any eigensolver) fixes arbitrarily.  The
reference averages them over degenerate phonon branches, then initial bands,
then final bands (|E - E'| < 1e-6 eV).  Its loops run in place, so a later
member of a group averages values its predecessors have already replaced
(mode REFERENCE, restated literally); mode MEAN takes every mean from the
values before the pass and is gauge invariant.

CPU: known answers of one group in both modes; on the symmetric model the
oracle's averaged list keeps its shape and MEAN is idempotent; on a random
crystal (no degeneracies but the zero acoustic modes at Gamma, whose |g|^2 is
zero) both modes leave the list as it is.
GPU (through the C ABI, FP64 on the device):
- the library's averaging of the oracle's own list equals the oracle's, both
  modes (same inputs, same summation order: 1e-14 relative);
- MEAN-averaged lists of the library's FP64 and split forms against the
  oracle's, per vertex: FP64 |a-b| <= 1e-10 |b| + 1e-12 max, split
  |a-b| <= 1e-5 |b| + 1e-6 max -- although the raw lists differ by far more
  inside the degenerate subspaces (the gauges differ).
"""
import numpy as np
import pytest

from elphbolt_gb300 import _lib
from tests.test_symmetry import symmetric_case


def test_group_known_answers(oracle_lib):
    O = oracle_lib
    e = [0.0, 0.0, 1.0, 0.5e-6]           # members 0, 1, 3 are degenerate (< 1e-6 apart)
    v = [1.0, 2.0, 3.0, 4.0]
    ref = O.degenerate_group(v, e, 0)
    a0 = (1 + 2 + 4) / 3
    a1 = (a0 + 2 + 4) / 3
    a3 = (a0 + a1 + 4) / 3
    assert np.allclose(ref, [a0, a1, 3.0, a3], rtol=0, atol=1e-15)
    assert np.allclose(O.degenerate_group(v, e, 1), [7 / 3, 7 / 3, 3.0, 7 / 3], rtol=0, atol=1e-15)
    # no partners: unchanged (a value divided by one)
    assert np.array_equal(O.degenerate_group(v, [0, 1, 2, 3], 0), v)


@pytest.fixture(scope="module")
def sym_lists(oracle_lib):
    import os
    wd, req = symmetric_case()
    R = oracle_lib.RatesRun(oracle_lib.Wannier(wd), req, nthreads=os.cpu_count() or 1)
    raw = R.run(0, -1, literal=False, vertices=True)
    out = {"raw": raw, "ref": R.average_degenerate(raw["g2"], 0), "mean": R.average_degenerate(raw["g2"], 1)}
    out["mean2"] = R.average_degenerate(out["mean"], 1)
    R.close()
    return wd, req, out


def test_oracle_averaging_on_symmetric_model(sym_lists):
    wd, req, L = sym_lists
    g = L["raw"]["g2"]
    assert len(g) == L["raw"]["vertices"] > 0
    for k in ("ref", "mean"):
        assert L[k].shape == g.shape and np.all(np.isfinite(L[k])) and np.all(L[k] >= 0)
    # the model has degenerate subspaces in the window: averaging changes the list
    assert np.max(np.abs(L["mean"] - g)) > 1e-6 * g.max()
    # MEAN is idempotent
    assert np.max(np.abs(L["mean2"] - L["mean"])) <= 1e-13 * g.max()


def test_no_degeneracy_no_change(oracle_lib):
    import os
    from tests.cases import case
    wd, req = case("si8")
    R = oracle_lib.RatesRun(oracle_lib.Wannier(wd), req, nthreads=os.cpu_count() or 1)
    g = R.run(0, -1, literal=False, vertices=True)["g2"]
    for mode in (0, 1):
        assert np.array_equal(R.average_degenerate(g, mode), g)
    with pytest.raises(ValueError):
        R.average_degenerate(g[:-1], 1)
    R.close()


@pytest.mark.gpu
def test_gpu_averaging_matches_oracle(sym_lists):
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    wd, req, L = sym_lists
    g_or = L["raw"]["g2"]
    W = Wannier(wd)
    try:
        # the same input list: the averaging arithmetic itself
        for mode, key in ((_lib.DEGAVG_REFERENCE, "ref"), (_lib.DEGAVG_MEAN, "mean")):
            got = W.average_degenerate(req, g_or, mode)
            assert np.max(np.abs(got - L[key]) / (np.abs(L[key]) + 1e-30 * g_or.max())) <= 1e-14, mode
        # the library's own lists, gauge fixed, against the oracle's
        mx = L["mean"].max()
        for prec, rel, absf in ((_lib.PREC_FP64, 1e-10, 1e-12), (_lib.PREC_SPLIT_TF32, 1e-5, 1e-6)):
            out = W.el_rates(req, precision=prec, vertices=True, cap=len(g_or))
            assert np.array_equal(out["indexlist"], L["raw"]["indexlist"])
            raw = out["g2"]
            avg = W.average_degenerate(req, raw, _lib.DEGAVG_MEAN)
            err = np.abs(avg - L["mean"])
            assert np.all(err <= rel * np.abs(L["mean"]) + absf * mx), (prec, float(np.max(err / mx)))
            if prec == _lib.PREC_FP64:
                # raw |g|^2 in degenerate subspaces carry the gauge: far apart
                assert np.max(np.abs(raw - g_or)) > 1e3 * max(np.max(err), 1e-300)
        with pytest.raises(_lib.EphgError):
            W.average_degenerate(req, g_or[:-1])
    finally:
        W.deallocate_wannier()
