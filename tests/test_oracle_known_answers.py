"""Known answers of the reference's unit tests, restated against the oracle.

test/test_misc.f90:128-244 (mux/demux/state/binsearch/expm1/Bose/Fermi) and
:306-319 (.umklapp.); test/test_vector.f90:21-199 (vector_allreps).
"""
import numpy as np
import pytest

from elphbolt_gb300 import constants as C


def test_mux_demux_vector(oracle_lib):
    O = oracle_lib
    assert O.mux_vector([1, 2, 3], [4, 4, 4], 0) == 58      # test_misc.f90:131-135
    assert O.mux_vector([1, 2, 3], [4, 4, 4], 1) == 37
    assert O.demux_vector(58, [4, 4, 4], 0) == [1, 2, 3]    # :139-145
    assert O.demux_vector(37, [4, 4, 4], 1) == [1, 2, 3]


def test_demux_mesh(oracle_lib):
    O = oracle_lib                                          # :149-171
    m0 = [O.demux_vector(i, [2, 2, 2], 0) for i in range(1, 9)]
    m1 = [O.demux_vector(i, [2, 2, 2], 1) for i in range(1, 9)]
    exp0 = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1], [1, 1, 1]]
    assert m0 == exp0
    assert m1 == [[a + 1 for a in v] for v in exp0]


def test_mux_demux_state(oracle_lib):
    O = oracle_lib                                          # :174-190
    assert [O.mux_state(12, 1, 1), O.mux_state(12, 12, 1), O.mux_state(6, 3, 6)] == [1, 12, 33]
    assert O.demux_state(1, 12) == (1, 1)
    assert O.demux_state(12, 12) == (12, 1)
    assert O.demux_state(33, 6) == (3, 6)


def test_binsearch(oracle_lib):
    O = oracle_lib                                          # :112-118
    arr = sorted([-105, 105, 105, 105, 0])
    assert O.binsearch(arr, 105) == 3
    assert O.binsearch([1, 3, 5, 7], 4) == -1


def test_expm1_bose_fermi(oracle_lib):
    O = oracle_lib                                          # :221-244
    got = [O.expm1(np.pi), O.expm1(1.0e-8), O.expm1(1.0e-10)]
    exp = [22.140692632779267, 1.0000000050000001e-08, 1.0000000050000000e-08]
    # the reference's testify tolerance 1e-8 (absolute)
    assert all(abs(g - e) <= 1e-8 for g, e in zip(got, exp))
    assert abs(1e-10 * O.Bose(1.0e-6, 1.0e8) - 1e-10 * C.kB * 1.0e8 / 1.0e-6) <= 1e-10
    assert abs(O.Bose(1.0, 1.0e-2) - 0.0) <= 1e-10
    assert abs(O.Fermi(1.0, 1.0, 300.0) - 0.5) <= 1e-8
    assert abs(O.Fermi(1.0, 1.0, 1.0e-2) - 0.5) <= 1e-8


def test_umklapp(oracle_lib):
    O = oracle_lib                                          # :288-319
    q1 = [[0.5, 0, 0], [0.5, 0.5, 0], [0.5, 0.5, 0.5], [0.1, 0.2, 0.0]]
    q2 = [[0.5, 0, 0], [0.5, 0.5, 0], [0.5, 0.5, 0.5], [-0.5, -0.5, -0.1]]
    q3 = [[0, 0, 0], [0, 0, 0], [0, 0, 0], [0.6, 0.7, 0.9]]
    for a, b, c in zip(q1, q2, q3):
        assert np.allclose(O.umklapp(a, b), c, atol=1e-12, rtol=0)


PRIM = np.array([[-0.5, 0.0, 0.5], [0.0, 0.5, 0.5], [-0.5, 0.5, 0.0]]).T   # columns


def test_vector_allreps(oracle_lib):
    O = oracle_lib                                          # test_vector.f90:21-199
    g = [4, 4, 4]
    v0 = O.vector_create(1, g, PRIM)
    assert v0["int"] == [0, 0, 0] and np.allclose(v0["frac"], 0) and np.allclose(v0["cart"], 0)
    v1 = O.vector_create(2, g, PRIM)
    assert v1["int"] == [1, 0, 0]
    assert np.allclose(v1["frac"], [0.25, 0, 0]) and np.allclose(v1["cart"], [-0.125, 0, 0.125])
    v2 = O.vector_create(64, g, PRIM)
    assert v2["int"] == [3, 3, 3]
    assert np.allclose(v2["frac"], [0.75] * 3) and np.allclose(v2["cart"], [-0.75, 0.75, 0.75])
    a = O.vector_addsub(2, 64, +1, g, PRIM)
    assert a["muxed"] == 61 and a["int"] == [0, 3, 3]
    assert np.allclose(a["frac"], np.array([0, 3, 3]) / 4) and np.allclose(a["cart"], np.array([-3, 6, 3]) / 8)
    s = O.vector_addsub(2, 64, -1, g, PRIM)
    assert s["muxed"] == 23 and s["int"] == [2, 1, 1]
    assert np.allclose(s["frac"], [0.5, 0.25, 0.25]) and np.allclose(s["cart"], np.array([-3, 2, 3]) / 8)
    c0 = O.vector_change_grid(v0["frac"], [12, 12, 12])
    assert c0["muxed"] == 1 and c0["int"] == [0, 0, 0]
    c1 = O.vector_change_grid(v2["frac"], [12, 12, 12])
    assert c1["muxed"] == 1414 and c1["int"] == [9, 9, 9]


def test_constants():
    # params.f90:27-57 expressions
    assert C.Ryd2eV == 13.6058
    assert abs(C.Ryd2amu - 2 * 9.1093837015e-31 / 1.66053906660e-27) == 0.0
    assert C.bohr2nm == 0.052917721092
