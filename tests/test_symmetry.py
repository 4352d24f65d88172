"""Crystal symmetry and the irreducible wedge (src/symmetry.f90, electron.f90:346-577).

CPU only (the finder and the wedge are host-side entry points of the library):
- the library's space-group finder against the reference's own spglib,
  compiled from its vendored sources into oracle/_ref (skipped where the
  reference tree is absent);
- the wedge against known answers and the oracle's literal find_irred_wedge;
- the oracle's rate driver with symmetry on a symmetric model: its rows equal
  the full-zone rates of the same points (summed over degenerate bands).
"""
import numpy as np
import pytest

from elphbolt_gb300 import _lib, synthetic as S, symmetry as Y


def _hexagonal(a=3.1, c=5.0):
    return np.array([[a, 0, 0], [-a / 2, a * np.sqrt(3) / 2, 0], [0, 0, c]]).T / 10.0


def crystals():
    rng = np.random.default_rng(17)
    si = S.make_crystal_si_like()
    out = {"si": si, "sic": S.make_crystal_sic_like(), "multi3": S.make_crystal_multi(3, rng)}
    # tetragonal strain of the diamond cell: fewer operations
    t = S.make_crystal_si_like()
    t.lattvecs = t.lattvecs * np.array([1.0, 1.0, 1.04])[:, None]
    out["tetragonal"] = t
    # a displaced atom: lower symmetry again
    d = S.make_crystal_si_like()
    d.basis = d.basis + np.array([[0.0, 0.0], [0.0, 0.0], [0.0, 0.013]])
    out["displaced"] = d
    # wurtzite-like hexagonal cell, 4 atoms of two types
    b = np.array([[1 / 3, 2 / 3, 0.0], [2 / 3, 1 / 3, 0.5], [1 / 3, 2 / 3, 0.375], [2 / 3, 1 / 3, 0.875]]).T
    out["wurtzite"] = S.Crystal(lattvecs=_hexagonal(), basis=b, masses=np.array([65.0, 65.0, 16.0, 16.0]))
    # conventional cubic diamond cell: 8 atoms, pure translations among the operations
    a = 0.543
    fcc = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    bb = np.concatenate([fcc, fcc + 0.25]).T
    out["cubic8"] = S.Crystal(lattvecs=a * np.eye(3), basis=bb, masses=np.full(8, 28.0))
    return out


def _key(R, T):
    return sorted((tuple(np.asarray(r).ravel()), tuple(np.round(np.mod(t, 1.0), 6) % 1.0)) for r, t in zip(R, T))


@pytest.mark.parametrize("name", list(crystals()))
def test_finder_matches_reference_spglib(oracle_lib, name):
    c = crystals()[name]
    _, types = np.unique(c.masses, return_inverse=True)
    ref = oracle_lib.spglib_symmetry(c.lattvecs, c.basis, types)
    if ref is None:
        pytest.skip("reference tree absent: its spglib was not compiled")
    R, T = Y.crystal_symmetry(c, atomtypes=types)
    assert R[0].tolist() == np.eye(3, dtype=int).tolist()     # identity first
    assert len(R) == len(ref[0])
    assert _key(R, T) == _key(*ref)


def test_finder_counts():
    """Operation counts: Fd-3m 48, F-43m 24, P1 1, wurtzite 12, conventional diamond 192."""
    c = crystals()
    want = {"si": 48, "sic": 24, "multi3": 1, "wurtzite": 12, "cubic8": 192}
    for name, n in want.items():
        assert len(Y.crystal_symmetry(c[name])[0]) == n, name


@pytest.mark.parametrize("mesh,n_oh,n_p1", [((8, 8, 8), 29, 260), ((4, 4, 4), 8, 36), ((6, 6, 6), 16, 112),
                                            ((5, 5, 5), 10, 63)])
def test_wedge_known_answers(mesh, n_oh, n_p1):
    """fcc with the full cubic group (time reversal adds nothing there) and with
    the identity alone (time reversal pairs k with -k: (N + N_TRIM) / 2 points)."""
    c = S.make_crystal_si_like()
    R, _ = Y.crystal_symmetry(c)
    irr, neq, f2i = Y.irred_wedge(c.lattvecs, R, mesh)
    assert len(irr) == n_oh and neq.sum() == np.prod(mesh)
    irr1, neq1, _ = Y.irred_wedge(c.lattvecs, R[:1], mesh)
    assert len(irr1) == n_p1
    # fbz2ibz maps every point to the irreducible point of its orbit
    assert np.all(irr[f2i - 1] <= np.arange(1, np.prod(mesh) + 1))


@pytest.mark.parametrize("name", ["si", "sic", "tetragonal", "wurtzite", "multi3"])
@pytest.mark.parametrize("mesh", [(4, 4, 4), (6, 6, 6), (5, 5, 5), (4, 4, 6), (3, 4, 5)])
def test_wedge_matches_oracle(oracle_lib, name, mesh):
    """The library's wedge (orbit minima) against the oracle's literal
    find_irred_wedge (running list), over the mesh and over a window-like list
    closed under the group."""
    c = crystals()[name]
    R, _ = Y.crystal_symmetry(c)
    st, irr_o, neq_o = oracle_lib.irred_wedge(c.lattvecs, R, mesh)
    irr, neq, _ = Y.irred_wedge(c.lattvecs, R, mesh)
    assert st == 0 and np.array_equal(irr, irr_o) and np.array_equal(neq, neq_o)
    # a closed list: the orbits of a few points
    full_irr, _, f2i = Y.irred_wedge(c.lattvecs, R, mesh)
    pick = set(full_irr[::3].tolist())
    lst = np.array([i + 1 for i in range(np.prod(mesh)) if full_irr[f2i[i] - 1] in pick], dtype=np.int64)
    st, irr_o, neq_o = oracle_lib.irred_wedge(c.lattvecs, R, mesh, lst)
    irr, neq, _ = Y.irred_wedge(c.lattvecs, R, mesh, lst)
    assert st == 0 and np.array_equal(irr, irr_o) and np.array_equal(neq, neq_o)


def test_wedge_refuses_open_list(oracle_lib):
    """A point list that is not a union of orbits has no wedge: the reference
    stops ("Could not find irreducible wedge.", symmetry.f90:417)."""
    c = S.make_crystal_si_like()
    R, _ = Y.crystal_symmetry(c)
    lst = np.array([2, 3], dtype=np.int64)
    st, _, _ = oracle_lib.irred_wedge(c.lattvecs, R, (4, 4, 4), lst)
    assert st == 1
    with pytest.raises(_lib.EphgError) as ei:
        Y.irred_wedge(c.lattvecs, R, (4, 4, 4), lst)
    assert ei.value.code == _lib.EPHG_ERR_ARG


def degenerate_groups(E, tol=1e-7):
    order = np.argsort(E)
    out, cur = [], [order[0]]
    for i in order[1:]:
        if abs(E[i] - E[cur[-1]]) < tol:
            cur.append(i)
        else:
            out.append(cur)
            cur = [i]
    out.append(cur)
    return out


def symmetric_case():
    wd = S.make_wannier_symmetric(S.make_crystal_si_like(), 4, supercell=(4, 4, 4), seed=31)
    return wd, S.si_like_request(wd, (6, 6, 6), window=0.6, shift=0.8)


def test_symmetric_model_is_symmetric(oracle_lib):
    """The symmetric model: E(Sk) = E(k) for every rotation kept for the mesh,
    and full-zone rates agree on equivalent points (summed over degenerate bands)."""
    wd, req = symmetric_case()
    c = wd.crystal
    R, _ = Y.crystal_symmetry(c)
    W = oracle_lib.Wannier(wd)
    q = oracle_lib.symmetry_qrotations(c.lattvecs, R, req.mesh)
    assert q.shape[2] == 48
    ks = S.mesh_kvecs(req.mesh)
    e, _, _ = W.el_wann(ks, evecs=False)
    f = W.el_rates(req, literal=False, nthreads=4)
    pos = {int(k): i for i, k in enumerate(f["indexlist"])}
    m = np.asarray(req.mesh)
    scale = f["rates"].max()
    for k in f["indexlist"][::7]:
        v = np.array([(k - 1) % m[0], ((k - 1) // m[0]) % m[1], (k - 1) // (m[0] * m[1])])
        for s in range(q.shape[2]):
            v2 = np.rint(m * (q[:, :, s] @ (v / m))).astype(int) % m
            k2 = v2[0] + m[0] * (v2[1] + m[1] * v2[2]) + 1
            assert np.max(np.abs(e[k2 - 1] - e[k - 1])) < 1e-12
            for g in degenerate_groups(e[k - 1]):
                assert abs(f["rates"][pos[int(k)], g].sum() - f["rates"][pos[int(k2)], g].sum()) <= 1e-12 * scale


def test_ibz_rates_equal_full_zone_rows(oracle_lib):
    """The rate driver with symmetry (IBZ blocks initial states) gives, on the
    symmetric model, the full-zone rates of its irreducible points."""
    wd, req = symmetric_case()
    R, _ = Y.crystal_symmetry(wd.crystal)
    W = oracle_lib.Wannier(wd)
    f = W.el_rates(req, literal=False, nthreads=4)
    a = W.el_rates_sym(req, R, nthreads=4, literal=False)
    assert a["status"] == 0 and a["nwv"] == 16 and f["nwv"] == 216
    irr, _, _ = Y.irred_wedge(wd.crystal.lattvecs, R, req.mesh, f["indexlist"])
    assert np.array_equal(a["indexlist"], irr)
    e, _, _ = W.el_wann(S.mesh_kvecs(req.mesh), evecs=False)
    pos = {int(k): i for i, k in enumerate(f["indexlist"])}
    scale = f["rates"].max()
    for r, k in enumerate(a["indexlist"]):
        for g in degenerate_groups(e[k - 1]):
            assert abs(a["rates"][r, g].sum() - f["rates"][pos[int(k)], g].sum()) <= 1e-12 * scale
    assert a["vertices"] * f["nwv"] < f["vertices"] * a["nwv"] * 2   # the work shrinks with the wedge
