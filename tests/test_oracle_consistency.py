"""Oracle self-checks and physical invariants (CPU only)."""
import numpy as np
import pytest

from elphbolt_gb300 import synthetic as S
from tests.cases import case, CASES


@pytest.mark.parametrize("name", CASES)
def test_literal_vs_restructured(oracle_lib, name):
    """Per-vertex g2 exactly as wannier.f90:903 vs Fourier-then-rotate: FP64 rounding only."""
    wd, req = case(name)
    W = oracle_lib.Wannier(wd)
    a = W.el_rates(req, literal=True, vertices=True)
    b = W.el_rates(req, literal=False, vertices=True)
    assert a["vertices"] == b["vertices"] > 0
    assert np.array_equal(a["indexlist"], b["indexlist"])
    scale = np.abs(a["g2"]).max()
    assert np.max(np.abs(a["g2"] - b["g2"])) <= 1e-12 * scale
    assert np.allclose(a["rates"], b["rates"], rtol=1e-12, atol=1e-14 * np.abs(a["rates"]).max())


@pytest.mark.parametrize("name", CASES)
def test_eigen_vs_lapack(oracle_lib, name):
    """Jacobi eigenvalues against LAPACK (scipy zheevd) on the same H(k), D(q)."""
    wd, req = case(name)
    W = oracle_lib.Wannier(wd)
    ks = S.mesh_kvecs(req.mesh)
    e, v, _ = W.el_wann(ks)
    ph = np.exp(2j * np.pi * (ks @ wd.rcells_k.T)) / wd.elwsdeg[None, :]
    Hk = np.einsum("kr,rij->kij", ph, np.asarray(wd.Hwann))
    Hk = np.triu(Hk) + np.conj(np.transpose(np.triu(Hk, 1), (0, 2, 1)))
    ref = np.linalg.eigvalsh(Hk) * 13.6058
    assert np.max(np.abs(e - ref)) < 1e-11
    # eigenvectors: H v = e v
    for k in range(0, len(ks), 7):
        H = 0.5 * (Hk[k] + Hk[k].conj().T)
        V = v[k].T      # columns
        assert np.max(np.abs(H @ V - V * (e[k] / 13.6058))) < 1e-12


@pytest.mark.parametrize("name", CASES)
def test_phonon_invariants(oracle_lib, name):
    """omega^2 >= 0, three zero modes at Gamma, Hermitian D(q) eigen-system."""
    wd, req = case(name)
    W = oracle_lib.Wannier(wd)
    qs = S.mesh_kvecs(req.mesh)
    e, v, _, st = W.ph_wann(qs)
    assert st == 0
    assert np.all(e >= 0)
    assert np.all(e[0, :3] == 0) and e[0, 3:].min() > 1e-3
    assert e[1:].min() > 1e-4     # no floppy modes away from Gamma


def test_gauge_invariance(oracle_lib):
    """|g|^2 is unchanged by U_k -> U_k e^{i phi} and e_q -> e_q e^{i chi}."""
    wd, req = case("si8")
    W = oracle_lib.Wannier(wd)
    rng = np.random.default_rng(0)
    k = np.array([0.2, 0.4, 0.0])
    kp = np.array([0.6, 0.2, 0.8])
    q = (kp - k) % 1.0
    ek, vk, _ = W.el_wann(k[None])
    ekp, vkp, _ = W.el_wann(kp[None])
    eq, vq, _, _ = W.ph_wann(q[None])
    gm = W.gkRp(k)
    for m, n, s in [(0, 1, 3), (3, 5, 4), (7, 2, 5)]:
        a = W.g2(k, q, vk[0, m], vkp[0, n], vq[0, s], eq[0, s], gm)
        ph = np.exp(1j * rng.uniform(0, 2 * np.pi, 3))
        b = W.g2(k, q, vk[0, m] * ph[0], vkp[0, n] * ph[1], vq[0, s] * ph[2], eq[0, s], gm)
        assert abs(a - b) <= 1e-12 * abs(a)


def test_gaussian_delta_normalisation(oracle_lib):
    """Sum over a fine uniform energy grid of the Gaussian delta integrates to 1/N_k."""
    import math
    sigma, N = 0.01, 1000
    x = np.linspace(-0.2, 0.2, 40001)
    d = (1 / math.sqrt(2 * math.pi)) / sigma * np.exp(-0.5 * (x / sigma) ** 2) / N
    assert abs(np.trapezoid(d, x) * N - 1.0) < 1e-9


def test_triangle_delta_linear_band(oracle_lib):
    """A linear band on a 2D mesh gives a flat triangle-method DOS inside the band."""
    import ctypes as ct
    O = oracle_lib
    mesh = np.array([8, 8, 1], dtype=np.int64)
    nk = 64
    idx = np.arange(1, nk + 1, dtype=np.int64)
    ens = np.zeros((nk, 1), order="F")
    for i in range(nk):
        v = O.demux_vector(i + 1, list(mesh), 0)
        ens[i, 0] = v[0] + 0.5 * v[1]      # linear in both directions (periodic wrap aside)
    tri = np.zeros((2 * nk, 3), dtype=np.int64, order="F")
    cnt = np.zeros(nk, dtype=np.int64)
    mp = np.zeros((2, nk, 6), dtype=np.int64, order="F")
    P = lambda a, t=ct.c_int64: a.ctypes.data_as(ct.POINTER(t))
    O.lib().or_form_triangles(ct.c_int64(nk), P(mesh), P(idx), P(tri), P(cnt), P(mp))
    assert np.all(cnt == 6)
    se = np.zeros((2 * nk, 1, 3), order="F")
    O.lib().or_fill_simplices(ct.c_int64(2 * nk), ct.c_int64(3), P(tri), ct.c_int64(nk), ct.c_int64(1),
                              P(ens, ct.c_double), P(se, ct.c_double))
    O.lib().or_delta_triang.argtypes = [ct.c_double, ct.c_int64, ct.c_int64, ct.POINTER(ct.c_int64),
                                        ct.c_int64, ct.c_int64, ct.c_int64, ct.POINTER(ct.c_int64),
                                        ct.POINTER(ct.c_int64), ct.POINTER(ct.c_double)]
    # total DOS at energy e: sum over k of delta(e, k); interior energies only
    tot = []
    for e in (2.3, 3.1, 3.7):
        s = sum(O.lib().or_delta_triang(e, ik, 1, P(mesh), nk, 2 * nk, 1, P(mp), P(cnt), P(se, ct.c_double))
                for ik in range(1, nk + 1))
        tot.append(s)
    assert np.all(np.array(tot) > 0)


def _oracle_window(W, req, indexlist):
    i = np.asarray(indexlist) - 1
    m = np.asarray(req.mesh)
    k = np.stack([i % m[0], (i // m[0]) % m[1], i // (m[0] * m[1])], 1) / m
    e, _, _ = W.el_wann(k)
    return np.abs(e - req.enref) <= req.fsthick


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("delta", [0, 1, 2])
def test_ph_side_visits_el_vertices(oracle_lib, name, delta):
    """The ibzq loop (gReq + 'el' g2, phonon-state order) and the ibzk loop
    (gkRp + 'ph' g2, electron-state order) visit the same vertices with the same
    |g|^2: the electron-order list, reordered by ibzq_order, is the phonon-order
    list.  The library forms both sides in one sweep on this identity."""
    from elphbolt_gb300.interactions import ibzq_order
    wd, req = case(name)
    req = S.RateRequest(**{**req.__dict__, "delta_kind": delta})
    W = oracle_lib.Wannier(wd)
    el = W.el_rates(req, literal=False, vertices=True)
    ph = W.ph_rates(req, spindeg=2, nthreads=4, vertices=True)
    assert el["vertices"] == ph["vertices"] > 0
    win = _oracle_window(W, req, el["indexlist"])
    assert win.sum() == el["nstates_inwindow"]
    order, istate_ph, i1, i2 = ibzq_order(el["indexlist"], win, req.mesh, wd.numbranches)
    scale = np.abs(ph["g2"]).max()
    assert np.max(np.abs(el["g2"][order] - ph["g2"])) <= 1e-12 * scale
    # the phonon states run in demux_state order and every q of the mesh appears
    assert np.all(np.diff(istate_ph) >= 0)
    # rates: spindeg * sum of Y per phonon state, in list order
    N = int(np.prod(req.mesh))
    acc = np.zeros(N * wd.numbranches)
    np.add.at(acc, istate_ph - 1, 2 * ph["y"])
    r = ph["rates_phe"].reshape(-1, order="C")           # row-major (q, s) = istate order
    assert np.allclose(acc, r, rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("name", ["si8"])
def test_ph_rates_spindeg_and_detailed_balance(oracle_lib, name):
    """rates_phe is linear in spindeg, and each vertex obeys Y = X+ f(1 - f) / (n (1 + n))
    (f = f(E_km), n = n(omega_qs)): absorption by the electron and emission seen
    from the phonon are tied by detailed balance."""
    from elphbolt_gb300.interactions import ibzq_order
    from elphbolt_gb300 import constants as C
    wd, req = case(name)
    W = oracle_lib.Wannier(wd)
    a = W.ph_rates(req, spindeg=1, nthreads=4)
    b = W.ph_rates(req, spindeg=2, nthreads=4, vertices=True)
    assert np.allclose(2 * a["rates_phe"], b["rates_phe"], rtol=1e-14, atol=0)
    el = W.el_rates(req, literal=False, vertices=True)
    win = _oracle_window(W, req, el["indexlist"])
    order, istate_ph, i1, i2 = ibzq_order(el["indexlist"], win, req.mesh, wd.numbranches)
    i = np.asarray(el["indexlist"]) - 1
    m = np.asarray(req.mesh)
    k = np.stack([i % m[0], (i // m[0]) % m[1], i // (m[0] * m[1])], 1) / m
    e, _, _ = W.el_wann(k)
    E = e.reshape(-1)[i1 - 1]
    qs = S.mesh_kvecs(req.mesh)
    om, _, _, _ = W.ph_wann(qs)
    w = om.reshape(-1)[istate_ph - 1]
    kT = C.kB * req.T
    f = 1.0 / (np.exp((E - req.chempot) / kT) + 1.0)
    keep = w >= 0.5e-3
    n = 1.0 / np.expm1(w[keep] / kT)
    xp = el["xp"][order][keep]
    y = b["y"][keep]
    assert np.all(b["y"][~keep] == 0)
    pred = xp * f[keep] * (1 - f[keep]) / (n * (1 + n))
    assert np.max(np.abs(pred - y)) <= 1e-10 * np.abs(y).max()


def test_polar_terms_vs_numpy(oracle_lib):
    """dyn_nonanalytic and long_range_prefac (wannier.f90:784-901, 1013-1071): the
    oracle's loops against the vectorised numpy restatement of the golden
    generator, at random q and for random mode vectors."""
    from tests.golden.make_golden import np_polar, q_cart
    wd, _ = case("sic")
    W = oracle_lib.Wannier(wd)
    dyn, lvec = np_polar(wd.crystal, wd.coarse_qmesh)
    rng = np.random.default_rng(5)
    qfs = np.concatenate([rng.uniform(-1, 1, (6, 3)), [[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]]])
    # one scale for all q: at Gamma the vector is rounding noise (its G and -G terms cancel)
    lscale = max(np.abs(lvec(q_cart(wd.crystal, qf)[0])).sum() for qf in qfs)
    for qf in qfs:
        qc = W.q_cart_bohr(qf)
        assert np.allclose(qc, q_cart(wd.crystal, qf)[0], rtol=1e-14, atol=0)
        d = W.dyn_nonanalytic(qc)
        ref = dyn(qc)
        assert np.max(np.abs(d - ref)) <= 1e-12 * np.abs(ref).max()
        u = rng.standard_normal(wd.numbranches) + 1j * rng.standard_normal(wd.numbranches)
        gl = W.long_range_prefac(qc, u)
        glr = lvec(qc) @ u
        assert abs(gl - glr) <= 1e-12 * abs(glr) + 1e-13 * lscale * np.abs(u).max()


def test_polar_velocity_term_is_the_derivative(oracle_lib):
    """ddyn_l of dyn_nonanalytic is d(dyn_l)/dq (Cartesian): central differences."""
    wd, _ = case("sic")
    W = oracle_lib.Wannier(wd)
    rng = np.random.default_rng(6)
    h = 1e-5
    for qf in rng.uniform(-1, 1, (4, 3)):
        qc = W.q_cart_bohr(qf)
        _, dd = W.dyn_nonanalytic(qc, velocities=True)
        for x in range(3):
            e = np.zeros(3)
            e[x] = h
            fd = (W.dyn_nonanalytic(qc + e) - W.dyn_nonanalytic(qc - e)) / (2 * h)
            assert np.max(np.abs(fd - dd[:, :, x])) <= 1e-6 * np.abs(dd).max()


def test_polar_phonons(oracle_lib):
    """The polar crystal's phonons: the long-range term is Hermitian and keeps
    the acoustic sum rule (three zero modes at Gamma), and it changes the
    optical branches against the same crystal without it."""
    wd, req = case("sic")
    W = oracle_lib.Wannier(wd)
    for qf in [[0.1, 0.2, 0.3], [0.5, 0.5, 0.0]]:
        d = W.dyn_nonanalytic(W.q_cart_bohr(qf))
        assert np.max(np.abs(d - d.conj().T)) <= 1e-12 * np.abs(d).max()
    qs = S.mesh_kvecs(req.mesh)
    e, _, _, st = W.ph_wann(qs)
    assert st == 0 and np.all(e[0, :3] == 0) and np.all(e >= 0)
    c = wd.crystal
    wd0 = S.make_wannier(S.Crystal(c.lattvecs, c.basis, c.masses), 8, supercell=(3, 3, 3), seed=14)
    e0, _, _, _ = oracle_lib.Wannier(wd0).ph_wann(qs)
    assert np.abs(e - e0)[1:, 3:].max() > 1e-3
