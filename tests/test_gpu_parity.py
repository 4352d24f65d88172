"""FP64 drop-in on the GPU (through the C ABI) against the CPU oracle.

Tolerances (FP64 form): energies 1e-10 eV absolute; |g|^2 per vertex
|a-b| <= 1e-10 |b| + 1e-12 max|b| (eigen-gauge and summation order differ);
rates 1e-10 relative per state; integer tables bit-exact.
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


def ora(oracle_lib, name):
    return oracle_lib.Wannier(case(name)[0])


def close(a, b, rel, absfrac):
    a, b = np.asarray(a), np.asarray(b)
    tol = rel * np.abs(b) + absfrac * np.abs(b).max()
    return np.all(np.abs(a - b) <= tol), np.max(np.abs(a - b) / (np.abs(b) + 1e-300))


@pytest.mark.parametrize("name", CASES)
def test_el_wann(W_cache, oracle_lib, name):
    wd, req = case(name)
    ks = np.random.default_rng(1).uniform(-1, 1, (37, 3))
    ks[0] = 0
    e, v, ev = gpu(W_cache, name).el_wann(kvecs=ks, velocities=True, evecs=True)
    eo, evo, vo = ora(oracle_lib, name).el_wann(ks, velocities=True)
    assert np.max(np.abs(e - eo)) < 1e-10
    # eigenvectors agree up to a phase: |<v_o|v_g>| = 1
    ov = np.abs(np.einsum("kbc,kbc->kb", np.conj(evo), ev))
    assert np.max(np.abs(ov - 1)) < 1e-9
    assert np.max(np.abs(v - vo)) < 1e-8 * max(1.0, np.abs(vo).max())


@pytest.mark.parametrize("name", CASES)
def test_eigensolver_converges_everywhere(W_cache, oracle_lib, name):
    """el_wann / ph_wann over the whole mesh and 2000 random points: every
    Jacobi solve converges (the FP32-angle rotations leave the off-diagonal at
    the FP64 rounding floor, which the convergence test must accept) and the
    energies match the oracle."""
    wd, req = case(name)
    rng = np.random.default_rng(3)
    ks = np.concatenate([S.mesh_kvecs(req.mesh), rng.uniform(-1, 1, (2000, 3)),
                         np.round(rng.uniform(-1, 1, (500, 3)) * 8) / 8])
    e = gpu(W_cache, name).el_wann(kvecs=ks)
    eo, _, _ = ora(oracle_lib, name).el_wann(ks, evecs=False)
    assert np.max(np.abs(e - eo)) < 1e-10
    om = gpu(W_cache, name).ph_wann(qvecs=np.abs(ks) % 1.0)
    omo, _, _, st = ora(oracle_lib, name).ph_wann(np.abs(ks) % 1.0, evecs=False)
    assert st == 0
    assert np.max(np.abs(om - omo)) < 1e-10


@pytest.mark.parametrize("name", CASES)
def test_ph_wann(W_cache, oracle_lib, name):
    wd, req = case(name)
    qs = np.random.default_rng(2).uniform(0, 1, (23, 3))
    qs[0] = 0
    e, ev, v = gpu(W_cache, name).ph_wann(qvecs=qs, evecs=True, velocities=True)
    eo, evo, vo, st = ora(oracle_lib, name).ph_wann(qs, velocities=True)
    assert st == 0
    assert np.max(np.abs(e - eo)) < 1e-10
    nz = eo > 1e-3
    ov = np.abs(np.einsum("kbc,kbc->kb", np.conj(evo), ev))
    assert np.max(np.abs(ov[nz] - 1)) < 1e-8
    # (in a 2^3 supercell every wrap set is symmetric and the reference's
    # unwrapped-R velocity formula cancels to ~0, hence the absolute floor)
    assert np.max(np.abs(v[1:] - vo[1:])) < 1e-7 * max(np.abs(vo).max(), 1e-3)


@pytest.mark.parametrize("name", CASES)
def test_gkRp_gReq(W_cache, oracle_lib, name):
    ks = np.random.default_rng(3).uniform(0, 1, (3, 3))
    G = gpu(W_cache, name).gkRp(kvec=ks)
    O = ora(oracle_lib, name)
    for i in range(3):
        go = O.gkRp(ks[i])
        assert np.max(np.abs(G[..., i] - go)) <= 1e-12 * np.abs(go).max()
    R = gpu(W_cache, name).gReq(qvec=ks)
    for i in range(3):
        ro = O.gReq(ks[i])
        assert np.max(np.abs(R[..., i] - ro)) <= 1e-12 * np.abs(ro).max()


@pytest.mark.parametrize("name", CASES)
def test_g2_batch(W_cache, oracle_lib, name):
    wd, req = case(name)
    O = ora(oracle_lib, name)
    rng = np.random.default_rng(4)
    nv = 40
    k = rng.uniform(0, 1, (2, 3))
    gms = np.stack([O.gkRp(k[0]), O.gkRp(k[1])], axis=-1)
    kp = rng.uniform(0, 1, (nv, 3))
    gi = rng.integers(1, 3, nv)
    kv = k[gi - 1]
    q = (kp - kv) % 1.0
    _, vk, _ = O.el_wann(kv)
    _, vkp, _ = O.el_wann(kp)
    eq, vq, _, _ = O.ph_wann(q)
    m, n, s = rng.integers(0, wd.numwannbands, nv), rng.integers(0, wd.numwannbands, nv), rng.integers(0, wd.numbranches, nv)
    a = [vk[i, m[i]] for i in range(nv)]
    b = [vkp[i, n[i]] for i in range(nv)]
    c = [vq[i, s[i]] for i in range(nv)]
    en = np.array([eq[i, s[i]] for i in range(nv)])
    en[0] = 0.0
    got = gpu(W_cache, name).g2_batch(kv, q, np.array(a), np.array(b), np.array(c), en, gms, gi)
    ref = np.array([O.g2(kv[i], q[i], a[i], b[i], c[i], en[i], gms[..., gi[i] - 1]) for i in range(nv)])
    assert got[0] == 0.0
    ok, worst = close(got, ref, 1e-10, 1e-12)
    assert ok, worst


def test_kq_index_bit_exact(W_cache, oracle_lib):
    O = oracle_lib
    mesh = [6, 5, 4]
    N = 120
    k = np.arange(1, N + 1)
    kp = np.arange(1, N + 1)[::-1].copy()
    got = gpu(W_cache, "tiny").kq_index(mesh, k, kp)
    prim = np.eye(3)
    ref = np.array([[O.vector_addsub(b, a, -1, mesh, prim)["muxed"] for b in kp] for a in k])
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("delta", [0, 1, 2])
def test_el_rates_fp64(W_cache, oracle_lib, name, delta):
    wd, req0 = case(name)
    req = S.RateRequest(**{**req0.__dict__, "delta_kind": delta})
    o = ora(oracle_lib, name).el_rates(req, literal=True, vertices=True)
    g = gpu(W_cache, name).el_rates(req, precision=_lib.PREC_FP64, vertices=True)
    assert g["nwv"] == o["nwv"] and np.array_equal(g["indexlist"], o["indexlist"])
    assert g["vertices"] == o["vertices"] > 0
    ok, worst = close(g["g2"], o["g2"], 1e-10, 1e-12)
    assert ok, worst
    for key in ("xp", "xm"):
        ok, worst = close(g[key], o[key], 1e-9, 1e-12)
        assert ok, (key, worst)
    ok, worst = close(g["rates"], o["rates"], 1e-10, 1e-13)
    assert ok, worst


def test_empty_window_refused(W_cache):
    wd, req0 = case("tiny")
    req = S.RateRequest(**{**req0.__dict__, "enref": 1e3})
    with pytest.raises(_lib.EphgError) as ei:
        gpu(W_cache, "tiny").el_rates(req)
    assert ei.value.code == _lib.EPHG_ERR_EMPTY_WINDOW
