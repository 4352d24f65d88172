"""ephg_el_wann_noalloc: electron interpolation for callers that cannot allocate.

Such a caller owns its device buffers (OpenACC / CUDA Fortran arrays, a
framework's memory pool, system memory the GPU reaches over C2C) and cannot
call cudaMalloc where it needs the electrons.  This checks, through the C ABI:
- the energies of two calls in a row against the CPU oracle's el_wann
  (wannier.f90:430-524 restated) and against the ordinary ephg_el_wann; the
  fixed scratch is reused, so the second call must not see the first one's
  leftovers;
- the eigenvectors against ephg_el_wann's, up to a phase;
- a call without eigenvectors (evecs NULL) gives the same energies;
- a request larger than the fixed scratch is refused.
Tolerances: energies 1e-12 eV absolute against the oracle (FP64 Jacobi on
both sides) and against ephg_el_wann; eigenvectors |<v|v'>| = 1 within 1e-10.

This file is collected last on purpose: when a run stops at the first failure,
every other test has already run.
"""
import numpy as np
import pytest

from elphbolt_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_el_wann_noalloc_matches_el_wann_and_oracle():
    torch = pytest.importorskip("torch")
    from elphbolt_gb300.build import build
    from elphbolt_gb300 import synthetic as S
    from elphbolt_gb300.wannier import Wannier
    from oracle import oracle as O
    build()
    L = _lib.load()
    wd = S.make_wannier(S.make_crystal_si_like(), 8, supercell=(3, 3, 3), seed=12)
    W = Wannier(wd)
    ref = O.Wannier(wd)
    nw = wd.numwannbands
    rng = np.random.default_rng(3)
    dev = torch.device("cuda", 0)
    try:
        for call, nk in enumerate((37, 53)):        # two calls in a row, different sizes
            ks = rng.uniform(-1, 1, (nk, 3))
            e_or, _, _ = ref.el_wann(ks, evecs=False)
            e_ref, v_ref = W.el_wann(kvecs=ks, evecs=True)
            kv = torch.from_numpy(np.asfortranarray(ks).ravel(order="F").copy()).to(dev)
            e = torch.full((nk * nw,), float("nan"), dtype=torch.float64, device=dev)
            v = torch.full((2 * nk * nw * nw,), float("nan"), dtype=torch.float64, device=dev)
            torch.cuda.synchronize()        # kvecs written on torch's stream: complete before the call
            rc = L.ephg_el_wann_noalloc(W._h, nk, kv.data_ptr(), e.data_ptr(), v.data_ptr())
            assert rc == 0, L.ephg_last_error()
            en = e.cpu().numpy().reshape((nk, nw), order="F")
            vv = v.cpu().numpy().view(np.complex128).reshape((nk, nw, nw), order="F")
            assert np.max(np.abs(en - e_or)) <= 1e-12, call
            assert np.max(np.abs(en - e_ref)) <= 1e-12, call
            ov = np.abs(np.einsum("kbc,kbc->kb", np.conj(v_ref), vv))
            assert np.max(np.abs(ov - 1)) <= 1e-10, call
            # the same k-points without eigenvectors
            e2 = torch.full((nk * nw,), float("nan"), dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            rc = L.ephg_el_wann_noalloc(W._h, nk, kv.data_ptr(), e2.data_ptr(), None)
            assert rc == 0, L.ephg_last_error()
            assert np.array_equal(e2.cpu().numpy().reshape((nk, nw), order="F"), en), call
        # beyond the fixed scratch: refused, nothing launched
        big = 10 ** 6
        rc = L.ephg_el_wann_noalloc(W._h, big, kv.data_ptr(), e.data_ptr(), v.data_ptr())
        assert rc == _lib.EPHG_ERR_ARG
        assert b"scratch" in L.ephg_last_error()
    finally:
        W.deallocate_wannier()
