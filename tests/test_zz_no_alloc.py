"""ephg_el_wann_noalloc: electron interpolation for callers that cannot allocate.

Such a caller owns its device buffers (OpenACC / CUDA Fortran arrays, a
framework's memory pool, system memory the GPU reaches over C2C) and cannot
call cudaMalloc where it needs the electrons.  This checks, through the C ABI,
that the allocation-free entry point gives the energies and eigenvectors of
the ordinary ephg_el_wann on two calls in a row (the fixed scratch is reused,
so the second call must not see the first one's leftovers), and that a request
larger than the fixed scratch is refused.  Tolerances: energies 1e-12 eV
absolute, eigenvectors equal up to a phase (|<v|v'>| = 1 within 1e-10); the
kernels are the same, so both are met with room to spare.

This file is collected last on purpose: when a run stops at the first failure,
every other test has already run.
"""
import ctypes as ct

import numpy as np
import pytest

from elphbolt_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_el_wann_noalloc_matches_el_wann():
    torch = pytest.importorskip("torch")
    from elphbolt_gb300.build import build
    from elphbolt_gb300 import synthetic as S
    from elphbolt_gb300.wannier import Wannier
    build()
    L = _lib.load()
    wd = S.make_wannier(S.make_crystal_si_like(), 8, supercell=(3, 3, 3), seed=12)
    W = Wannier(wd)
    nw = wd.numwannbands
    rng = np.random.default_rng(3)
    dev = torch.device("cuda", 0)
    try:
        for call, nk in enumerate((37, 53)):        # two calls in a row, different sizes
            ks = rng.uniform(-1, 1, (nk, 3))
            e_ref, v_ref = W.el_wann(kvecs=ks, evecs=True)
            kv = torch.from_numpy(np.asfortranarray(ks).ravel(order="F").copy()).to(dev)
            e = torch.full((nk * nw,), float("nan"), dtype=torch.float64, device=dev)
            v = torch.full((2 * nk * nw * nw,), float("nan"), dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            rc = L.ephg_el_wann_noalloc(W._h, nk, kv.data_ptr(), e.data_ptr(), v.data_ptr())
            assert rc == 0, L.ephg_last_error()
            torch.cuda.synchronize()
            en = e.cpu().numpy().reshape((nk, nw), order="F")
            vv = v.cpu().numpy().view(np.complex128).reshape((nk, nw, nw), order="F")
            assert np.max(np.abs(en - e_ref)) <= 1e-12, call
            ov = np.abs(np.einsum("kbc,kbc->kb", np.conj(v_ref), vv))
            assert np.max(np.abs(ov - 1)) <= 1e-10, call
        # beyond the fixed scratch: refused, nothing launched
        big = 10 ** 6
        rc = L.ephg_el_wann_noalloc(W._h, big, kv.data_ptr(), e.data_ptr(), v.data_ptr())
        assert rc == _lib.EPHG_ERR_ARG
        assert b"scratch" in L.ephg_last_error()
    finally:
        W.deallocate_wannier()
