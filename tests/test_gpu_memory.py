"""Device memory of the library: handles and workspaces come from a pool that
keeps freed memory mapped for the next handle; ephg_trim_memory gives the
unused part back to the driver (a caller that needs it for other allocations).

Checked: after a request and ephg_destroy the device's free memory is below
what it is after ephg_trim_memory (the pool held the handle's memory), and a
handle created after the trim still computes the same rates.
"""
import numpy as np
import pytest

from elphbolt_gb300 import _lib
from elphbolt_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def test_trim_returns_pooled_memory():
    torch = pytest.importorskip("torch")
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    L = _lib.load()
    wd = S.si_like()
    req = S.si_like_request(wd, (12, 12, 12))
    W = Wannier(wd)
    try:
        ref = W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)["rates"]
    finally:
        W.deallocate_wannier()
    torch.cuda.synchronize()
    free_pooled, _ = torch.cuda.mem_get_info()
    assert L.ephg_trim_memory() == _lib.EPHG_OK, L.ephg_last_error()
    free_trimmed, _ = torch.cuda.mem_get_info()
    assert free_trimmed - free_pooled >= 256 << 20   # the handle's g(Re,Rp) alone is ~1 GB
    W = Wannier(wd)
    try:
        again = W.el_rates(req, precision=_lib.PREC_SPLIT_TF32)["rates"]
    finally:
        W.deallocate_wannier()
    assert np.array_equal(again, ref)
