"""The batched form's round logic on the CPU (no GPU): the gate that gathers the
GEMMs of concurrently running requests into grouped launches, driven by host
threads that activate, submit with random pauses, and deactivate
(ephg_debug_batcher_selftest).  Every submission must be launched exactly once,
in its member's order, before its submit returns, and no member may stay
blocked."""
import ctypes as ct

import pytest

from elphbolt_gb300 import _lib, build


@pytest.fixture(scope="module")
def lib():
    build.build()
    L = _lib.load()
    L.ephg_debug_batcher_selftest.argtypes = [ct.c_int, ct.c_int, ct.c_uint64, ct.POINTER(ct.c_int64),
                                              ct.POINTER(ct.c_int64)]
    L.ephg_debug_batcher_selftest.restype = ct.c_int
    return L


@pytest.mark.parametrize("members,iters,seed", [(1, 20, 1), (2, 40, 2), (8, 30, 3), (16, 15, 4), (64, 4, 5)])
def test_gate_rounds(lib, members, iters, seed):
    rounds, max_group = ct.c_int64(), ct.c_int64()
    rc = lib.ephg_debug_batcher_selftest(members, iters, seed, ct.byref(rounds), ct.byref(max_group))
    assert rc == _lib.EPHG_OK, lib.ephg_last_error()
    assert rounds.value > 0 and 1 <= max_group.value <= members
    if members >= 8:
        assert max_group.value >= 2   # concurrent members met in a round


def test_gate_refuses_bad_arguments(lib):
    assert lib.ephg_debug_batcher_selftest(0, 1, 0, None, None) == _lib.EPHG_ERR_ARG
    assert lib.ephg_debug_batcher_selftest(65, 1, 0, None, None) == _lib.EPHG_ERR_ARG
