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


def test_group_tile_lookup(lib):
    """The grouped GEMM kernel's tile -> (problem, row tile, column tile) lookup,
    run on the host over random problem sets: every tile of every problem is
    hit exactly once, and its operand rows and output offset agree."""
    import numpy as np
    lib.ephg_debug_group_tiles.argtypes = [ct.c_int, ct.POINTER(ct.c_int), ct.POINTER(ct.c_int),
                                           ct.POINTER(ct.c_int)]
    lib.ephg_debug_group_tiles.restype = ct.c_int
    rng = np.random.default_rng(11)
    for np_ in (1, 2, 3, 7, 8, 31, 64):
        m = rng.integers(1, 40, np_).astype(np.int32)
        n = rng.integers(1, 300, np_).astype(np.int32)
        hits = np.zeros(int((m.astype(np.int64) * n).sum()), dtype=np.int32)
        rc = lib.ephg_debug_group_tiles(np_, m.ctypes.data_as(ct.POINTER(ct.c_int)),
                                        n.ctypes.data_as(ct.POINTER(ct.c_int)),
                                        hits.ctypes.data_as(ct.POINTER(ct.c_int)))
        assert rc == _lib.EPHG_OK
        assert np.all(hits == 1)
