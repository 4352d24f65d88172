"""ctypes binding of ``libephg.so`` (the C ABI declared in ``include/ephg.h``).

The library is the only compute path: if it is missing, or no GPU is visible,
calls raise instead of falling back to anything on the CPU.
"""
from __future__ import annotations

import ctypes as ct
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libephg.so")

EPHG_OK = 0
EPHG_ERR_ARG = 1
EPHG_ERR_CUDA = 2
EPHG_ERR_NEG_PHONON = 3
EPHG_ERR_EMPTY_WINDOW = 4
EPHG_ERR_EIG = 5
EPHG_ERR_NOMEM = 6
EPHG_ERR_TIMEOUT = 7
EPHG_ERR_INDEX = 8

PREC_FP64 = 0
PREC_SPLIT_TF32 = 1
DELTA_GAUSSIAN, DELTA_TRIANGLE, DELTA_TETRA = 0, 1, 2
WANNSPACE_EL, WANNSPACE_PH = 0, 1

c_i64p = ct.POINTER(ct.c_int64)
c_dp = ct.POINTER(ct.c_double)

# every symbol include/ephg.h declares
EXPORTS = ["ephg_create", "ephg_destroy", "ephg_last_error", "ephg_device_count", "ephg_el_wann",
           "ephg_ph_wann", "ephg_gkRp", "ephg_gReq", "ephg_g2", "ephg_kq_index", "ephg_el_rates",
           "ephg_server_create", "ephg_server_destroy", "ephg_submit", "ephg_poll", "ephg_wait",
           "ephg_server_stats_get", "ephg_el_wann_noalloc", "ephg_ph_rates", "ephg_set_polar",
           "ephg_crystal_symmetry", "ephg_set_symmetry", "ephg_irred_wedge", "ephg_el_rates_batch",
           "ephg_g2_average_degenerate", "ephg_el_rates_sets", "ephg_server_set_merge", "ephg_trim_memory"]

TICKET_QUEUED, TICKET_RUNNING, TICKET_DONE, TICKET_FAILED = 0, 1, 2, 3
DEGAVG_REFERENCE, DEGAVG_MEAN = 0, 1
MAX_SETS = 8   # EPHG_MAX_SETS


class EphgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("ephg error %d: %s" % (code, msg))
        self.code = code


class WannierDesc(ct.Structure):
    _fields_ = [("numwannbands", ct.c_int64), ("numbranches", ct.c_int64),
                ("nwsk", ct.c_int64), ("nwsq", ct.c_int64), ("nwsg", ct.c_int64),
                ("numatoms", ct.c_int64), ("coarse_qmesh", ct.c_int64 * 3),
                ("lattvecs", c_dp), ("basis", c_dp), ("masses", c_dp),
                ("rcells_k", c_i64p), ("rcells_q", c_i64p), ("rcells_g", c_i64p),
                ("elwsdeg", c_i64p), ("phwsdeg", c_i64p), ("gwsdeg", c_i64p),
                ("Hwann", c_dp), ("Dphwann", c_dp), ("gwann", c_dp)]


class RateRequest(ct.Structure):
    _fields_ = [("mesh", ct.c_int64 * 3), ("enref", ct.c_double), ("fsthick", ct.c_double),
                ("chempot", ct.c_double), ("T", ct.c_double), ("delta_kind", ct.c_int64),
                ("sigma", ct.c_double), ("precision", ct.c_int64)]


class RateStats(ct.Structure):
    _fields_ = [("nwv", ct.c_int64), ("nstates_inwindow", ct.c_int64), ("nstates", ct.c_int64),
                ("vertices", ct.c_int64), ("pairs", ct.c_int64), ("kernel_launches", ct.c_int64),
                ("ms_setup", ct.c_double), ("ms_stage_a", ct.c_double),
                ("ms_stage_bc", ct.c_double), ("ms_total", ct.c_double),
                ("stage_b_gflop", ct.c_double), ("stage_a_gflop", ct.c_double),
                ("ms_gemm_a", ct.c_double), ("ms_gemm_b", ct.c_double),
                ("gemm_a_launches", ct.c_int64), ("gemm_b_launches", ct.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerStats(ct.Structure):
    _fields_ = [("submitted", ct.c_int64), ("completed", ct.c_int64), ("failed", ct.c_int64),
                ("rejected", ct.c_int64), ("vertices", ct.c_int64), ("p50_ms", ct.c_double),
                ("p99_ms", ct.c_double), ("max_ms", ct.c_double), ("mean_ms", ct.c_double),
                ("wall_s", ct.c_double), ("vertices_per_s", ct.c_double), ("peak_device_bytes", ct.c_int64),
                ("merged", ct.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class BatchOpts(ct.Structure):
    _fields_ = [("nslots", ct.c_int64), ("hbm_budget_bytes", ct.c_int64), ("grouped", ct.c_int64)]


class BatchStats(ct.Structure):
    _fields_ = [("requests", ct.c_int64), ("failed", ct.c_int64), ("vertices", ct.c_int64),
                ("wall_ms", ct.c_double), ("vertices_per_s", ct.c_double), ("group_launches", ct.c_int64),
                ("group_problems", ct.c_int64), ("group_tiles", ct.c_int64), ("max_group", ct.c_int64),
                ("retried_alone", ct.c_int64), ("peak_workspace_bytes", ct.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def load(path: str = LIB_PATH):
    """Load the library (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libephg.so is not built: run elphbolt_gb300.build.build() "
                           "(there is no CPU fallback)")
    L = ct.CDLL(path)
    L.ephg_last_error.restype = ct.c_char_p
    L.ephg_device_count.restype = ct.c_int
    vp = ct.c_void_p
    L.ephg_create.argtypes = [ct.POINTER(WannierDesc), ct.POINTER(vp)]
    L.ephg_destroy.argtypes = [vp]
    L.ephg_el_wann.argtypes = [vp, ct.c_int64, c_dp, c_dp, c_dp, c_dp, c_dp]
    L.ephg_ph_wann.argtypes = [vp, ct.c_int64, c_dp, c_dp, c_dp, c_dp]
    L.ephg_gkRp.argtypes = [vp, ct.c_int64, c_dp, c_dp]
    L.ephg_gReq.argtypes = [vp, ct.c_int64, c_dp, c_dp]
    L.ephg_g2.argtypes = [vp, ct.c_int64, ct.c_int64, c_dp, c_dp, c_dp, c_dp, c_dp, c_dp,
                          ct.c_int64, c_dp, c_i64p, c_dp]
    L.ephg_kq_index.argtypes = [vp, c_i64p, ct.c_int64, c_i64p, ct.c_int64, c_i64p, c_i64p]
    L.ephg_el_rates.argtypes = [vp, ct.POINTER(RateRequest), c_dp, c_i64p, ct.POINTER(RateStats),
                                c_dp, c_dp, c_dp, ct.c_int64]
    L.ephg_el_rates_sets.argtypes = [vp, ct.c_int64, ct.POINTER(RateRequest), ct.POINTER(c_dp), c_i64p,
                                     ct.POINTER(RateStats)]
    L.ephg_ph_rates.argtypes = [vp, ct.POINTER(RateRequest), ct.c_int64, c_dp, c_dp, c_i64p, ct.POINTER(RateStats),
                                c_dp, c_dp, ct.c_int64]
    L.ephg_set_polar.argtypes = [vp, c_dp, c_dp]
    L.ephg_g2_average_degenerate.argtypes = [vp, ct.POINTER(RateRequest), ct.c_int64, ct.c_double, ct.c_int64, c_dp]
    L.ephg_crystal_symmetry.argtypes = [c_dp, ct.c_int64, c_dp, c_i64p, ct.c_double, ct.c_int64, c_i64p, c_i64p,
                                        c_dp]
    L.ephg_set_symmetry.argtypes = [vp, ct.c_int64, c_i64p]
    L.ephg_irred_wedge.argtypes = [c_dp, ct.c_int64, c_i64p, c_i64p, ct.c_int64, c_i64p, c_i64p, c_i64p, c_i64p,
                                   c_i64p]
    L.ephg_el_wann_noalloc.argtypes = [vp, ct.c_int64, ct.c_void_p, ct.c_void_p, ct.c_void_p]
    L.ephg_el_rates_batch.argtypes = [ct.c_int64, ct.POINTER(vp), ct.POINTER(RateRequest), ct.POINTER(c_dp),
                                      ct.POINTER(c_i64p), ct.POINTER(RateStats), ct.POINTER(ct.c_int),
                                      ct.POINTER(BatchOpts), ct.POINTER(BatchStats)]
    L.ephg_server_set_merge.argtypes = [vp, ct.c_int]
    L.ephg_trim_memory.argtypes = []
    L.ephg_server_create.argtypes = [ct.POINTER(vp), ct.c_int, ct.c_int64, ct.c_int, ct.POINTER(vp)]
    L.ephg_server_destroy.argtypes = [vp]
    L.ephg_submit.argtypes = [vp, ct.c_int, ct.POINTER(RateRequest), c_i64p]
    L.ephg_poll.argtypes = [vp, ct.c_int64, ct.POINTER(ct.c_int)]
    L.ephg_wait.argtypes = [vp, ct.c_int64, c_dp, c_i64p, ct.POINTER(RateStats), c_dp]
    L.ephg_server_stats_get.argtypes = [vp, ct.POINTER(ServerStats)]
    for name in EXPORTS:
        getattr(L, name).restype = getattr(L, name).restype or ct.c_int
    L.ephg_last_error.restype = ct.c_char_p
    _lib = L
    return L


def check(rc: int):
    if rc != EPHG_OK:
        raise EphgError(rc, load().ephg_last_error().decode(errors="replace"))
