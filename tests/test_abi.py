"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
header declares; without a GPU every entry point refuses loudly (no fallback)."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

from elphbolt_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "ephg.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(ephg_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_header_symbols_exported(lib):
    syms = header_symbols()
    assert len(syms) >= 11
    assert set(syms) == set(_lib.EXPORTS)
    for s in syms:
        assert hasattr(lib, s), s


def test_library_is_sm103a():
    # the fatbin of the linked library was built with -gencode compute_103a/sm_103a only
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert os.path.exists(build.LIB)


def test_no_device_refuses(lib):
    if lib.ephg_device_count() > 0:
        pytest.skip("a GPU is visible")
    from elphbolt_gb300 import synthetic as S
    from elphbolt_gb300.wannier import Wannier
    wd = S.make_wannier(S.make_crystal_si_like(), 4, supercell=(2, 2, 2), seed=1)
    with pytest.raises(_lib.EphgError):
        Wannier(wd)
    h = ct.c_void_p()
    d = _lib.WannierDesc()
    rc = lib.ephg_create(ct.byref(d), ct.byref(h))
    assert rc == _lib.EPHG_ERR_CUDA
    assert b"no CUDA device" in lib.ephg_last_error()


def test_null_arguments(lib):
    assert lib.ephg_create(None, None) == _lib.EPHG_ERR_ARG
    assert lib.ephg_el_wann(None, 1, None, None, None, None, None) == _lib.EPHG_ERR_ARG
    assert lib.ephg_el_rates(None, None, None, None, None, None, None, None, 0) == _lib.EPHG_ERR_ARG
    assert lib.ephg_destroy(None) == _lib.EPHG_OK


def test_batch_refuses_bad_arguments(lib):
    """ephg_el_rates_batch checks its arguments before touching a device."""
    n = 2
    H = (ct.c_void_p * n)(None, None)
    R = (_lib.RateRequest * n)()
    RP = (_lib.c_dp * n)()
    IP = (_lib.c_i64p * n)()
    st = (ct.c_int * n)()
    assert lib.ephg_el_rates_batch(0, H, R, RP, IP, None, st, None, None) == _lib.EPHG_ERR_ARG
    assert lib.ephg_el_rates_batch(n, None, R, RP, IP, None, st, None, None) == _lib.EPHG_ERR_ARG
    assert lib.ephg_el_rates_batch(n, H, R, RP, IP, None, None, None, None) == _lib.EPHG_ERR_ARG
    # null crystal handles
    assert lib.ephg_el_rates_batch(n, H, R, RP, IP, None, st, None, None) == _lib.EPHG_ERR_ARG
    assert b"null crystal" in lib.ephg_last_error()


def test_debug_header_symbols_exported(lib):
    txt = open(os.path.join(ROOT, "include", "ephg_debug.h")).read()
    syms = sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(ephg_debug_\w+)\s*\(", txt, re.M)))
    assert "ephg_debug_wait_timeout" in syms
    for s in syms:
        assert hasattr(lib, s), s


def test_fortran_binding_covers_the_header():
    """include/wannier_gpu.f90 has a bind(C) interface for every entry point of
    include/ephg.h, and its bind(C) types have the C structs' fields in order."""
    f90 = open(os.path.join(ROOT, "include", "wannier_gpu.f90")).read()
    bound = set(re.findall(r'bind\(C,\s*name="(ephg_\w+)"\)', f90))
    assert set(header_symbols()) <= bound, set(header_symbols()) - bound
    hdr = open(os.path.join(ROOT, "include", "ephg.h")).read()

    def c_fields(name):
        body = re.search(r"typedef struct \{([^{}]*)\}\s*%s;" % name, hdr).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        out = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            names = decl.split(None, 1)[1] if not decl.startswith("const") else decl.split(None, 2)[2]
            for n in names.split(","):
                out.append(re.sub(r"[\s*]|\[.*\]", "", n))
        return out

    def f_fields(name):
        body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type" % name, f90, re.S).group(1)
        out = []
        for line in body.replace("&\n", " ").splitlines():
            if "::" in line:
                out += [re.sub(r"\(.*\)", "", n).strip() for n in line.split("::")[1].split(",")]
        return out

    for t in ("ephg_wannier_desc", "ephg_rate_request", "ephg_rate_stats", "ephg_batch_opts", "ephg_batch_stats",
              "ephg_server_stats"):
        assert c_fields(t) == f_fields(t), t
