"""File-format interop (elphbolt_gb300/epw_io.py): EPW's Wannier files and the
per-state stream files of the reference's passes.

CPU: list-directed parsing (Fortran's READ(*) rules), EPW round trips, the
byte layout of the stream files.  GPU: the library's results dumped as the
reference's files and summed back into rates the way the reference's rate
routines read them.
"""
import os

import numpy as np
import pytest

from elphbolt_gb300 import epw_io as E, synthetic as S
from tests.cases import case


def test_list_directed_values():
    txt = " (1.0000000000000000,-2.5000000000000000)  3*0.5, 1.0D-03 ,( 2.0E+00 , 1d1 ) 7"
    v = E.list_directed_values(txt)
    assert v == [complex(1.0, -2.5), 0.5, 0.5, 0.5, 1e-3, complex(2.0, 10.0), 7.0]


def _epwdata_text(ef, header, be, H, D, extra_on_records=False, style="gfortran"):
    """A hand-written epwdata.fmt: gfortran- or ifort-style list-directed output."""
    def c(z):
        if style == "gfortran":
            return "             (%.17g,%.17g)" % (z.real, z.imag)
        return " (%.16E,%.16E)" % (z.real, z.imag)
    lines = ["   %.17g     " % ef, " ".join("%11d" % n for n in header)]
    be = list(be)
    while be:
        lines.append("  ".join("%.17g" % x for x in be[:4]))
        be = be[4:]
    nwsk, nw, _ = H.shape
    nwsq, nb, _ = D.shape
    for ib in range(nw):
        for jb in range(nw):
            for r in range(nwsk):
                lines.append(c(H[r, ib, jb]) + (c(complex(99.0, 99.0)) if extra_on_records else ""))
    for ib in range(nb):
        for jb in range(nb):
            for r in range(nwsq):
                lines.append(c(D[r, ib, jb]))
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("style,extra", [("gfortran", False), ("ifort", False), ("gfortran", True)])
def test_read_epwdata_follows_list_directed_reads(tmp_path, style, extra):
    """One value per READ for H and D (wannier.f90:322-346): a record with more
    values gives only its first; Born / epsilon span records."""
    rng = np.random.default_rng(0)
    nw, nwsk, nb, nwsq, nwsg = 2, 3, 6, 4, 4
    H = rng.standard_normal((nwsk, nw, nw)) + 1j * rng.standard_normal((nwsk, nw, nw))
    D = rng.standard_normal((nwsq, nb, nb)) + 1j * rng.standard_normal((nwsq, nb, nb))
    be = rng.standard_normal((nb // 3 + 1) * 9)
    p = tmp_path / "epwdata.fmt"
    p.write_text(_epwdata_text(6.25, (nw, nwsk, nb, nwsq, nwsg), be, H, D, extra, style))
    ef, a, b, c, d, e, be2, H2, D2 = E.read_epwdata(str(p))
    assert (ef, a, b, c, d, e) == (6.25, nw, nwsk, nb, nwsq, nwsg)
    assert np.array_equal(be2, be) and np.array_equal(H2, H) and np.array_equal(D2, D)


def test_epw_round_trip(tmp_path, oracle_lib):
    """write_epw_wannier -> read_epw_wannier gives the arrays back bit for bit,
    and the oracle's rates on them are the same."""
    wd, req = case("tiny")
    E.write_epw_wannier(str(tmp_path), wd, ef=6.0)
    wd2, ef, _ = E.read_epw_wannier(str(tmp_path), wd.crystal, wd.coarse_qmesh)
    assert ef == 6.0
    for f in ("rcells_k", "rcells_q", "rcells_g", "elwsdeg", "phwsdeg", "gwsdeg", "Hwann", "Dphwann", "gwann"):
        assert np.array_equal(np.asarray(getattr(wd2, f)), np.asarray(getattr(wd, f))), f
    a = oracle_lib.Wannier(wd).el_rates(req, literal=False)
    b = oracle_lib.Wannier(wd2).el_rates(req, literal=False)
    assert np.array_equal(a["rates"], b["rates"])
    # the integer files in EPW's layout, "(3(I10,x))"
    first = (tmp_path / "rcells_k").read_text().splitlines()[0]
    assert len(first.split()) == 3 and len(first) == 33


def test_epw_size_checks(tmp_path):
    wd, _ = case("tiny")
    E.write_epw_wannier(str(tmp_path), wd)
    with open(tmp_path / "wsdeg_q", "a") as f:
        f.write("%10d \n" % 1)
    with pytest.raises(ValueError):
        E.read_epw_wannier(str(tmp_path), wd.crystal, wd.coarse_qmesh)


def test_stream_files_byte_layout(tmp_path):
    """int64 count, then the arrays back to back, no record markers (access='stream')."""
    x = np.array([1.5, -2.0, 3.25])
    E.write_X_istate(str(tmp_path), 7, x, 2 * x, np.array([4, 5, 6]), np.array([7, 8, 9]))
    raw = (tmp_path / "Xplus.istate7").read_bytes()
    assert len(raw) == 8 + 3 * 8 + 2 * 3 * 8
    assert np.frombuffer(raw[:8], dtype=np.int64)[0] == 3
    assert np.array_equal(np.frombuffer(raw[8:32], dtype=np.float64), x)
    n, v, a, b = E.read_istate(str(tmp_path / "Xminus.istate7"), with_indices=True)
    assert n == 3 and np.array_equal(v, 2 * x) and list(a) == [4, 5, 6] and list(b) == [7, 8, 9]
    E.write_gk2_istate(str(tmp_path), 1, x)
    assert E.read_istate(str(tmp_path / "gk2.istate1"))[0] == 3
    E.write_Y_istate(str(tmp_path), 2, x, [1, 2, 3], [3, 2, 1])
    assert list(E.read_istate(str(tmp_path / "Y.istate2"), with_indices=True)[3]) == [3, 2, 1]


def test_gk2_istate_writes_the_whole_buffer(tmp_path):
    """The ibzk 'g' pass writes count and then all of g2_istate(nprocs)
    (interactions.f90:2343-2348): entries past count keep the values an earlier
    state left (the buffer is zeroed once, :2146-2148); readers take count."""
    buf = np.zeros(5)
    E.write_gk2_istate(str(tmp_path), 1, [1.0, 2.0, 3.0, 4.0], buf)
    E.write_gk2_istate(str(tmp_path), 2, [9.0, 8.0], buf)
    raw = (tmp_path / "gk2.istate2").read_bytes()
    assert len(raw) == 8 + 5 * 8
    assert np.frombuffer(raw[:8], dtype=np.int64)[0] == 2
    assert np.array_equal(np.frombuffer(raw[8:], dtype=np.float64), [9.0, 8.0, 3.0, 4.0, 0.0])
    n, v = E.read_istate(str(tmp_path / "gk2.istate2"))
    assert n == 2 and list(v) == [9.0, 8.0]
    with pytest.raises(ValueError):
        E.write_gk2_istate(str(tmp_path), 3, np.ones(6), buf)


@pytest.mark.gpu
def test_dumped_files_give_the_rates(tmp_path, oracle_lib):
    """The library's vertex lists written as gk2 / X / gq2 / Y files; summed back
    as calculate_el_rta_rates and calculate_ph_rta_rates read them, they give
    the library's rates; the tags are the reference's mux_state indices."""
    from elphbolt_gb300.build import build
    from elphbolt_gb300.wannier import Wannier
    build()
    wd, req = case("tiny")
    W = Wannier(wd)
    try:
        out = E.dump_el_side(W, req, str(tmp_path / "g2"), str(tmp_path / "X"))
        rates = E.el_rates_from_files(str(tmp_path / "X"), out["nwv"], wd.numwannbands)
        assert np.allclose(rates, out["rates"], rtol=1e-13, atol=0)
        n, _, ist_el, ist_ph = E.read_istate(str(tmp_path / "X" / os.listdir(tmp_path / "X")[0]), with_indices=True)
        nin = out["stats"]["nstates_inwindow"]
        assert n == nin * wd.numbranches
        raw = (tmp_path / "g2" / sorted(os.listdir(tmp_path / "g2"))[0]).read_bytes()
        assert len(raw) == 8 + 8 * nin * wd.numbranches      # count, then g2_istate(nprocs)
        assert ist_el.min() >= 1 and ist_el.max() <= out["nwv"] * wd.numwannbands
        assert ist_ph.min() >= 1 and ist_ph.max() <= np.prod(req.mesh) * wd.numbranches
        rph = E.dump_ph_side(W, req, str(tmp_path / "gq2"), str(tmp_path / "Y"))
        back = E.ph_rates_from_files(str(tmp_path / "Y"), int(np.prod(req.mesh)), wd.numbranches)
        assert np.allclose(back, rph, rtol=1e-12, atol=1e-300)
        o = oracle_lib.Wannier(wd).ph_rates(req, spindeg=2)
        assert np.allclose(back, o["rates_phe"], rtol=1e-10, atol=1e-300)
    finally:
        W.deallocate_wannier()
