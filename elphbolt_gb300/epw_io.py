"""File-format interop with elphbolt and EPW.

Readers of the Wannier data EPW writes for elphbolt (``read_EPW_Wannier``,
src/wannier.f90:289-428), and writers / readers of the per-state files
through which the reference's passes hand results to one another
(src/interactions.f90), so that the unmodified BTE and Eliashberg codes can
consume what the library computes:

* ``epwdata.fmt`` -- list-directed text: E_F; nw, nwsk, nb, nwsq, nwsg; the
  Born charges (3,3,nat) and dielectric tensor (3,3); H(Re) as (ib, jb, Re)
  loops of complex values; D(Rp) likewise;
* ``epmatwp1`` -- stream of complex(r64) g(nw, nw, nwsk, nb, nwsg), column-major;
* ``rcells_k|q|g``, ``wsdeg_k|q|g`` -- integer text, one cell per line
  (ephwann_shuffle.f90:385-420);
* ``gk2.istate<n>`` (ibzk 'g', interactions.f90:2337-2348): int64 count, g2;
* ``Xplus.istate<n>``, ``Xminus.istate<n>`` ('X', :2351-2377): int64 count,
  X (THz), istate_el, istate_ph (int64);
* ``gq2.istate<n>`` (ibzq 'g', :1884-1894): int64 count, g2(1:count);
* ``Y.istate<n>`` ('Y', :1896-1911): int64 count, Y (THz), istate1, istate2.

Stream files carry no record markers (``access='stream'``); integers are
int64 and reals float64 in the machine's byte order, as gfortran writes them.
"""
from __future__ import annotations

import os
import re

import numpy as np

from . import synthetic as S

# ------------------------------------------------------------ list-directed text
_TOKEN = re.compile(r"""
    (?:(\d+)\*)?                                            # repeat count r*
    (?:\(\s*([^,()\s]+)\s*,\s*([^,()\s]+)\s*\)              # complex (re, im)
       |([^\s,()/]+))                                       # or a plain value
    """, re.VERBOSE)


def _num(s):
    return float(s.replace("D", "E").replace("d", "e"))


def list_directed_values(text):
    """The values of Fortran list-directed input, in order: complex numbers for
    '(re,im)', floats otherwise; 'r*value' repeats, commas and blanks separate."""
    out = []
    for m in _TOKEN.finditer(text):
        rep = int(m.group(1)) if m.group(1) else 1
        if m.group(2) is not None:
            v = complex(_num(m.group(2)), _num(m.group(3)))
        else:
            v = _num(m.group(4))
        out.extend([v] * rep)
    return out


class _ListDirected:
    """Fortran list-directed READ over the records (lines) of a file: every READ
    starts at a new record, takes values until its items are filled (continuing
    over records) and discards the rest of the record it ends in."""

    def __init__(self, path):
        with open(path) as f:
            self.lines = f.read().splitlines()
        self.path = path
        self.row = 0

    def read(self, n):
        out = []
        while len(out) < n:
            if self.row >= len(self.lines):
                raise ValueError("%s: file ends before %d values" % (self.path, n))
            out.extend(list_directed_values(self.lines[self.row]))
            self.row += 1
        return out[:n]


def read_epwdata(path):
    """epwdata.fmt: (ef, nw, nwsk, nb, nwsq, nwsg, born_eps, Hwann (nwsk,nw,nw),
    Dphwann (nwsq,nb,nb)), with the READ statements of wannier.f90:314-346: one
    value per READ for H and D, whole lists for the header and Born / epsilon."""
    rd = _ListDirected(path)
    ef = float(np.real(rd.read(1)[0]))
    nw, nwsk, nb, nwsq, nwsg = (int(np.real(x)) for x in rd.read(5))
    born_eps = np.real(np.array(rd.read((nb // 3 + 1) * 9), dtype=complex))
    if all(len(list_directed_values(line)) <= 1 for line in rd.lines[rd.row:rd.row + 4]):
        # one value per record, the layout EPW writes: read the rest at once
        vals = []
        for line in rd.lines[rd.row:]:
            vals.extend(list_directed_values(line)[:1])
        need = nw * nw * nwsk + nb * nb * nwsq
        if len(vals) < need:
            raise ValueError("%s: %d values for H and D, %d needed" % (path, len(vals), need))
        H = np.array(vals[:nw * nw * nwsk], dtype=np.complex128)
        D = np.array(vals[nw * nw * nwsk:need], dtype=np.complex128)
    else:
        H = np.array([rd.read(1)[0] for _ in range(nw * nw * nwsk)], dtype=np.complex128)
        D = np.array([rd.read(1)[0] for _ in range(nb * nb * nwsq)], dtype=np.complex128)
    # loop order ib, jb, iuc with iuc innermost: Hwann(iuc, ib, jb) -> C order (ib, jb, iuc)
    Hwann = np.asfortranarray(H.reshape(nw, nw, nwsk).transpose(2, 0, 1))
    Dphwann = np.asfortranarray(D.reshape(nb, nb, nwsq).transpose(2, 0, 1))
    return ef, nw, nwsk, nb, nwsq, nwsg, born_eps, Hwann, Dphwann


def _fmt_real(x):
    return "%26.17E" % x


def _fmt_complex(z):
    return " (%s,%s)" % (_fmt_real(z.real).strip(), _fmt_real(z.imag).strip())


def write_epwdata(path, ef, Hwann, Dphwann, nwsg, born=None, epsilon=None):
    """epwdata.fmt in list-directed style (one record per value after the header)."""
    nwsk, nw, _ = Hwann.shape
    nwsq, nb, _ = Dphwann.shape
    nat = nb // 3
    be = np.zeros((nat + 1) * 9)
    if born is not None:
        be[:9 * nat] = np.asarray(born, dtype=float).reshape(-1, order="F")
    if epsilon is not None:
        be[9 * nat:] = np.asarray(epsilon, dtype=float).reshape(-1, order="F")
    with open(path, "w") as f:
        f.write(_fmt_real(ef) + "\n")
        f.write("%12d%12d%12d%12d%12d\n" % (nw, nwsk, nb, nwsq, nwsg))
        for i in range(0, len(be), 3):
            f.write("".join(_fmt_real(x) for x in be[i:i + 3]) + "\n")
        for ib in range(nw):
            for jb in range(nw):
                f.write("\n".join(_fmt_complex(z) for z in Hwann[:, ib, jb]) + "\n")
        for ib in range(nb):
            for jb in range(nb):
                f.write("\n".join(_fmt_complex(z) for z in Dphwann[:, ib, jb]) + "\n")


def _read_ints(path, ncol):
    a = np.loadtxt(path, dtype=np.int64, ndmin=2)
    return a[:, :ncol] if ncol > 1 else a[:, 0]


def read_epw_wannier(dirpath, crystal, coarse_qmesh):
    """The Wannier data of an EPW run (read_EPW_Wannier, wannier.f90:289-428) as
    ``synthetic.WannierData``; the crystal and the coarse phonon mesh come from
    the elphbolt input, as in the reference (crystal.f90, numerics qmesh).
    Returns (wannier_data, ef, born_eps) -- the last two read but, as in the
    reference, not used on the path."""
    ef, nw, nwsk, nb, nwsq, nwsg, born_eps, H, D = read_epwdata(os.path.join(dirpath, "epwdata.fmt"))
    g = np.fromfile(os.path.join(dirpath, "epmatwp1"), dtype=np.complex128)
    if g.size != nw * nw * nwsk * nb * nwsg:
        raise ValueError("epmatwp1: %d values, expected %d" % (g.size, nw * nw * nwsk * nb * nwsg))
    gwann = np.asfortranarray(g.reshape((nw, nw, nwsk, nb, nwsg), order="F"))
    rk = _read_ints(os.path.join(dirpath, "rcells_k"), 3)
    rq = _read_ints(os.path.join(dirpath, "rcells_q"), 3)
    rg = _read_ints(os.path.join(dirpath, "rcells_g"), 3)
    dk = _read_ints(os.path.join(dirpath, "wsdeg_k"), 1)
    dq = _read_ints(os.path.join(dirpath, "wsdeg_q"), 1)
    dg = _read_ints(os.path.join(dirpath, "wsdeg_g"), 1)
    for name, a, n in (("rcells_k", rk, nwsk), ("rcells_q", rq, nwsq), ("rcells_g", rg, nwsg),
                       ("wsdeg_k", dk, nwsk), ("wsdeg_q", dq, nwsq), ("wsdeg_g", dg, nwsg)):
        if len(a) != n:
            raise ValueError("%s: %d cells, epwdata.fmt says %d" % (name, len(a), n))
    wd = S.WannierData(crystal=crystal, numwannbands=nw, numbranches=nb,
                       coarse_qmesh=np.asarray(coarse_qmesh, dtype=np.int64),
                       rcells_k=rk, rcells_q=rq, rcells_g=rg, elwsdeg=dk, phwsdeg=dq, gwsdeg=dg,
                       Hwann=H, Dphwann=D, gwann=gwann)
    return wd, ef, born_eps


def write_epw_wannier(dirpath, wd, ef=0.0, born=None, epsilon=None):
    """The EPW files of a Wannier data set (the inverse of read_epw_wannier)."""
    os.makedirs(dirpath, exist_ok=True)
    write_epwdata(os.path.join(dirpath, "epwdata.fmt"), ef, np.asarray(wd.Hwann), np.asarray(wd.Dphwann),
                  wd.nwsg, born, epsilon)
    np.asfortranarray(wd.gwann, dtype=np.complex128).reshape(-1, order="F").tofile(os.path.join(dirpath, "epmatwp1"))
    for name, a in (("rcells_k", wd.rcells_k), ("rcells_q", wd.rcells_q), ("rcells_g", wd.rcells_g)):
        with open(os.path.join(dirpath, name), "w") as f:
            for r in np.asarray(a):
                f.write("%10d %10d %10d \n" % tuple(int(x) for x in r))
    for name, a in (("wsdeg_k", wd.elwsdeg), ("wsdeg_q", wd.phwsdeg), ("wsdeg_g", wd.gwsdeg)):
        with open(os.path.join(dirpath, name), "w") as f:
            for d in np.asarray(a):
                f.write("%10d \n" % int(d))


# ------------------------------------------------------------ per-state stream files
def _write_stream(path, count, *arrays):
    with open(path, "wb") as f:
        np.array([count], dtype=np.int64).tofile(f)
        for a, dt in arrays:
            np.ascontiguousarray(a, dtype=dt).tofile(f)


def write_gk2_istate(dirpath, istate, g2, g2_istate=None):
    """gk2.istate<n> as the ibzk 'g' pass writes it (interactions.f90:2337-2348):
    int64 count, then the whole g2_istate buffer -- not 1:count.  The buffer is
    allocated once per image with nprocs = nstates_inwindow * numbranches
    entries and zeroed once (:2146-2148); each state overwrites 1:count, so
    entries past count keep an earlier state's values.  ``g2_istate``, if given,
    is that running buffer (updated in place); otherwise the file holds count
    values.  With q on the k mesh (mesh_ref = 1) every window k' is a final
    state of every initial state, so count = nprocs and both agree."""
    g2 = np.asarray(g2, dtype=np.float64)
    if g2_istate is None:
        _write_stream(os.path.join(dirpath, "gk2.istate%d" % istate), len(g2), (g2, np.float64))
        return
    if len(g2) > len(g2_istate):
        raise ValueError("count %d exceeds the g2_istate buffer (%d)" % (len(g2), len(g2_istate)))
    g2_istate[:len(g2)] = g2
    _write_stream(os.path.join(dirpath, "gk2.istate%d" % istate), len(g2), (g2_istate, np.float64))


def write_gq2_istate(dirpath, istate, g2):
    _write_stream(os.path.join(dirpath, "gq2.istate%d" % istate), len(g2), (g2, np.float64))


def write_X_istate(dirpath, istate, xplus, xminus, istate_el, istate_ph):
    for name, x in (("Xplus", xplus), ("Xminus", xminus)):
        _write_stream(os.path.join(dirpath, "%s.istate%d" % (name, istate)), len(x), (x, np.float64),
                      (istate_el, np.int64), (istate_ph, np.int64))


def write_Y_istate(dirpath, istate, y, istate1, istate2):
    _write_stream(os.path.join(dirpath, "Y.istate%d" % istate), len(y), (y, np.float64), (istate1, np.int64),
                  (istate2, np.int64))


def read_istate(path, with_indices=False):
    """A per-state file: (count, values[, istate_a, istate_b]) -- what
    read_transition_probs_e (interactions.f90:3065-3091) and the 'X' / 'Y'
    passes read back."""
    with open(path, "rb") as f:
        count = int(np.fromfile(f, dtype=np.int64, count=1)[0])
        v = np.fromfile(f, dtype=np.float64, count=count)
        if not with_indices:
            return count, v
        a = np.fromfile(f, dtype=np.int64, count=count)
        b = np.fromfile(f, dtype=np.int64, count=count)
        return count, v, a, b


# ------------------------------------------------------------ dumps of library results
def dump_el_side(wann, req, g2dir, xdir, precision=None):
    """Run the electron side once (ephg_el_rates with vertex lists) and write the
    files the ibzk 'g' and 'X' passes write: gk2.istate<n> into g2dir and
    Xplus / Xminus.istate<n> into xdir, n the IBZ-blocks state index
    (demux_state order, interactions.f90:2169-2191).  Returns the rates."""
    from . import _lib
    from .interactions import _window
    if precision is None:
        precision = _lib.PREC_FP64
    out = wann.el_rates(req, precision=precision, vertices=True)
    nw, nb = wann.numwannbands, wann.numbranches
    idx = out["indexlist"]
    win = _window(wann, req, idx)
    mesh = np.asarray(req.mesh)
    nin = int(win.sum())
    per = nin * nb
    kint = np.stack([(idx - 1) % mesh[0], ((idx - 1) // mesh[0]) % mesh[1], (idx - 1) // (mesh[0] * mesh[1])], 1)
    ikp, n = np.nonzero(win)                                    # final states (window k', band), in order
    os.makedirs(g2dir, exist_ok=True)
    os.makedirs(xdir, exist_ok=True)
    g2_istate = np.zeros(nin * nb)                             # nprocs = nstates_inwindow * numbranches
    j = 0
    for ik in range(len(idx)):
        for m in range(nw):
            if not win[ik, m]:
                continue
            istate = ik * nw + m + 1                            # mux_state(nw, m, ik)
            sl = slice(j * per, (j + 1) * per)
            dq = (kint[ikp] - kint[ik]) % mesh
            iq = dq[:, 0] + mesh[0] * (dq[:, 1] + mesh[1] * dq[:, 2]) + 1
            ist_el = np.repeat(ikp * nw + n + 1, nb)
            ist_ph = ((np.repeat(iq, nb) - 1) * nb + np.tile(np.arange(1, nb + 1), len(iq)))
            write_gk2_istate(g2dir, istate, out["g2"][sl], g2_istate)
            write_X_istate(xdir, istate, out["xp"][sl], out["xm"][sl], ist_el, ist_ph)
            j += 1
    return out


def el_rates_from_files(xdir, nwv, nw):
    """calculate_el_rta_rates from the X files (interactions.f90:2958-3063 with
    read_transition_probs_e): rate(ik, m) = sum X+ + sum X-."""
    rates = np.zeros((nwv, nw))
    for ik in range(nwv):
        for m in range(nw):
            p = os.path.join(xdir, "Xplus.istate%d" % (ik * nw + m + 1))
            if not os.path.exists(p):
                continue
            _, xp = read_istate(p)
            _, xm = read_istate(os.path.join(xdir, "Xminus.istate%d" % (ik * nw + m + 1)))
            rates[ik, m] = xp.sum() + xm.sum()
    return rates


def dump_ph_side(wann, req, g2dir, ydir, spindeg=2, precision=None):
    """Run the phonon side once (ephg_ph_rates with vertex lists) and write the
    ibzq 'g' and 'Y' files: gq2.istate<n> and Y.istate<n>, n = (iq - 1) * nb + s
    over every q of the mesh.  Returns the phonon rates."""
    from . import _lib
    from .interactions import calculate_eph_interaction_ibzq
    if precision is None:
        precision = _lib.PREC_FP64
    g2, iph = calculate_eph_interaction_ibzq(wann, req, "g", precision=precision)
    y, i1, i2, iph2 = calculate_eph_interaction_ibzq(wann, req, "Y", precision=precision)
    os.makedirs(g2dir, exist_ok=True)
    os.makedirs(ydir, exist_ok=True)
    nstates = int(np.prod(req.mesh)) * wann.numbranches
    bounds = np.searchsorted(iph, np.arange(1, nstates + 2))
    for st in range(1, nstates + 1):
        a, b = bounds[st - 1], bounds[st]
        write_gq2_istate(g2dir, st, g2[a:b])
        write_Y_istate(ydir, st, y[a:b], i1[a:b], i2[a:b])
    return wann.ph_rates(req, precision=precision, spindeg=spindeg)["rates_phe"]


def ph_rates_from_files(ydir, nq, nb, spindeg=2):
    """The ph-e part of calculate_ph_rta_rates from the Y files (:2723-2828)."""
    rates = np.zeros((nq, nb))
    for iq in range(nq):
        for s in range(nb):
            _, y = read_istate(os.path.join(ydir, "Y.istate%d" % (iq * nb + s + 1)))
            rates[iq, s] = np.sum(spindeg * y)
    return rates
