"""Host-side mirror of elphbolt's ``type Wannier`` (``src/wannier.f90:46-93``).

Same procedure names and argument meaning as the reference, computed on the
GPU through the C ABI of ``libephg.so``:

==========================  =======================================
reference                   here
==========================  =======================================
``wann%read``               ``Wannier(wd)`` (upload once, resident)
``wann%el_wann``            ``Wannier.el_wann``
``wann%ph_wann``            ``Wannier.ph_wann``
``wann%gkRp``               ``Wannier.gkRp`` (returns gmixed; no file)
``wann%gReq``               ``Wannier.gReq`` (returns gmixed; no file)
``wann%g2``                 ``Wannier.g2`` / ``Wannier.g2_batch``
``wann%deallocate_wannier`` ``Wannier.deallocate_wannier``
==========================  =======================================

Arrays follow the reference's shapes (``kvecs(nk,3)``, ``energies(nk,nw)``,
``evecs(nk,nw,nw)`` with ``evecs[k,b,:]`` the eigenvector of band b, ...).
Where the reference stops with ``exit_with_message`` these raise ``EphgError``.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib
from ._lib import c_dp, c_i64p, check


def _f(a, dtype=np.float64):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def _p(a, t=c_dp):
    return a.ctypes.data_as(t) if a is not None else None


def _vecs(a, what, n=None):
    """Wave vectors (n, 3) in crystal coordinates as a column-major float64
    array; refuses a missing or misshaped array (the library reads n x 3)."""
    if a is None:
        raise ValueError("%s: wave vectors missing" % what)
    v = _f(np.atleast_2d(a))
    if v.ndim != 2 or v.shape[1] != 3:
        raise ValueError("%s: wave vectors must be (n, 3), got %s" % (what, v.shape))
    if n is not None and int(n) > v.shape[0]:
        raise ValueError("%s: %d wave vectors requested, %d given" % (what, int(n), v.shape[0]))
    return v


class Wannier:
    """Wannier data resident on the GPU behind one library handle."""

    def __init__(self, wd):
        L = _lib.load()
        if L.ephg_device_count() <= 0:
            raise _lib.EphgError(_lib.EPHG_ERR_CUDA, "no CUDA device visible (no CPU fallback)")
        c = wd.crystal
        self.numwannbands = int(wd.numwannbands)
        self.numbranches = int(wd.numbranches)
        self.nwsk, self.nwsq, self.nwsg = int(wd.nwsk), int(wd.nwsq), int(wd.nwsg)
        self.coarse_qmesh = np.asarray(wd.coarse_qmesh, dtype=np.int64)
        self.crystal = c
        keep = [_f(c.lattvecs), _f(c.basis), _f(c.masses),
                _f(wd.rcells_k, np.int64), _f(wd.rcells_q, np.int64), _f(wd.rcells_g, np.int64),
                _f(wd.elwsdeg, np.int64), _f(wd.phwsdeg, np.int64), _f(wd.gwsdeg, np.int64),
                _f(wd.Hwann, np.complex128), _f(wd.Dphwann, np.complex128),
                _f(wd.gwann, np.complex128)]
        d = _lib.WannierDesc()
        d.numwannbands, d.numbranches = self.numwannbands, self.numbranches
        d.nwsk, d.nwsq, d.nwsg, d.numatoms = self.nwsk, self.nwsq, self.nwsg, c.numatoms
        for i in range(3):
            d.coarse_qmesh[i] = int(self.coarse_qmesh[i])
        d.lattvecs, d.basis, d.masses = _p(keep[0]), _p(keep[1]), _p(keep[2])
        d.rcells_k, d.rcells_q, d.rcells_g = (_p(keep[i], c_i64p) for i in (3, 4, 5))
        d.elwsdeg, d.phwsdeg, d.gwsdeg = (_p(keep[i], c_i64p) for i in (6, 7, 8))
        d.Hwann, d.Dphwann, d.gwann = _p(keep[9]), _p(keep[10]), _p(keep[11])
        h = ct.c_void_p()
        check(L.ephg_create(ct.byref(d), ct.byref(h)))
        self._h = h
        self._L = L
        if getattr(c, "polar", False):
            self.set_polar(c.epsilon, c.born)

    def set_symmetry(self, rotations):
        """The crystal's real-space rotations (nops,3,3) (``ephg_set_symmetry``);
        None or an empty list: the identity only.  Rate requests then start
        from the irreducible window points (see include/ephg.h)."""
        from .symmetry import rotations_fortran
        if rotations is None or len(rotations) == 0:
            check(self._L.ephg_set_symmetry(self._h, 0, None))
            return
        R = rotations_fortran(rotations)
        check(self._L.ephg_set_symmetry(self._h, R.shape[2], _p(R, c_i64p)))

    def set_polar(self, epsilon, born):
        """crys%polar, epsilon (3,3), born (3,3,numatoms) (``ephg_set_polar``);
        epsilon None switches the long-range terms off."""
        if epsilon is None:
            check(self._L.ephg_set_polar(self._h, None, None))
            return
        e = _f(epsilon)
        b = _f(born)
        if e.shape != (3, 3) or b.shape != (3, 3, self.crystal.numatoms):
            raise ValueError("set_polar: epsilon must be (3,3) and born (3,3,numatoms)")
        check(self._L.ephg_set_polar(self._h, _p(e), _p(b)))

    # ---- wannier.f90:430 ----
    def el_wann(self, crys=None, nk=None, kvecs=None, velocities=False, evecs=False, scissor=None):
        """Energies (nk,nw) eV [, velocities (nk,nw,3) km/s] [, evecs (nk,nw,nw)]."""
        k = _vecs(kvecs, "el_wann", nk)
        nk = k.shape[0] if nk is None else int(nk)
        nw = self.numwannbands
        e = np.zeros((nk, nw), order="F")
        v = np.zeros((nk, nw, 3), order="F") if velocities else None
        ev = np.zeros((nk, nw, nw), dtype=np.complex128, order="F") if (evecs or velocities) else None
        sc = _f(scissor) if scissor is not None else None
        check(self._L.ephg_el_wann(self._h, nk, _p(k), _p(e), _p(v), _p(ev), _p(sc)))
        out = [e]
        if velocities:
            out.append(v)
        if evecs:
            out.append(ev)
        return out[0] if len(out) == 1 else tuple(out)

    # ---- wannier.f90:585 ----
    def ph_wann(self, crys=None, nq=None, qvecs=None, evecs=False, velocities=False):
        """Energies (nq,nb) eV [, evecs (nq,nb,nb)] [, velocities (nq,nb,3) km/s]."""
        q = _vecs(qvecs, "ph_wann", nq)
        nq = q.shape[0] if nq is None else int(nq)
        nb = self.numbranches
        e = np.zeros((nq, nb), order="F")
        ev = np.zeros((nq, nb, nb), dtype=np.complex128, order="F") if (evecs or velocities) else None
        v = np.zeros((nq, nb, 3), order="F") if velocities else None
        check(self._L.ephg_ph_wann(self._h, nq, _p(q), _p(e), _p(ev), _p(v)))
        out = [e]
        if evecs:
            out.append(ev)
        if velocities:
            out.append(v)
        return out[0] if len(out) == 1 else tuple(out)

    # ---- wannier.f90:1073 ----
    def gkRp(self, num=None, ik=None, kvec=None):
        """g(k,Rp) = gmixed(nw,nw,nb,nwsq) for one k, or (...,nk) for kvec (nk,3)."""
        k = _vecs(kvec, "gkRp")
        nk = k.shape[0]
        nw, nb = self.numwannbands, self.numbranches
        out = np.zeros((nw, nw, nb, self.nwsq, nk), dtype=np.complex128, order="F")
        check(self._L.ephg_gkRp(self._h, nk, _p(k), _p(out)))
        return out[..., 0] if np.ndim(kvec) == 1 else out

    # ---- wannier.f90:1134 ----
    def gReq(self, num=None, iq=None, qvec=None):
        """g(Re,q) = gmixed(nw,nw,nb,nwsk) for one q, or (...,nq)."""
        q = _vecs(qvec, "gReq")
        nq = q.shape[0]
        nw, nb = self.numwannbands, self.numbranches
        out = np.zeros((nw, nw, nb, self.nwsk, nq), dtype=np.complex128, order="F")
        check(self._L.ephg_gReq(self._h, nq, _p(q), _p(out)))
        return out[..., 0] if np.ndim(qvec) == 1 else out

    # ---- wannier.f90:903 ----
    def g2_batch(self, kvecs, qvecs, el_evec_k, el_evec_kp, ph_evec_q, ph_en, gmixed, gm_index,
                 wannspace="ph"):
        """|g|^2 (eV^2) for nv vertices; gmixed (...,ngm), gm_index 1-based (nv)."""
        ws = {"ph": _lib.WANNSPACE_PH, "el": _lib.WANNSPACE_EL}.get(wannspace)
        if ws is None:
            raise _lib.EphgError(_lib.EPHG_ERR_ARG, "Invalid value of wannspace in call to g2_epw. Exiting.")
        kv, qv = _vecs(kvecs, "g2"), _vecs(qvecs, "g2")
        nv = qv.shape[0]
        a = _f(np.atleast_2d(el_evec_k), np.complex128)
        b = _f(np.atleast_2d(el_evec_kp), np.complex128)
        c = _f(np.atleast_2d(ph_evec_q), np.complex128)
        en = _f(np.atleast_1d(ph_en))
        gm = _f(gmixed, np.complex128)
        if gm.ndim == 4:
            gm = gm[..., None]
        gi = np.ascontiguousarray(np.atleast_1d(gm_index), dtype=np.int64)
        nw, nb = self.numwannbands, self.numbranches
        if (kv.shape[0] != nv or a.shape != (nv, nw) or b.shape != (nv, nw) or c.shape != (nv, nb)
                or en.shape != (nv,) or gi.shape != (nv,) or gm.shape[:4] != (nw, nw, nb, gm.shape[3])):
            raise ValueError("g2_batch: inconsistent shapes for %d vertices" % nv)
        out = np.zeros(nv)
        check(self._L.ephg_g2(self._h, ws, nv, _p(kv), _p(qv), _p(a), _p(b), _p(c), _p(en),
                              gm.shape[-1], _p(gm), _p(gi, c_i64p), _p(out)))
        return out

    def g2(self, crys, kvec, qvec, el_evec_k, el_evec_kp, ph_evec_q, ph_en, gmixed, wannspace):
        return float(self.g2_batch(kvec, qvec, el_evec_k, el_evec_kp, ph_evec_q, ph_en,
                                   gmixed, [1], wannspace)[0])

    def kq_index(self, mesh, k_idx, kp_idx):
        """q(i,j) = muxed index of k'(j) - k(i) on the mesh (vector.f90:86-102)."""
        m = np.ascontiguousarray(mesh, dtype=np.int64)
        a = np.ascontiguousarray(k_idx, dtype=np.int64)
        b = np.ascontiguousarray(kp_idx, dtype=np.int64)
        out = np.zeros((len(a), len(b)), dtype=np.int64, order="F")
        check(self._L.ephg_kq_index(self._h, _p(m, c_i64p), len(a), _p(a, c_i64p), len(b),
                                    _p(b, c_i64p), _p(out, c_i64p)))
        return out

    def el_rates(self, req, precision=_lib.PREC_FP64, vertices=False, cap=None):
        """Fused ibzk 'g' + 'X' + RTA rates; see interactions.calculate_el_rta_rates."""
        r = _lib.RateRequest()
        for i in range(3):
            r.mesh[i] = int(req.mesh[i])
        r.enref, r.fsthick, r.chempot, r.T = req.enref, req.fsthick, req.chempot, req.T
        r.delta_kind, r.sigma, r.precision = int(req.delta_kind), float(req.sigma), int(precision)
        N = int(np.prod(req.mesh))
        nw = self.numwannbands
        rates = np.zeros((N, nw), order="F")
        idx = np.zeros(N, dtype=np.int64)
        st = _lib.RateStats()
        g2 = xp = xm = None
        c = 0
        if vertices:
            c = int(cap) if cap is not None else N * nw * N * nw * self.numbranches
            g2, xp, xm = np.zeros(c), np.zeros(c), np.zeros(c)
        check(self._L.ephg_el_rates(self._h, ct.byref(r), _p(rates), _p(idx, c_i64p),
                                    ct.byref(st), _p(g2), _p(xp), _p(xm), c))
        nwv = int(st.nwv)
        out = dict(nwv=nwv, indexlist=idx[:nwv].copy(), rates=np.asfortranarray(rates[:nwv]),
                   stats=st.as_dict(), nstates=int(st.nstates), vertices=int(st.vertices))
        if vertices:
            nv = min(int(st.vertices), c)
            out.update(g2=g2[:nv], xp=xp[:nv], xm=xm[:nv])
        return out

    def el_rates_sets(self, reqs, precision=_lib.PREC_FP64):
        """``el_rates`` for requests that differ only in T, sigma and chempot
        (``ephg_el_rates_sets``): one contraction, one rate epilogue per request.
        Returns one output per request, laid out as ``el_rates``'s; the
        indexlist and stats are common to all."""
        n = len(reqs)
        R = (_lib.RateRequest * n)(*[_rate_request(q, precision) for q in reqs])
        N = int(np.prod(reqs[0].mesh))
        nw = self.numwannbands
        rates = [np.zeros((N, nw), order="F") for _ in range(n)]
        RP = (c_dp * n)(*[_p(a) for a in rates])
        idx = np.zeros(N, dtype=np.int64)
        st = _lib.RateStats()
        check(self._L.ephg_el_rates_sets(self._h, n, R, RP, _p(idx, c_i64p), ct.byref(st)))
        nwv = int(st.nwv)
        return [dict(nwv=nwv, indexlist=idx[:nwv].copy(), rates=np.asfortranarray(r[:nwv]), stats=st.as_dict(),
                     nstates=int(st.nstates), vertices=int(st.vertices)) for r in rates]

    def average_degenerate(self, req, g2, mode=_lib.DEGAVG_MEAN, thres=1e-6):
        """Degenerate-subspace gauge fixing of an ``el_rates`` |g|^2 vertex list
        (``ephg_g2_average_degenerate``; plot_along_path, wannier.f90:1332-1384):
        returns the averaged copy.  ``mode``: ``DEGAVG_REFERENCE`` (the
        reference's in-place loops) or ``DEGAVG_MEAN`` (gauge-invariant means)."""
        r = _rate_request(req, _lib.PREC_FP64)
        out = np.array(g2, dtype=np.float64, copy=True)
        check(self._L.ephg_g2_average_degenerate(self._h, ct.byref(r), int(mode), float(thres), out.size, _p(out)))
        return out

    def ph_rates(self, req, precision=_lib.PREC_FP64, spindeg=2, electrons=False, vertices=False, cap=None):
        """Fused ibzq 'g' + 'Y' + ph-e RTA rates (``ephg_ph_rates``).

        Returns rates_phe (N, nb) in THz, row iq - 1 = the phonon of muxed q index
        iq; with ``electrons`` also the electron rates and window index list of
        the same sweep; with ``vertices`` the |g|^2 and Y lists in the electron
        side's vertex order (``interactions.ibzq_order`` maps them to the
        reference's phonon order)."""
        r = _lib.RateRequest()
        for i in range(3):
            r.mesh[i] = int(req.mesh[i])
        r.enref, r.fsthick, r.chempot, r.T = req.enref, req.fsthick, req.chempot, req.T
        r.delta_kind, r.sigma, r.precision = int(req.delta_kind), float(req.sigma), int(precision)
        N = int(np.prod(req.mesh))
        nw, nb = self.numwannbands, self.numbranches
        rph = np.zeros((N, nb), order="F")
        rates = np.zeros((N, nw), order="F") if electrons else None
        idx = np.zeros(N, dtype=np.int64) if electrons else None
        st = _lib.RateStats()
        g2 = y = None
        c = 0
        if vertices:
            c = int(cap) if cap is not None else N * nw * N * nw * nb
            g2, y = np.zeros(c), np.zeros(c)
        check(self._L.ephg_ph_rates(self._h, ct.byref(r), int(spindeg), _p(rph), _p(rates), _p(idx, c_i64p),
                                    ct.byref(st), _p(g2), _p(y), c))
        nwv = int(st.nwv)
        out = dict(nwv=nwv, rates_phe=rph, stats=st.as_dict(), vertices=int(st.vertices))
        if electrons:
            out.update(indexlist=idx[:nwv].copy(), rates=np.asfortranarray(rates[:nwv]))
        if vertices:
            nv = min(int(st.vertices), c)
            out.update(g2=g2[:nv], y=y[:nv])
        return out

    def deallocate_wannier(self, num=None):
        if getattr(self, "_h", None):
            self._L.ephg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.deallocate_wannier()
        except Exception:
            pass


def _rate_request(req, precision):
    r = _lib.RateRequest()
    for i in range(3):
        r.mesh[i] = int(req.mesh[i])
    r.enref, r.fsthick, r.chempot, r.T = req.enref, req.fsthick, req.chempot, req.T
    r.delta_kind, r.sigma, r.precision = int(req.delta_kind), float(req.sigma), int(precision)
    return r


def el_rates_batch(crystals, reqs, precision=_lib.PREC_SPLIT_TF32, nslots=8, grouped=True, budget=0,
                   raise_on_error=True):
    """The batched form (``ephg_el_rates_batch``): request i against crystal
    ``crystals[i]`` (a ``Wannier``; repeats allowed), all solved in one call.
    Returns (outputs, batch stats, status codes); output i is laid out as
    ``Wannier.el_rates``'s (None where the request failed)."""
    n = len(reqs)
    if len(crystals) != n or n == 0:
        raise ValueError("one crystal per request")
    L = _lib.load()
    R = (_lib.RateRequest * n)(*[_rate_request(q, precision) for q in reqs])
    H = (ct.c_void_p * n)(*[c._h for c in crystals])
    rates = [np.zeros((int(np.prod(q.mesh)), c.numwannbands), order="F") for q, c in zip(reqs, crystals)]
    idx = [np.zeros(int(np.prod(q.mesh)), dtype=np.int64) for q in reqs]
    RP = (c_dp * n)(*[_p(a) for a in rates])
    IP = (c_i64p * n)(*[_p(a, c_i64p) for a in idx])
    st = (_lib.RateStats * n)()
    status = (ct.c_int * n)()
    opts = _lib.BatchOpts(int(nslots), int(budget), 1 if grouped else 0)
    bs = _lib.BatchStats()
    rc = L.ephg_el_rates_batch(n, H, R, RP, IP, st, status, ct.byref(opts), ct.byref(bs))
    if rc != _lib.EPHG_OK and raise_on_error:
        check(rc)
    outs = []
    for i in range(n):
        if status[i] != _lib.EPHG_OK:
            outs.append(None)
            continue
        nwv = int(st[i].nwv)
        outs.append(dict(nwv=nwv, indexlist=idx[i][:nwv].copy(), rates=np.asfortranarray(rates[i][:nwv]),
                         stats=st[i].as_dict(), nstates=int(st[i].nstates), vertices=int(st[i].vertices)))
    return outs, bs.as_dict(), list(status)
