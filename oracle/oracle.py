"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this module; it is the checker for the CUDA library, never part of
the product path.  See ``ephg_oracle.h`` for the reference functions it
restates and its parity status.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libephg_oracle.so")
_lib = None

c_i64p = ct.POINTER(ct.c_int64)
c_dp = ct.POINTER(ct.c_double)


class OrWannier(ct.Structure):
    _fields_ = [("nw", ct.c_int64), ("nb", ct.c_int64), ("nwsk", ct.c_int64),
                ("nwsq", ct.c_int64), ("nwsg", ct.c_int64), ("natoms", ct.c_int64),
                ("coarse_qmesh", ct.c_int64 * 3),
                ("lattvecs", c_dp), ("basis", c_dp), ("masses", c_dp),
                ("rcells_k", c_i64p), ("rcells_q", c_i64p), ("rcells_g", c_i64p),
                ("elwsdeg", c_i64p), ("phwsdeg", c_i64p), ("gwsdeg", c_i64p),
                ("Hwann", c_dp), ("Dphwann", c_dp), ("gwann", c_dp),
                ("polar", ct.c_int64), ("epsilon", c_dp), ("born", c_dp)]


class OrRequest(ct.Structure):
    _fields_ = [("mesh", ct.c_int64 * 3), ("enref", ct.c_double), ("fsthick", ct.c_double),
                ("chempot", ct.c_double), ("T", ct.c_double), ("delta_kind", ct.c_int64),
                ("sigma", ct.c_double)]


# the elphbolt source tree (read only, for its vendored spglib): ELPHBOLT_REFERENCE
_REF_ROOT = os.environ.get("ELPHBOLT_REFERENCE", "/root/reference")
_SPGLIB = os.path.join(_HERE, "_ref", "libspglib_ref.so")


def build():
    """Compile the oracle with its Makefile (gcc, OpenMP), and the reference's
    own spglib into oracle/_ref/ where the reference tree is present."""
    subprocess.check_call(["make", "-s", "-C", _HERE])
    if os.path.isdir(os.path.join(_REF_ROOT, "thirdparty", "spglib", "src")) and not os.path.exists(_SPGLIB):
        subprocess.check_call(["make", "-s", "-C", _HERE, "ref", "REFROOT=" + _REF_ROOT])


def spglib_symmetry(lattvecs, basis, types, symprec=1e-5):
    """The reference's spglib (oracle/_ref, compiled from its vendored sources):
    spg_get_symmetry on the crystal, (rotations (n,3,3), translations (n,3)) with
    x' = W x + t; None where the reference tree was not there to compile it."""
    if not os.path.exists(_SPGLIB):
        return None
    # lazy binding: the magnetic-space-group functions of spglib.c refer to a
    # database file the vendored copy does not carry; they are never called
    L = ct.CDLL(_SPGLIB, mode=os.RTLD_LAZY)
    L.spg_get_symmetry.restype = ct.c_int
    nat = np.asarray(basis).shape[1]
    maxn = 192
    rot = np.zeros((maxn, 3, 3), dtype=np.intc)
    tr = np.zeros((maxn, 3))
    lat = np.ascontiguousarray(lattvecs, dtype=np.float64)        # lattice[i][j]: row i = i-th component
    pos = np.ascontiguousarray(np.asarray(basis, dtype=np.float64).T)
    typ = np.ascontiguousarray(types, dtype=np.intc)
    n = L.spg_get_symmetry(rot.ctypes.data_as(ct.c_void_p), tr.ctypes.data_as(ct.c_void_p), maxn,
                           lat.ctypes.data_as(ct.c_void_p), pos.ctypes.data_as(ct.c_void_p),
                           typ.ctypes.data_as(ct.c_void_p), nat, ct.c_double(symprec))
    return rot[:n].astype(np.int64), tr[:n].copy()


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ct.CDLL(_LIB_PATH)
        L.or_mux_vector.restype = ct.c_int64
        L.or_mux_state.restype = ct.c_int64
        L.or_binsearch.restype = ct.c_int64
        L.or_expm1.restype = ct.c_double
        L.or_expm1.argtypes = [ct.c_double]
        L.or_Bose.restype = ct.c_double
        L.or_Bose.argtypes = [ct.c_double, ct.c_double]
        L.or_Fermi.restype = ct.c_double
        L.or_Fermi.argtypes = [ct.c_double, ct.c_double, ct.c_double]
        L.or_g2.restype = ct.c_double
        L.or_g2.argtypes = [ct.c_void_p, c_dp, c_dp, c_dp, c_dp, c_dp, ct.c_double, c_dp, ct.c_int]
        L.or_delta_triang.restype = ct.c_double
        L.or_delta_tetra.restype = ct.c_double
        _lib = L
    return _lib


def _p(a, t=c_dp):
    return a.ctypes.data_as(t)


def _f64(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def _c128_view(a):
    a = np.asfortranarray(np.asarray(a, dtype=np.complex128))
    return a


class Wannier:
    """Oracle-side holder of one synthetic Wannier data set."""

    def __init__(self, wd):
        self.wd = wd
        c = wd.crystal
        self._keep = []

        def keep(a):
            self._keep.append(a)
            return a

        self.lattvecs = keep(_f64(c.lattvecs))
        self.basis = keep(_f64(c.basis))
        self.masses = keep(_f64(c.masses))
        self.rk = keep(np.asfortranarray(wd.rcells_k, dtype=np.int64))
        self.rq = keep(np.asfortranarray(wd.rcells_q, dtype=np.int64))
        self.rg = keep(np.asfortranarray(wd.rcells_g, dtype=np.int64))
        self.dk = keep(np.ascontiguousarray(wd.elwsdeg, dtype=np.int64))
        self.dq = keep(np.ascontiguousarray(wd.phwsdeg, dtype=np.int64))
        self.dg = keep(np.ascontiguousarray(wd.gwsdeg, dtype=np.int64))
        self.H = keep(_c128_view(wd.Hwann))
        self.D = keep(_c128_view(wd.Dphwann))
        self.G = keep(_c128_view(wd.gwann))
        s = OrWannier()
        s.nw, s.nb = wd.numwannbands, wd.numbranches
        s.nwsk, s.nwsq, s.nwsg = wd.nwsk, wd.nwsq, wd.nwsg
        s.natoms = c.numatoms
        for i in range(3):
            s.coarse_qmesh[i] = int(wd.coarse_qmesh[i])
        s.lattvecs, s.basis, s.masses = _p(self.lattvecs), _p(self.basis), _p(self.masses)
        s.rcells_k, s.rcells_q, s.rcells_g = _p(self.rk, c_i64p), _p(self.rq, c_i64p), _p(self.rg, c_i64p)
        s.elwsdeg, s.phwsdeg, s.gwsdeg = _p(self.dk, c_i64p), _p(self.dq, c_i64p), _p(self.dg, c_i64p)
        s.Hwann, s.Dphwann, s.gwann = _p(self.H), _p(self.D), _p(self.G)
        if getattr(c, "polar", False):
            self.eps = keep(_f64(c.epsilon))
            self.born = keep(_f64(c.born))
            s.polar, s.epsilon, s.born = 1, _p(self.eps), _p(self.born)
        self.s = s
        self.nw, self.nb = wd.numwannbands, wd.numbranches

    # ---- wannier.f90 restatements ----
    def el_wann(self, kvecs, evecs=True, velocities=False, scissor=None):
        k = _f64(kvecs).reshape(-1, 3, order="F") if np.ndim(kvecs) == 2 else _f64(np.atleast_2d(kvecs))
        nk = k.shape[0]
        e = np.zeros((nk, self.nw), order="F")
        v = np.zeros((nk, self.nw, self.nw), dtype=np.complex128, order="F") if evecs else None
        vel = np.zeros((nk, self.nw, 3), order="F") if velocities else None
        sc = _f64(scissor) if scissor is not None else None
        lib().or_el_wann(ct.byref(self.s), ct.c_int64(nk), _p(k), _p(e),
                         _p(v) if v is not None else None, _p(vel) if vel is not None else None,
                         _p(sc) if sc is not None else None)
        return e, v, vel

    def ph_wann(self, qvecs, evecs=True, velocities=False):
        q = _f64(np.atleast_2d(qvecs))
        nq = q.shape[0]
        e = np.zeros((nq, self.nb), order="F")
        v = np.zeros((nq, self.nb, self.nb), dtype=np.complex128, order="F") if evecs else None
        vel = np.zeros((nq, self.nb, 3), order="F") if velocities else None
        st = lib().or_ph_wann(ct.byref(self.s), ct.c_int64(nq), _p(q), _p(e),
                              _p(v) if v is not None else None, _p(vel) if vel is not None else None)
        return e, v, vel, st

    def dyn_nonanalytic(self, q_cart_bohr, velocities=False):
        """dyn_l (nb,nb) [, ddyn_l (nb,nb,3)] for q Cartesian in 1/bohr."""
        L = lib()
        L.or_dyn_nonanalytic.argtypes = [ct.c_void_p, c_dp, c_dp, c_dp]
        q = np.ascontiguousarray(q_cart_bohr, dtype=np.float64)
        d = np.zeros((self.nb, self.nb), dtype=np.complex128, order="F")
        dd = np.zeros((self.nb, self.nb, 3), dtype=np.complex128, order="F") if velocities else None
        L.or_dyn_nonanalytic(ct.byref(self.s), _p(q), _p(d), _p(dd) if dd is not None else None)
        return (d, dd) if velocities else d

    def long_range_prefac(self, q_cart_bohr, uqs):
        L = lib()
        L.or_long_range_prefac.argtypes = [ct.c_void_p, c_dp, c_dp, c_dp]
        q = np.ascontiguousarray(q_cart_bohr, dtype=np.float64)
        u = np.ascontiguousarray(uqs, dtype=np.complex128)
        out = np.zeros(1, dtype=np.complex128)
        L.or_long_range_prefac(ct.byref(self.s), _p(q), _p(u), _p(out))
        return complex(out[0])

    def q_cart_bohr(self, qf):
        L = lib()
        L.or_q_cart_bohr.argtypes = [ct.c_void_p, c_dp, c_dp]
        q = np.ascontiguousarray(qf, dtype=np.float64)
        out = np.zeros(3)
        L.or_q_cart_bohr(ct.byref(self.s), _p(q), _p(out))
        return out

    def gkRp(self, kvec):
        out = np.zeros((self.nw, self.nw, self.nb, self.wd.nwsq), dtype=np.complex128, order="F")
        k = np.ascontiguousarray(kvec, dtype=np.float64)
        lib().or_gkRp(ct.byref(self.s), _p(k), _p(out))
        return out

    def gReq(self, qvec):
        out = np.zeros((self.nw, self.nw, self.nb, self.wd.nwsk), dtype=np.complex128, order="F")
        q = np.ascontiguousarray(qvec, dtype=np.float64)
        lib().or_gReq(ct.byref(self.s), _p(q), _p(out))
        return out

    def g2(self, kvec, qvec, ev_k, ev_kp, ev_q, ph_en, gmixed, wannspace="ph"):
        a = [np.ascontiguousarray(x) for x in (kvec, qvec)]
        b = [np.ascontiguousarray(x, dtype=np.complex128) for x in (ev_k, ev_kp, ev_q)]
        gm = np.asfortranarray(gmixed, dtype=np.complex128)
        return lib().or_g2(ct.byref(self.s), _p(a[0]), _p(a[1]), _p(b[0]), _p(b[1]), _p(b[2]),
                           float(ph_en), _p(gm), 1 if wannspace == "ph" else 0)

    def el_rates(self, req, max_states=-1, nthreads=1, literal=True, vertices=False, cap=None):
        """Full 'g' + 'X' + rates driver; returns a dict of results."""
        r = OrRequest()
        for i in range(3):
            r.mesh[i] = int(req.mesh[i])
        r.enref, r.fsthick, r.chempot, r.T = req.enref, req.fsthick, req.chempot, req.T
        r.delta_kind, r.sigma = int(req.delta_kind), req.sigma
        N = int(np.prod(req.mesh))
        rates = np.zeros((N, self.nw), order="F")
        idx = np.zeros(N, dtype=np.int64)
        info = np.zeros(8, dtype=np.int64)
        g2 = xp = xm = None
        c = 0
        if vertices:
            c = int(cap) if cap is not None else N * self.nw * N * self.nw * self.nb
            g2, xp, xm = (np.zeros(c) for _ in range(3))
        st = lib().or_el_rates(ct.byref(self.s), ct.byref(r), ct.c_int64(max_states),
                               ct.c_int(nthreads), ct.c_int(1 if literal else 0), _p(rates),
                               _p(idx, c_i64p), _p(info, c_i64p),
                               _p(g2) if g2 is not None else None,
                               _p(xp) if xp is not None else None,
                               _p(xm) if xm is not None else None, ct.c_int64(c))
        nwv = int(info[0])
        out = dict(status=int(st), nwv=nwv, nstates_inwindow=int(info[1]),
                   nstates=int(info[2]), vertices=int(info[3]), pairs=int(info[4]),
                   indexlist=idx[:nwv].copy(), rates=np.asfortranarray(rates[:nwv, :]),
                   us_setup=int(info[6]), us_loop=int(info[7]))
        if vertices:
            nv = min(int(info[3]), c)
            out.update(g2=g2[:nv], xp=xp[:nv], xm=xm[:nv])
        return out


    def el_rates_sym(self, req, rotations, nthreads=1, literal=False, vertices=False, cap=None):
        """The rate driver with crystal symmetry (or_rates_setup_sym): rows are
        the irreducible window points (IBZ blocks)."""
        L = lib()
        L.or_rates_setup_sym.restype = ct.c_void_p
        L.or_rates_setup_sym.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int64, c_dp, ct.c_int]
        L.or_rates_run.argtypes = [ct.c_void_p, ct.c_int64, ct.c_int64, ct.c_int, ct.c_int, c_dp, c_i64p,
                                   c_i64p, c_dp, c_dp, c_dp, ct.c_int64]
        L.or_rates_free.argtypes = [ct.c_void_p]
        q = symmetry_qrotations(self.lattvecs, rotations, req.mesh)
        r = _request(req)
        N = int(np.prod(req.mesh))
        rates = np.zeros((N, self.nw), order="F")
        idx = np.zeros(N, dtype=np.int64)
        info = np.zeros(8, dtype=np.int64)
        c = 0
        g2 = xp = xm = None
        if vertices:
            c = int(cap) if cap is not None else N * self.nw * N * self.nw * self.nb
            g2, xp, xm = (np.zeros(c) for _ in range(3))
        ctx = L.or_rates_setup_sym(ct.byref(self.s), ct.byref(r), q.shape[2], _p(q), int(nthreads))
        try:
            st = L.or_rates_run(ctx, 0, -1, int(nthreads), 1 if literal else 0, _p(rates), _p(idx, c_i64p),
                                _p(info, c_i64p), _p(g2) if g2 is not None else None,
                                _p(xp) if xp is not None else None, _p(xm) if xm is not None else None, c)
        finally:
            L.or_rates_free(ctx)
        n = int(info[0])
        out = dict(status=int(st), nwv=n, nstates_inwindow=int(info[1]), nstates=int(info[2]),
                   vertices=int(info[3]), pairs=int(info[4]), indexlist=idx[:n].copy(),
                   rates=np.asfortranarray(rates[:n]), nsym=q.shape[2])
        if vertices:
            nv = min(int(info[3]), c)
            out.update(g2=g2[:nv], xp=xp[:nv], xm=xm[:nv])
        return out

    def ph_rates(self, req, spindeg=2, nthreads=1, vertices=False, cap=None):
        """ibzq 'g' + 'Y' and the ph-e RTA rates (or_ph_rates); rates_phe (N, nb)."""
        L = lib()
        L.or_ph_rates.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_double, ct.c_int, c_dp, c_i64p, c_dp, c_dp,
                                  ct.c_int64]
        r = _request(req)
        N = int(np.prod(req.mesh))
        rates = np.zeros((N, self.nb), order="F")
        info = np.zeros(8, dtype=np.int64)
        g2 = y = None
        c = 0
        if vertices:
            c = int(cap) if cap is not None else N * self.nb * N * self.nw * self.nw
            g2, y = np.zeros(c), np.zeros(c)
        st = L.or_ph_rates(ct.byref(self.s), ct.byref(r), float(spindeg), int(nthreads), _p(rates),
                           _p(info, c_i64p), _p(g2) if g2 is not None else None,
                           _p(y) if y is not None else None, ct.c_int64(c))
        out = dict(status=int(st), nwv=int(info[0]), nstates_inwindow=int(info[1]), nstates=int(info[2]),
                   vertices=int(info[3]), pairs=int(info[4]), rates_phe=rates, us_setup=int(info[6]),
                   us_loop=int(info[7]))
        if vertices:
            nv = min(int(info[3]), c)
            out.update(g2=g2[:nv], y=y[:nv])
        return out


def symmetry_qrotations(lattvecs, rotations, mesh):
    """or_symmetry_qrotations: the reciprocal rotations (3,3,n) kept for the mesh."""
    L = lib()
    L.or_symmetry_qrotations.restype = ct.c_int64
    L.or_symmetry_qrotations.argtypes = [c_dp, ct.c_int64, c_i64p, c_i64p, c_dp]
    A = _f64(lattvecs)
    R = np.asfortranarray(np.transpose(np.asarray(rotations, dtype=np.int64), (1, 2, 0)))
    m = np.ascontiguousarray(mesh, dtype=np.int64)
    q = np.zeros((3, 3, 2 * R.shape[2] + 1), order="F")
    n = L.or_symmetry_qrotations(_p(A), R.shape[2], _p(R, c_i64p), _p(m, c_i64p), _p(q))
    return np.asfortranarray(q[:, :, :n])


def irred_wedge(lattvecs, rotations, mesh, indexlist=None):
    """or_find_irred_wedge with the rotations kept for the mesh:
    (status, indexlist_irred, nequiv)."""
    L = lib()
    L.or_find_irred_wedge.argtypes = [c_i64p, ct.c_int64, c_dp, ct.c_int64, c_i64p, c_i64p, c_i64p, c_i64p, c_i64p]
    q = symmetry_qrotations(lattvecs, rotations, mesh)
    m = np.ascontiguousarray(mesh, dtype=np.int64)
    n = int(np.prod(m)) if indexlist is None else len(indexlist)
    idx = None if indexlist is None else np.ascontiguousarray(indexlist, dtype=np.int64)
    irr = np.zeros(n, dtype=np.int64)
    neq = np.zeros(n, dtype=np.int64)
    nir = ct.c_int64()
    st = L.or_find_irred_wedge(_p(m, c_i64p), q.shape[2], _p(q), n, _p(idx, c_i64p) if idx is not None else None,
                               ct.byref(nir), _p(irr, c_i64p), _p(neq, c_i64p), None)
    return st, irr[:nir.value].copy(), neq[:nir.value].copy()


def _request(req):
    r = OrRequest()
    for i in range(3):
        r.mesh[i] = int(req.mesh[i])
    r.enref, r.fsthick, r.chempot, r.T = req.enref, req.fsthick, req.chempot, req.T
    r.delta_kind, r.sigma = int(req.delta_kind), req.sigma
    return r


# ---- misc.f90 / vector.f90 restatements ----
def degenerate_group(values, energies, mode, thres=1e-6):
    """One group of the degenerate-subspace passes (or_degenerate_group)."""
    L = lib()
    L.or_degenerate_group.argtypes = [ct.c_int, ct.c_double, ct.c_int64, c_dp, ct.c_int64, c_dp, c_dp]
    v = np.array(values, dtype=np.float64, copy=True)
    e = np.ascontiguousarray(energies, dtype=np.float64)
    tmp = np.zeros(len(v))
    L.or_degenerate_group(int(mode), float(thres), len(v), _p(v), 1, _p(e), _p(tmp))
    return v


def mux_vector(v, mesh, base):
    a = (ct.c_int64 * 3)(*v)
    m = (ct.c_int64 * 3)(*mesh)
    return lib().or_mux_vector(a, m, ct.c_int64(base))


def demux_vector(i, mesh, base):
    v = (ct.c_int64 * 3)()
    m = (ct.c_int64 * 3)(*mesh)
    lib().or_demux_vector(ct.c_int64(i), v, m, ct.c_int64(base))
    return list(v)


def mux_state(nbands, iband, ik):
    return lib().or_mux_state(ct.c_int64(nbands), ct.c_int64(iband), ct.c_int64(ik))


def demux_state(m, nbands):
    ib, ik = ct.c_int64(), ct.c_int64()
    lib().or_demux_state(ct.c_int64(m), ct.c_int64(nbands), ct.byref(ib), ct.byref(ik))
    return ib.value, ik.value


def binsearch(array, e):
    a = np.ascontiguousarray(array, dtype=np.int64)
    return lib().or_binsearch(_p(a, c_i64p), ct.c_int64(len(a)), ct.c_int64(e))


def umklapp(q1, q2):
    a = np.ascontiguousarray(q1, dtype=np.float64)
    b = np.ascontiguousarray(q2, dtype=np.float64)
    c = np.zeros(3)
    lib().or_umklapp(_p(a), _p(b), _p(c))
    return c


def vector_create(ind, grid, prim):
    iv = (ct.c_int64 * 3)()
    mx = ct.c_int64()
    fr, ca = np.zeros(3), np.zeros(3)
    g = (ct.c_int64 * 3)(*grid)
    P = np.asfortranarray(prim, dtype=np.float64)
    lib().or_vector_create(ct.c_int64(ind), g, _p(P), iv, ct.byref(mx), _p(fr), _p(ca))
    return dict(int=list(iv), muxed=mx.value, frac=fr, cart=ca)


def vector_addsub(ind1, ind2, sign, grid, prim):
    iv = (ct.c_int64 * 3)()
    mx = ct.c_int64()
    fr, ca = np.zeros(3), np.zeros(3)
    g = (ct.c_int64 * 3)(*grid)
    P = np.asfortranarray(prim, dtype=np.float64)
    lib().or_vector_addsub(ct.c_int64(ind1), ct.c_int64(ind2), ct.c_int(sign), g, _p(P), iv,
                           ct.byref(mx), _p(fr), _p(ca))
    return dict(int=list(iv), muxed=mx.value, frac=fr, cart=ca)


def vector_change_grid(frac, grid):
    iv = (ct.c_int64 * 3)()
    mx = ct.c_int64()
    f = np.ascontiguousarray(frac, dtype=np.float64)
    g = (ct.c_int64 * 3)(*grid)
    lib().or_vector_change_grid(_p(f), g, iv, ct.byref(mx))
    return dict(int=list(iv), muxed=mx.value)


def expm1(x):
    return lib().or_expm1(float(x))


def Bose(e, T):
    return lib().or_Bose(float(e), float(T))


def Fermi(e, mu, T):
    return lib().or_Fermi(float(e), float(mu), float(T))


def herm_eig(A):
    A = np.asfortranarray(A, dtype=np.complex128)
    n = A.shape[0]
    w = np.zeros(n)
    V = np.zeros((n, n), dtype=np.complex128, order="F")
    sw = lib().or_herm_eig(ct.c_int64(n), _p(A), _p(w), _p(V))
    return w, V, sw


class RatesRun:
    """The oracle's rate driver with its set-up done once (or_rates_setup), so
    that a timed sample of initial states (or_rates_run) excludes it."""

    def __init__(self, W, req, nthreads=1):
        L = lib()
        L.or_rates_setup.restype = ct.c_void_p
        L.or_rates_setup.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int]
        L.or_rates_run.argtypes = [ct.c_void_p, ct.c_int64, ct.c_int64, ct.c_int, ct.c_int, c_dp, c_i64p,
                                   c_i64p, c_dp, c_dp, c_dp, ct.c_int64]
        L.or_rates_free.argtypes = [ct.c_void_p]
        self.W = W
        r = OrRequest()
        for i in range(3):
            r.mesh[i] = int(req.mesh[i])
        r.enref, r.fsthick, r.chempot, r.T = req.enref, req.fsthick, req.chempot, req.T
        r.delta_kind, r.sigma = int(req.delta_kind), req.sigma
        self.r = r
        self.N = int(np.prod(req.mesh))
        self.nthreads = nthreads
        self.ctx = L.or_rates_setup(ct.byref(W.s), ct.byref(r), nthreads)

    def run(self, state_begin, nstates, literal=True, vertices=False):
        N, nw = self.N, self.W.nw
        rates = np.zeros((N, nw), order="F")
        idx = np.zeros(N, dtype=np.int64)
        info = np.zeros(8, dtype=np.int64)
        cap = 0
        g2 = xp = xm = None
        if vertices:   # room for every vertex of the states asked for
            cap = N * nw * N * nw * self.W.nb if nstates < 0 else nstates * N * nw * self.W.nb
            g2, xp, xm = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        lib().or_rates_run(self.ctx, state_begin, nstates, self.nthreads, 1 if literal else 0, _p(rates),
                           _p(idx, c_i64p), _p(info, c_i64p), _p(g2) if vertices else None,
                           _p(xp) if vertices else None, _p(xm) if vertices else None, cap)
        nwv = int(info[0])
        out = dict(nwv=nwv, nstates_inwindow=int(info[1]), nstates=int(info[2]), vertices=int(info[3]),
                   status=int(info[5]), us_setup=int(info[6]), us_loop=int(info[7]),
                   rates=np.asfortranarray(rates[:nwv]), indexlist=idx[:nwv].copy())
        if vertices:
            nv = int(info[3])
            out.update(g2=g2[:nv].copy(), xp=xp[:nv].copy(), xm=xm[:nv].copy())
        return out

    def average_degenerate(self, g2, mode=1, thres=1e-6):
        """or_average_degenerate on a copy of an all-states |g|^2 list (mode 0:
        the reference's in-place loops, wannier.f90:1332-1384; 1: the means of
        the values before each pass)."""
        L = lib()
        L.or_average_degenerate.argtypes = [ct.c_void_p, ct.c_int, ct.c_double, c_dp, ct.c_int64]
        out = np.array(g2, dtype=np.float64, copy=True)
        if L.or_average_degenerate(self.ctx, int(mode), float(thres), _p(out), out.size):
            raise ValueError("the list is not the request's whole vertex list")
        return out

    def run_ph(self, q_begin, nq, spindeg=2):
        """Phonon-side states of the q-points [q_begin, q_begin + nq) (or_ph_rates_run)."""
        L = lib()
        L.or_ph_rates_run.argtypes = [ct.c_void_p, ct.c_int64, ct.c_int64, ct.c_int, ct.c_double, c_dp, c_i64p,
                                      c_dp, c_dp, ct.c_int64]
        rates = np.zeros((self.N, self.W.nb), order="F")
        info = np.zeros(8, dtype=np.int64)
        L.or_ph_rates_run(self.ctx, q_begin, nq, self.nthreads, float(spindeg), _p(rates), _p(info, c_i64p),
                          None, None, 0)
        return dict(nwv=int(info[0]), nstates=int(info[2]), vertices=int(info[3]), pairs=int(info[4]),
                    status=int(info[5]), us_setup=int(info[6]), us_loop=int(info[7]), rates_phe=rates)

    def close(self):
        if self.ctx:
            lib().or_rates_free(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
