"""Host-side mirror of elphbolt's e-ph drivers (``src/interactions.f90``).

The reference runs the chain as separate passes that talk through files:

* ``calculate_gkRp`` (:1632) writes ``gkRp.ik<ik>``;
* ``calculate_eph_interaction_ibzk(..., 'g')`` (:2095) writes ``gk2.istate<n>``;
* ``calculate_eph_interaction_ibzk(..., 'X')`` writes ``Xplus/Xminus.istate<n>``;
* ``calculate_el_rta_rates`` (:2958) sums them into ``rta_rates_eph(nwv_irred, nw)``.

Here the whole chain is one device-resident call (``ephg_el_rates``).  The
per-pass functions below return what the reference writes to disk, in the
same order (initial state, k', n in window, s), for callers that consume the
lists (e.g. the Eliashberg path reads ``gk2.istate*``).

The phonon side mirrors it:

* ``calculate_gReq`` (:1603) writes ``gReq.iq<iq>``;
* ``calculate_eph_interaction_ibzq(..., 'g')`` (:1673) writes ``gq2.istate<n>``;
* ``calculate_eph_interaction_ibzq(..., 'Y')`` or ``calculate_Y_OTF`` (:1932)
  give ``Y.istate<n>``;
* ``calculate_ph_rta_rates`` (:2723) sums them into ``rta_rates_phe(nwv_irred, nb)``.

With the identity point group and q mesh = k mesh the phonon side visits the
electron side's vertices ((k, m, k + q, n, s) of phonon state (q, s) is
(k, m, k', n, s) with k' = k + q), so ``ephg_ph_rates`` forms both in one
sweep; ``ibzq_order`` maps its vertex lists to the reference's phonon order.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def calculate_el_rta_rates(wann, req, precision=_lib.PREC_FP64):
    """RTA e-ph rates (nwv, nw) in THz for the window k-points of ``req``.

    Returns ``(rates, indexlist, stats)``: rates(ik, m) for the ik-th window
    k-point (muxed mesh index ``indexlist[ik]``, 1-based) and band m; bands
    outside the window carry 0 as in the reference.
    """
    out = wann.el_rates(req, precision=precision)
    return out["rates"], out["indexlist"], out["stats"]


def calculate_eph_interaction_ibzk(wann, req, key, precision=_lib.PREC_FP64, cap=None):
    """'g' -> |g|^2 list (eV^2); 'X' -> (X+, X-) lists (THz), reference order."""
    if key not in ("g", "X"):
        raise _lib.EphgError(_lib.EPHG_ERR_ARG,
                             "Invalid value of key in call to calculate_eph_interaction_ibzk. Exiting.")
    out = wann.el_rates(req, precision=precision, vertices=True, cap=cap)
    if key == "g":
        return out["g2"]
    return out["xp"], out["xm"]


def ibzq_order(indexlist, window, mesh, nb):
    """Reference order of the phonon side's vertices.

    ``indexlist``: muxed 1-based indices of the window k-points; ``window``:
    (nwv, nw) bool, band b of window k-point ik inside the energy window.
    The electron side lists its vertices by initial state (ik, m), k', n, s;
    the reference's phonon side by phonon state istate = (iq - 1) * nb + s,
    then k, m, n (interactions.f90:1746-1880).  Returns ``(order, istate_ph,
    istate1, istate2)``: ``lst[order]`` is an electron-order list in phonon
    order, and per vertex in phonon order the phonon state and the initial /
    final electron states (mux_state(nw, m, ik), misc.f90:965, as written to
    ``Y.istate*``)."""
    idx = np.asarray(indexlist, dtype=np.int64) - 1
    window = np.asarray(window, dtype=bool)
    mesh = np.asarray(mesh, dtype=np.int64)
    nwv, nw = window.shape
    kint = np.stack([idx % mesh[0], (idx // mesh[0]) % mesh[1], idx // (mesh[0] * mesh[1])], 1)
    ik, m = np.nonzero(window)                       # window states, ik-major (demux_state order)
    nst = len(ik)
    # electron order: state j, final state f (same window-state list), s
    J = np.repeat(np.arange(nst), nst)
    F = np.tile(np.arange(nst), nst)
    dq = (kint[ik[F]] - kint[ik[J]]) % mesh
    iq = dq[:, 0] + mesh[0] * (dq[:, 1] + mesh[1] * dq[:, 2])              # 0-based muxed q
    iqv = np.repeat(iq, nb)
    sv = np.tile(np.arange(nb), nst * nst)
    ikv, mv = np.repeat(ik[J], nb), np.repeat(m[J], nb)
    nv = np.repeat(m[F], nb)
    ikpv = np.repeat(ik[F], nb)
    order = np.lexsort((nv, mv, ikv, sv, iqv))
    istate_ph = iqv[order] * nb + sv[order] + 1
    istate1 = ikv[order] * nw + mv[order] + 1
    istate2 = ikpv[order] * nw + nv[order] + 1
    return order, istate_ph, istate1, istate2


def _window(wann, req, indexlist):
    """Window bands of the window k-points, from the library's el_wann."""
    mesh = np.asarray(req.mesh)
    i = np.asarray(indexlist) - 1
    k = np.stack([i % mesh[0], (i // mesh[0]) % mesh[1], i // (mesh[0] * mesh[1])], 1) / mesh
    e = wann.el_wann(kvecs=k)
    return np.abs(e - req.enref) <= req.fsthick


def calculate_ph_rta_rates(wann, req, spindeg=2, precision=_lib.PREC_FP64):
    """The ph-e part of calculate_ph_rta_rates (interactions.f90:2723-2828):
    rta_rates_phe (N, nb) in THz for every q of the mesh (identity point group:
    the IBZ phonons are the mesh), row iq - 1 = muxed q index iq.  The 3-phonon
    part is not on this path.  Returns ``(rates_phe, stats)``."""
    out = wann.ph_rates(req, precision=precision, spindeg=spindeg)
    return out["rates_phe"], out["stats"]


def calculate_eph_interaction_ibzq(wann, req, key, precision=_lib.PREC_FP64, cap=None):
    """'g' -> |g|^2 list (eV^2); 'Y' -> (Y (THz), istate1, istate2) lists, in
    the reference's phonon order, with the phonon state of every entry
    (``istate_ph``, the file tag of ``gq2.istate*`` / ``Y.istate*``)."""
    if key not in ("g", "Y"):
        raise _lib.EphgError(_lib.EPHG_ERR_ARG,
                             "Invalid value of key in call to calculate_eph_interaction_ibzq. Exiting.")
    out = wann.ph_rates(req, precision=precision, electrons=True, vertices=True, cap=cap)
    if cap is not None and out["vertices"] > cap:
        raise _lib.EphgError(_lib.EPHG_ERR_ARG, "calculate_eph_interaction_ibzq: cap below the vertex count")
    win = _window(wann, req, out["indexlist"])
    nst = int(win.sum())
    if nst != out["stats"]["nstates_inwindow"]:
        raise _lib.EphgError(_lib.EPHG_ERR_ARG, "calculate_eph_interaction_ibzq: window bands do not match")
    order, istate_ph, i1, i2 = ibzq_order(out["indexlist"], win, req.mesh, wann.numbranches)
    if key == "g":
        return out["g2"][order], istate_ph
    return out["y"][order], i1, i2, istate_ph
