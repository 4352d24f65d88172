"""Host-side mirror of elphbolt's electron e-ph drivers (``src/interactions.f90``).

The reference runs the chain as separate passes that talk through files:

* ``calculate_gkRp`` (:1632) writes ``gkRp.ik<ik>``;
* ``calculate_eph_interaction_ibzk(..., 'g')`` (:2095) writes ``gk2.istate<n>``;
* ``calculate_eph_interaction_ibzk(..., 'X')`` writes ``Xplus/Xminus.istate<n>``;
* ``calculate_el_rta_rates`` (:2958) sums them into ``rta_rates_eph(nwv_irred, nw)``.

Here the whole chain is one device-resident call (``ephg_el_rates``).  The
per-pass functions below return what the reference writes to disk, in the
same order (initial state, k', n in window, s), for callers that consume the
lists (e.g. the Eliashberg path reads ``gk2.istate*``).
"""
from __future__ import annotations

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
