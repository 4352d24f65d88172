"""Crystal symmetry and irreducible wedges (``src/symmetry.f90``) through the C ABI.

Host-only entry points of the library (no device needed):

* ``crystal_symmetry`` -- the space-group operations of a crystal, what
  ``spg_get_dataset`` gives ``calculate_symmetries`` (symmetry.f90:66-110);
* ``irred_wedge`` -- ``find_irred_wedge`` + ``create_fbz2ibz_map``
  (symmetry.f90:303-452, 480-503) for a mesh and a rotation set.

``Wannier.set_symmetry(rotations)`` hands the rotations to a device handle, so
that rate requests take initial states on the irreducible wedge.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib
from ._lib import c_dp, c_i64p, check


def _p(a, t=c_dp):
    return a.ctypes.data_as(t) if a is not None else None


def crystal_symmetry(crystal, atomtypes=None, symprec=1e-5):
    """(rotations (nops,3,3) int, translations (nops,3)) with x' = W x + t in
    crystal coordinates.  ``atomtypes`` defaults to one type per distinct mass."""
    L = _lib.load()
    A = np.asfortranarray(crystal.lattvecs, dtype=np.float64)
    B = np.asfortranarray(crystal.basis, dtype=np.float64)
    nat = B.shape[1]
    if atomtypes is None:
        _, atomtypes = np.unique(np.asarray(crystal.masses), return_inverse=True)
    t = np.ascontiguousarray(atomtypes, dtype=np.int64)
    maxops = 192
    rot = np.zeros(9 * maxops, dtype=np.int64)
    tr = np.zeros(3 * maxops)
    n = ct.c_int64()
    check(L.ephg_crystal_symmetry(_p(A), nat, _p(B), _p(t, c_i64p), float(symprec), maxops, ct.byref(n),
                                  _p(rot, c_i64p), _p(tr)))
    n = n.value
    R = rot[:9 * n].reshape(n, 3, 3).transpose(0, 2, 1)   # column-major 3x3 -> W[i, j]
    return np.ascontiguousarray(R), tr[:3 * n].reshape(n, 3).copy()


def rotations_fortran(R):
    """(nops,3,3) W[i, j] -> the (3,3,nops) column-major array the ABI takes."""
    R = np.asarray(R, dtype=np.int64)
    return np.asfortranarray(np.transpose(R, (1, 2, 0)))


def irred_wedge(lattvecs, rotations, mesh, indexlist=None):
    """find_irred_wedge: (indexlist_irred, nequiv, fbz2ibz), all 1-based, for the
    mesh (``indexlist`` None) or its sorted 1-based points ``indexlist``."""
    L = _lib.load()
    A = np.asfortranarray(lattvecs, dtype=np.float64)
    R = rotations_fortran(rotations) if len(rotations) else np.zeros((3, 3, 0), dtype=np.int64, order="F")
    m = np.ascontiguousarray(mesh, dtype=np.int64)
    n = int(np.prod(m)) if indexlist is None else len(indexlist)
    idx = None if indexlist is None else np.ascontiguousarray(indexlist, dtype=np.int64)
    irr = np.zeros(n, dtype=np.int64)
    neq = np.zeros(n, dtype=np.int64)
    f2i = np.zeros(n, dtype=np.int64)
    nirr = ct.c_int64()
    check(L.ephg_irred_wedge(_p(A), R.shape[2], _p(R, c_i64p), _p(m, c_i64p), n, _p(idx, c_i64p) if idx is not None
                             else None, ct.byref(nirr), _p(irr, c_i64p), _p(neq, c_i64p), _p(f2i, c_i64p)))
    k = nirr.value
    return irr[:k].copy(), neq[:k].copy(), f2i
