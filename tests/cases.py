"""Small seeded workloads shared by the CPU and GPU tests.

Sizes are chosen so that the oracle's literal per-vertex path finishes in
seconds.  Each case fixes its window explicitly (enref, fsthick, chempot).
"""
import functools

import numpy as np

from elphbolt_gb300 import synthetic as S


@functools.lru_cache(maxsize=None)
def case(name):
    if name == "tiny":          # nw 4, 2 atoms, 2^3 WS supercell
        wd = S.make_wannier(S.make_crystal_si_like(), 4, supercell=(2, 2, 2), seed=11)
        mesh, win, shift = (4, 4, 4), 1.0, 0.3
    elif name == "si8":         # nw 8, 2 atoms, 3^3 WS supercell, odd mesh
        wd = S.make_wannier(S.make_crystal_si_like(), 8, supercell=(3, 3, 3), seed=12)
        mesh, win, shift = (5, 5, 5), 0.5, 0.6
    elif name == "sic":         # polar SiC-like crystal: the long-range terms on, nw 8, 3^3 WS supercell
        wd = S.make_wannier(S.make_crystal_sic_like(), 8, supercell=(3, 3, 3), seed=14)
        mesh, win, shift = (4, 4, 4), 0.6, 0.5
    elif name == "odd":         # nw 5 (odd Jacobi), 3 atoms (nb 9), non-cubic mesh
        rng = np.random.Generator(np.random.PCG64(7))
        crys = S.make_crystal_multi(3, rng)
        wd = S.make_wannier(crys, 5, supercell=(2, 2, 3), seed=13)
        mesh, win, shift = (3, 4, 5), 1.5, 0.0
    else:
        raise KeyError(name)
    req = S.si_like_request(wd, mesh, window=win, shift=shift)
    return wd, req


CASES = ["tiny", "si8", "odd", "sic"]
