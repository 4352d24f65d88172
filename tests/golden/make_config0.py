"""Generate tests/golden/golden_config0.npz (run from the repository root).

    python tests/golden/make_config0.py

The fixture pins the library at the CPU-runnable benchmark configuration
itself, not a shrunken test crystal: the seeded Si-like fcc crystal (nw 8,
nb 6, 279 Re / 279 Rp Wigner-Seitz cells of a 6x6x6 supercell), a 12x12x12
k = q mesh, window +-0.5 eV about mid-gap + 0.6 eV, Gaussian delta of 10 meV,
T = 300 K.  The oracle (oracle/ephg_oracle.c, the CPU FP64 restatement of
interactions.f90:2095-2400 and :2958-3063) computes the RTA rates of a
deterministic sample of initial states -- 16 runs of 8 consecutive states
spread over the window, each rate a full sum over every window k' -- in its
restructured form, after checking on the first run that the literal
per-vertex g2 form (wannier.f90:903-1011) agrees to 1e-12.

Stored: the request's parameters (so that the test does not recompute the
window centre from the band structure), the window k-point list, and the
sampled states' (row, band) positions, energies and rates.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from elphbolt_gb300 import synthetic as S  # noqa: E402

MESH = (12, 12, 12)
RUNS, PER_RUN = 16, 8


def window_states(ens, enref, fsthick):
    """(row, band) of every in-window initial state in istate order
    (demux_state: band fastest, interactions.f90:2169-2191)."""
    rows, bands = np.nonzero(np.abs(ens - enref) <= fsthick)
    return rows, bands


def main():
    from oracle import oracle as O
    O.build()
    wd = S.si_like()
    req = S.si_like_request(wd, MESH)
    W = O.Wannier(wd)
    nthreads = os.cpu_count() or 1
    t0 = time.time()
    R = O.RatesRun(W, req, nthreads=nthreads)
    a = R.run(0, 1)
    nst = a["nstates_inwindow"] if "nstates_inwindow" in a else None
    idx = a["indexlist"]
    nwv = len(idx)
    i = idx - 1
    m = np.asarray(MESH)
    kf = np.stack([i % m[0], (i // m[0]) % m[1], i // (m[0] * m[1])], 1) / m
    ens, _, _ = W.el_wann(kf, evecs=False)
    rows, bands = window_states(ens, req.enref, req.fsthick)
    nstates = len(rows)
    starts = np.linspace(0, nstates - PER_RUN, RUNS).astype(np.int64)
    rates = np.zeros((nwv, wd.numwannbands))
    for r, s0 in enumerate(starts):
        out = R.run(int(s0), PER_RUN, literal=False)
        got = out["rates"]
        if r == 0:
            lit = R.run(int(s0), PER_RUN, literal=True)["rates"]
            sel = got != 0
            rel = np.max(np.abs(lit[sel] - got[sel]) / np.abs(lit[sel]))
            assert rel < 1e-12, rel
            print("literal vs restructured on the first run: %.2e" % rel)
        rates += got
    R.close()
    pick = np.concatenate([np.arange(s0, s0 + PER_RUN) for s0 in starts])
    prow, pband = rows[pick], bands[pick]
    vals = rates[prow, pband]
    assert np.all(vals > 0), "a sampled state has no rate"
    mask = np.zeros_like(rates, dtype=bool)
    mask[prow, pband] = True
    assert np.all(rates[~mask] == 0), "the oracle computed states outside the sample"
    np.savez_compressed(os.path.join(HERE, "golden_config0.npz"),
                        mesh=m, enref=req.enref, fsthick=req.fsthick, chempot=req.chempot, T=req.T,
                        sigma=req.sigma, indexlist=idx, nstates=nstates, rows=prow, bands=pband,
                        ens=ens[prow, pband], rates=vals)
    print("config 0: %d window k, %d initial states, %d sampled, rates %.3e .. %.3e THz, %.1f s on %d threads"
          % (nwv, nstates, len(pick), vals.min(), vals.max(), time.time() - t0, nthreads))
    del nst


if __name__ == "__main__":
    main()
