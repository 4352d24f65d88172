"""Generate the golden fixtures of tests/golden/ (run from the repository root).

    python tests/golden/make_golden.py [el | ph | polar | all]

For each small seeded workload this script computes the e-ph path twice:
- with the C oracle (oracle/ephg_oracle.c, literal per-vertex g2);
- with an independent numpy restatement written here: vectorised,
  scipy/LAPACK eigensolver, and the reference's loop order only where it
  matters for the integer bookkeeping.

It checks that the two agree (energies 1e-10 eV, |g|^2 and rates 1e-10
relative) before writing:
- the request parameters;
- window energies, phonon energies, rates;
- a deterministic sample of |g|^2, X+ and X- vertices.

The reference ships no |g|^2 or rate vectors (its regression data is a network
download), so these fixtures pin the oracle against a second, independent
restatement of the same Fortran rather than against the reference's output.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from elphbolt_gb300 import constants as C  # noqa: E402
from elphbolt_gb300 import synthetic as S  # noqa: E402


# ---------------------------------------------------------------- numpy path
def np_el_wann(wd, k):
    """H(k) (wannier.f90:466-486) diagonalised with LAPACK: energies (eV), U[k,b,:]."""
    ph = np.exp(2j * np.pi * (k @ wd.rcells_k.T)) / wd.elwsdeg[None, :]
    H = np.einsum("kr,rij->kij", ph, np.asarray(wd.Hwann))
    Hu = np.triu(H, 1)
    H = Hu + np.conj(np.transpose(Hu, (0, 2, 1))) + np.einsum("kii->ki", H).real[:, :, None] * np.eye(H.shape[1])
    w, V = np.linalg.eigh(H)
    return w * C.Ryd2eV, np.transpose(V, (0, 2, 1))


def np_polar(crys, nqc):
    """The polar long-range terms, vectorised over the G box (wannier.f90:784-901,
    1013-1071): returns dyn(q) -> (nb, nb) and lvec(q) -> (nb,), q Cartesian in
    1/bohr, with long_range_prefac(q, u) = lvec(q) @ u."""
    rec, vol = crys.reclattvecs, crys.volume
    bc = crys.lattvecs @ crys.basis                                # nm
    nat = crys.numatoms
    nb = 3 * nat
    tpiba = 2 * math.pi / np.linalg.norm(crys.lattvecs[:, 0]) * C.bohr2nm
    alph, gmax = tpiba ** 2, 14.0
    fac = 8 * math.pi / (vol / C.bohr2nm ** 3)
    r = [np.arange(-n, n + 1) for n in nqc]
    m = np.stack(np.meshgrid(*r, indexing="ij"), -1).reshape(-1, 3)
    G = (m @ rec.T) * C.bohr2nm
    eps, born = np.asarray(crys.epsilon), np.asarray(crys.born)
    rr = (bc[:, :, None] - bc[:, None, :]) / C.bohr2nm              # rr[:, i, j]

    def terms(g):
        qeq = np.einsum("gi,ij,gj->g", g, eps, g)
        sel = (qeq > 0) & (qeq / alph / 4 < gmax)
        g, qeq = g[sel], qeq[sel]
        f = np.exp(-qeq / alph / 4) / qeq
        Z = np.einsum("gi,ija->gaj", g, born)                        # (g, atom, j)
        ph = np.exp(1j * np.einsum("gd,dij->gij", g, rr))            # e^{i g.r_ij}
        return g, f, Z, ph

    _, fa, Za, pha = terms(G)
    fnat = np.einsum("gbj,gab->gaj", Za, pha)
    Da = np.zeros((nb, nb), dtype=complex)
    for a in range(nat):
        Da[3 * a:3 * a + 3, 3 * a:3 * a + 3] -= np.einsum("g,gi,gj->ij", fa, Za[:, a, :], fnat[:, a, :])

    def dyn(q):
        _, f, Z, ph = terms(G + q)
        Db = np.einsum("g,gab,gai,gbj->aibj", f, ph, Z, Z).reshape(nb, nb)
        return (Da + Db) * fac

    def lvec(q):
        g, f, Z, _ = terms(G + q)
        pa = np.exp(-1j * (g @ bc) / C.bohr2nm)                       # (g, atom)
        return (1j * fac) * np.einsum("g,ga,gaj->aj", f, pa, Z).reshape(nb)

    return dyn, lvec


def q_cart(crys, qf):
    return (np.atleast_2d(qf) @ crys.reclattvecs.T) * C.bohr2nm


def np_ph_wann(wd, q):
    """D(q) with WS wrapping (wannier.f90:631-665), the non-analytic term for a
    polar crystal (:684-705), mass-normalised, LAPACK eigen."""
    c = wd.crystal
    nat, nb = c.numatoms, wd.numbranches
    D = np.zeros((len(q), nb, nb), dtype=complex)
    for iuc in range(wd.nwsq):
        R = wd.rcells_q[iuc]
        for jat in range(nat):
            for iat in range(nat):
                dist = (R - c.basis[:, iat] + c.basis[:, jat]) / wd.coarse_qmesh
                wr = S.ws_wrapping_vectors(c.lattvecs, dist)
                cs = np.zeros(len(q), dtype=complex)
                for w in wr:
                    cs += np.exp(2j * np.pi * (q @ (R + w * wd.coarse_qmesh)))
                cs /= (wd.phwsdeg[iuc] * len(wr))
                D[:, 3 * iat:3 * iat + 3, 3 * jat:3 * jat + 3] += cs[:, None, None] * \
                    np.asarray(wd.Dphwann)[iuc, 3 * iat:3 * iat + 3, 3 * jat:3 * jat + 3]
    if getattr(c, "polar", False):
        dyn, _ = np_polar(c, wd.coarse_qmesh)
        D = D + np.array([dyn(qc) for qc in q_cart(c, q)])
    Du = np.triu(0.5 * (D + np.conj(np.transpose(D, (0, 2, 1)))), 1)
    D = Du + np.conj(np.transpose(Du, (0, 2, 1))) + np.einsum("kii->ki", D).real[:, :, None] * np.eye(nb)
    m = np.repeat(c.masses, 3)
    D = D / np.sqrt(np.outer(m, m))[None] * C.Ryd2amu
    w2, V = np.linalg.eigh(D)
    om = np.sign(w2) * np.sqrt(np.abs(w2)) * C.Ryd2eV
    gam = np.all(q == 0, axis=1)
    om[gam, :3] = 0.0
    om[(om < 0) & (om > -0.005)] = 0.0
    return om, np.transpose(V, (0, 2, 1))


def np_rates(wd, req):
    """ibzk 'g' + 'X' and the RTA rates for a Gaussian delta, vectorised per state."""
    mesh = np.asarray(req.mesh)
    N = int(np.prod(mesh))
    ks = S.mesh_kvecs(mesh)
    e_all, _ = np_el_wann(wd, ks)
    inw = np.any(np.abs(e_all - req.enref) <= req.fsthick, axis=1)
    idx = np.nonzero(inw)[0]                       # 0-based mesh indices, ascending
    ens, U = np_el_wann(wd, ks[idx])
    om, V = np_ph_wann(wd, ks)
    u = V / np.sqrt(np.repeat(wd.crystal.masses, 3))[None, None, :]
    nw, nb = wd.numwannbands, wd.numbranches
    kint = np.stack([idx % mesh[0], (idx // mesh[0]) % mesh[1], idx // (mesh[0] * mesh[1])], 1)
    g = np.asarray(wd.gwann)
    ph_k = np.exp(2j * np.pi * (ks[idx] @ wd.rcells_k.T)) / wd.elwsdeg[None, :]
    kT = C.kB * req.T
    polar = getattr(wd.crystal, "polar", False)
    if polar:   # long_range_prefac(q, u_s) for every q of the mesh and mode s
        _, lvec = np_polar(wd.crystal, wd.coarse_qmesh)
        glp = np.array([u[i] @ lvec(qc) for i, qc in enumerate(q_cart(wd.crystal, ks))])   # (N, nb)
    rates = np.zeros((len(idx), nw))
    g2_all, xp_all, xm_all = [], [], []
    win_kp = np.abs(ens - req.enref) <= req.fsthick
    for ik in range(len(idx)):
        gk = np.einsum("r,ijrsp->ijsp", ph_k[ik], g)          # gkRp (nw, nw, nb, nwsq)
        for m in range(nw):
            E = ens[ik, m]
            if abs(E - req.enref) > req.fsthick:
                continue
            qint = (kint - kint[ik]) % mesh
            iq = qint[:, 0] + mesh[0] * (qint[:, 1] + mesh[1] * qint[:, 2])
            qf = qint / mesh
            phq = np.exp(2j * np.pi * (qf @ wd.rcells_q.T)) / wd.phwsdeg[None, :]   # (nkp, nwsq)
            gm = np.einsum("j,ijsp->isp", U[ik, m], gk)        # rotate initial band
            G = np.einsum("kp,isp->kis", phq, gm)              # Rp Fourier, (nkp, n', s')
            for ikp in range(len(idx)):
                for n in range(nw):
                    if not win_kp[ikp, n]:
                        continue
                    h = np.conj(U[ikp, n]) @ G[ikp]            # (s')
                    gs = u[iq[ikp]] @ h                         # (s)
                    if polar:                                   # + glprefac * unm (wannier.f90:998-1006)
                        gs = gs + glp[iq[ikp]] * (np.conj(U[ikp, n]) @ U[ik, m])
                    o = om[iq[ikp]]
                    with np.errstate(divide="ignore", invalid="ignore"):
                        g2 = np.where(o == 0, 0.0, 0.5 * np.abs(gs) ** 2 / o * C.g2unitfactor)
                    bose = np.where(o != 0, 1.0 / np.expm1(np.where(o != 0, o, 1.0) / C.kB / req.T), 0.0)
                    fp = 1.0 / (np.exp((E + o - req.chempot) / C.kB / req.T) + 1.0)
                    fm = 1.0 / (np.exp((E - o - req.chempot) / C.kB / req.T) + 1.0)
                    eps = ens[ikp, n]
                    dp = (1 / math.sqrt(2 * math.pi)) / req.sigma * np.exp(-0.5 * ((E + o - eps) / req.sigma) ** 2) / N
                    dm = (1 / math.sqrt(2 * math.pi)) / req.sigma * np.exp(-0.5 * ((E - o - eps) / req.sigma) ** 2) / N
                    cut = o >= 0.5e-3
                    xp = np.where(cut, g2 * (bose + fp) * dp, 0.0) * (2 * math.pi / C.hbar_eVps)
                    xm = np.where(cut, g2 * (1 + bose - fm) * dm, 0.0) * (2 * math.pi / C.hbar_eVps)
                    g2_all.append(g2)
                    xp_all.append(xp)
                    xm_all.append(xm)
                    rates[ik, m] += xp.sum() + xm.sum()
    return dict(indexlist=idx + 1, ens=ens, om=om, rates=rates, g2=np.concatenate(g2_all),
                xp=np.concatenate(xp_all), xm=np.concatenate(xm_all))


def np_ph_rates(wd, req, spindeg=2):
    """ibzq 'g' + 'Y' and the ph-e rates for a Gaussian delta, q-major as the
    reference walks them: g(Re,q) by an Rp sum (gReq), the 'el' Re sum per k,
    vertices in the order (q, s, k, m, n)."""
    mesh = np.asarray(req.mesh)
    N = int(np.prod(mesh))
    ks = S.mesh_kvecs(mesh)
    e_all, _ = np_el_wann(wd, ks)
    idx = np.nonzero(np.any(np.abs(e_all - req.enref) <= req.fsthick, axis=1))[0]
    ens, U = np_el_wann(wd, ks[idx])
    om, V = np_ph_wann(wd, ks)
    u = V / np.sqrt(np.repeat(wd.crystal.masses, 3))[None, None, :]
    nw, nb = wd.numwannbands, wd.numbranches
    pos = -np.ones(N, dtype=np.int64)
    pos[idx] = np.arange(len(idx))
    kint = np.stack([idx % mesh[0], (idx // mesh[0]) % mesh[1], idx // (mesh[0] * mesh[1])], 1)
    g = np.asarray(wd.gwann)                                       # (n', m', Re, s, Rp)
    phk = np.exp(2j * np.pi * (ks[idx] @ wd.rcells_k.T)) / wd.elwsdeg[None, :]
    win = np.abs(ens - req.enref) <= req.fsthick
    kT = C.kB * req.T
    fermi = lambda e: 1.0 / (np.exp((e - req.chempot) / kT) + 1.0)
    polar = getattr(wd.crystal, "polar", False)
    if polar:
        _, lvec = np_polar(wd.crystal, wd.coarse_qmesh)
    rates = np.zeros((N, nb))
    g2_all, y_all = [], []
    for iq in range(N):
        qi = np.array([iq % mesh[0], (iq // mesh[0]) % mesh[1], iq // (mesh[0] * mesh[1])])
        phq = np.exp(2j * np.pi * (wd.rcells_g @ (qi / mesh))) / wd.gwsdeg
        gReq = np.einsum("p,ijrsp->ijsr", phq, g)                  # (n', m', s, Re)
        kp = (kint + qi) % mesh
        ikp_all = pos[kp[:, 0] + mesh[0] * (kp[:, 1] + mesh[1] * kp[:, 2])]
        g2q, occ_delta = [], []                                    # per vertex: (nb,) arrays
        o = om[iq]
        glp = u[iq] @ lvec(q_cart(wd.crystal, qi / mesh)[0]) if polar else None
        with np.errstate(divide="ignore", invalid="ignore"):
            invb = np.where(o != 0, 1.0 / (1.0 + 1.0 / np.expm1(np.where(o != 0, o, 1.0) / kT)), 0.0)
        for ik in range(len(idx)):
            ikp = ikp_all[ik]
            if ikp < 0:
                continue
            gk = np.einsum("r,ijsr->ijs", phk[ik], gReq)
            for m in range(nw):
                if not win[ik, m]:
                    continue
                E = ens[ik, m]
                for n in range(nw):
                    if not win[ikp, n]:
                        continue
                    h = np.einsum("i,ijs,j->s", np.conj(U[ikp, n]), gk, U[ik, m])
                    gs = u[iq] @ h
                    if polar:
                        gs = gs + glp * (np.conj(U[ikp, n]) @ U[ik, m])
                    with np.errstate(divide="ignore", invalid="ignore"):
                        g2 = np.where(o == 0, 0.0, 0.5 * np.abs(gs) ** 2 / o * C.g2unitfactor)
                    x = (ens[ikp, n] - o - E) / req.sigma
                    delta = (1 / math.sqrt(2 * math.pi)) / req.sigma * np.exp(-0.5 * x * x) / N
                    occ = fermi(E) * (1.0 - fermi(E + o)) * invb
                    g2q.append(g2)
                    occ_delta.append(np.where(o >= 0.5e-3, occ * delta, 0.0))
        if not g2q:
            continue
        g2q = np.array(g2q)                                       # (count, nb)
        yq = g2q * np.array(occ_delta) * (2 * math.pi / C.hbar_eVps)
        for s in range(nb):
            g2_all.append(g2q[:, s])
            y_all.append(yq[:, s])
            rates[iq, s] = np.sum(spindeg * yq[:, s])
    return dict(indexlist=idx + 1, rates_phe=rates, g2=np.concatenate(g2_all), y=np.concatenate(y_all))


CASES = {
    "tiny": dict(nw=4, supercell=(2, 2, 2), seed=11, mesh=(4, 4, 4), window=1.0, shift=0.3),
    "si8": dict(nw=8, supercell=(3, 3, 3), seed=12, mesh=(4, 4, 4), window=0.5, shift=0.6),
}
# polar (SiC-like, long-range terms on): written by "polar", not by "el" / "ph"
POLAR_CASES = {
    "sic": dict(nw=8, supercell=(3, 3, 3), seed=14, mesh=(4, 4, 4), window=0.6, shift=0.5, crystal="sic"),
}


def build_case(name):
    c = CASES[name] if name in CASES else POLAR_CASES[name]
    crys = S.make_crystal_sic_like() if c.get("crystal") == "sic" else S.make_crystal_si_like()
    wd = S.make_wannier(crys, c["nw"], supercell=c["supercell"], seed=c["seed"])
    req = S.si_like_request(wd, c["mesh"], window=c["window"], shift=c["shift"])
    return wd, req


def main_ph(names=tuple(CASES)):
    """golden_ph_<case>.npz: the phonon side (ibzq 'g' + 'Y', ph-e rates), spindeg 2."""
    from oracle import oracle as O
    for name in names:
        wd, req = build_case(name)
        ref = np_ph_rates(wd, req, spindeg=2)
        o = O.Wannier(wd).ph_rates(req, spindeg=2, nthreads=os.cpu_count(), vertices=True)
        rel = lambda a, b: np.max(np.abs(a - b)) / max(np.abs(b).max(), 1e-300)
        assert o["vertices"] == len(ref["g2"]), name
        assert rel(o["g2"], ref["g2"]) < 1e-10, (name, rel(o["g2"], ref["g2"]))
        assert rel(o["y"], ref["y"]) < 1e-10, (name, rel(o["y"], ref["y"]))
        assert rel(o["rates_phe"], ref["rates_phe"]) < 1e-10, (name, rel(o["rates_phe"], ref["rates_phe"]))
        sel = np.arange(0, len(ref["g2"]), 7)
        np.savez_compressed(os.path.join(HERE, "golden_ph_%s.npz" % name), spindeg=2,
                            mesh=np.asarray(req.mesh), indexlist=ref["indexlist"], rates_phe=ref["rates_phe"],
                            vsel=sel, g2=ref["g2"][sel], y=ref["y"][sel], nvert=len(ref["g2"]))
        print(name, "ph vertices", len(ref["g2"]), "max|rate_phe|", ref["rates_phe"].max(),
              "oracle-vs-numpy g2 %.2e y %.2e rates %.2e" % (rel(o["g2"], ref["g2"]), rel(o["y"], ref["y"]),
                                                             rel(o["rates_phe"], ref["rates_phe"])))


def main(names=tuple(CASES)):
    from oracle import oracle as O
    for name in names:
        wd, req = build_case(name)
        ref = np_rates(wd, req)
        o = O.Wannier(wd).el_rates(req, literal=True, vertices=True)
        assert np.array_equal(o["indexlist"], ref["indexlist"]), name
        rel = lambda a, b: np.max(np.abs(a - b)) / max(np.abs(b).max(), 1e-300)
        assert rel(o["g2"], ref["g2"]) < 1e-10, (name, rel(o["g2"], ref["g2"]))
        assert rel(o["rates"], ref["rates"]) < 1e-10, (name, rel(o["rates"], ref["rates"]))
        # vertex sample: every 7th vertex
        sel = np.arange(0, len(ref["g2"]), 7)
        np.savez_compressed(os.path.join(HERE, "golden_%s.npz" % name),
                            enref=req.enref, fsthick=req.fsthick, chempot=req.chempot, T=req.T,
                            sigma=req.sigma, mesh=np.asarray(req.mesh), indexlist=ref["indexlist"],
                            ens=ref["ens"], om=ref["om"], rates=ref["rates"], vsel=sel,
                            g2=ref["g2"][sel], xp=ref["xp"][sel], xm=ref["xm"][sel],
                            nvert=len(ref["g2"]))
        print(name, "vertices", len(ref["g2"]), "max|rate|", ref["rates"].max(),
              "oracle-vs-numpy g2 %.2e rates %.2e" % (rel(o["g2"], ref["g2"]), rel(o["rates"], ref["rates"])))


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("el", "all"):
        main()
    if what in ("ph", "all"):
        main_ph()
    if what in ("polar", "all"):
        main(tuple(POLAR_CASES))
        main_ph(tuple(POLAR_CASES))
