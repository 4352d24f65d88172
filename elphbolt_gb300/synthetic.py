"""Seeded synthetic Wannier-space inputs for the e-ph vertex path.

No real EPW data exists for this path, so every workload is generated here from
a seed, in the reference's own units and array layouts, and the same arrays feed
both the CUDA library and the CPU oracle:

* lattice vectors in nm as columns (``crystal.f90`` ``lattvecs``), basis in
  crystal coordinates, masses in amu;
* Wigner-Seitz sets of a coarse supercell with integer degeneracies
  (``rcells_k/q/g``, ``elwsdeg/phwsdeg/gwsdeg``, read at ``wannier.f90:384-427``);
  the vertex set equals the phonon set (``rcells_g = rcells_q``), which the
  reference's ``g2`` assumes (``wannier.f90:947-951,988-990``);
* ``Hwann(nwsk, nw, nw)`` in Ry, Hermitian-paired (H(-R) = H(R)^dagger);
* ``Dphwann(nwsq, nb, nb)`` in Ry/bohr^2 from positive central springs (so the
  dynamical matrix is positive semi-definite at every q) with the acoustic sum
  rule; the block (i, j) of cell R holds the spring of the bond from atom i in
  cell 0 to atom j in cell R, wrapped exactly as ``ph_wann`` wraps it
  (``wannier.f90:631-665``);
* ``gwann(nw, nw, nwsk, nb, nwsg)`` in Ry/bohr, the order of EPW's ``epmatwp``
  stream (``wannier.f90:355-371``).

All arrays are numpy, Fortran (column-major) ordered where the reference is.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import constants as C

ANG_PER_NM = 10.0
BOHR_ANG = C.bohr2nm * 10.0
# eV/Angstrom -> Ry/bohr and eV/Angstrom^2 -> Ry/bohr^2
EV_PER_ANG_TO_RY_PER_BOHR = BOHR_ANG / C.Ryd2eV
EV_PER_ANG2_TO_RY_PER_BOHR2 = BOHR_ANG ** 2 / C.Ryd2eV


@dataclasses.dataclass
class Crystal:
    """Crystal data used on the path (``crystal.f90:115-298``)."""
    lattvecs: np.ndarray        # (3,3) nm, columns are a1, a2, a3
    basis: np.ndarray           # (3, numatoms) crystal coordinates
    masses: np.ndarray          # (numatoms,) amu, one per atom
    T: float = 300.0            # K
    polar: bool = False         # crys%polar: add the long-range dipole terms
    epsilon: np.ndarray = None  # (3,3) high-frequency dielectric tensor
    born: np.ndarray = None     # (3,3,numatoms) Born effective charges, born(:, ipol, iat)

    @property
    def numatoms(self) -> int:
        return self.basis.shape[1]

    @property
    def reclattvecs(self) -> np.ndarray:
        """Reciprocal vectors (1/nm) as columns, ``crystal.f90:284-293``."""
        a = self.lattvecs
        rec = np.empty((3, 3))
        for i in range(3):
            j = (i + 1) % 3
            k = (j + 1) % 3
            rec[:, i] = np.cross(a[:, j], a[:, k])
        vol = abs(float(a[:, 0] @ rec[:, 0]))
        return (C.twopi / vol) * rec

    @property
    def volume(self) -> float:
        a = self.lattvecs
        return abs(float(a[:, 0] @ np.cross(a[:, 1], a[:, 2])))


@dataclasses.dataclass
class WannierData:
    """Real-space Wannier data in the reference's layouts and units."""
    crystal: Crystal
    numwannbands: int
    numbranches: int
    coarse_qmesh: np.ndarray    # (3,) int64
    rcells_k: np.ndarray        # (nwsk, 3) int64
    rcells_q: np.ndarray        # (nwsq, 3) int64
    rcells_g: np.ndarray        # (nwsg, 3) int64
    elwsdeg: np.ndarray         # (nwsk,) int64
    phwsdeg: np.ndarray         # (nwsq,) int64
    gwsdeg: np.ndarray          # (nwsg,) int64
    Hwann: np.ndarray           # (nwsk, nw, nw) complex128, F-order, Ry
    Dphwann: np.ndarray         # (nwsq, nb, nb) complex128, F-order, Ry/bohr^2
    gwann: np.ndarray           # (nw, nw, nwsk, nb, nwsg) complex128, F-order, Ry/bohr
    midgap: float = 0.0         # eV, (VBM + CBM)/2 of the valence/conduction split

    @property
    def nwsk(self) -> int:
        return self.rcells_k.shape[0]

    @property
    def nwsq(self) -> int:
        return self.rcells_q.shape[0]

    @property
    def nwsg(self) -> int:
        return self.rcells_g.shape[0]


def fcc_lattvecs(a_ang: float) -> np.ndarray:
    """fcc primitive vectors a/2*[(-1,0,1),(0,1,1),(-1,1,0)] as columns, in nm."""
    a = a_ang / ANG_PER_NM
    return 0.5 * a * np.array([[-1.0, 0.0, -1.0],
                               [0.0, 1.0, 1.0],
                               [1.0, 1.0, 0.0]])


def wigner_seitz(lattvecs: np.ndarray, supercell, tol: float = 1e-8):
    """Wigner-Seitz cell vectors of a supercell with integer degeneracies.

    R (integer, lattice coordinates) is kept when no supercell translation T
    brings it closer to the origin; its degeneracy is the number of T at the
    same shortest distance.  The sum of 1/deg equals the supercell volume
    (number of cells), which the caller may check.
    """
    n = np.asarray(supercell, dtype=np.int64)
    rng = [np.arange(-2 * n[d], 2 * n[d] + 1) for d in range(3)]
    # all supercell translations with coefficients in [-2, 2]
    ts = np.array([[i, j, k] for k in range(-2, 3) for j in range(-2, 3)
                   for i in range(-2, 3)], dtype=np.int64) * n
    cells, degs = [], []
    for r3 in rng[2]:
        for r2 in rng[1]:
            for r1 in rng[0]:
                r = np.array([r1, r2, r3], dtype=np.int64)
                d = np.linalg.norm(lattvecs @ (r[None, :] - ts).T, axis=0)
                d0 = np.linalg.norm(lattvecs @ r)
                dmin = d.min()
                if d0 <= dmin + tol:
                    cells.append(r)
                    degs.append(int(np.sum(np.abs(d - dmin) < tol)))
    cells = np.array(cells, dtype=np.int64)
    degs = np.array(degs, dtype=np.int64)
    assert abs(np.sum(1.0 / degs) - float(np.prod(n))) < 1e-9
    return cells, degs


_WRAP_SHIFTS = np.array([(i, j, k) for k in range(-3, 4) for j in range(-3, 4) for i in range(-3, 4)],
                        dtype=np.int64)


def ws_wrapping_vectors(lvec: np.ndarray, vl: np.ndarray, eps: float = 1e-6):
    """Shortest lattice wraps of a vector given in lattice coordinates.

    Same search as ``wannier.f90:532-582`` (supercell range [-3, 3]^3,
    truncation of vl toward zero, tolerance eps); used here only to place the
    synthetic springs where ``ph_wann`` will look for them.
    """
    iv0 = np.trunc(vl).astype(np.int64)
    wl = vl - iv0
    # all 343 shifts at once (i fastest, then j, then k), then the reference's
    # running minimum over them in the same order
    wc = lvec @ (wl[:, None] + _WRAP_SHIFTS.T)
    norms = np.sqrt(np.einsum("ij,ij->j", wc, wc)).tolist()
    d = np.finfo(np.float64).max
    for nrm in norms:
        if abs(nrm - d) < eps:
            continue
        if nrm < d:
            d = nrm
    keep = np.abs(np.asarray(norms) - d) < eps
    return (_WRAP_SHIFTS[keep] - iv0).astype(np.int64)


def _springs(crys: Crystal, rcells_q: np.ndarray, coarse_qmesh, rng,
             kmin_ev_ang2: float, kmax_ev_ang2: float, bond_tol: float = 1.08,
             shell2=(1.75, 1.0, 3.0)):
    """Central-spring force constants Dphwann(R) in Ry/bohr^2 (F-order).

    Nearest-neighbour bonds (distance within ``bond_tol`` of the shortest
    interatomic distance) draw springs in [kmin, kmax]; second-shell bonds (up
    to ``shell2[0]`` times the shortest distance) draw weaker springs in
    [shell2[1], shell2[2]].  Central nearest-neighbour springs alone leave the
    diamond structure with zero-frequency transverse acoustic modes at every q,
    for which |g|^2 ~ 1/omega is ill-conditioned; the second shell removes them.
    Each undirected bond draws one constant, so Phi_ij(R) = Phi_ji(-R)^T exactly.
    """
    nat = crys.numatoms
    nb = 3 * nat
    nwsq = rcells_q.shape[0]
    L = crys.lattvecs * ANG_PER_NM          # Angstrom
    tau = L @ crys.basis                    # (3, nat) Angstrom
    # shortest distance over a small neighbourhood
    dmin = np.inf
    rr = range(-2, 3)
    for i in range(nat):
        for j in range(nat):
            for a in rr:
                for b in rr:
                    for c in rr:
                        if i == j and a == 0 and b == 0 and c == 0:
                            continue
                        v = tau[:, j] + L @ np.array([a, b, c]) - tau[:, i]
                        dmin = min(dmin, float(np.linalg.norm(v)))
    cut = bond_tol * dmin
    cut2 = shell2[0] * dmin
    # enumerate directed bonds (i, j, R) with R small; one constant per undirected bond
    bonds = {}
    for i in range(nat):
        for j in range(nat):
            for a in rr:
                for b in rr:
                    for c in rr:
                        R = (a, b, c)
                        if i == j and R == (0, 0, 0):
                            continue
                        v = tau[:, j] + L @ np.array(R, dtype=float) - tau[:, i]
                        dv = np.linalg.norm(v)
                        if dv <= cut2:
                            key = (i, j, R)
                            rkey = (j, i, (-a, -b, -c))
                            if rkey in bonds:
                                bonds[key] = bonds[rkey]
                            elif dv <= cut:
                                bonds[key] = float(rng.uniform(kmin_ev_ang2, kmax_ev_ang2))
                            else:
                                bonds[key] = float(rng.uniform(shell2[1], shell2[2]))
    # Phi blocks (eV/A^2) by (i, j, R)
    phi = {}
    for (i, j, R), kb in bonds.items():
        v = tau[:, j] + L @ np.array(R, dtype=float) - tau[:, i]
        e = v / np.linalg.norm(v)
        blk = -kb * np.outer(e, e)
        phi[(i, j, R)] = phi.get((i, j, R), 0.0) + blk
        self_key = (i, i, (0, 0, 0))
        phi[self_key] = phi.get(self_key, 0.0) - blk
    D = np.zeros((nwsq, nb, nb), dtype=np.complex128, order="F")
    cq = np.asarray(coarse_qmesh, dtype=np.int64)
    for iuc in range(nwsq):
        R0 = rcells_q[iuc]
        for jat in range(nat):
            for iat in range(nat):
                dist = (R0 - crys.basis[:, iat] + crys.basis[:, jat]) / cq
                wr = ws_wrapping_vectors(crys.lattvecs, dist)
                # the spring seen by ph_wann for this (R, i, j): the shortest image
                found = None
                for w in wr:
                    Rs = tuple(int(x) for x in (R0 + w * cq))
                    if (iat, jat, Rs) in phi:
                        found = phi[(iat, jat, Rs)]
                        break
                if found is not None:
                    D[iuc, 3 * iat:3 * iat + 3, 3 * jat:3 * jat + 3] = found
    return D * EV_PER_ANG2_TO_RY_PER_BOHR2


def _hermitian_paired(rng, cells, nw, amp):
    """Complex H(R) with H(-R) = H(R)^dagger; amp(R) scales entries (eV)."""
    idx = {tuple(int(x) for x in r): i for i, r in enumerate(cells)}
    nws = cells.shape[0]
    H = np.zeros((nws, nw, nw), dtype=np.complex128)
    done = np.zeros(nws, dtype=bool)
    for i, r in enumerate(cells):
        if done[i]:
            continue
        a = rng.standard_normal((nw, nw)) + 1j * rng.standard_normal((nw, nw))
        a *= amp[i] / math.sqrt(2.0)
        j = idx[tuple(int(-x) for x in r)]
        if j == i:
            H[i] = 0.5 * (a + a.conj().T)
        else:
            H[i] = a
            H[j] = a.conj().T
            done[j] = True
        done[i] = True
    return np.asfortranarray(H)


def make_crystal_si_like() -> Crystal:
    """Diamond-Si-like fcc 2-atom cell, a = 5.43 A, masses 28 amu."""
    return Crystal(lattvecs=fcc_lattvecs(5.43),
                   basis=np.array([[0.0, 0.25], [0.0, 0.25], [0.0, 0.25]]),
                   masses=np.array([28.0, 28.0]), T=300.0)


def make_crystal_sic_like() -> Crystal:
    """Zincblende SiC-like polar fcc cell: the lattice, masses, dielectric
    constant and Born charges of 3C-SiC's input (test/3C-SiC/input.nml)."""
    born = np.zeros((3, 3, 2))
    born[:, :, 0] = 2.7514963 * np.eye(3)
    born[:, :, 1] = -2.7514963 * np.eye(3)
    return Crystal(lattvecs=fcc_lattvecs(4.33909462),
                   basis=np.array([[0.0, 0.25], [0.0, 0.25], [0.0, 0.25]]),
                   masses=np.array([28.0855, 12.011]), T=300.0,
                   polar=True, epsilon=7.4190074 * np.eye(3), born=np.asfortranarray(born))


def make_crystal_multi(natoms: int, rng, mass_range=(12.0, 60.0)) -> Crystal:
    """fcc cell with ``natoms`` atoms spread along the body diagonal plus jitter."""
    basis = np.zeros((3, natoms))
    for i in range(natoms):
        basis[:, i] = (i / natoms) * np.ones(3) + rng.uniform(-0.03, 0.03, 3) * (i > 0)
    masses = rng.uniform(mass_range[0], mass_range[1], natoms)
    return Crystal(lattvecs=fcc_lattvecs(5.43), basis=basis, masses=masses)


def make_wannier(crys: Crystal, nw: int, supercell=(6, 6, 6), seed: int = 20260101,
                 h_sigma_ev: float = 1.0, g_sigma_ev_ang: float = 0.1,
                 decay_ang: float = 2.0, spring_range=(5.0, 15.0),
                 nvalence: int | None = None, lean: bool = False) -> WannierData:
    """Build the synthetic Wannier data for a crystal.

    H(Re) entries are N(0, h_sigma) eV * exp(-|Re|/decay); g(Re, Rp) entries
    are N(0, g_sigma) eV/A * exp(-|Re|/decay - |Rp|/decay); springs are
    uniform in ``spring_range`` eV/A^2.  Converted to Ry, Ry/bohr^2, Ry/bohr.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    cells, degs = wigner_seitz(crys.lattvecs, supercell)
    nb = 3 * crys.numatoms
    rlen = np.linalg.norm((crys.lattvecs * ANG_PER_NM) @ cells.T, axis=0)  # Angstrom
    amp = h_sigma_ev * np.exp(-rlen / decay_ang)
    H_ev = _hermitian_paired(rng, cells, nw, amp)
    Hwann = np.asfortranarray(H_ev / C.Ryd2eV)
    D = _springs(crys, cells, supercell, rng, *spring_range)
    nws = cells.shape[0]
    shape = (nw, nw, nws, nb, nws)
    env = np.exp(-rlen / decay_ang)
    if not lean:
        # draw in C order of (Rp, s, Re, j, i) so the stream is the F-order layout
        gr = rng.standard_normal(shape[::-1]) + 1j * rng.standard_normal(shape[::-1])
        g = np.asfortranarray(gr.T) * (g_sigma_ev_ang / math.sqrt(2.0))
        g *= env[None, None, :, None, None]
        g *= env[None, None, None, None, :]
        g *= EV_PER_ANG_TO_RY_PER_BOHR
    else:
        # one Rp slab at a time (same distribution, a different stream): the
        # peak host memory is g itself plus one slab
        g = np.empty(shape, dtype=np.complex128, order="F")
        slab = shape[:4]
        for rp in range(nws):
            x = rng.standard_normal(slab[::-1]) + 1j * rng.standard_normal(slab[::-1])
            x *= (g_sigma_ev_ang / math.sqrt(2.0)) * env[rp] * EV_PER_ANG_TO_RY_PER_BOHR
            x *= env[None, :, None, None]            # C-order (s, Re, j, i): Re on axis 1
            g[:, :, :, :, rp] = x.T
    wd = WannierData(crystal=crys, numwannbands=nw, numbranches=nb,
                     coarse_qmesh=np.asarray(supercell, dtype=np.int64),
                     rcells_k=cells.copy(), rcells_q=cells.copy(), rcells_g=cells.copy(),
                     elwsdeg=degs.copy(), phwsdeg=degs.copy(), gwsdeg=degs.copy(),
                     Hwann=Hwann, Dphwann=np.asfortranarray(D), gwann=np.asfortranarray(g))
    wd.midgap = _midgap(wd, nvalence if nvalence is not None else nw // 2)
    return wd


def make_wannier_symmetric(crys: Crystal, n_orb: int = 4, supercell=(4, 4, 4), seed: int = 20260201,
                           t_ev: float = 2.0, decay_ang: float = 1.2, shells: float = 1.75,
                           k_nn: float = 10.0, k_2nd: float = 2.0, nvalence: int | None = None) -> WannierData:
    """Wannier data of a symmetric tight-binding model: the space group of
    ``crys`` is a symmetry of H(k), D(q) and g(k,q), as for real EPW data.

    n_orb s-like Wannier functions per atom (nw = n_orb * natoms).  Hopping
    between orbital a of atom i (cell 0) and b of atom j (cell R) is
    t = c_ab(types) exp(-d/decay) for bond length 0 < d <= ``shells`` times the
    shortest distance, with c symmetric under (i,a) <-> (j,b); on-site blocks
    are random symmetric matrices per atom type.  Springs are central, one
    constant per shell (``k_nn``, ``k_2nd`` eV/A^2).  The e-ph coupling is the
    bond-stretching derivative of the hopping, g = dt/du = t'(d) e_d for atom j
    in cell R and -t'(d) e_d for atom i in cell 0 (Ry/bohr).  Every bond lies
    inside the Wigner-Seitz cell of the supercell (degeneracy 1), so the
    interpolation reproduces the model exactly.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    cells, degs = wigner_seitz(crys.lattvecs, supercell)
    nat = crys.numatoms
    nw, nb = n_orb * nat, 3 * nat
    L = crys.lattvecs * ANG_PER_NM
    tau = L @ crys.basis
    _, types = np.unique(np.asarray(crys.masses), return_inverse=True)
    ntype = int(types.max()) + 1
    # bond shells
    dmin = np.inf
    for i in range(nat):
        for j in range(nat):
            for R in cells:
                v = tau[:, j] + L @ R - tau[:, i]
                dv = float(np.linalg.norm(v))
                if dv > 1e-9:
                    dmin = min(dmin, dv)
    cut = shells * dmin
    # hopping prefactors c[ti][tj][a][b] with c[tj][ti] = c[ti][tj]^T; on-site blocks per type
    c = np.zeros((ntype, ntype, n_orb, n_orb))
    for ti in range(ntype):
        for tj in range(ti, ntype):
            m = rng.uniform(-1.0, 1.0, (n_orb, n_orb)) * t_ev
            if ti == tj:
                m = 0.5 * (m + m.T)
            c[ti, tj], c[tj, ti] = m, m.T
    eps = []
    for t in range(ntype):
        m = rng.normal(0.0, 1.5, (n_orb, n_orb))
        eps.append(0.5 * (m + m.T))
    nws = cells.shape[0]
    H = np.zeros((nws, nw, nw), dtype=np.complex128, order="F")
    g = np.zeros((nw, nw, nws, nb, nws), dtype=np.complex128, order="F")
    index = {tuple(int(x) for x in R): r for r, R in enumerate(cells)}
    r0 = index[(0, 0, 0)]
    lam = decay_ang / BOHR_ANG            # bohr
    for r, R in enumerate(cells):
        for i in range(nat):
            for j in range(nat):
                v = tau[:, j] + L @ R - tau[:, i]
                d = float(np.linalg.norm(v))
                blk_h = np.zeros((n_orb, n_orb))
                if d < 1e-9:
                    blk_h = eps[types[i]]
                elif d <= cut * (1 + 1e-9):
                    if degs[r] != 1:
                        raise ValueError("a bond reaches a Wigner-Seitz boundary cell: enlarge the supercell")
                    t = c[types[i], types[j]] * math.exp(-d / decay_ang)          # eV
                    blk_h = t
                    e = v / d
                    tp = -t / C.Ryd2eV / lam                                        # Ry/bohr, d t / d d
                    for x in range(3):
                        # atom j in cell R moves: d -> d + u.e ; atom i in cell 0 moves: d -> d - u.e
                        g[n_orb * i:n_orb * (i + 1), n_orb * j:n_orb * (j + 1), r, 3 * j + x, r] += tp * e[x]
                        g[n_orb * i:n_orb * (i + 1), n_orb * j:n_orb * (j + 1), r, 3 * i + x, r0] -= tp * e[x]
                H[r, n_orb * i:n_orb * (i + 1), n_orb * j:n_orb * (j + 1)] = blk_h / C.Ryd2eV
    D = _springs(crys, cells, supercell, rng, k_nn, k_nn, shell2=(shells, k_2nd, k_2nd))
    wd = WannierData(crystal=crys, numwannbands=nw, numbranches=nb,
                     coarse_qmesh=np.asarray(supercell, dtype=np.int64),
                     rcells_k=cells.copy(), rcells_q=cells.copy(), rcells_g=cells.copy(),
                     elwsdeg=degs.copy(), phwsdeg=degs.copy(), gwsdeg=degs.copy(),
                     Hwann=np.asfortranarray(H), Dphwann=np.asfortranarray(D), gwann=np.asfortranarray(g))
    wd.midgap = _midgap(wd, nvalence if nvalence is not None else nw // 2)
    return wd


def _midgap(wd: WannierData, nval: int, mesh=(6, 6, 6)) -> float:
    """(VBM + CBM)/2 of the split after ``nval`` bands on a coarse mesh (eV).

    Generator-side helper only: it fixes the chemical potential of a workload.
    """
    ks = mesh_kvecs(np.asarray(mesh))
    ph = np.exp(2j * np.pi * (ks @ wd.rcells_k.T)) / wd.elwsdeg[None, :]
    Hk = np.einsum("kr,rij->kij", ph, np.asarray(wd.Hwann))
    Hk = 0.5 * (Hk + np.conj(np.transpose(Hk, (0, 2, 1))))
    e = np.linalg.eigvalsh(Hk) * C.Ryd2eV
    vbm = e[:, nval - 1].max()
    cbm = e[:, nval].min()
    return 0.5 * (vbm + cbm)


def mesh_kvecs(mesh) -> np.ndarray:
    """All mesh points in crystal coordinates, muxed order of ``misc.f90:906``."""
    m = np.asarray(mesh, dtype=np.int64)
    n = int(np.prod(m))
    i = np.arange(n)
    v1 = i % m[0]
    v2 = (i // m[0]) % m[1]
    v3 = i // (m[0] * m[1])
    return np.stack([v1 / m[0], v2 / m[1], v3 / m[2]], axis=1)


@dataclasses.dataclass
class RateRequest:
    """One scattering-rate request: mesh, window, occupations, delta kind."""
    mesh: tuple
    enref: float          # eV, window centre
    fsthick: float        # eV, window half width
    chempot: float        # eV
    T: float              # K
    delta_kind: int = 0   # 0 gaussian, 1 triangle, 2 tetrahedron
    sigma: float = 0.010  # eV, gaussian width


def si_like(nw: int = 8, supercell=(6, 6, 6), seed: int = 20260101) -> WannierData:
    """Synthetic Si-like crystal: fcc, 2 atoms, masses 28 amu, nw Wannier bands."""
    return make_wannier(make_crystal_si_like(), nw, supercell=supercell, seed=seed)


def si_like_request(wd: WannierData, mesh=(12, 12, 12), T: float = 300.0,
                    sigma: float = 0.010, window: float = 0.5, shift: float = 0.6,
                    delta_kind: int = 0) -> RateRequest:
    """Window of +-window eV about mu = mid-gap + shift (enref = mu)."""
    mu = wd.midgap + shift
    return RateRequest(mesh=tuple(int(x) for x in mesh), enref=mu, fsthick=window,
                       chempot=mu, T=T, delta_kind=delta_kind, sigma=sigma)


def large_instance(supercell=(6, 6, 6), seed: int = 20260103) -> WannierData:
    """The large single instance: a 6-atom fcc cell (``make_crystal_multi``,
    masses U[12, 60] amu), nw = 32 Wannier bands, nb = 18 modes, Re and Rp
    Wigner-Seitz sets of a 6x6x6 supercell (279 cells each): g(Re,Rp) is
    32^2 x 18 x 279^2 complex128 = 23 GB.  Value distributions as si_like."""
    rng = np.random.Generator(np.random.PCG64(seed))
    crys = make_crystal_multi(6, rng)
    return make_wannier(crys, 32, supercell=supercell, seed=seed + 1, lean=True)


# The batched workload: many requests of uneven size on random crystals.
# (nw, natoms, WS supercell) of each crystal; nb = 3 natoms.
BATCH_CRYSTALS = [(8, 2, (6, 6, 6)), (8, 4, (5, 5, 5)), (16, 2, (5, 5, 5)), (16, 4, (5, 5, 5)),
                  (8, 6, (5, 5, 5)), (24, 2, (5, 5, 5)), (16, 6, (4, 4, 4)), (24, 4, (4, 4, 4))]


def batch_workload(n_requests: int = 64, mesh_range=(8, 16), window_range=(0.2, 1.0), seed: int = 20260102,
                   crystals=None):
    """Random crystals (``make_crystal_multi``: fcc cell, masses U[12, 60] amu)
    with nw in {8, 16, 24}, nb in {6, 12, 18} and WS sets of 93-279 vectors,
    and ``n_requests`` requests drawn over them: crystal i % len(crystals), a
    cubic mesh uniform in ``mesh_range``, a full window width uniform in
    ``window_range`` eV about mid-gap + 0.6 eV, 300 K, Gaussian delta 10 meV.
    Returns (list of WannierData, list of (crystal index, RateRequest))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = crystals if crystals is not None else BATCH_CRYSTALS
    wds = []
    for c, (nw, nat, sc) in enumerate(specs):
        crys = make_crystal_multi(nat, rng)
        wds.append(make_wannier(crys, nw, supercell=sc, seed=seed + 1 + c))
    reqs = []
    for i in range(n_requests):
        c = i % len(wds)
        m = int(rng.integers(mesh_range[0], mesh_range[1] + 1))
        width = float(rng.uniform(*window_range))
        reqs.append((c, si_like_request(wds[c], (m, m, m), window=0.5 * width)))
    return wds, reqs
