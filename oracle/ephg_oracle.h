/*
 * ephg_oracle.h - CPU FP64 restatement of elphbolt's e-ph vertex path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA library
 * and the timed CPU baseline; nothing in the product links or calls it.
 *
 * It restates, function by function, the reference's Fortran (all FP64):
 *   el_wann               src/wannier.f90:430-524
 *   ws_wrapping_vectors   src/wannier.f90:532-582
 *   ph_wann               src/wannier.f90:585-782
 *   dyn_nonanalytic       src/wannier.f90:784-901
 *   g2                    src/wannier.f90:903-1011
 *   long_range_prefac     src/wannier.f90:1013-1071
 *   gkRp                  src/wannier.f90:1073-1132
 *   gReq                  src/wannier.f90:1134-1188
 *   ibzk 'g' + 'X'        src/interactions.f90:2095-2400
 *   el RTA rates          src/interactions.f90:2958-3063
 *   ibzq 'g' + 'Y'        src/interactions.f90:1673-1930, 1932-2093
 *   ph-e RTA rates        src/interactions.f90:2723-2828
 *   triangles / tetra     src/delta.f90:61-225,494-646,648-881
 *   symmetry / IBZ        src/symmetry.f90:134-289,303-452, src/electron.f90:346-577
 *   index helpers         src/misc.f90:588-610,738-763,906-1019, src/vector.f90:38-120
 *   window                src/electron.f90:597-636
 * plus a Gaussian delta of fixed width with the reference's Gaussian
 * convention (src/bz_sums.f90:73-83) divided by the number of mesh points.
 *
 * The reference's own LAPACK zheev is replaced by a cyclic complex Jacobi
 * eigensolver (Golub & Van Loan, 4th ed., sec. 8.5); only gauge-invariant
 * quantities may be compared across eigensolvers.
 *
 * Parity status: the reference ships no |g|^2, X or rate golden vectors, and
 * its Fortran cannot be compiled here (no Fortran compiler).  The integer
 * indexing, occupations and expm1 are pinned against the known answers of
 * test/test_misc.f90 and test/test_vector.f90; |g|^2 and rates are pinned
 * only by this restatement, cross-checked against an independent numpy
 * restatement (tests/golden/make_golden.py).
 *
 * Conventions: Fortran layouts (column-major, 1-based integer indices where
 * the reference uses them), complex numbers as interleaved (re, im) doubles.
 */
#ifndef EPHG_ORACLE_H
#define EPHG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int64_t nw, nb, nwsk, nwsq, nwsg, natoms;
  int64_t coarse_qmesh[3];
  const double *lattvecs;   /* (3,3) nm, columns a1 a2 a3 */
  const double *basis;      /* (3,natoms) crystal coordinates */
  const double *masses;     /* (natoms) amu */
  const int64_t *rcells_k;  /* (nwsk,3) */
  const int64_t *rcells_q;  /* (nwsq,3) */
  const int64_t *rcells_g;  /* (nwsg,3) */
  const int64_t *elwsdeg, *phwsdeg, *gwsdeg;
  const double *Hwann;      /* complex (nwsk,nw,nw) Ry */
  const double *Dphwann;    /* complex (nwsq,nb,nb) Ry/bohr^2 */
  const double *gwann;      /* complex (nw,nw,nwsk,nb,nwsg) Ry/bohr */
  int64_t polar;            /* crys%polar: add the long-range terms */
  const double *epsilon;    /* (3,3) high-frequency dielectric tensor */
  const double *born;       /* (3,3,natoms) Born effective charges */
} or_wannier;

typedef struct {
  int64_t mesh[3];
  double enref, fsthick, chempot, T;
  int64_t delta_kind;       /* 0 gaussian, 1 triangle, 2 tetrahedron */
  double sigma;             /* eV, gaussian only */
} or_request;

/* ---- index helpers (misc.f90, vector.f90) ---- */
int64_t or_mux_vector(const int64_t v[3], const int64_t mesh[3], int64_t base);
void or_demux_vector(int64_t i, int64_t v[3], const int64_t mesh[3], int64_t base);
int64_t or_mux_state(int64_t nbands, int64_t iband, int64_t ik);
void or_demux_state(int64_t m, int64_t nbands, int64_t *iband, int64_t *ik);
int64_t or_binsearch(const int64_t *array, int64_t n, int64_t e);
void or_umklapp(const double q1[3], const double q2[3], double q3[3]);
/* vector_allreps: create/add/sub/change_grid; out: int[3], muxed, frac[3], cart[3] */
void or_vector_create(int64_t ind, const int64_t grid[3], const double prim[9],
                      int64_t iv[3], int64_t *muxed, double frac[3], double cart[3]);
void or_vector_addsub(int64_t ind1, int64_t ind2, int sign, const int64_t grid[3],
                      const double prim[9], int64_t iv[3], int64_t *muxed,
                      double frac[3], double cart[3]);
void or_vector_change_grid(const double frac[3], const int64_t grid[3],
                           int64_t iv[3], int64_t *muxed);
double or_expm1(double x);
double or_Bose(double e, double T);
double or_Fermi(double e, double chempot, double T);

/* ---- eigen solver ---- */
int or_herm_eig(int64_t n, double *A, double *w, double *V);

/* ---- Wannier interpolation ---- */
void or_el_wann(const or_wannier *w, int64_t nk, const double *kvecs, double *energies,
                double *evecs, double *velocities, const double *scissor);
int or_ws_wrapping_vectors(const double lvec[9], const double vl[3], double eps,
                           int64_t *wrappers, int maxw);
int or_ph_wann(const or_wannier *w, int64_t nq, const double *qvecs, double *energies,
               double *evecs, double *velocities);
void or_gkRp(const or_wannier *w, const double kvec[3], double *gmixed);
void or_gReq(const or_wannier *w, const double qvec[3], double *gmixed);
/* polar: dyn_nonanalytic (wannier.f90:784-901) and long_range_prefac
 * (:1013-1071), q Cartesian in 1/bohr (or_q_cart_bohr converts crystal q) */
void or_q_cart_bohr(const or_wannier *w, const double qf[3], double qc[3]);
void or_dyn_nonanalytic(const or_wannier *w, const double q[3], double *dyn_l, double *ddyn_l);
void or_long_range_prefac(const or_wannier *w, const double q[3], const double *uqs, double *glprefac);
double or_g2(const or_wannier *w, const double kvec[3], const double qvec[3],
             const double *el_evec_k, const double *el_evec_kp, const double *ph_evec_q,
             double ph_en, const double *gmixed, int wannspace_ph);

/* ---- delta functions ---- */
void or_form_triangles(int64_t nk, const int64_t mesh[3], const int64_t *indexlist,
                       int64_t *triang, int64_t *triangcount, int64_t *triangmap);
void or_form_tetrahedra_3d(int64_t nk, const int64_t mesh[3], const int64_t *indexlist,
                           int64_t *tetra, int64_t *tetracount, int64_t *tetramap);
void or_fill_simplices(int64_t nsimplex, int64_t nv, const int64_t *simplex,
                       int64_t nk, int64_t nbands, const double *evals, double *simplex_evals);
double or_delta_triang(double e, int64_t ik, int64_t ib, const int64_t mesh[3], int64_t nk,
                       int64_t nsimplex, int64_t nbands, const int64_t *map,
                       const int64_t *count, const double *evals);
double or_delta_tetra(double e, int64_t ik, int64_t ib, const int64_t mesh[3], int64_t nk,
                      int64_t nsimplex, int64_t nbands, const int64_t *map,
                      const int64_t *count, const double *evals);

/* ---- full driver: ibzk 'g' + 'X' + rates ----
 * info[0]  nwv         window k-points (FBZ blocks = IBZ blocks, identity group)
 * info[1]  nstates_inwindow (FBZ blocks states in window)
 * info[2]  nstates_irred_inwindow (initial states processed, after max_states)
 * info[3]  vertices    total count increments (interactions.f90:2261)
 * info[4]  pairs       (initial state, k') pairs
 * info[5]  status      0 ok, 1 large negative phonon energy, 2 empty window
 * info[6]  microseconds of set-up (meshes, eigensolves, phonons, simplices)
 * info[7]  microseconds of the per-state loop (gkRp + |g|^2 + X + rates)
 * rates:      (N_k, nw) column-major, first info[0] rows valid (IBZ block order)
 * indexlist:  (N_k) muxed 1-based indices of the window k-points
 * g2/xp/xm:   optional per-vertex lists in the reference's order, capacity cap
 * max_states: process only the first max_states in-window initial states (<0: all)
 * nthreads:   OpenMP threads over initial states (distribute_points analogue)
 * literal:    1 = per-vertex g2 exactly as wannier.f90:903 (O(N_Rp nb nw^2) per
 *             vertex); 0 = restructured CPU form (Fourier over Rp once per
 *             (state, k'), then rotation), equal within FP64 rounding
 */
int or_el_rates(const or_wannier *w, const or_request *req, int64_t max_states,
                int nthreads, int literal, double *rates, int64_t *indexlist,
                int64_t *info, double *g2, double *xp, double *xm, int64_t cap);

/* The same driver split in two, so that a timed sample of states does not
 * repeat the set-up: or_rates_setup (steps up to the simplices), then
 * or_rates_run on the in-window states of rank [state_begin, state_begin +
 * nstates) (nstates < 0: all), or_rates_free.  Arguments as above. */
typedef struct or_rates_ctx or_rates_ctx;
or_rates_ctx *or_rates_setup(const or_wannier *w, const or_request *req, int nthreads);
int or_rates_run(or_rates_ctx *cx, int64_t state_begin, int64_t nstates, int nthreads,
                 int literal, double *rates, int64_t *indexlist, int64_t *info,
                 double *g2, double *xp, double *xm, int64_t cap);
void or_rates_free(or_rates_ctx *cx);
/* Degenerate-subspace averaging (wannier.f90:1332-1384) of the |g|^2 list of
 * or_rates_run over all in-window states, in place: phonon branches, then
 * initial bands, then final bands, each group |E - E'| < thres (eV).  mode 0:
 * the reference's in-place loops; mode 1: each member the mean of the group's
 * values before the pass.  Returns 1 if nv is not the list's length. */
int or_average_degenerate(or_rates_ctx *cx, int mode, double thres, double *g2, int64_t nv);
/* One group of those passes: c values v[0], v[st], ... with energies e; tmp
 * holds c doubles of scratch. */
void or_degenerate_group(int mode, double thres, int64_t c, double *v, int64_t st, const double *e, double *tmp);

/* ---- symmetry (symmetry.f90) ----
 * qrot / rotations: (3,3,n) column-major; indices 1-based muxed. */
void or_find_equiv_map(int64_t nsym, const double *qrot, const int64_t mesh[3], int64_t n,
                       const int64_t *indexlist, int64_t *equiv);
int64_t or_symmetry_qrotations(const double lattvecs[9], int64_t nsymm, const int64_t *rot, const int64_t mesh[3],
                               double *qrot);
int or_find_irred_wedge(const int64_t mesh[3], int64_t nsym, const double *qrot, int64_t n, const int64_t *indexlist,
                        int64_t *nirr, int64_t *indexlist_irred, int64_t *nequiv, int64_t *ibz2fbz);
/* The rate driver's set-up with nsym > 0 reciprocal rotations (from
 * or_symmetry_qrotations): or_rates_run then takes the initial states on the
 * irreducible window points only, and info[0] / indexlist / the rate rows are
 * those points (IBZ blocks, electron.f90:346-577).  status 3: no wedge. */
or_rates_ctx *or_rates_setup_sym(const or_wannier *w, const or_request *req, int64_t nsym, const double *qrot,
                                 int nthreads);

/* ---- phonon side: ibzq 'g' + 'Y' + the ph-e RTA rates ----
 * calculate_eph_interaction_ibzq (interactions.f90:1673-1930), calculate_Y_OTF
 * (:1932-2093) and the ph-e part of calculate_ph_rta_rates (:2723-2828) with
 * g(Re,q) from gReq (:1603-1630), identity point group, q mesh = k mesh.
 * info[0] nwv, [1] window final states, [2] phonon states (q, s) processed,
 * [3] vertices (the count of :1850), [4] (q, k) pairs with k, k + q in the
 * window, [5] status, [6] us set-up, [7] us loop.
 * rates_phe: (N, nb) column-major, row iq - 1 = the q-point of muxed index iq
 *            (the phonon side has no window: every q of the mesh); rows of q
 *            outside [q_begin, q_begin + nq) are zero.
 * g2/y:      optional per-vertex lists in the reference's order (phonon state
 *            (iq - 1) * nb + s, then k, m, n), capacity cap; y in THz.
 * spindeg:   el%spindeg (electron.f90), the factor of each Y in the rate sum. */
int or_ph_rates_run(or_rates_ctx *cx, int64_t q_begin, int64_t nq, int nthreads, double spindeg,
                    double *rates_phe, int64_t *info, double *g2, double *y, int64_t cap);
int or_ph_rates(const or_wannier *w, const or_request *req, double spindeg, int nthreads,
                double *rates_phe, int64_t *info, double *g2, double *y, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
