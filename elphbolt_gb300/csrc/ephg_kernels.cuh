// ephg_kernels.cuh - launchers of the library's kernels (internal interface).
#pragma once
#include "ephg_common.cuh"

namespace ephg {

// ---- phases ----
void launch_roots(int L, double2 *roots, cudaStream_t st);
// out[row*ldo + r] = e^{2 pi i k_row . R_r} (/ deg_r if deg) (conjugated if conj);
// k on the mesh (row -> mesh index rowp[row], or row itself if rowp == nullptr)
void launch_phase_mesh(int nrows, const int *rowp, const int mesh[3], int L, int nR,
                       const int *R, const double *deg, int conj, const double2 *roots,
                       double2 *out, int64_t ldo, cudaStream_t st);
// same for arbitrary fractional k: kv (nrows,3) column-major as the reference
void launch_phase_frac(int nrows, const double *kv, int nR, const int *R, const double *deg,
                       double2 *out, int64_t ldo, cudaStream_t st);

// out[p][e] = sum_R e^{2 pi i k_p.R} X(R)[e] for every point p of the mesh (muxed
// order), X given on the box of cell coordinates [lo, lo + ext) per dimension
// (box[((r1 ext2 + r2) ext3 + r3) nn + e], zero where there is no cell); three
// 1-D passes through t1 (ext1 ext2 m3 nn) and t2 (ext1 m2 m3 nn).
void launch_mesh_fourier(const double2 *box, const int lo[3], const int ext[3], int nn, const int mesh[3], int L,
                         const double2 *roots, double2 *t1, double2 *t2, double2 *out, cudaStream_t st);

// ---- FP64 complex GEMM: C[M][N] = A[M][K] * B[K][N], row-major ----
void launch_zgemm(int M, int N, int K, const double2 *A, int64_t lda, const double2 *B,
                  int64_t ldb, double2 *C, int64_t ldc, cudaStream_t st);

// ---- Hermitian eigensolver (batched, one warp per matrix, n <= 32) ----
// A: batch matrices (n,n) column-major at stride n*n, upper triangle forced
// Hermitian as in wannier.f90:481-486.  w: (batch, n) ascending;
// V: (batch, n, n) column-major, columns = eigenvectors.
void launch_heig(int batch, int n, const double2 *A, int64_t stride, double *w, double2 *V,
                 int *err, cudaStream_t st);

// ---- electron / phonon post-processing ----
// C: (nk, 4*nw*nw) from the H(k) GEMM (H, dH_x, dH_y, dH_z), nvel = 0 or 3
void launch_el_post(int nk, int nw, const double *w, const double2 *V, const double2 *C,
                    int64_t ldc, int with_vel, const double *scissor, double *energies_f,
                    double *vel_f, double2 *evecs_f, double *ens_i, cudaStream_t st);

struct PhTerms {
  int npair;            // natoms^2, pair = iat + nat*jat
  const int *pair_off;  // (npair+1) offsets into the entry list
  const int *ent_iuc;   // entry -> WS cell
  const int *ent_woff;  // entry -> first wrap vector (wrap list offsets, nent+1)
  const int *wrapR;     // wrap vectors R + w*N_c, 3 ints each
  const double *ent_rden;// 1 / (phwsdeg * nwrap)
  const double2 *D;     // (nwsq, nb, nb) column-major
  const double *rcart;  // (nwsq, 3) lattvecs @ R, nm
  const double *masses; // per atom
  int nwsq, nb, nat;
};
// Build the mass-normalised dynamical matrix D(q) (and dD/dq with vel);
// mesh mode if qp != nullptr (exact integer phases), else fractional qv (nq,3).
void launch_dbuild(int nq, const int *qp, const int mesh[3], int L, const double2 *roots,
                   const double *qv, const PhTerms &t, int with_vel, double2 *Dq, double2 *dDq,
                   cudaStream_t st);
// omega, Gamma / negative handling, velocities; outputs in reference layout
// (energies_f (nq,nb), evecs_f (nq,nb,nb), vel_f (nq,nb,3)) and/or internal
// (om_i [q][s], u_i [q][s][c] = evec/sqrt(M_c)).
void launch_ph_post(int nq, int nb, const int *qp, const double *qv, const double *w,
                    const double2 *V, const double2 *dDq, int with_vel, const double *masses,
                    double *energies_f, double2 *evecs_f, double *vel_f, double *om_i,
                    double2 *u_i, float2 *u_f, int *err, cudaStream_t st);

// ---- gkRp / gReq layout helpers ----
void launch_permute_gwann(int nw, int nb, int nwsk, int nwsg, const double2 *raw, double2 *G,
                          cudaStream_t st);
// gReq GEMM output (nq, [i,j,Re,s]) -> (nw,nw,nb,nwsk,nq) column-major
void launch_permute_greq(int nq, int nw, int nb, int nwsk, const double2 *in, double2 *out,
                         cudaStream_t st);

// ---- g2 batched (wannier.f90:903-1011) ----
// Lv (nv, nb), nullable: the polar long-range vector of each vertex's q (launch_polar_q)
void launch_g2_batch(int nv, int nw, int nb, int nws, const double *qv, const int *R,
                     const double *deg, const double2 *ek, const double2 *ekp,
                     const double2 *eq, const double *ph_en, const double *masses,
                     const double2 *gm, const int64_t *gm_index, int64_t gm_stride,
                     const double2 *Lv, double *g2, cudaStream_t st);

// ---- polar long-range terms (wannier.f90:784-901, 1013-1071) ----
// Crystal data of a polar crystal on the device (ephg_set_polar).  The Ewald
// sums run over the box of reciprocal-lattice vectors m1 b1 + m2 b2 + m3 b3,
// |m_i| <= coarse_qmesh(i), with the cut qeq / (4 alph) < gmax.
struct PolarDev {
  int nat = 0, nb = 0, M = 0;
  const double *G = nullptr;      // [M][3] box vectors, Cartesian 1/bohr, in the reference's loop order
  const double *Gcell = nullptr;  // [Mcell][3] those of them that can pass the cut for q in the first cell
  int Mcell = 0;
  const double *born = nullptr;   // born(x, ipol, at) at x + 3 ipol + 9 at
  const double *tau = nullptr;    // [nat][3] Cartesian basis, bohr
  const double2 *Da = nullptr;    // (nb,nb) column-major: the q-independent sum (before fac)
  const double *masses = nullptr; // per atom, amu
  double eps[9];                  // dielectric tensor, column-major
  double rec[9];                  // reciprocal vectors (columns, 1/nm, with 2 pi)
  double alph = 0, gmax = 14.0, fac = 0;   // tpiba^2 (1/bohr^2), cut, 8 pi / volume (1/bohr^3)
};
// Per q (mesh index qp[q] on `mesh`, else crystal coordinates qv (nq,3)
// column-major): Dq[q] += massnorm * dyn_l(q) (nullable; layout of
// launch_dbuild), dDq[q] += massnorm * ddyn_l(q) * bohr2nm (nullable), and
// Lq[q][c] (nullable) with long_range_prefac(q, u) = sum_c Lq[q][c] u[c].
void launch_polar_q(const PolarDev &P, int nq, const int *qp, const int mesh[3], const double *qv,
                    double2 *Dq, double2 *dDq, double2 *Lq, cudaStream_t st);
// The q-independent part of dyn_nonanalytic into Da (nb,nb), once per crystal.
void launch_polar_da(const PolarDev &P, double2 *Da, cudaStream_t st);
// glp[q][s] = sum_c Lq[q][c] u[q][s][c] (u = evec / sqrt(M)), and its fp32 copy (nullable)
void launch_glprefac(int nq, int nb, const double2 *Lq, const double2 *u, double2 *glp, float2 *glpf,
                     cudaStream_t st);

// ---- q index table (vector.f90:86-102 on integers) ----
void launch_kq_index(const int mesh[3], int nk, const int64_t *k_idx, int nkp,
                     const int64_t *kp_idx, int64_t *q_idx, int *err, cudaStream_t st);

// ---- rate pipeline ----
void launch_window_flags(int N, int nw, const double *ens, double enref, double fsthick,
                         int *flag, cudaStream_t st);
void launch_state_flags(int nwv, int nw, const int *widx, const double *ens, double enref,
                        double fsthick, int *flag, int *nin_k, cudaStream_t st);
void launch_iota(int n, int *out, cudaStream_t st);
// Stage A rotation: B[Rp][c] (ldb) for states j in [j0,j1) of k-chunk [i0, i0+kc):
// B = conj(e^{2 pi i k.Rp})/deg(Rp) * sum_m' U_k[m][m'] gk(n',m',s',Rp)
void launch_rotate_states_fp64(int j0, int j1, int i0, const int *st_code, int nw, int nb,
                               int nws, const int *widx, const double2 *U, const double2 *gk,
                               int64_t ldgk, const int mesh[3], int L, const double2 *roots,
                               const int *Rq, const double *degq, double2 *B, int64_t ldb,
                               cudaStream_t st);
struct EpiData {
  const int *widx;      // window (k' row) -> mesh index
  const int *st_code;   // state -> i*nw + m, i the state's k row (an A-row)
  const int *sidx;      // A-row (the k of initial states) -> mesh index
  const int *swin;      // A-row -> window index (simplices); null: the identity
  const int *cum;       // window k' -> first (k',n) final-state rank
  const double *ens;    // [p][b] eV
  const double2 *U;     // [p][b][c]
  const float2 *Uf;     // same in fp32 (split path)
  const double *om;     // [q][s] eV
  const double2 *u;     // [q][s][c] evec/sqrt(M)
  const float2 *uf;     // same in fp32
  const double *bose;   // [q][s]
  // triangle / tetrahedron delta data (window-k indexed, 0-based)
  const int *smap;      // (nwv, maxc, 2): simplex, vertex(1-based)
  const int *scount;    // (nwv)
  const double *sevals; // (nsimplex, nw, nv) sorted vertex energies
  int nsimplex, maxc, nvx;
  int64_t per_state;    // vertices per initial state
  double *g2, *xp, *xm; // optional vertex lists
  int64_t cap;
  // phonon side (ibzq 'Y' + the ph-e rates), both nullable: phr (N, nb)
  // column-major receives ph_scale * Y summed over the vertices of each (q, s)
  // (device atomics); yv is the optional per-vertex Y list in the order of g2
  double *phr, *yv;
  double ph_scale;      // el%spindeg
  // polar crystals: glp[q][s] = long_range_prefac(q, u_s), added to each vertex
  // as glp * <U_k'[n]|U_k[m]> (wannier.f90:998-1006); nullable
  const double2 *glp;
  const float2 *glpf;   // same in fp32 (split path)
};
// Parameter sets of a merged request (ephg_el_rates_sets): requests that differ
// only in T, sigma and chempot share their vertices and |g|^2, so the
// contractions run once and the rate epilogue once per set.  Set 0 is the
// request itself (its RateParams, EpiData.bose and partial buffer); sets 1..n-1
// carry their own parameters, FP64 Bose factors and rate partials.
constexpr int MAX_SETS = 8;   // EPHG_MAX_SETS
struct RateSets {
  int n;
  RateParams rp[MAX_SETS];
  double *bose[MAX_SETS];      // [q][s] per set (set 0: EpiData.bose)
  double *partial[MAX_SETS];   // [j][iblk] per set (set 0: the caller's partial)
};
// per (k', state) epilogue on an FP64 C chunk: rates partial sums [j][iblk]
void launch_epilogue_fp64(int nwv, int j0, int j1, const double2 *C, int64_t ldc,
                          const RateParams &rp, const EpiData &d, double *partial,
                          int nblk, cudaStream_t st);
void launch_epilogue_fp32(int nwv, int j0, int j1, const float *Cr, const float *Ci,
                          int64_t ldc, const RateParams &rp, const EpiData &d, double *partial,
                          int nblk, cudaStream_t st);
void launch_bose(int N, int nb, const double *om, double T, double *bose, cudaStream_t st);
void launch_rate_final(int nst, int nblk, const double *partial, const int *st_code, int nw,
                       int N, double *rates_f, cudaStream_t st);
// degenerate-subspace averaging of a vertex list (3 launches); 1 if nw or nb > 64
int launch_degenerate_average(double *g2, int64_t per, int nin, const int *st_code, const int *arow, const int *widx,
                              const int *cum, const int *first_state, const double *ens, const double *om, int nst,
                              int nA, int nwv, int nw, int nb, const int mesh[3], double enref, double fsthick,
                              double thres, int mode, cudaStream_t st);

}  // namespace ephg
