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
void launch_g2_batch(int nv, int nw, int nb, int nws, const double *qv, const int *R,
                     const double *deg, const double2 *ek, const double2 *ekp,
                     const double2 *eq, const double *ph_en, const double *masses,
                     const double2 *gm, const int64_t *gm_index, int64_t gm_stride,
                     double *g2, cudaStream_t st);

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
  const int *widx;      // window -> mesh index
  const int *st_code;   // state -> i*nw + m
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

}  // namespace ephg
