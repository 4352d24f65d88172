/*
 * ephg_oracle.c - CPU FP64 restatement of elphbolt's e-ph vertex path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed
 * CPU baseline.  Nothing in the product links, loads or calls this file.
 * See ephg_oracle.h for the list of reference functions restated here and for
 * the parity status.  Every function names the reference lines it follows.
 */
#include "ephg_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double wall_us(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e6 + ts.tv_nsec * 1e-3;
}

typedef double complex cplx;

/* ---- constants: src/params.f90:27-57 ---- */
static const double qe = 1.602176634e-19;
static const double me = 9.1093837015e-31;
static const double amu = 1.66053906660e-27;
static const double hbar = 1.05457172647e-22;
#define HBAR_EVPS (hbar / qe)
#define KB (1.380649e-23 / qe)
#define PI (4.0 * atan(1.0))
#define TWOPI (2.0 * PI)
#define HARTREE2RADTHZ (27.2116 * qe / hbar)
#define RYD2RADTHZ (0.5 * HARTREE2RADTHZ)
#define RYD2EV (0.5 * 27.2116)
#define RYD2AMU (2.0 * me / amu)
#define BOHR2NM 0.052917721092   /* params.f90:53 */

static inline cplx cget(const double *p, int64_t i) { return p[2 * i] + I * p[2 * i + 1]; }
static inline void cset(double *p, int64_t i, cplx v) { p[2 * i] = creal(v); p[2 * i + 1] = cimag(v); }
/* expi: misc.f90:588-594 */
static inline cplx expi(double x) { return cos(x) + I * sin(x); }

/* ======================= index helpers ======================= */

/* mux_vector: misc.f90:906-923 */
int64_t or_mux_vector(const int64_t v[3], const int64_t mesh[3], int64_t base) {
  if (base == 0) return (v[2] * mesh[1] + v[1]) * mesh[0] + v[0] + 1;
  return ((v[2] - 1) * mesh[1] + (v[1] - 1)) * mesh[0] + v[0];
}

/* demux_vector: misc.f90:925-942 (int_div = Fortran truncating / and mod) */
void or_demux_vector(int64_t i, int64_t v[3], const int64_t mesh[3], int64_t base) {
  int64_t aux = (i - 1) / mesh[0];
  v[0] = (i - 1) % mesh[0];
  v[2] = aux / mesh[1];
  v[1] = aux % mesh[1];
  if (base == 1) { v[0] += 1; v[1] += 1; v[2] += 1; }
}

/* mux_state / demux_state: misc.f90:965-990 */
int64_t or_mux_state(int64_t nbands, int64_t iband, int64_t ik) { return (ik - 1) * nbands + iband; }
void or_demux_state(int64_t m, int64_t nbands, int64_t *iband, int64_t *ik) {
  int64_t r = (m - 1) % nbands;
  if (r < 0) r += nbands;             /* Fortran modulo */
  *iband = r + 1;
  *ik = (m - 1) / nbands + 1;
}

/* binsearch: misc.f90:738-763.  Returns the 1-based position or -1. */
int64_t or_binsearch(const int64_t *array, int64_t n, int64_t e) {
  int64_t a = 1, b = n, m = (b + a) / 2;
  int64_t mid = array[m - 1];
  while (mid != e) {
    if (e > mid) a = m + 1;
    else if (e < mid) b = m - 1;
    if (a > b) return -1;
    m = (b + a) / 2;
    mid = array[m - 1];
  }
  return m;
}

/* .umklapp. = add_and_fold: misc.f90:596-610 */
void or_umklapp(const double q1[3], const double q2[3], double q3[3]) {
  for (int i = 0; i < 3; ++i) {
    q3[i] = q1[i] + q2[i];
    if (q3[i] >= 1.0) q3[i] = q3[i] - 1.0;
    if (q3[i] < 0.0) q3[i] = q3[i] + 1.0;
  }
}

static void matvec3(const double m[9], const double v[3], double o[3]) {
  for (int i = 0; i < 3; ++i) o[i] = m[i] * v[0] + m[i + 3] * v[1] + m[i + 6] * v[2];
}

/* vector_allreps create: vector.f90:38-56 */
void or_vector_create(int64_t ind, const int64_t grid[3], const double prim[9],
                      int64_t iv[3], int64_t *muxed, double frac[3], double cart[3]) {
  *muxed = ind;
  or_demux_vector(ind, iv, grid, 0);
  for (int i = 0; i < 3; ++i) frac[i] = (double)iv[i] / (double)grid[i];
  matvec3(prim, frac, cart);
}

/* vector_allreps_add (sign=+1) / _sub (sign=-1): vector.f90:68-102 */
void or_vector_addsub(int64_t ind1, int64_t ind2, int sign, const int64_t grid[3],
                      const double prim[9], int64_t iv[3], int64_t *muxed,
                      double frac[3], double cart[3]) {
  int64_t i1[3], i2[3], mx;
  double f1[3], f2[3], c[3];
  or_vector_create(ind1, grid, prim, i1, &mx, f1, c);
  or_vector_create(ind2, grid, prim, i2, &mx, f2, c);
  if (sign < 0) for (int i = 0; i < 3; ++i) f2[i] = -f2[i];
  or_umklapp(f1, f2, frac);
  matvec3(prim, frac, cart);
  for (int i = 0; i < 3; ++i) iv[i] = (int64_t)llround(frac[i] * (double)grid[i]);
  *muxed = or_mux_vector(iv, grid, 0);
}

/* vector_allreps_change_grid: vector.f90:104-120 */
void or_vector_change_grid(const double frac[3], const int64_t grid[3], int64_t iv[3], int64_t *muxed) {
  for (int i = 0; i < 3; ++i) iv[i] = (int64_t)llround(frac[i] * (double)grid[i]);
  *muxed = or_mux_vector(iv, grid, 0);
}

/* expm1: misc.f90:1011-1019.  The reference evaluates exp(x) - 1 in real128
 * and rounds to real64; C's expm1 returns that value to within one ulp
 * (80-bit long double, the x86 fallback, loses ~1e-9 relative at x ~ 1e-10). */
double or_expm1(double x) { return expm1(x); }
/* Bose: misc.f90:992-999 */
double or_Bose(double e, double T) { return 1.0 / or_expm1(e / KB / T); }
/* Fermi: misc.f90:1001-1009 */
double or_Fermi(double e, double chempot, double T) { return 1.0 / (exp((e - chempot) / KB / T) + 1.0); }

/* ======================= eigen solver ======================= */

/*
 * Hermitian eigenproblem by cyclic complex Jacobi rotations (Golub & Van Loan
 * sec. 8.5), standing in for LAPACK zheev('V','U') at wannier.f90:489,732.
 * A: (n,n) column-major complex; only the upper triangle is read (zheev 'U').
 * w: ascending eigenvalues; V: (n,n) eigenvectors as columns.
 * Returns the number of sweeps, or -1 if not converged.
 */
int or_herm_eig(int64_t n, double *A_in, double *w, double *V_out) {
  cplx *A = (cplx *)malloc(sizeof(cplx) * n * n);
  cplx *V = (cplx *)malloc(sizeof(cplx) * n * n);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) {
      cplx u = (i <= j) ? cget(A_in, i + n * j) : conj(cget(A_in, j + n * i));
      if (i == j) u = creal(u);
      A[i + n * j] = u;
      V[i + n * j] = (i == j) ? 1.0 : 0.0;
    }
  int sweeps = 0, ok = 0;
  for (; sweeps < 100; ++sweeps) {
    double off = 0.0, tot = 0.0;
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < n; ++i) {
        double a2 = creal(A[i + n * j]) * creal(A[i + n * j]) + cimag(A[i + n * j]) * cimag(A[i + n * j]);
        tot += a2;
        if (i != j) off += a2;
      }
    if (off <= 1e-32 * tot || off == 0.0) { ok = 1; break; }
    for (int64_t p = 0; p < n - 1; ++p)
      for (int64_t q = p + 1; q < n; ++q) {
        cplx apq = A[p + n * q];
        double r = cabs(apq);
        if (r == 0.0) continue;
        cplx ph = apq / r;                       /* e^{i phi} */
        double app = creal(A[p + n * p]), aqq = creal(A[q + n * q]);
        double tau = (aqq - app) / (2.0 * r);
        double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        /* J = [[c, s], [-s e^{-i phi}, c e^{-i phi}]] on (p, q); A <- J^H A J, V <- V J */
        cplx phc = conj(ph);
        for (int64_t k = 0; k < n; ++k) {      /* columns: A <- A J */
          cplx akp = A[k + n * p], akq = A[k + n * q];
          A[k + n * p] = c * akp - s * phc * akq;
          A[k + n * q] = s * akp + c * phc * akq;
          cplx vkp = V[k + n * p], vkq = V[k + n * q];
          V[k + n * p] = c * vkp - s * phc * vkq;
          V[k + n * q] = s * vkp + c * phc * vkq;
        }
        for (int64_t k = 0; k < n; ++k) {      /* rows: A <- J^H A */
          cplx apk = A[p + n * k], aqk = A[q + n * k];
          A[p + n * k] = c * apk - s * ph * aqk;
          A[q + n * k] = s * apk + c * ph * aqk;
        }
        A[p + n * q] = 0.0;
        A[q + n * p] = 0.0;
        A[p + n * p] = creal(A[p + n * p]);
        A[q + n * q] = creal(A[q + n * q]);
      }
  }
  /* sort ascending (selection sort keeps it simple and deterministic) */
  int64_t *ord = (int64_t *)malloc(sizeof(int64_t) * n);
  double *ev = (double *)malloc(sizeof(double) * n);
  for (int64_t i = 0; i < n; ++i) { ord[i] = i; ev[i] = creal(A[i + n * i]); }
  for (int64_t i = 0; i < n; ++i) {
    int64_t b = i;
    for (int64_t j = i + 1; j < n; ++j) if (ev[ord[j]] < ev[ord[b]]) b = j;
    int64_t t = ord[i]; ord[i] = ord[b]; ord[b] = t;
  }
  for (int64_t j = 0; j < n; ++j) {
    w[j] = ev[ord[j]];
    for (int64_t i = 0; i < n; ++i) cset(V_out, i + n * j, V[i + n * ord[j]]);
  }
  free(ord); free(ev); free(A); free(V);
  return ok ? sweeps : -1;
}

/* ======================= Wannier interpolation ======================= */

/* el_wann: wannier.f90:430-524 */
void or_el_wann(const or_wannier *w, int64_t nk, const double *kvecs, double *energies,
                double *evecs, double *velocities, const double *scissor) {
  const int64_t nw = w->nw, nwsk = w->nwsk;
  /* the k-points are independent: OpenMP over them, buffers per thread */
#pragma omp parallel
  {
  double *H = (double *)malloc(sizeof(double) * 2 * nw * nw);
  double *dH = (double *)malloc(sizeof(double) * 2 * 3 * nw * nw);
  double *V = (double *)malloc(sizeof(double) * 2 * nw * nw);
  double *ev = (double *)malloc(sizeof(double) * nw);
#pragma omp for schedule(dynamic, 16)
  for (int64_t ik = 0; ik < nk; ++ik) {
    cplx *Hc = (cplx *)calloc(nw * nw, sizeof(cplx));
    cplx *dHc = (cplx *)calloc(3 * nw * nw, sizeof(cplx));
    for (int64_t iuc = 0; iuc < nwsk; ++iuc) {
      double dot = 0.0;
      for (int d = 0; d < 3; ++d) dot += kvecs[ik + nk * d] * (double)w->rcells_k[iuc + nwsk * d];
      cplx caux = expi(TWOPI * dot) / (double)w->elwsdeg[iuc];
      double rcart[3] = {0, 0, 0};
      if (velocities) {
        double r[3] = {(double)w->rcells_k[iuc], (double)w->rcells_k[iuc + nwsk], (double)w->rcells_k[iuc + 2 * nwsk]};
        matvec3(w->lattvecs, r, rcart);
      }
      for (int64_t jb = 0; jb < nw; ++jb)
        for (int64_t ib = 0; ib < nw; ++ib) {
          cplx h = cget(w->Hwann, iuc + nwsk * (ib + nw * jb));
          Hc[ib + nw * jb] += caux * h;
          if (velocities)
            for (int p = 0; p < 3; ++p) dHc[p + 3 * (ib + nw * jb)] += I * rcart[p] * caux * h;
        }
    }
    /* force Hermiticity on the upper triangle (:481-486) */
    for (int64_t ib = 0; ib < nw; ++ib)
      for (int64_t jb = ib + 1; jb < nw; ++jb) {
        Hc[ib + nw * jb] = (Hc[ib + nw * jb] + conj(Hc[jb + nw * ib])) * 0.5;
        Hc[jb + nw * ib] = Hc[ib + nw * jb];
      }
    for (int64_t i = 0; i < nw * nw; ++i) cset(H, i, Hc[i]);
    or_herm_eig(nw, H, ev, V);
    /* evecs(ik,b,:) = column b of the eigenvector matrix (transpose at :501) */
    for (int64_t b = 0; b < nw; ++b) {
      if (evecs)
        for (int64_t c = 0; c < nw; ++c) cset(evecs, ik + nk * (b + nw * c), cget(V, c + nw * b));
      if (velocities)
        for (int p = 0; p < 3; ++p) {
          cplx acc = 0.0;
          for (int64_t r = 0; r < nw; ++r) {
            cplx mv = 0.0;
            for (int64_t c = 0; c < nw; ++c) mv += dHc[p + 3 * (r + nw * c)] * cget(V, c + nw * b);
            acc += conj(cget(V, r + nw * b)) * mv;
          }
          velocities[ik + nk * (b + nw * p)] = creal(acc) * RYD2RADTHZ;
        }
      energies[ik + nk * b] = ev[b] * RYD2EV;
      if (scissor) energies[ik + nk * b] += scissor[b];
    }
    free(Hc); free(dHc);
  }
  free(H); free(dH); free(V); free(ev);
  }
}

/* ws_wrapping_vectors: wannier.f90:532-582.  Returns the number of wrappers.
 * The reference counts them in a first pass and fills them in a second; with
 * distances within 2 eps of each other the two counts can differ, and this
 * restatement returns the second-pass count. */
int or_ws_wrapping_vectors(const double lvec[9], const double vl[3], double eps,
                           int64_t *wrappers, int maxw) {
  int64_t iv0[3];
  double wl[3];
  for (int i = 0; i < 3; ++i) { iv0[i] = (int64_t)trunc(vl[i]); wl[i] = vl[i] - (double)iv0[i]; }
  double d = 1.79769313486231570815e308;
  int n = 0;
  for (int k = -3; k <= 3; ++k)
    for (int j = -3; j <= 3; ++j)
      for (int i = -3; i <= 3; ++i) {
        double v[3] = {wl[0] + i, wl[1] + j, wl[2] + k}, wc[3];
        matvec3(lvec, v, wc);
        double nr = sqrt(wc[0] * wc[0] + wc[1] * wc[1] + wc[2] * wc[2]);
        if (fabs(nr - d) < eps) n++;
        else if (nr < d) { n = 1; d = nr; }
      }
  n = 0;
  for (int k = -3; k <= 3; ++k)
    for (int j = -3; j <= 3; ++j)
      for (int i = -3; i <= 3; ++i) {
        double v[3] = {wl[0] + i, wl[1] + j, wl[2] + k}, wc[3];
        matvec3(lvec, v, wc);
        double nr = sqrt(wc[0] * wc[0] + wc[1] * wc[1] + wc[2] * wc[2]);
        if (fabs(nr - d) < eps) {
          if (n < maxw) {
            wrappers[3 * n + 0] = i - iv0[0];
            wrappers[3 * n + 1] = j - iv0[1];
            wrappers[3 * n + 2] = k - iv0[2];
          }
          n++;
        }
      }
  return n;
}

/* ph_wann (non-polar branch): wannier.f90:585-782.  Returns 1 on a large
 * negative phonon energy (the reference stops there), else 0. */
/* ======================= polar long-range terms ======================= */

/* Reciprocal vectors (columns, 1/nm, with 2 pi) and cell volume (nm^3):
 * crystal.f90:284-293.  Cartesian basis (nm): crystal.f90:282. */
static void polar_cell(const or_wannier *w, double rec[9], double *vol, double *bc) {
  const double *a = w->lattvecs;
  for (int i = 0; i < 3; ++i) {
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    rec[0 + 3 * i] = a[1 + 3 * j] * a[2 + 3 * k] - a[2 + 3 * j] * a[1 + 3 * k];
    rec[1 + 3 * i] = a[2 + 3 * j] * a[0 + 3 * k] - a[0 + 3 * j] * a[2 + 3 * k];
    rec[2 + 3 * i] = a[0 + 3 * j] * a[1 + 3 * k] - a[1 + 3 * j] * a[0 + 3 * k];
  }
  *vol = fabs(a[0] * rec[0] + a[1] * rec[1] + a[2] * rec[2]);
  for (int i = 0; i < 9; ++i) rec[i] *= TWOPI / *vol;
  for (int64_t at = 0; at < w->natoms; ++at) matvec3(a, w->basis + 3 * at, bc + 3 * at);
}

/* q in crystal coordinates -> Cartesian 1/bohr: matmul(reclattvecs, q) * bohr2nm */
void or_q_cart_bohr(const or_wannier *w, const double qf[3], double qc[3]) {
  double rec[9], vol, bc[3 * 64];
  polar_cell(w, rec, &vol, bc);
  matvec3(rec, qf, qc);
  for (int d = 0; d < 3; ++d) qc[d] *= BOHR2NM;
}

/* z(j) = sum_i g(i) born(i, j, at): matmul(g, born(:,:,at)) */
static void gdotz(const double *born, int64_t at, const double g[3], double z[3]) {
  for (int j = 0; j < 3; ++j) z[j] = g[0] * born[0 + 3 * j + 9 * at] + g[1] * born[1 + 3 * j + 9 * at] +
                                     g[2] * born[2 + 3 * j + 9 * at];
}

static double geg(const double *eps, const double g[3]) {   /* dot_product(g, matmul(epsilon, g)) */
  double acc = 0.0;
  for (int i = 0; i < 3; ++i) acc += g[i] * (eps[i] * g[0] + eps[i + 3] * g[1] + eps[i + 6] * g[2]);
  return acc;
}

/* dyn_nonanalytic: wannier.f90:784-901.  q Cartesian (1/bohr); dyn_l (nb,nb)
 * complex, ddyn_l (nb,nb,3) complex or NULL, both in Ry / bohr units. */
void or_dyn_nonanalytic(const or_wannier *w, const double q[3], double *dyn_l, double *ddyn_l) {
  const int64_t nat = w->natoms, nb = 3 * nat;
  const double *born = w->born, *eps = w->epsilon;
  double rec[9], vol, bc[3 * 64];
  polar_cell(w, rec, &vol, bc);
  const double a1 = sqrt(w->lattvecs[0] * w->lattvecs[0] + w->lattvecs[1] * w->lattvecs[1] +
                         w->lattvecs[2] * w->lattvecs[2]);
  const double tpiba = TWOPI / a1 * BOHR2NM;
  const double gmax = 14.0, alph = tpiba * tpiba;
  const double fac = 8.0 * PI / (vol / (BOHR2NM * BOHR2NM * BOHR2NM));
  cplx *D = (cplx *)calloc(nb * nb, sizeof(cplx));
  cplx *dD = (cplx *)calloc(nb * nb * 3, sizeof(cplx));
  const int64_t n1 = w->coarse_qmesh[0], n2 = w->coarse_qmesh[1], n3 = w->coarse_qmesh[2];
  for (int64_t m1 = -n1; m1 <= n1; ++m1)
    for (int64_t m2 = -n2; m2 <= n2; ++m2)
      for (int64_t m3 = -n3; m3 <= n3; ++m3) {
        double g[3];
        for (int d = 0; d < 3; ++d)
          g[d] = ((double)m1 * rec[d] + (double)m2 * rec[d + 3] + (double)m3 * rec[d + 6]) * BOHR2NM;
        double qeq = geg(eps, g);
        if (qeq > 0.0 && qeq / alph / 4.0 < gmax) {     /* the q-independent term (:843-867) */
          const double facqd = exp(-qeq / alph / 4.0) / qeq;
          for (int64_t iat = 0; iat < nat; ++iat) {
            double zig[3], zjg[3];
            gdotz(born, iat, g, zig);
            cplx fnat[3] = {0, 0, 0};
            for (int64_t jat = 0; jat < nat; ++jat) {
              double rr[3];
              for (int d = 0; d < 3; ++d) rr[d] = (bc[d + 3 * iat] - bc[d + 3 * jat]) / BOHR2NM;
              const double arg = g[0] * rr[0] + g[1] * rr[1] + g[2] * rr[2];
              gdotz(born, jat, g, zjg);
              for (int d = 0; d < 3; ++d) fnat[d] += zjg[d] * expi(arg);
            }
            for (int ip = 0; ip < 3; ++ip)
              for (int jp = 0; jp < 3; ++jp) D[(3 * iat + ip) + nb * (3 * iat + jp)] -= facqd * zig[ip] * fnat[jp];
          }
        }
        for (int d = 0; d < 3; ++d) g[d] += q[d];
        qeq = geg(eps, g);
        if (qeq > 0.0 && qeq / alph / 4.0 < gmax) {     /* the G + q term (:869-897) */
          const double facqd = exp(-qeq / alph / 4.0) / qeq;
          double dgeg[3];
          for (int i = 0; i < 3; ++i)
            dgeg[i] = (eps[i] + eps[3 * i]) * g[0] + (eps[i + 3] + eps[3 * i + 1]) * g[1] +
                      (eps[i + 6] + eps[3 * i + 2]) * g[2];
          const double dgeg_coeff = 0.25 / alph + 1.0 / qeq;
          for (int64_t iat = 0; iat < nat; ++iat) {
            double zig[3], zjg[3];
            gdotz(born, iat, g, zig);
            for (int64_t jat = 0; jat < nat; ++jat) {
              double rr[3];
              for (int d = 0; d < 3; ++d) rr[d] = (bc[d + 3 * iat] - bc[d + 3 * jat]) / BOHR2NM;
              gdotz(born, jat, g, zjg);
              const double arg = g[0] * rr[0] + g[1] * rr[1] + g[2] * rr[2];
              const cplx facq = facqd * expi(arg);
              for (int ip = 0; ip < 3; ++ip)
                for (int jp = 0; jp < 3; ++jp) {
                  const int64_t ij = (3 * iat + ip) + nb * (3 * jat + jp);
                  D[ij] += facq * zig[ip] * zjg[jp];
                  if (ddyn_l)
                    for (int x = 0; x < 3; ++x)
                      dD[ij + nb * nb * x] += facq * (zjg[jp] * born[x + 3 * ip + 9 * iat] +
                                                      zig[ip] * born[x + 3 * jp + 9 * jat] +
                                                      zig[ip] * zjg[jp] * (I * rr[x] - dgeg_coeff * dgeg[x]));
                }
            }
          }
        }
      }
  for (int64_t i = 0; i < nb * nb; ++i) cset(dyn_l, i, D[i] * fac);
  if (ddyn_l)
    for (int64_t i = 0; i < 3 * nb * nb; ++i) cset(ddyn_l, i, dD[i] * fac);
  free(D);
  free(dD);
}

/* long_range_prefac: wannier.f90:1013-1071.  q Cartesian (1/bohr), uqs (nb)
 * complex = the mass-scaled phonon eigenvector; returns glprefac (Ry units). */
void or_long_range_prefac(const or_wannier *w, const double q[3], const double *uqs, double *glprefac) {
  const int64_t nat = w->natoms;
  const double *born = w->born, *eps = w->epsilon;
  double rec[9], vol, bc[3 * 64];
  polar_cell(w, rec, &vol, bc);
  const double a1 = sqrt(w->lattvecs[0] * w->lattvecs[0] + w->lattvecs[1] * w->lattvecs[1] +
                         w->lattvecs[2] * w->lattvecs[2]);
  const double tpiba = TWOPI / a1 * BOHR2NM;
  const double gmax = 14.0, alph = tpiba * tpiba;
  const cplx fac = 8.0 * PI / (vol / (BOHR2NM * BOHR2NM * BOHR2NM)) * I;
  cplx acc = 0.0;
  const int64_t n1 = w->coarse_qmesh[0], n2 = w->coarse_qmesh[1], n3 = w->coarse_qmesh[2];
  for (int64_t m1 = -n1; m1 <= n1; ++m1)
    for (int64_t m2 = -n2; m2 <= n2; ++m2)
      for (int64_t m3 = -n3; m3 <= n3; ++m3) {
        double g[3];
        for (int d = 0; d < 3; ++d)
          g[d] = ((double)m1 * rec[d] + (double)m2 * rec[d + 3] + (double)m3 * rec[d + 6]) * BOHR2NM + q[d];
        const double qeq = geg(eps, g);
        if (qeq > 0.0 && qeq / alph / 4.0 < gmax) {
          const double facqd = exp(-qeq / alph / 4.0) / qeq;
          for (int64_t na = 0; na < nat; ++na) {
            const double arg = -(g[0] * bc[3 * na] + g[1] * bc[3 * na + 1] + g[2] * bc[3 * na + 2]) / BOHR2NM;
            const cplx facq = facqd * expi(arg);
            for (int ip = 0; ip < 3; ++ip) {
              const double zaq = g[0] * born[0 + 3 * ip + 9 * na] + g[1] * born[1 + 3 * ip + 9 * na] +
                                 g[2] * born[2 + 3 * ip + 9 * na];
              acc += facq * zaq * cget(uqs, 3 * na + ip);
            }
          }
        }
      }
  cset(glprefac, 0, acc * fac);
}

int or_ph_wann(const or_wannier *w, int64_t nq, const double *qvecs, double *energies,
               double *evecs, double *velocities) {
  const int64_t nb = w->nb, nwsq = w->nwsq, nat = w->natoms;
  int status = 0;
  cplx *caux_mat = (cplx *)malloc(sizeof(cplx) * nb * nb);
  cplx *dyn = (cplx *)malloc(sizeof(cplx) * nb * nb);
  cplx *ddyn = (cplx *)malloc(sizeof(cplx) * nb * nb * 3);
  double *Dd = (double *)malloc(sizeof(double) * 2 * nb * nb);
  double *V = (double *)malloc(sizeof(double) * 2 * nb * nb * 3);
  double *om2 = (double *)malloc(sizeof(double) * nb);
  /* ws_wrapping_vectors depends on the cell and the atom pair, not on q: the
   * reference calls it per q (:642); here it runs once per call, with the same
   * wrappers in the same order, so every sum below is unchanged */
  const int64_t npair = nwsq * nat * nat;
  int *wn = (int *)malloc(sizeof(int) * npair);
  int64_t *woff = (int64_t *)malloc(sizeof(int64_t) * (npair + 1));
  int64_t wcap = 8 * npair + 512, wtot = 0;
  int64_t *wall = (int64_t *)malloc(sizeof(int64_t) * 3 * wcap);
  {
    int64_t wr[3 * 512];
    for (int64_t iuc = 0; iuc < nwsq; ++iuc)
      for (int64_t jat = 0; jat < nat; ++jat)
        for (int64_t iat = 0; iat < nat; ++iat) {
          double dist[3];
          for (int d = 0; d < 3; ++d)
            dist[d] = ((double)w->rcells_q[iuc + nwsq * d] - w->basis[d + 3 * iat] + w->basis[d + 3 * jat]) /
                      (double)w->coarse_qmesh[d];
          const int64_t pi = iat + nat * (jat + nat * iuc);
          int nwrap = or_ws_wrapping_vectors(w->lattvecs, dist, 1.0e-6, wr, 512);
          if (wtot + nwrap > wcap) {
            wcap = 2 * (wtot + nwrap);
            wall = (int64_t *)realloc(wall, sizeof(int64_t) * 3 * wcap);
          }
          wn[pi] = nwrap;
          woff[pi] = wtot;
          for (int i = 0; i < 3 * nwrap; ++i) wall[3 * wtot + i] = wr[i];
          wtot += nwrap;
        }
  }
  for (int64_t iq = 0; iq < nq; ++iq) {
    for (int64_t i = 0; i < nb * nb; ++i) dyn[i] = 0.0;
    for (int64_t i = 0; i < 3 * nb * nb; ++i) ddyn[i] = 0.0;
    for (int64_t iuc = 0; iuc < nwsq; ++iuc) {
      for (int64_t i = 0; i < nb * nb; ++i) caux_mat[i] = 0.0;
      for (int64_t jat = 0; jat < nat; ++jat)
        for (int64_t iat = 0; iat < nat; ++iat) {
          const int64_t pi = iat + nat * (jat + nat * iuc);
          const int nwrap = wn[pi];
          const int64_t *wr = wall + 3 * woff[pi];
          for (int iw = 0; iw < nwrap; ++iw) {
            double dot = 0.0;
            for (int d = 0; d < 3; ++d)
              dot += qvecs[iq + nq * d] *
                     (double)(w->rcells_q[iuc + nwsq * d] + wr[3 * iw + d] * w->coarse_qmesh[d]);
            cplx caux = expi(TWOPI * dot);
            double den = (double)(w->phwsdeg[iuc] * nwrap);
            for (int64_t b = 0; b < 3; ++b)
              for (int64_t a = 0; a < 3; ++a)
                caux_mat[(3 * iat + a) + nb * (3 * jat + b)] += caux / den;
          }
        }
      double rcart[3] = {0, 0, 0};
      if (velocities) {
        double r[3] = {(double)w->rcells_q[iuc], (double)w->rcells_q[iuc + nwsq], (double)w->rcells_q[iuc + 2 * nwsq]};
        matvec3(w->lattvecs, r, rcart);
      }
      for (int64_t j = 0; j < nb; ++j)
        for (int64_t i = 0; i < nb; ++i) {
          cplx t = caux_mat[i + nb * j] * cget(w->Dphwann, iuc + nwsq * (i + nb * j));
          dyn[i + nb * j] += t;
          if (velocities)
            for (int p = 0; p < 3; ++p) ddyn[i + nb * (j + nb * p)] += I * rcart[p] * t;
        }
    }
    /* non-analytic correction (:684-705) */
    if (w->polar) {
      const double qf[3] = {qvecs[iq], qvecs[iq + nq], qvecs[iq + 2 * nq]};
      double qc[3];
      or_q_cart_bohr(w, qf, qc);
      or_dyn_nonanalytic(w, qc, Dd, velocities ? V : NULL);   /* Dd, V as scratch */
      if (velocities)
        for (int64_t i = 0; i < 3 * nb * nb; ++i) ddyn[i] += cget(V, i) * BOHR2NM;
      for (int64_t i = 0; i < nb * nb; ++i) dyn[i] += cget(Dd, i);
    }
    /* force Hermiticity (:708-713) */
    for (int64_t ib = 0; ib < nb; ++ib)
      for (int64_t jb = ib + 1; jb < nb; ++jb) {
        dyn[ib + nb * jb] = (dyn[ib + nb * jb] + conj(dyn[jb + nb * ib])) * 0.5;
        dyn[jb + nb * ib] = dyn[ib + nb * jb];
      }
    /* mass normalise (:716-729) */
    for (int64_t na = 0; na < nat; ++na)
      for (int64_t nbb = 0; nbb < nat; ++nbb) {
        double massnorm = 1.0 / sqrt(w->masses[na] * w->masses[nbb]) * RYD2AMU;
        for (int64_t b = 0; b < 3; ++b)
          for (int64_t a = 0; a < 3; ++a) {
            int64_t idx = (3 * na + a) + nb * (3 * nbb + b);
            dyn[idx] *= massnorm;
            if (velocities) for (int p = 0; p < 3; ++p) ddyn[idx + nb * nb * p] *= massnorm;
          }
      }
    for (int64_t i = 0; i < nb * nb; ++i) cset(Dd, i, dyn[i]);
    or_herm_eig(nb, Dd, om2, V);
    for (int64_t s = 0; s < nb; ++s) {
      double e = sqrt(fabs(om2[s]));
      energies[iq + nq * s] = (om2[s] >= 0 && !signbit(om2[s])) ? e : -e;
    }
    if (evecs)
      for (int64_t s = 0; s < nb; ++s)
        for (int64_t c = 0; c < nb; ++c) cset(evecs, iq + nq * (s + nb * c), cget(V, c + nb * s));
    if (velocities)
      for (int64_t s = 0; s < nb; ++s) {
        for (int p = 0; p < 3; ++p) {
          cplx acc = 0.0;
          for (int64_t r = 0; r < nb; ++r) {
            cplx mv = 0.0;
            for (int64_t c = 0; c < nb; ++c) mv += ddyn[r + nb * (c + nb * p)] * cget(V, c + nb * s);
            acc += conj(cget(V, r + nb * s)) * mv;
          }
          velocities[iq + nq * (s + nb * p)] = creal(acc) / (2.0 * energies[iq + nq * s]);
        }
      }
    for (int64_t s = 0; s < nb; ++s) energies[iq + nq * s] *= RYD2EV;
    if (velocities)
      for (int64_t s = 0; s < nb; ++s)
        for (int p = 0; p < 3; ++p) velocities[iq + nq * (s + nb * p)] *= RYD2RADTHZ;
    /* Gamma point (:767-771) */
    if (qvecs[iq] == 0 && qvecs[iq + nq] == 0 && qvecs[iq + 2 * nq] == 0) {
      for (int64_t s = 0; s < 3 && s < nb; ++s) energies[iq + nq * s] = 0.0;
      if (velocities)
        for (int64_t s = 0; s < nb; ++s)
          for (int p = 0; p < 3; ++p) velocities[iq + nq * (s + nb * p)] = 0.0;
    }
    /* negative energies (:774-780) */
    for (int64_t s = 0; s < nb; ++s) {
      double e = energies[iq + nq * s];
      if (e < -0.005) status = 1;
      else if (e < 0 && e > -0.005) energies[iq + nq * s] = 0.0;
    }
  }
  free(caux_mat); free(dyn); free(ddyn); free(Dd); free(V); free(om2);
  free(wn); free(woff); free(wall);
  return status;
}

/* gkRp: wannier.f90:1073-1132 (gmixed(nw,nw,nb,nwsq); nwsg cells filled) */
void or_gkRp(const or_wannier *w, const double kvec[3], double *gmixed) {
  const int64_t nw = w->nw, nb = w->nb, nwsk = w->nwsk, nwsg = w->nwsg;
  const int64_t blk = nw * nw * nb;
  cplx *acc = (cplx *)calloc(blk * w->nwsq, sizeof(cplx));
  cplx *caux = (cplx *)malloc(sizeof(cplx) * nwsk);
  for (int64_t iuc = 0; iuc < nwsk; ++iuc) {
    double dot = 0.0;
    for (int d = 0; d < 3; ++d) dot += kvec[d] * (double)w->rcells_k[iuc + nwsk * d];
    caux[iuc] = expi(TWOPI * dot) / (double)w->elwsdeg[iuc];
  }
  /* the Rp blocks are independent: OpenMP over them, each element still summed over Re in order */
#pragma omp parallel for schedule(static)
  for (int64_t rp = 0; rp < nwsg; ++rp)
    for (int64_t iuc = 0; iuc < nwsk; ++iuc)
      for (int64_t s = 0; s < nb; ++s)
        for (int64_t j = 0; j < nw; ++j)
          for (int64_t i = 0; i < nw; ++i)
            acc[i + nw * (j + nw * (s + nb * rp))] +=
                caux[iuc] * cget(w->gwann, i + nw * (j + nw * (iuc + nwsk * (s + nb * rp))));
  for (int64_t i = 0; i < blk * w->nwsq; ++i) cset(gmixed, i, acc[i]);
  free(acc);
  free(caux);
}

/* gReq: wannier.f90:1134-1188 (gmixed(nw,nw,nb,nwsk)) */
void or_gReq(const or_wannier *w, const double qvec[3], double *gmixed) {
  const int64_t nw = w->nw, nb = w->nb, nwsk = w->nwsk, nwsg = w->nwsg;
  cplx *acc = (cplx *)calloc(nw * nw * nb * nwsk, sizeof(cplx));
  for (int64_t iuc = 0; iuc < nwsg; ++iuc) {
    double dot = 0.0;
    for (int d = 0; d < 3; ++d) dot += qvec[d] * (double)w->rcells_g[iuc + nwsg * d];
    cplx phase = expi(TWOPI * dot) / (double)w->gwsdeg[iuc];
    for (int64_t s = 0; s < nb; ++s)
      for (int64_t re = 0; re < nwsk; ++re)
        for (int64_t j = 0; j < nw; ++j)
          for (int64_t i = 0; i < nw; ++i)
            acc[i + nw * (j + nw * (s + nb * re))] +=
                phase * cget(w->gwann, i + nw * (j + nw * (re + nwsk * (s + nb * iuc))));
  }
  for (int64_t i = 0; i < nw * nw * nb * nwsk; ++i) cset(gmixed, i, acc[i]);
  free(acc);
}

/* g2 (non-polar): wannier.f90:903-1011 */
double or_g2(const or_wannier *w, const double kvec[3], const double qvec[3],
             const double *el_evec_k, const double *el_evec_kp, const double *ph_evec_q,
             double ph_en, const double *gmixed, int wannspace_ph) {
  const int64_t nw = w->nw, nb = w->nb;
  const double g2unitfactor = RYD2EV * RYD2EV * RYD2EV * RYD2AMU;
  cplx u[64], overlap[32 * 32];
  for (int64_t ip = 0; ip < nb; ++ip) u[ip] = cget(ph_evec_q, ip) / sqrt(w->masses[ip / 3]);
  if (ph_en == 0) return 0.0;
  const int64_t nws = wannspace_ph ? w->nwsg : w->nwsk;
  for (int64_t np = 0; np < nw; ++np)
    for (int64_t mp = 0; mp < nw; ++mp) overlap[mp + nw * np] = conj(cget(el_evec_kp, np)) * cget(el_evec_k, mp);
  cplx gbloch = 0.0;
  cplx *ukg = (cplx *)malloc(sizeof(cplx) * nb);
  for (int64_t iws = 0; iws < nws; ++iws) {
    for (int64_t sp = 0; sp < nb; ++sp) {
      cplx caux = 0.0;
      for (int64_t np = 0; np < nw; ++np)
        for (int64_t mp = 0; mp < nw; ++mp)
          caux += overlap[mp + nw * np] * cget(gmixed, np + nw * (mp + nw * (sp + nb * iws)));
      ukg[sp] = caux;
    }
    cplx ukgu = 0.0;
    for (int64_t sp = 0; sp < nb; ++sp) ukgu += u[sp] * ukg[sp];   /* dot_product(conjg(u), .) */
    double dot = 0.0;
    cplx caux;
    if (wannspace_ph) {
      for (int d = 0; d < 3; ++d) dot += qvec[d] * (double)w->rcells_q[iws + w->nwsq * d];
      caux = expi(TWOPI * dot) / (double)w->phwsdeg[iws];
    } else {
      for (int d = 0; d < 3; ++d) dot += kvec[d] * (double)w->rcells_k[iws + w->nwsk * d];
      caux = expi(TWOPI * dot) / (double)w->elwsdeg[iws];
    }
    gbloch += caux * ukgu;
  }
  free(ukg);
  if (w->polar) {   /* long-range correction (:998-1006) */
    cplx unm = 0.0;   /* dot_product(el_evec_kp, el_evec_k) */
    for (int64_t c = 0; c < nw; ++c) unm += conj(cget(el_evec_kp, c)) * cget(el_evec_k, c);
    double qc[3], uu[128], gl[2];
    or_q_cart_bohr(w, qvec, qc);
    for (int64_t ip = 0; ip < nb; ++ip) cset(uu, ip, u[ip]);
    or_long_range_prefac(w, qc, uu, gl);
    gbloch += (gl[0] + I * gl[1]) * unm;
  }
  return 0.5 * creal(gbloch * conj(gbloch)) / ph_en * g2unitfactor;
}

/* ======================= delta functions ======================= */

/* form_triangles: delta.f90:648-747 (blocks = true).
 * triang (2nk,3), triangcount (nk), triangmap (2,nk,6), all column-major. */
void or_form_triangles(int64_t nk, const int64_t mesh[3], const int64_t *indexlist,
                       int64_t *triang, int64_t *triangcount, int64_t *triangmap) {
  static const int lab[2][3] = {{1, 2, 3}, {1, 3, 4}};
  memset(triang, 0, sizeof(int64_t) * 2 * nk * 3);
  memset(triangcount, 0, sizeof(int64_t) * nk);
  memset(triangmap, 0, sizeof(int64_t) * 2 * nk * 6);
  int64_t count = 1;
  for (int64_t ik = 1; ik <= nk; ++ik) {
    int64_t ijk[3];
    or_demux_vector(indexlist[ik - 1], ijk, mesh, 1);
    int64_t i = ijk[0], j = ijk[1], k = ijk[2];
    int64_t ip1 = (i == mesh[0]) ? 1 : i + 1;
    int64_t jp1 = (j == mesh[1]) ? 1 : j + 1;
    int64_t sc[4][3] = {{i, j, k}, {ip1, j, k}, {i, jp1, k}, {ip1, jp1, k}};
    for (int tk = 0; tk < 2; ++tk) {
      for (int tl = 0; tl < 3; ++tl) {
        int a = lab[tk][tl] - 1;
        int64_t aux = or_mux_vector(sc[a], mesh, 1);
        int64_t tmp = or_binsearch(indexlist, nk, aux);
        triang[(count - 1) + 2 * nk * tl] = tmp;
        if (tmp > 0) {
          triangcount[tmp - 1] += 1;
          int64_t c = triangcount[tmp - 1];
          triangmap[0 + 2 * ((tmp - 1) + nk * (c - 1))] = count;
          triangmap[1 + 2 * ((tmp - 1) + nk * (c - 1))] = tl + 1;
        }
      }
      count++;
    }
  }
}

/* form_tetrahedra_3d: delta.f90:494-605 (blocks = true).
 * tetra (6nk,4), tetracount (nk), tetramap (2,nk,24). */
void or_form_tetrahedra_3d(int64_t nk, const int64_t mesh[3], const int64_t *indexlist,
                           int64_t *tetra, int64_t *tetracount, int64_t *tetramap) {
  static const int lab[6][4] = {{1, 2, 3, 6}, {1, 3, 5, 6}, {3, 5, 6, 7},
                                {3, 6, 7, 8}, {3, 4, 6, 8}, {2, 3, 4, 6}};
  memset(tetra, 0, sizeof(int64_t) * 6 * nk * 4);
  memset(tetracount, 0, sizeof(int64_t) * nk);
  memset(tetramap, 0, sizeof(int64_t) * 2 * nk * 24);
  int64_t count = 1;
  for (int64_t ik = 1; ik <= nk; ++ik) {
    int64_t ijk[3];
    or_demux_vector(indexlist[ik - 1], ijk, mesh, 1);
    int64_t i = ijk[0], j = ijk[1], k = ijk[2];
    int64_t ip1 = (i == mesh[0]) ? 1 : i + 1;
    int64_t jp1 = (j == mesh[1]) ? 1 : j + 1;
    int64_t kp1 = (k == mesh[2]) ? 1 : k + 1;
    int64_t sc[8][3] = {{i, j, k}, {ip1, j, k}, {i, jp1, k}, {ip1, jp1, k},
                        {i, j, kp1}, {ip1, j, kp1}, {i, jp1, kp1}, {ip1, jp1, kp1}};
    for (int tk = 0; tk < 6; ++tk) {
      for (int tl = 0; tl < 4; ++tl) {
        int a = lab[tk][tl] - 1;
        int64_t aux = or_mux_vector(sc[a], mesh, 1);
        int64_t tmp = or_binsearch(indexlist, nk, aux);
        tetra[(count - 1) + 6 * nk * tl] = tmp;
        if (tmp > 0) {
          tetracount[tmp - 1] += 1;
          int64_t c = tetracount[tmp - 1];
          tetramap[0 + 2 * ((tmp - 1) + nk * (c - 1))] = count;
          tetramap[1 + 2 * ((tmp - 1) + nk * (c - 1))] = tl + 1;
        }
      }
      count++;
    }
  }
}

/* fill_triangles / fill_tetrahedra_3d: delta.f90:607-646,749-788.
 * simplex (nsimplex,nv), evals (nk,nbands) -> simplex_evals (nsimplex,nbands,nv),
 * vertices outside the window left at zero, then sorted per (simplex, band). */
void or_fill_simplices(int64_t nsimplex, int64_t nv, const int64_t *simplex,
                       int64_t nk, int64_t nbands, const double *evals, double *se) {
  memset(se, 0, sizeof(double) * nsimplex * nbands * nv);
  for (int64_t it = 0; it < nsimplex; ++it)
    for (int64_t iv = 0; iv < nv; ++iv) {
      int64_t aux = simplex[it + nsimplex * iv];
      if (aux > 0)
        for (int64_t ib = 0; ib < nbands; ++ib)
          se[it + nsimplex * (ib + nbands * iv)] = evals[(aux - 1) + nk * ib];
    }
  for (int64_t it = 0; it < nsimplex; ++it)
    for (int64_t ib = 0; ib < nbands; ++ib) {
      /* insertion sort of nv values (misc.f90 sort_real gives ascending order) */
      for (int64_t a = 1; a < nv; ++a) {
        double x = se[it + nsimplex * (ib + nbands * a)];
        int64_t b = a - 1;
        while (b >= 0 && se[it + nsimplex * (ib + nbands * b)] > x) {
          se[it + nsimplex * (ib + nbands * (b + 1))] = se[it + nsimplex * (ib + nbands * b)];
          b--;
        }
        se[it + nsimplex * (ib + nbands * (b + 1))] = x;
      }
    }
}

/* delta_fn_triang: delta.f90:790-881.  ik, ib 1-based. */
double or_delta_triang(double e, int64_t ik, int64_t ib, const int64_t mesh[3], int64_t nk,
                       int64_t nsimplex, int64_t nbands, const int64_t *map,
                       const int64_t *count, const double *ev) {
  double d = 0.0;
  int64_t numtriangs = mesh[0] * mesh[1] * mesh[2] * 2;
  int64_t num = count[ik - 1];
  for (int64_t itk = 1; itk <= num; ++itk) {
    int64_t it = map[0 + 2 * ((ik - 1) + nk * (itk - 1))];
    int64_t iv = map[1 + 2 * ((ik - 1) + nk * (itk - 1))];
    double e1 = ev[(it - 1) + nsimplex * ((ib - 1) + nbands * 0)];
    double e2 = ev[(it - 1) + nsimplex * ((ib - 1) + nbands * 1)];
    double e3 = ev[(it - 1) + nsimplex * ((ib - 1) + nbands * 2)];
    int c1 = e <= e1, c2 = e1 < e && e <= e2, c3 = e2 < e && e <= e3, c4 = e3 < e;
    double tmp = 0.0;
    if (c1 || c4) continue;
    double E12 = (e - e2) / (e1 - e2), E21 = (e - e1) / (e2 - e1), E13 = (e - e3) / (e1 - e3);
    double E31 = (e - e1) / (e3 - e1), E23 = (e - e3) / (e2 - e3), E32 = (e - e2) / (e3 - e2);
    switch (iv) {
      case 1:
        if (c2) tmp = E21 * (E12 + E13) / (e3 - e1);
        else if (c3) tmp = E23 * E13 / (e3 - e1);
        break;
      case 2:
        if (c2) tmp = E21 * E21 / (e3 - e1);
        else if (c3) tmp = E23 * E23 / (e3 - e1);
        break;
      case 3:
        if (c2) tmp = E21 * E31 / (e3 - e1);
        else if (c3) tmp = E23 * (E31 + E32) / (e3 - e1);
        break;
    }
    d += tmp;
  }
  if (d < 1.0e-12) d = 0.0;
  return d / (double)numtriangs;
}

/* delta_fn_tetra: delta.f90:61-225.  ik, ib 1-based. */
double or_delta_tetra(double e, int64_t ik, int64_t ib, const int64_t mesh[3], int64_t nk,
                      int64_t nsimplex, int64_t nbands, const int64_t *map,
                      const int64_t *count, const double *ev) {
  double d = 0.0, tmp = 0.0;
  int64_t numtetra = mesh[0] * mesh[1] * mesh[2] * 6;
  int64_t num = count[ik - 1];
  for (int64_t itk = 1; itk <= num; ++itk) {
    int64_t it = map[0 + 2 * ((ik - 1) + nk * (itk - 1))];
    int64_t iv = map[1 + 2 * ((ik - 1) + nk * (itk - 1))];
    double e1 = ev[(it - 1) + nsimplex * ((ib - 1) + nbands * 0)];
    double e2 = ev[(it - 1) + nsimplex * ((ib - 1) + nbands * 1)];
    double e3 = ev[(it - 1) + nsimplex * ((ib - 1) + nbands * 2)];
    double e4 = ev[(it - 1) + nsimplex * ((ib - 1) + nbands * 3)];
    double e1e = e1 - e, e2e = e2 - e, e3e = e3 - e, e4e = e4 - e;
    double e21 = e2 - e1, e31 = e3 - e1, e41 = e4 - e1, e32 = e3 - e2, e42 = e4 - e2, e43 = e4 - e3;
    int c1 = e1 <= e && e <= e2, c2 = e2 <= e && e <= e3, c3 = e3 <= e && e <= e4;
    if (!(e < e1 || e > e4)) {
      switch (iv) {
        case 1:
          if (c1) {
            tmp = (e2e / e21 + e3e / e31 + e4e / e41) * (e1e * e1e) / e41 / e31 / e21;
            if (e1 == e2) tmp = 0.0;
          } else if (c2) {
            tmp = -0.5 * (e3e / (e31 * e31) * (e3e * e2e / e42 / e32 + e4e * e1e / e41 / e42 + e3e * e1e / e32 / e41) +
                          e4e / (e41 * e41) * (e4e * e1e / e42 / e31 + e4e * e2e / e42 / e32 + e3e * e1e / e31 / e32));
            if (e2 == e3)
              tmp = -0.5 * (e4e * e1e / e41 / e42 + e1e / e41 +
                            e4e / (e41 * e41) * (e4e * e1e / e42 / e31 + e4e / e42 + e1e / e31));
          } else if (c3) {
            tmp = (e4e * e4e * e4e) / (e41 * e41) / e42 / e43;
            if (e3 == e4) tmp = (e4e * e4e) / (e41 * e41) / e42;
          }
          break;
        case 2:
          if (c1) {
            tmp = -(e1e * e1e * e1e) / (e21 * e21) / e31 / e41;
            if (e1 == e2) tmp = 0.0;
          } else if (c2) {
            tmp = -0.5 * (e3e / (e32 * e32) * (e3e * e2e / e42 / e31 + e4e * e2e / e42 / e41 + e3e * e1e / e31 / e41) +
                          e4e / (e42 * e42) * (e3e * e2e / e32 / e31 + e4e * e1e / e41 / e31 + e4e * e2e / e32 / e41));
            if (e2 == e3) tmp = -0.5 * (0.0 + e4e / e42 / e41 + 0.0 + e4e / (e42 * e42) * (0.0 + e4e * e1e / e41 / e31 + 1.0));
          } else if (c3) {
            tmp = (e4e * e4e * e4e) / e41 / (e42 * e42) / e43;
            if (e3 == e4) tmp = 0.0;
          }
          break;
        case 3:
          if (c1) {
            tmp = -(e1e * e1e * e1e) / e21 / (e31 * e31) / e41;
            if (e1 == e2) tmp = 0.0;
          } else if (c2) {
            tmp = 0.5 * (e2e / (e32 * e32) * (e3e * e2e / e42 / e31 + e4e * e2e / e42 / e41 + e3e * e1e / e31 / e41) +
                         e1e / (e31 * e31) * (e3e * e2e / e42 / e32 + e4e * e1e / e41 / e42 + e3e * e1e / e32 / e41));
            if (e2 == e3)
              tmp = 0.5 * (0.0 + e4e / e42 / e41 + e1e / e31 / e41 + e1e / (e31 * e31) * (0.0 + e4e * e1e / e41 / e42 + e1e / e41));
          } else if (c3) {
            tmp = (e4e * e4e * e4e) / e41 / e42 / (e43 * e43);
            if (e3 == e4) tmp = 0.0;
          }
          break;
        case 4:
          if (c1) {
            tmp = -(e1e * e1e * e1e) / e21 / e31 / (e41 * e41);
            if (e1 == e2) tmp = 0.0;
          } else if (c2) {
            tmp = 0.5 * (e2e / (e42 * e42) * (e3e * e2e / e32 / e31 + e4e * e1e / e41 / e31 + e4e * e2e / e32 / e41) +
                         e1e / (e41 * e41) * (e4e * e1e / e42 / e31 + e4e * e2e / e42 / e32 + e3e * e1e / e31 / e32));
            if (e2 == e3) tmp = 0.5 * (0.0 + e1e / (e41 * e41) * (e4e * e1e / e42 / e31 + e4e / e42 + e1e / e31));
          } else if (c3) {
            tmp = -(e3e / e43 + e2e / e42 + e1e / e41) * (e4e * e4e) / e41 / e42 / e43;
            if (e3 == e4) tmp = 0.0;
          }
          break;
      }
      if (e1 == e2 && e1 == e3 && e1 == e4 && e == e1) tmp = 0.25;
      d += tmp;
    }
  }
  if (d < 1.0e-12) d = 0.0;
  return d / (double)numtetra;
}

/* ======================= symmetry ======================= */

/* find_star + find_equiv_map: symmetry.f90:215-289.  equiv (nsym, n): the
 * 1-based muxed image of point i under rotation s, or -1 off the mesh. */
void or_find_equiv_map(int64_t nsym, const double *qrot, const int64_t mesh[3], int64_t n,
                       const int64_t *indexlist, int64_t *equiv) {
  for (int64_t i = 0; i < n; ++i) {
    int64_t v[3];
    or_demux_vector(indexlist ? indexlist[i] : i + 1, v, mesh, 0);
    for (int64_t s = 0; s < nsym; ++s) {
      const double *q = qrot + 9 * s;
      double vec[3];
      int64_t iv[3];
      double nrm = 0.0;
      for (int r = 0; r < 3; ++r) {
        vec[r] = (double)mesh[r] * (q[r] * ((double)v[0] / mesh[0]) + q[r + 3] * ((double)v[1] / mesh[1]) +
                                    q[r + 6] * ((double)v[2] / mesh[2]));
        iv[r] = (int64_t)llround(vec[r]);
        nrm += (vec[r] - iv[r]) * (vec[r] - iv[r]);
      }
      if (sqrt(nrm) >= 1e-2) {
        equiv[s + nsym * i] = -1;
      } else {
        for (int r = 0; r < 3; ++r) iv[r] = ((iv[r] % mesh[r]) + mesh[r]) % mesh[r];
        equiv[s + nsym * i] = or_mux_vector(iv, mesh, 0);
      }
    }
  }
}

/* calculate_symmetries after spg_get_dataset (symmetry.f90:134-212): the
 * reciprocal rotations M^-1 R^T M transposed (M = A^T A) of the nsymm
 * real-space rotations rot (3,3,nsymm, crystal coordinates), time reversal
 * appended as the negatives, then the rotations that send a mesh point off the
 * mesh or repeat an earlier valid rotation dropped.  qrot (3,3,2 nsymm)
 * receives the kept ones; returns their number. */
int64_t or_symmetry_qrotations(const double lattvecs[9], int64_t nsymm, const int64_t *rot, const int64_t mesh[3],
                               double *qrot) {
  const double *A = lattvecs;
  double M[9], Mi[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[i + 3 * j] = A[3 * i] * A[3 * j] + A[3 * i + 1] * A[3 * j + 1] + A[3 * i + 2] * A[3 * j + 2];
  const double det = M[0] * (M[4] * M[8] - M[7] * M[5]) - M[3] * (M[1] * M[8] - M[7] * M[2]) +
                     M[6] * (M[1] * M[5] - M[4] * M[2]);
  Mi[0] = (M[4] * M[8] - M[7] * M[5]) / det;
  Mi[3] = -(M[3] * M[8] - M[6] * M[5]) / det;
  Mi[6] = (M[3] * M[7] - M[6] * M[4]) / det;
  Mi[1] = -(M[1] * M[8] - M[7] * M[2]) / det;
  Mi[4] = (M[0] * M[8] - M[6] * M[2]) / det;
  Mi[7] = -(M[0] * M[7] - M[6] * M[1]) / det;
  Mi[2] = (M[1] * M[5] - M[4] * M[2]) / det;
  Mi[5] = -(M[0] * M[5] - M[3] * M[2]) / det;
  Mi[8] = (M[0] * M[4] - M[3] * M[1]) / det;
  const int64_t n2 = 2 * nsymm;
  double *q = (double *)calloc(9 * n2 + 1, sizeof(double));
  int64_t *r = (int64_t *)calloc(9 * n2 + 1, sizeof(int64_t));
  for (int64_t s = 0; s < nsymm; ++s) {
    double t2[9], t3[9];   /* t2 = M^-1 R^T, qrot = transpose(t2 M) */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc += Mi[i + 3 * k] * (double)rot[9 * s + j + 3 * k];
        t2[i + 3 * j] = acc;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc += t2[i + 3 * k] * M[k + 3 * j];
        t3[i + 3 * j] = acc;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        q[9 * s + i + 3 * j] = t3[j + 3 * i];
        q[9 * (s + nsymm) + i + 3 * j] = -t3[j + 3 * i];
      }
    for (int k = 0; k < 9; ++k) {
      r[9 * s + k] = rot[9 * s + k];
      r[9 * (s + nsymm) + k] = -rot[9 * s + k];
    }
  }
  const int64_t N = mesh[0] * mesh[1] * mesh[2];
  int64_t *eq = (int64_t *)malloc(sizeof(int64_t) * n2 * N);
  or_find_equiv_map(n2, q, mesh, N, NULL, eq);
  int *valid = (int *)malloc(sizeof(int) * n2);
  for (int64_t s = 0; s < n2; ++s) {
    valid[s] = 1;
    for (int64_t i = 0; i < N && valid[s]; ++i)
      if (eq[s + n2 * i] == -1) valid[s] = 0;
  }
  for (int64_t ii = 1; ii < n2; ++ii)
    for (int64_t i = 0; i < ii; ++i) {
      if (!valid[i]) continue;
      int same = 1;
      for (int k = 0; k < 9; ++k) same &= r[9 * ii + k] == r[9 * i + k];
      if (same) { valid[ii] = 0; break; }
    }
  int64_t kk = 0;
  for (int64_t s = 0; s < n2; ++s)
    if (valid[s]) {
      for (int k = 0; k < 9; ++k) qrot[9 * kk + k] = q[9 * s + k];
      kk++;
    }
  free(q); free(r); free(eq); free(valid);
  return kk;
}

/* find_irred_wedge: symmetry.f90:303-452 (serial form of its running list).
 * Over the mesh (indexlist NULL) or the n sorted points of indexlist (blocks):
 * indexlist_irred (nirr), nequiv (nirr), ibz2fbz (nsym, n, 2) nullable.
 * Returns 0, or 1 ("Could not find irreducible wedge.", :417). */
int or_find_irred_wedge(const int64_t mesh[3], int64_t nsym, const double *qrot, int64_t n, const int64_t *indexlist,
                        int64_t *nirr, int64_t *indexlist_irred, int64_t *nequiv, int64_t *ibz2fbz) {
  const int64_t N = mesh[0] * mesh[1] * mesh[2];
  int64_t *eq = (int64_t *)malloc(sizeof(int64_t) * (nsym * n > 0 ? nsym * n : 1));
  or_find_equiv_map(nsym, qrot, mesh, n, indexlist, eq);
  char *running = (char *)calloc(N + 1, 1);   /* membership of the running list, by muxed index */
  int64_t *imagelist = (int64_t *)malloc(sizeof(int64_t) * (nsym > 0 ? nsym : 1));
  int64_t nir = 0, counter = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t imux = indexlist ? indexlist[i] : i + 1;
    if (running[imux]) continue;
    const int64_t ir = nir++;
    indexlist_irred[ir] = imux;
    int64_t ne = 0;
    for (int64_t s = 0; s < nsym; ++s) {
      const int64_t image = eq[s + nsym * i];
      int seen = 0;
      for (int64_t l = 0; l < ne; ++l) seen |= imagelist[l] == image;
      if (seen) continue;
      imagelist[ne] = image;
      if (image >= 1 && image <= N) running[image] = 1;
      if (ibz2fbz) {
        ibz2fbz[ne + nsym * (ir + n * 0)] = s + 1;
        ibz2fbz[ne + nsym * (ir + n * 1)] = image;
      }
      ne++;
    }
    nequiv[ir] = ne;
    counter += ne;
  }
  *nirr = nir;
  free(eq); free(running); free(imagelist);
  return counter == n ? 0 : 1;
}

/* ======================= driver ======================= */

typedef struct {
  int kind;
  int64_t mesh[3], nk, nsimplex, nbands;
  const int64_t *map, *count;
  const double *se, *ens;
  double sigma, inv_nk;
} delta_ctx;

static double delta_eval(const delta_ctx *c, double e, int64_t ikp, int64_t n) {
  if (c->kind == 0) {
    /* fixed-sigma Gaussian, bz_sums.f90:73-83 convention, / N_k */
    double x = (e - c->ens[(ikp - 1) + c->nk * (n - 1)]) / c->sigma;
    return (1.0 / sqrt(TWOPI)) / c->sigma * exp(-0.5 * x * x) * c->inv_nk;
  }
  if (c->kind == 1)
    return or_delta_triang(e, ikp, n, c->mesh, c->nk, c->nsimplex, c->nbands, c->map, c->count, c->se);
  return or_delta_tetra(e, ikp, n, c->mesh, c->nk, c->nsimplex, c->nbands, c->map, c->count, c->se);
}

/*
 * calculate_eph_interaction_ibzk ('g' then 'X', interactions.f90:2095-2400) and
 * calculate_el_rta_rates (interactions.f90:2958-3063), with the identity point
 * group (IBZ blocks = FBZ blocks), q on the electron mesh (mesh_ref = 1) and no
 * disk: |g|^2, X+- and rates are formed state by state in memory.
 */
struct or_rates_ctx {
  const or_wannier *w;
  or_request req;
  int64_t N, nwv, nin, status, us_setup;
  int64_t *indexlist;
  double *kfull, *ens_full, *kw, *ens, *evecs, *phe, *phv;
  int64_t *simplex, *scount, *smap;
  double *se;
  delta_ctx dc;
  int64_t nirr;       /* with symmetry: irreducible window points (IBZ blocks) */
  int64_t *irr_pos;   /* (nwv) their row in the IBZ list, -1 for the others; NULL without symmetry */
};

/* Set-up of the ibzk driver: FBZ energies, window, window eigenvectors,
 * phonons on the q mesh, simplices (electron.f90:321-595, phonon.f90:159-230). */
or_rates_ctx *or_rates_setup(const or_wannier *w, const or_request *req, int nthreads) {
  return or_rates_setup_sym(w, req, 0, NULL, nthreads);
}

/* With nsym > 0 reciprocal rotations qrot (or_symmetry_qrotations): the
 * electron set-up of calculate_electrons (electron.f90:346-577) -- FBZ energies
 * from the IBZ of the full mesh mapped onto its images, the window on them,
 * FBZ blocks eigenvectors computed directly, the IBZ of the window blocks and
 * its energies mapped again -- so that or_rates_run takes initial states on
 * the irreducible window points only. */
or_rates_ctx *or_rates_setup_sym(const or_wannier *w, const or_request *req, int64_t nsym, const double *qrot,
                                 int nthreads) {
  const int64_t nw = w->nw, nb = w->nb;
  const int64_t *mesh = req->mesh;
  const int64_t N = mesh[0] * mesh[1] * mesh[2];
  or_rates_ctx *cx = (or_rates_ctx *)calloc(1, sizeof(or_rates_ctx));
  cx->w = w;
  cx->req = *req;
  cx->N = N;
  double t_start = wall_us();
  int64_t *indexlist = (int64_t *)malloc(sizeof(int64_t) * (N > 0 ? N : 1));
  cx->indexlist = indexlist;
  /* 1. FBZ wave vectors (crystal.f90:377-408) and energies */
  double *kfull = (double *)malloc(sizeof(double) * N * 3);
  for (int64_t i = 1; i <= N; ++i) {
    int64_t v[3];
    or_demux_vector(i, v, mesh, 0);
    for (int d = 0; d < 3; ++d) kfull[(i - 1) + N * d] = (double)v[d] / (double)mesh[d];
  }
  double *ens_full = (double *)malloc(sizeof(double) * N * nw);
  or_el_wann(w, N, kfull, ens_full, NULL, NULL, NULL);
  if (nsym > 0) {   /* IBZ of the full mesh, its energies mapped onto the FBZ (:351-385) */
    int64_t nir = 0, *irr = (int64_t *)malloc(sizeof(int64_t) * N), *neq = (int64_t *)malloc(sizeof(int64_t) * N);
    int64_t *map = (int64_t *)malloc(sizeof(int64_t) * nsym * N * 2);
    if (or_find_irred_wedge(mesh, nsym, qrot, N, NULL, &nir, irr, neq, map)) cx->status = 3;
    double *kir = (double *)malloc(sizeof(double) * nir * 3), *eir = (double *)malloc(sizeof(double) * nir * nw);
    for (int64_t i = 0; i < nir; ++i)
      for (int d = 0; d < 3; ++d) kir[i + nir * d] = kfull[(irr[i] - 1) + N * d];
    or_el_wann(w, nir, kir, eir, NULL, NULL, NULL);
    for (int64_t i = 0; i < nir; ++i)
      for (int64_t l = 0; l < neq[i]; ++l) {
        const int64_t il = map[l + nsym * (i + N * 1)];
        for (int64_t b = 0; b < nw; ++b) ens_full[(il - 1) + N * b] = eir[i + nir * b];
      }
    free(irr); free(neq); free(map); free(kir); free(eir);
  }
  /* 2. window: apply_energy_window (electron.f90:597-636), sorted index list */
  int64_t nwv = 0;
  for (int64_t ik = 0; ik < N; ++ik) {
    int in = 0;
    for (int64_t b = 0; b < nw; ++b) if (fabs(ens_full[ik + N * b] - req->enref) <= req->fsthick) in = 1;
    if (in) indexlist[nwv++] = ik + 1;
  }
  cx->nwv = nwv;
  cx->kfull = kfull;
  cx->ens_full = ens_full;
  if (nwv == 0) { cx->status = 2; return cx; }
  /* 3. window quantities: wave vectors, energies, eigenvectors */
  double *kw = (double *)malloc(sizeof(double) * nwv * 3);
  for (int64_t i = 0; i < nwv; ++i)
    for (int d = 0; d < 3; ++d) kw[i + nwv * d] = kfull[(indexlist[i] - 1) + N * d];
  double *ens = (double *)malloc(sizeof(double) * nwv * nw);
  double *evecs = (double *)malloc(sizeof(double) * 2 * nwv * nw * nw);
  or_el_wann(w, nwv, kw, ens, evecs, NULL, NULL);
  if (nsym > 0) {
    /* FBZ blocks energies: the mapped ones (fbz_blocks_quantities, :424); then the
     * IBZ of the blocks (:450-454), its energies computed and mapped onto the
     * blocks (:513-529) */
    for (int64_t i = 0; i < nwv; ++i)
      for (int64_t b = 0; b < nw; ++b) ens[i + nwv * b] = ens_full[(indexlist[i] - 1) + N * b];
    int64_t nir = 0, *irr = (int64_t *)malloc(sizeof(int64_t) * nwv), *neq = (int64_t *)malloc(sizeof(int64_t) * nwv);
    int64_t *map = (int64_t *)malloc(sizeof(int64_t) * nsym * nwv * 2);
    if (or_find_irred_wedge(mesh, nsym, qrot, nwv, indexlist, &nir, irr, neq, map)) cx->status = 3;
    double *kir = (double *)malloc(sizeof(double) * (nir > 0 ? nir : 1) * 3);
    double *eir = (double *)malloc(sizeof(double) * (nir > 0 ? nir : 1) * nw);
    for (int64_t i = 0; i < nir; ++i)
      for (int d = 0; d < 3; ++d) kir[i + nir * d] = kfull[(irr[i] - 1) + N * d];
    or_el_wann(w, nir, kir, eir, NULL, NULL, NULL);
    for (int64_t i = 0; i < nir; ++i)
      for (int64_t l = 0; l < neq[i]; ++l) {
        const int64_t il = map[l + nsym * (i + nwv * 1)];
        const int64_t aux = or_binsearch(indexlist, nwv, il);
        if (aux > 0)
          for (int64_t b = 0; b < nw; ++b) ens[(aux - 1) + nwv * b] = eir[i + nir * b];
      }
    cx->nirr = nir;
    cx->irr_pos = (int64_t *)malloc(sizeof(int64_t) * nwv);
    for (int64_t i = 0; i < nwv; ++i) cx->irr_pos[i] = -1;
    for (int64_t i = 0; i < nir; ++i) cx->irr_pos[or_binsearch(indexlist, nwv, irr[i]) - 1] = i;
    free(irr); free(neq); free(map); free(kir); free(eir);
  }
  int64_t nin = 0;
  for (int64_t i = 0; i < nwv; ++i)
    for (int64_t b = 0; b < nw; ++b) if (fabs(ens[i + nwv * b] - req->enref) <= req->fsthick) nin++;
  cx->nin = nin;
  cx->kw = kw;
  cx->ens = ens;
  cx->evecs = evecs;
  /* 4. phonons on the full q mesh (phonon.f90:208-214, q mesh = k mesh) */
  double *phe = (double *)malloc(sizeof(double) * N * nb);
  double *phv = (double *)malloc(sizeof(double) * 2 * N * nb * nb);
  int phs = 0;
  {
    int nt = nthreads > 0 ? nthreads : 1;
    int64_t chunk = (N + nt - 1) / nt;
#pragma omp parallel for num_threads(nt) schedule(static) reduction(| : phs)
    for (int t = 0; t < nt; ++t) {
      int64_t a = t * chunk, b = a + chunk < N ? a + chunk : N;
      if (a >= b) continue;
      int64_t n = b - a;
      double *q = (double *)malloc(sizeof(double) * n * 3);
      double *e = (double *)malloc(sizeof(double) * n * nb);
      double *v = (double *)malloc(sizeof(double) * 2 * n * nb * nb);
      for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) q[i + n * d] = kfull[(a + i) + N * d];
      phs |= or_ph_wann(w, n, q, e, v, NULL);
      for (int64_t i = 0; i < n; ++i)
        for (int64_t s = 0; s < nb; ++s) {
          phe[(a + i) + N * s] = e[i + n * s];
          for (int64_t c = 0; c < nb; ++c) {
            phv[2 * ((a + i) + N * (s + nb * c))] = v[2 * (i + n * (s + nb * c))];
            phv[2 * ((a + i) + N * (s + nb * c)) + 1] = v[2 * (i + n * (s + nb * c)) + 1];
          }
        }
      free(q); free(e); free(v);
    }
  }
  cx->phe = phe;
  cx->phv = phv;
  if (phs) cx->status = 1;
  /* 5. simplices for the triangle / tetrahedron deltas */
  delta_ctx dc;
  memset(&dc, 0, sizeof dc);
  dc.kind = (int)req->delta_kind;
  for (int d = 0; d < 3; ++d) dc.mesh[d] = mesh[d];
  dc.nk = nwv; dc.nbands = nw; dc.ens = ens; dc.sigma = req->sigma; dc.inv_nk = 1.0 / (double)N;
  int64_t *simplex = NULL, *scount = NULL, *smap = NULL;
  double *se = NULL;
  if (dc.kind == 1 || dc.kind == 2) {
    int64_t nv = dc.kind == 1 ? 3 : 4, per = dc.kind == 1 ? 2 : 6, maxc = dc.kind == 1 ? 6 : 24;
    dc.nsimplex = per * nwv;
    simplex = (int64_t *)malloc(sizeof(int64_t) * dc.nsimplex * nv);
    scount = (int64_t *)malloc(sizeof(int64_t) * nwv);
    smap = (int64_t *)malloc(sizeof(int64_t) * 2 * nwv * maxc);
    se = (double *)malloc(sizeof(double) * dc.nsimplex * nw * nv);
    if (dc.kind == 1) or_form_triangles(nwv, mesh, indexlist, simplex, scount, smap);
    else or_form_tetrahedra_3d(nwv, mesh, indexlist, simplex, scount, smap);
    or_fill_simplices(dc.nsimplex, nv, simplex, nwv, nw, ens, se);
    dc.map = smap; dc.count = scount; dc.se = se;
  }
  cx->simplex = simplex;
  cx->scount = scount;
  cx->smap = smap;
  cx->se = se;
  cx->dc = dc;
  cx->us_setup = (int64_t)(wall_us() - t_start);
  return cx;
}

/* One group of a degenerate-subspace pass: c values v[0], v[st], ..., with
 * energies e[0..c-1].  mode 0 restates the reference's loop literally, in
 * place: member a becomes the mean over the members b with |e_a - e_b| <
 * thres, summed in member order, of the values as they are at that moment, so
 * later members see their predecessors' new values (wannier.f90:1335-1347,
 * 1352-1364, 1369-1381).  mode 1: the same means, all of them taken from the
 * values before the pass. */
void or_degenerate_group(int mode, double thres, int64_t c, double *v, int64_t st, const double *e, double *tmp) {
  for (int64_t a = 0; a < c; ++a) tmp[a] = v[a * st];
  for (int64_t a = 0; a < c; ++a) {
    int64_t cnt = 0;
    double aux = 0.0;
    for (int64_t b = 0; b < c; ++b)
      if (fabs(e[a] - e[b]) < thres) {
        ++cnt;
        aux += mode == 0 ? v[b * st] : tmp[b];
      }
    v[a * st] = aux / (double)cnt;
  }
}

/* Degenerate-subspace averaging of |g|^2 (plot_along_path, wannier.f90:1332-
 * 1384; the same loops in test/check_interactions_symmetries.f90:330-384),
 * applied to the vertex list of or_rates_run over every in-window initial
 * state: (state j, final state f = (k', n), branch s), per_state = nin * nb
 * entries per state.  Three passes in the reference's order: over phonon
 * branches s of q = k' - k (|omega_s - omega_s'| < thres, eV); over the initial
 * bands m of each k (with k', n, s fixed); over the final bands n of each k'
 * (with the state and s fixed).  The band groups are the window bands, the
 * only ones the list holds.  Returns 1 if nv is not the list's length. */
int or_average_degenerate(or_rates_ctx *cx, int mode, double thres, double *g2, int64_t nv) {
  const or_wannier *w = cx->w;
  const or_request *req = &cx->req;
  const int64_t nw = w->nw, nb = w->nb, nwv = cx->nwv, N = cx->N;
  const int64_t *mesh = req->mesh;
  const double *ens = cx->ens, *phe = cx->phe;
  int64_t *sk = (int64_t *)malloc(sizeof(int64_t) * nwv * nw), *sm = (int64_t *)malloc(sizeof(int64_t) * nwv * nw);
  int64_t nst = 0;
  for (int64_t istate = 1; istate <= nwv * nw; ++istate) {   /* initial states in rank order */
    int64_t m, ik;
    or_demux_state(istate, nw, &m, &ik);
    if (cx->irr_pos && cx->irr_pos[ik - 1] < 0) continue;
    if (fabs(ens[(ik - 1) + nwv * (m - 1)] - req->enref) > req->fsthick) continue;
    sk[nst] = ik;
    sm[nst] = m;
    ++nst;
  }
  int64_t *fcum = (int64_t *)malloc(sizeof(int64_t) * (nwv + 1)), *fn = (int64_t *)malloc(sizeof(int64_t) * nwv * nw);
  int64_t nin = 0;
  for (int64_t ikp = 1; ikp <= nwv; ++ikp) {                   /* final states, row-major */
    fcum[ikp - 1] = nin;
    for (int64_t n = 1; n <= nw; ++n)
      if (fabs(ens[(ikp - 1) + nwv * (n - 1)] - req->enref) <= req->fsthick) fn[nin++] = n;
  }
  fcum[nwv] = nin;
  const int64_t per = nin * nb;
  if (nv != nst * per) {
    free(sk); free(sm); free(fcum); free(fn);
    return 1;
  }
  const int64_t gmax = nw > nb ? nw : nb;
  double *e = (double *)malloc(sizeof(double) * gmax), *tmp = (double *)malloc(sizeof(double) * gmax);
  double prim[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  /* 1. phonon branches, per (state, final state) */
  for (int64_t j = 0; j < nst; ++j)
    for (int64_t ikp = 1; ikp <= nwv; ++ikp) {
      int64_t qi[3], iq;
      double qf[3], qc[3];
      or_vector_addsub(cx->indexlist[ikp - 1], cx->indexlist[sk[j] - 1], -1, mesh, prim, qi, &iq, qf, qc);
      for (int64_t s = 0; s < nb; ++s) e[s] = phe[(iq - 1) + N * s];
      for (int64_t f = fcum[ikp - 1]; f < fcum[ikp]; ++f) or_degenerate_group(mode, thres, nb, g2 + j * per + f * nb, 1, e, tmp);
    }
  /* 2. initial bands, per (k, final state, s): the states of one k are consecutive */
  for (int64_t j0 = 0; j0 < nst;) {
    int64_t j1 = j0;
    while (j1 < nst && sk[j1] == sk[j0]) ++j1;
    for (int64_t j = j0; j < j1; ++j) e[j - j0] = ens[(sk[j] - 1) + nwv * (sm[j] - 1)];
    for (int64_t f = 0; f < nin; ++f)
      for (int64_t s = 0; s < nb; ++s) or_degenerate_group(mode, thres, j1 - j0, g2 + j0 * per + f * nb + s, per, e, tmp);
    j0 = j1;
  }
  /* 3. final bands, per (state, k', s) */
  for (int64_t j = 0; j < nst; ++j)
    for (int64_t ikp = 1; ikp <= nwv; ++ikp) {
      const int64_t f0 = fcum[ikp - 1], c = fcum[ikp] - f0;
      for (int64_t f = 0; f < c; ++f) e[f] = ens[(ikp - 1) + nwv * (fn[f0 + f] - 1)];
      for (int64_t s = 0; s < nb; ++s) or_degenerate_group(mode, thres, c, g2 + j * per + f0 * nb + s, nb, e, tmp);
    }
  free(e); free(tmp); free(sk); free(sm); free(fcum); free(fn);
  return 0;
}

void or_rates_free(or_rates_ctx *cx) {
  if (!cx) return;
  free(cx->indexlist); free(cx->kfull); free(cx->ens_full); free(cx->kw); free(cx->ens);
  free(cx->evecs); free(cx->phe); free(cx->phv); free(cx->simplex); free(cx->scount);
  free(cx->smap); free(cx->se); free(cx->irr_pos);
  free(cx);
}

/* The per-state part of the ibzk driver ('g' + 'X', interactions.f90:2169-2400)
 * and the rate sums (interactions.f90:3001-3034) for the in-window initial
 * states of rank [state_begin, state_begin + nstates) (nstates < 0: all). */
int or_rates_run(or_rates_ctx *cx, int64_t state_begin, int64_t nstates, int nthreads,
                 int literal, double *rates, int64_t *indexlist, int64_t *info,
                 double *g2out, double *xpout, double *xmout, int64_t cap) {
  const or_wannier *w = cx->w;
  const or_request *req = &cx->req;
  const int64_t nw = w->nw, nb = w->nb, nwsq = w->nwsq;
  const int64_t *mesh = req->mesh;
  const int64_t N = cx->N, nwv = cx->nwv, nin = cx->nin;
  const double const_tp = TWOPI / HBAR_EVPS;
  const double g2unitfactor = RYD2EV * RYD2EV * RYD2EV * RYD2AMU;
  const double *kw = cx->kw, *ens = cx->ens, *evecs = cx->evecs, *phe = cx->phe, *phv = cx->phv;
  const delta_ctx dc = cx->dc;
  for (int i = 0; i < 8; ++i) info[i] = 0;
  info[0] = cx->irr_pos ? cx->nirr : nwv;   /* rows of the rates: the IBZ blocks with symmetry */
  info[1] = nin;
  info[5] = cx->status;
  info[6] = cx->us_setup;
  for (int64_t i = 0; i < nwv; ++i) {
    if (!cx->irr_pos) indexlist[i] = cx->indexlist[i];
    else if (cx->irr_pos[i] >= 0) indexlist[cx->irr_pos[i]] = cx->indexlist[i];
  }
  if (cx->status == 2) return 2;
  /* 6. in-window initial states in istate order, optionally truncated; with
   *    symmetry those of the irreducible window points (interactions.f90:2169) */
  int64_t nst_all = nwv * nw;
  int64_t *rank = (int64_t *)malloc(sizeof(int64_t) * nst_all);
  int64_t nsel = 0;
  for (int64_t istate = 1; istate <= nst_all; ++istate) {
    int64_t m, ik;
    or_demux_state(istate, nw, &m, &ik);
    rank[istate - 1] = -1;
    if (cx->irr_pos && cx->irr_pos[ik - 1] < 0) continue;
    if (fabs(ens[(ik - 1) + nwv * (m - 1)] - req->enref) > req->fsthick) continue;
    int64_t k = nsel++;
    if (k < state_begin || (nstates >= 0 && k >= state_begin + nstates)) continue;
    rank[istate - 1] = k - state_begin;
  }
  nsel = 0;
  for (int64_t i = 0; i < nst_all; ++i) nsel += rank[i] >= 0;
  info[2] = nsel;
  int64_t per_state = nin * nb;     /* count per initial state: same for every state */
  info[3] = nsel * per_state;
  info[4] = nsel * nwv;
  for (int64_t i = 0; i < N * nw; ++i) rates[i] = 0.0;
  double t_loop = wall_us();
  /* 7. per IBZ k (serial, as one image walks its states): gkRp, then for each
   *    in-window state the k' loop, split over OpenMP threads; X+- are stored per
   *    vertex and summed in the reference's order afterwards. */
  int nt = nthreads > 0 ? nthreads : 1;
  int64_t *koff = (int64_t *)malloc(sizeof(int64_t) * (nwv + 1));   /* first vertex of k' */
  koff[0] = 0;
  for (int64_t ikp = 1; ikp <= nwv; ++ikp) {
    int64_t c = 0;
    for (int64_t n = 1; n <= nw; ++n) c += fabs(ens[(ikp - 1) + nwv * (n - 1)] - req->enref) <= req->fsthick;
    koff[ikp] = koff[ikp - 1] + c * nb;
  }
  const int64_t gsz = nw * nw * nb * nwsq;
  double *gk = (double *)malloc(sizeof(double) * 2 * gsz);
  double *xp = (double *)malloc(sizeof(double) * (per_state > 0 ? per_state : 1));
  double *xm = (double *)malloc(sizeof(double) * (per_state > 0 ? per_state : 1));
  double *g2l = (double *)malloc(sizeof(double) * (per_state > 0 ? per_state : 1));
  cplx *gkm = (cplx *)malloc(sizeof(cplx) * nw * nb * nwsq);   /* restructured form */
  double *evk = (double *)malloc(sizeof(double) * 2 * nw);
  for (int64_t ik = 1; ik <= nwv; ++ik) {
    int any = 0;
    for (int64_t m = 1; m <= nw; ++m) if (rank[(ik - 1) * nw + m - 1] >= 0) any = 1;
    if (!any) continue;
    double kv[3] = {kw[ik - 1], kw[(ik - 1) + nwv], kw[(ik - 1) + 2 * nwv]};
    or_gkRp(w, kv, gk);
    for (int64_t m = 1; m <= nw; ++m) {
      int64_t istate = (ik - 1) * nw + m;
      int64_t r = rank[istate - 1];
      if (r < 0) continue;
      double en_el = ens[(ik - 1) + nwv * (m - 1)];
      for (int64_t c = 0; c < nw; ++c) {
        evk[2 * c] = evecs[2 * ((ik - 1) + nwv * ((m - 1) + nw * c))];
        evk[2 * c + 1] = evecs[2 * ((ik - 1) + nwv * ((m - 1) + nw * c)) + 1];
      }
      if (!literal) {
        /* rotate the initial band once: gkm(n', s', Rp) = sum_m' U_k[m][m'] g(n', m', s', Rp) */
        for (int64_t rp = 0; rp < nwsq; ++rp)
          for (int64_t s = 0; s < nb; ++s)
            for (int64_t np = 0; np < nw; ++np) {
              cplx a = 0.0;
              for (int64_t mp = 0; mp < nw; ++mp)
                a += cget(evk, mp) * cget(gk, np + nw * (mp + nw * (s + nb * rp)));
              gkm[np + nw * (s + nb * rp)] = a;
            }
      }
#pragma omp parallel num_threads(nt)
      {
        double *evkp = (double *)malloc(sizeof(double) * 2 * nw);
        double *evq = (double *)malloc(sizeof(double) * 2 * nb);
        cplx *ph = (cplx *)malloc(sizeof(cplx) * nwsq);
#pragma omp for schedule(dynamic, 4)
        for (int64_t ikp = 1; ikp <= nwv; ++ikp) {
          /* q = k' - k on the electron mesh (vector.f90:86-102), ph mesh = el mesh */
          int64_t qi[3], qmux;
          double qf[3], qc[3];
          double prim[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
          or_vector_addsub(cx->indexlist[ikp - 1], cx->indexlist[ik - 1], -1, mesh, prim, qi, &qmux, qf, qc);
          int64_t iq = qmux;   /* change_grid to the same mesh keeps the index */
          double qv[3] = {qf[0], qf[1], qf[2]};
          if (!literal) {
            for (int64_t rp = 0; rp < nwsq; ++rp) {
              double dot = 0.0;
              for (int d = 0; d < 3; ++d) dot += qv[d] * (double)w->rcells_q[rp + nwsq * d];
              ph[rp] = expi(TWOPI * dot) / (double)w->phwsdeg[rp];
            }
          }
          int64_t cnt = koff[ikp - 1];
          for (int64_t n = 1; n <= nw; ++n) {
            if (fabs(ens[(ikp - 1) + nwv * (n - 1)] - req->enref) > req->fsthick) continue;
            for (int64_t c = 0; c < nw; ++c) {
              evkp[2 * c] = evecs[2 * ((ikp - 1) + nwv * ((n - 1) + nw * c))];
              evkp[2 * c + 1] = evecs[2 * ((ikp - 1) + nwv * ((n - 1) + nw * c)) + 1];
            }
            cplx hs[64];
            if (!literal) {
              /* h(s') = sum_Rp phase * sum_n' conj(U_k'[n][n']) gkm(n', s', Rp) */
              for (int64_t s = 0; s < nb; ++s) hs[s] = 0.0;
              for (int64_t rp = 0; rp < nwsq; ++rp)
                for (int64_t s = 0; s < nb; ++s) {
                  cplx a = 0.0;
                  for (int64_t np = 0; np < nw; ++np) a += conj(cget(evkp, np)) * gkm[np + nw * (s + nb * rp)];
                  hs[s] += ph[rp] * a;
                }
            }
            for (int64_t s = 1; s <= nb; ++s) {
              double en_ph = phe[(iq - 1) + N * (s - 1)];
              for (int64_t c = 0; c < nb; ++c) {
                evq[2 * c] = phv[2 * ((iq - 1) + N * ((s - 1) + nb * c))];
                evq[2 * c + 1] = phv[2 * ((iq - 1) + N * ((s - 1) + nb * c)) + 1];
              }
              double g2;
              if (literal) {
                g2 = or_g2(w, kv, qv, evk, evkp, evq, en_ph, gk, 1);
              } else if (en_ph == 0) {
                g2 = 0.0;
              } else {
                cplx gb = 0.0;
                for (int64_t sp = 0; sp < nb; ++sp) gb += cget(evq, sp) / sqrt(w->masses[sp / 3]) * hs[sp];
                if (w->polar) {   /* long-range term of g2 (wannier.f90:998-1006) */
                  cplx unm = 0.0;
                  for (int64_t c = 0; c < nw; ++c) unm += conj(cget(evkp, c)) * cget(evk, c);
                  double qc[3], uu[128], gl[2];
                  or_q_cart_bohr(w, qv, qc);
                  for (int64_t sp = 0; sp < nb; ++sp) cset(uu, sp, cget(evq, sp) / sqrt(w->masses[sp / 3]));
                  or_long_range_prefac(w, qc, uu, gl);
                  gb += (gl[0] + I * gl[1]) * unm;
                }
                g2 = 0.5 * creal(gb * conj(gb)) / en_ph * g2unitfactor;
              }
              /* 'X' (:2278-2332) */
              double bosefac = (en_ph != 0.0) ? or_Bose(en_ph, req->T) : 0.0;
              double fp = or_Fermi(en_el + en_ph, req->chempot, req->T);
              double fm = or_Fermi(en_el - en_ph, req->chempot, req->T);
              double dp = delta_eval(&dc, en_el + en_ph, ikp, n);
              double dm = delta_eval(&dc, en_el - en_ph, ikp, n);
              double xplus = 0.0, xminus = 0.0;
              if (en_ph >= 0.5e-3) {
                xplus = g2 * (bosefac + fp) * dp;
                xminus = g2 * (1.0 + bosefac - fm) * dm;
              }
              g2l[cnt] = g2;
              xp[cnt] = const_tp * xplus;
              xm[cnt] = const_tp * xminus;
              cnt++;
            }
          }
        }
        free(evkp); free(evq); free(ph);
      }
      /* rates: sum X+ then X- in order (:3012-3034) */
      double acc = 0.0;
      for (int64_t i = 0; i < per_state; ++i) acc += xp[i];
      for (int64_t i = 0; i < per_state; ++i) acc += xm[i];
      rates[(cx->irr_pos ? cx->irr_pos[ik - 1] : ik - 1) + N * (m - 1)] = acc;
      int64_t off = r * per_state;
      for (int64_t i = 0; i < per_state; ++i)
        if (off + i < cap) {
          if (g2out) g2out[off + i] = g2l[i];
          if (xpout) xpout[off + i] = xp[i];
          if (xmout) xmout[off + i] = xm[i];
        }
    }
  }
  free(gk); free(xp); free(xm); free(g2l); free(gkm); free(evk); free(koff);
  info[7] = (int64_t)(wall_us() - t_loop);
  free(rank);
  return (int)info[5];
}

int or_el_rates(const or_wannier *w, const or_request *req, int64_t max_states,
                int nthreads, int literal, double *rates, int64_t *indexlist,
                int64_t *info, double *g2out, double *xpout, double *xmout, int64_t cap) {
  or_rates_ctx *cx = or_rates_setup(w, req, nthreads);
  int rc = or_rates_run(cx, 0, max_states, nthreads, literal, rates, indexlist, info, g2out, xpout,
                        xmout, cap);
  or_rates_free(cx);
  return rc;
}

/*
 * calculate_eph_interaction_ibzq ('g' then 'Y', interactions.f90:1673-1930; the
 * 'Y' pass as calculate_Y_OTF, :1932-2093) and the ph-e part of
 * calculate_ph_rta_rates (interactions.f90:2723-2828), with the identity point
 * group (the IBZ phonons are all q of the mesh), q mesh = k mesh and no disk.
 * Per q, g(Re,q) from gReq (calculate_gReq, interactions.f90:1603-1630); per
 * phonon state (q, s) the loops over window k, k + q (vec_add + binsearch,
 * :1813-1822), m and n (:1825-1880) with the literal 'el' g2 (:1847-1852),
 * Y = g2 f(E)(1 - f(E + w)) / (1 + n(w)) delta(E' - w at (k, m)) for w >= 0.5 meV
 * (:1857-1870), times 2 pi / hbar (:1897), and the rate sum spindeg * Y in
 * list order (:2811-2813).  Phonon states of q in [q_begin, q_begin + nq).
 */
int or_ph_rates_run(or_rates_ctx *cx, int64_t q_begin, int64_t nq, int nthreads, double spindeg,
                    double *rates_phe, int64_t *info, double *g2out, double *yout, int64_t cap) {
  const or_wannier *w = cx->w;
  const or_request *req = &cx->req;
  const int64_t nw = w->nw, nb = w->nb, nwsk = w->nwsk, nwsg = w->nwsg;
  const int64_t *mesh = req->mesh;
  const int64_t N = cx->N, nwv = cx->nwv;
  const double const_tp = TWOPI / HBAR_EVPS;
  const double *kw = cx->kw, *ens = cx->ens, *evecs = cx->evecs, *phe = cx->phe, *phv = cx->phv;
  const int64_t *indexlist = cx->indexlist;
  const delta_ctx dc = cx->dc;
  for (int i = 0; i < 8; ++i) info[i] = 0;
  info[0] = nwv;
  info[1] = cx->nin;
  info[5] = cx->status;
  info[6] = cx->us_setup;
  for (int64_t i = 0; i < N * nb; ++i) rates_phe[i] = 0.0;
  if (cx->status == 2) return 2;
  const int64_t q0 = q_begin < 0 ? 0 : (q_begin > N ? N : q_begin);
  const int64_t q1 = nq < 0 ? N : (q0 + nq < N ? q0 + nq : N);
  const int nt = nthreads > 0 ? nthreads : 1;
  double t_loop = wall_us();
  int64_t *nin_k = (int64_t *)malloc(sizeof(int64_t) * (nwv > 0 ? nwv : 1));
  for (int64_t ik = 0; ik < nwv; ++ik) {
    int64_t c = 0;
    for (int64_t b = 0; b < nw; ++b) c += fabs(ens[ik + nwv * b] - req->enref) <= req->fsthick;
    nin_k[ik] = c;
  }
  const int64_t blk = nw * nw * nb;
  double *gm = (double *)malloc(sizeof(double) * 2 * blk * nwsk);   /* gReq(iq) */
  cplx *phase = (cplx *)malloc(sizeof(cplx) * (nwsg > 0 ? nwsg : 1));
  int64_t *kpw = (int64_t *)malloc(sizeof(int64_t) * (nwv > 0 ? nwv : 1));
  int64_t *koff = (int64_t *)malloc(sizeof(int64_t) * (nwv + 1));
  double *ybuf = (double *)malloc(sizeof(double) * (nwv * nw * nw > 0 ? nwv * nw * nw : 1));
  double *gbuf = (double *)malloc(sizeof(double) * (nwv * nw * nw > 0 ? nwv * nw * nw : 1));
  int64_t voff = 0, npairs = 0;
  for (int64_t iq = q0 + 1; iq <= q1; ++iq) {   /* muxed 1-based = IBZ index (identity group) */
    const double prim[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    int64_t qi[3];
    or_demux_vector(iq, qi, mesh, 0);
    double qf[3];
    for (int d = 0; d < 3; ++d) qf[d] = (double)qi[d] / (double)mesh[d];
    /* gReq (wannier.f90:1134-1188), each element summed over Rp in or_gReq's order */
    for (int64_t iuc = 0; iuc < nwsg; ++iuc) {
      double dot = 0.0;
      for (int d = 0; d < 3; ++d) dot += qf[d] * (double)w->rcells_g[iuc + nwsg * d];
      phase[iuc] = expi(TWOPI * dot) / (double)w->gwsdeg[iuc];
    }
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int64_t re = 0; re < nwsk; ++re)
      for (int64_t s = 0; s < nb; ++s)
        for (int64_t j = 0; j < nw; ++j)
          for (int64_t i = 0; i < nw; ++i) {
            cplx acc = 0.0;
            for (int64_t iuc = 0; iuc < nwsg; ++iuc)
              acc += phase[iuc] * cget(w->gwann, i + nw * (j + nw * (re + nwsk * (s + nb * iuc))));
            cset(gm, i + nw * (j + nw * (s + nb * re)), acc);
          }
    /* k + q in the window (vec_add + binsearch, interactions.f90:1813-1822) and the
     * first list position of each k's vertices */
    koff[0] = 0;
    for (int64_t ik = 0; ik < nwv; ++ik) {
      int64_t iv[3], kpmux;
      double f[3], cc[3];
      or_vector_addsub(indexlist[ik], iq, +1, mesh, prim, iv, &kpmux, f, cc);
      const int64_t ikp = or_binsearch(indexlist, nwv, kpmux);
      kpw[ik] = ikp;
      npairs += ikp > 0;
      koff[ik + 1] = koff[ik] + (ikp > 0 ? nin_k[ik] * nin_k[ikp - 1] : 0);
    }
    const int64_t count_q = koff[nwv];
    for (int64_t s = 1; s <= nb; ++s) {
      const double en_ph = phe[(iq - 1) + N * (s - 1)];
      double evq[2 * 64];
      for (int64_t c = 0; c < nb; ++c) {
        evq[2 * c] = phv[2 * ((iq - 1) + N * ((s - 1) + nb * c))];
        evq[2 * c + 1] = phv[2 * ((iq - 1) + N * ((s - 1) + nb * c)) + 1];
      }
      const double invboseplus1 = (en_ph != 0.0) ? 1.0 / (1.0 + or_Bose(en_ph, req->T)) : 0.0;
#pragma omp parallel num_threads(nt)
      {
        double *evk = (double *)malloc(sizeof(double) * 2 * nw);
        double *evkp = (double *)malloc(sizeof(double) * 2 * nw);
#pragma omp for schedule(dynamic, 4)
        for (int64_t ik = 1; ik <= nwv; ++ik) {
          const int64_t ikp = kpw[ik - 1];
          if (ikp < 0) continue;
          const double kv[3] = {kw[ik - 1], kw[(ik - 1) + nwv], kw[(ik - 1) + 2 * nwv]};
          int64_t count = koff[ik - 1];
          for (int64_t m = 1; m <= nw; ++m) {
            const double en_el = ens[(ik - 1) + nwv * (m - 1)];
            if (fabs(en_el - req->enref) > req->fsthick) continue;
            const double fermi1 = or_Fermi(en_el, req->chempot, req->T);
            const double fermi2 = or_Fermi(en_el + en_ph, req->chempot, req->T);
            for (int64_t c = 0; c < nw; ++c) {
              evk[2 * c] = evecs[2 * ((ik - 1) + nwv * ((m - 1) + nw * c))];
              evk[2 * c + 1] = evecs[2 * ((ik - 1) + nwv * ((m - 1) + nw * c)) + 1];
            }
            for (int64_t n = 1; n <= nw; ++n) {
              const double en_elp = ens[(ikp - 1) + nwv * (n - 1)];
              if (fabs(en_elp - req->enref) > req->fsthick) continue;
              for (int64_t c = 0; c < nw; ++c) {
                evkp[2 * c] = evecs[2 * ((ikp - 1) + nwv * ((n - 1) + nw * c))];
                evkp[2 * c + 1] = evecs[2 * ((ikp - 1) + nwv * ((n - 1) + nw * c)) + 1];
              }
              const double g2 = or_g2(w, kv, qf, evk, evkp, evq, en_ph, gm, 0);
              const double delta = delta_eval(&dc, en_elp - en_ph, ik, m);
              const double occup_fac = fermi1 * (1.0 - fermi2) * invboseplus1;
              double y = 0.0;
              if (en_ph >= 0.5e-3) y = g2 * occup_fac * delta;
              gbuf[count] = g2;
              ybuf[count] = const_tp * y;
              count++;
            }
          }
        }
        free(evk); free(evkp);
      }
      double acc = 0.0;
      for (int64_t i = 0; i < count_q; ++i) {
        acc = acc + spindeg * ybuf[i];
        if (voff + i < cap) {
          if (g2out) g2out[voff + i] = gbuf[i];
          if (yout) yout[voff + i] = ybuf[i];
        }
      }
      rates_phe[(iq - 1) + N * (s - 1)] = acc;
      voff += count_q;
    }
  }
  info[2] = (q1 - q0) * nb;
  info[3] = voff;
  info[4] = npairs;
  free(nin_k); free(gm); free(phase); free(kpw); free(koff); free(ybuf); free(gbuf);
  info[7] = (int64_t)(wall_us() - t_loop);
  return (int)info[5];
}

int or_ph_rates(const or_wannier *w, const or_request *req, double spindeg, int nthreads,
                double *rates_phe, int64_t *info, double *g2, double *y, int64_t cap) {
  or_rates_ctx *cx = or_rates_setup(w, req, nthreads);
  int rc = or_ph_rates_run(cx, 0, -1, nthreads, spindeg, rates_phe, info, g2, y, cap);
  or_rates_free(cx);
  return rc;
}
