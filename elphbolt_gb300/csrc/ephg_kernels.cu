// ephg_kernels.cu - FP64 set-up and drop-in kernels of the e-ph vertex path.
//
// Phase tables, H(k)/D(q) assembly, the batched warp-level Hermitian Jacobi
// eigensolver, the FP64 complex GEMM used by the plain drop-in, and the
// per-(k', state) epilogue that forms |g|^2, X+- and the RTA rate partials.
// Each kernel names the reference lines it restates.
#include <mutex>
#include <cstdio>

#include "ephg_kernels.cuh"

namespace ephg {

static constexpr double PI = 3.141592653589793;   // 4*atan(1), params.f90:44
static constexpr double TWOPI = 2.0 * PI;

// =================================================================== phases

__global__ void k_roots(int L, double2 *roots) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= L) return;
  double s, c;
  sincospi(2.0 * (double)t / (double)L, &s, &c);
  roots[t] = make_double2(c, s);
}

void launch_roots(int L, double2 *roots, cudaStream_t st) {
  k_roots<<<(L + 255) / 256, 256, 0, st>>>(L, roots);
}

// exact integer modular phase index of k (mesh index p) and integer R
__device__ inline int phase_index(int p, const int mesh[3], int L, int r1, int r2, int r3) {
  int v1 = p % mesh[0];
  int v2 = (p / mesh[0]) % mesh[1];
  int v3 = p / (mesh[0] * mesh[1]);
  int64_t t = (int64_t)v1 * r1 * (L / mesh[0]) + (int64_t)v2 * r2 * (L / mesh[1]) +
              (int64_t)v3 * r3 * (L / mesh[2]);
  return (int)floormod(t, L);
}

__global__ void k_phase_mesh(int nrows, const int *rowp, int m1, int m2, int m3, int L, int nR,
                             const int *R, const double *deg, int conj, const double2 *roots,
                             double2 *out, int64_t ldo) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nrows * nR) return;
  int row = (int)(idx / nR), r = (int)(idx % nR);
  int p = rowp ? rowp[row] : row;
  const int mesh[3] = {m1, m2, m3};
  int t = phase_index(p, mesh, L, R[3 * r], R[3 * r + 1], R[3 * r + 2]);
  double2 v = roots[t];
  if (conj) v.y = -v.y;
  if (deg) { v.x /= deg[r]; v.y /= deg[r]; }
  out[(int64_t)row * ldo + r] = v;
}

void launch_phase_mesh(int nrows, const int *rowp, const int mesh[3], int L, int nR,
                       const int *R, const double *deg, int conj, const double2 *roots,
                       double2 *out, int64_t ldo, cudaStream_t st) {
  int64_t n = (int64_t)nrows * nR;
  if (n == 0) return;
  k_phase_mesh<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nrows, rowp, mesh[0], mesh[1],
                                                             mesh[2], L, nR, R, deg, conj,
                                                             roots, out, ldo);
}

// ---- a Fourier sum over integer cells onto a whole mesh, one dimension at a time ----
// On a mesh, sum_R e^{2 pi i k.R} X(R) separates: with X placed on the box of
// cell coordinates [lo, lo + ext) per dimension (zero where there is no cell),
// three 1-D sums of ext terms each replace the N_k x N_R phase matrix and its
// GEMM (for H(k), wannier.f90:467-479: ~40x fewer FP64 flops at 24^3, 6^3 WS).
// Every factor e^{2 pi i v (r + lo) / m} is the exact integer-indexed root of
// unity.  One pass: out[a][v][b][e] = sum_r root(v (r + lo) L / m) in[a][r][b][e],
// or with TRANS out[a][b][v][e]: the second and third passes write [r1][v3][v2]
// and then [v3][v2][v1], the muxed mesh index v1 + m1 (v2 + m2 v3) in row order.
template <bool TRANS>
__global__ void k_dft1(int64_t total, int R, int B, int M, int nn, int lo, int Lm, int L,
                       const double2 *__restrict__ roots, const double2 *__restrict__ in,
                       double2 *__restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int e = (int)(idx % nn);
  int64_t t = idx / nn;
  const int b = (int)(t % B);
  t /= B;
  const int v = (int)(t % M);
  const int64_t a = t / M;
  double2 acc = make_double2(0.0, 0.0);
  for (int r = 0; r < R; ++r)
    cfma(acc, roots[floormod((int64_t)v * (r + lo) * Lm, L)], in[((a * R + r) * B + b) * nn + e]);
  out[TRANS ? ((a * B + b) * M + v) * nn + e : idx] = acc;
}

void launch_mesh_fourier(const double2 *box, const int lo[3], const int ext[3], int nn, const int mesh[3], int L,
                         const double2 *roots, double2 *t1, double2 *t2, double2 *out, cudaStream_t st) {
  const int64_t n1 = (int64_t)ext[0] * ext[1] * mesh[2] * nn, n2 = (int64_t)ext[0] * mesh[1] * mesh[2] * nn,
                n3 = (int64_t)mesh[0] * mesh[1] * mesh[2] * nn;
  // along R3: [r1 r2][r3][e] -> [r1 r2][v3][e]
  k_dft1<false><<<(unsigned)((n1 + 255) / 256), 256, 0, st>>>(n1, ext[2], 1, mesh[2], nn, lo[2], L / mesh[2], L,
                                                              roots, box, t1);
  // along R2: [r1][r2][v3][e] -> [r1][v3][v2][e]
  k_dft1<true><<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(n2, ext[1], mesh[2], mesh[1], nn, lo[1], L / mesh[1],
                                                             L, roots, t1, t2);
  // along R1: [r1][v3 v2][e] -> [v3 v2][v1][e], rows in muxed mesh order
  k_dft1<true><<<(unsigned)((n3 + 255) / 256), 256, 0, st>>>(n3, ext[0], mesh[1] * mesh[2], mesh[0], nn, lo[0],
                                                             L / mesh[0], L, roots, t2, out);
}

// expi(twopi * dot_product(k, R)) / deg, misc.f90:588 with wannier.f90:467,1097
__global__ void k_phase_frac(int nrows, const double *kv, int nR, const int *R,
                             const double *deg, double2 *out, int64_t ldo) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nrows * nR) return;
  int row = (int)(idx / nR), r = (int)(idx % nR);
  double dot = kv[row] * (double)R[3 * r];
  dot += kv[row + nrows] * (double)R[3 * r + 1];
  dot += kv[row + 2 * nrows] * (double)R[3 * r + 2];
  double s, c;
  sincos(TWOPI * dot, &s, &c);
  double2 v = make_double2(c, s);
  if (deg) { v.x /= deg[r]; v.y /= deg[r]; }
  out[(int64_t)row * ldo + r] = v;
}

void launch_phase_frac(int nrows, const double *kv, int nR, const int *R, const double *deg,
                       double2 *out, int64_t ldo, cudaStream_t st) {
  int64_t n = (int64_t)nrows * nR;
  if (n == 0) return;
  k_phase_frac<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nrows, kv, nR, R, deg, out, ldo);
}

// ============================================================ FP64 GEMM
// C[M][N] = A[M][K] * B[K][N], complex double, row-major.  64x64 tile per
// 256-thread block, 4x4 complex outputs per thread; FP64-FMA bound on GB300.
// 32-row tiles: the H(k) assembly (N = 64 columns) then spreads over ~3 waves of
// the 152 SMs instead of 1.4, which an FP64-bound kernel pays for in full.
constexpr int ZBM = 32, ZBN = 64, ZBK = 8, ZRM = ZBM / 16;

__global__ void __launch_bounds__(256) k_zgemm(int M, int N, int K, const double2 *__restrict__ A,
                                               int64_t lda, const double2 *__restrict__ B,
                                               int64_t ldb, double2 *__restrict__ C, int64_t ldc) {
  __shared__ double2 sA[ZBK][ZBM + 1];
  __shared__ double2 sB[ZBK][ZBN];
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  const int64_t m0 = (int64_t)blockIdx.y * ZBM, n0 = (int64_t)blockIdx.x * ZBN;
  double2 acc[ZRM][4];
#pragma unroll
  for (int i = 0; i < ZRM; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < K; k0 += ZBK) {
    for (int idx = t; idx < ZBM * ZBK; idx += 256) {
      int row = idx / ZBK, kk = idx % ZBK;
      int64_t gm = m0 + row;
      int gk = k0 + kk;
      sA[kk][row] = (gm < M && gk < K) ? A[gm * lda + gk] : make_double2(0.0, 0.0);
    }
    for (int idx = t; idx < ZBK * ZBN; idx += 256) {
      int kb = idx / ZBN, col = idx % ZBN;
      int64_t gn = n0 + col;
      int gkb = k0 + kb;
      sB[kb][col] = (gn < N && gkb < K) ? B[(int64_t)gkb * ldb + gn] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < ZBK; ++kk) {
      double2 a[ZRM], b[4];
#pragma unroll
      for (int i = 0; i < ZRM; ++i) a[i] = sA[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < ZRM; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < ZRM; ++i) {
    int64_t gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t gn = n0 + tx + 16 * j;
      if (gn < N) C[gm * ldc + gn] = acc[i][j];
    }
  }
}

void launch_zgemm(int M, int N, int K, const double2 *A, int64_t lda, const double2 *B,
                  int64_t ldb, double2 *C, int64_t ldc, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  dim3 grid((N + ZBN - 1) / ZBN, (M + ZBM - 1) / ZBM);
  k_zgemm<<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc);
}

// ====================================================== Jacobi eigensolver
// One warp per Hermitian matrix (n <= 32).  Parallel cyclic Jacobi with the
// round-robin ordering: n/2 disjoint rotations per step, n-1 steps per sweep
// (Golub & Van Loan sec. 8.5.4).  Stands in for zheev('V','U') at
// wannier.f90:489 and :732.
//
// Mixed precision, because GB300's FP64 rate is a sixtieth of its FP32 rate:
//  1. FP32 sweeps bring the matrix to near-diagonal form (off-diagonal norm
//     ~1e-5 of the total) and accumulate their rotations in Q;
//  2. two Newton-Schulz steps X <- X (3I - X^H X) / 2 in FP64 make Q unitary to
//     FP64 rounding (from ~1e-6);
//  3. B = Q^H A Q in FP64 has A's eigenvalues to FP64 rounding;
//  4. FP64 sweeps on B, accumulating into V = Q, converge quadratically from
//     there: two or three sweeps instead of six or seven from A.
constexpr int EIG_MAXSWEEP = 40;
constexpr int EIG_MAXSWEEP32 = 12;

// round-robin pair `lane` (< m / 2) of step r, m players: (p, q) with p < q
__device__ __forceinline__ void rr_pair(int r, int m, int lane, int &p, int &q) {
  int a, b;
  if (lane == 0) {
    a = 0;
    b = (r % (m - 1)) + 1;
  } else {
    a = ((r + lane) % (m - 1)) + 1;
    b = ((r - lane + (m - 1)) % (m - 1)) + 1;
  }
  p = min(a, b);
  q = max(a, b);
}

// FP32 sweeps on A (float2, column-major n x n) accumulating into Q until the
// off-diagonal norm is 1e-10 of the total or stalls below 1e-6 of it; P4 / PI:
// the step's rotations (c, s, e^{i phi}) and pairs.
__device__ void jacobi_f32(int n, float2 *A, float2 *Q, float4 *P4, int2 *PI, int lane) {
  const int nn = n * n, m = n + (n & 1), half = m / 2;
  float prev = INFINITY;
  for (int sweep = 0; sweep < EIG_MAXSWEEP32; ++sweep) {
    float off = 0.f, tot = 0.f;
    for (int idx = lane; idx < nn; idx += 32) {
      const float2 a = A[idx];
      const float a2 = a.x * a.x + a.y * a.y;
      tot += a2;
      if (idx % n != idx / n) off += a2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    // done at 1e-10 of the total, or once it stalls near FP32's floor; a
    // non-finite norm also stops it (Q is then not used)
    if (!(off > 1e-10f * tot) || (off <= 1e-6f * tot && off > 0.25f * prev)) return;
    prev = off;
    for (int r = 0; r < m - 1; ++r) {
      if (lane < half) {
        int p, q;
        rr_pair(r, m, lane, p, q);
        float c = 1.f, sn = 0.f, phx = 1.f, phy = 0.f;
        if (q < n) {
          const float2 apq = A[p + n * q];
          const float rr = hypotf(apq.x, apq.y);
          if (rr > 0.f) {
            const float tau = (A[q + n * q].x - A[p + n * p].x) / (2.f * rr);
            const float tf = fabsf(tau) > 1e18f ? 0.5f / tau
                                                : (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(1.f + tau * tau));
            c = rsqrtf(1.f + tf * tf);
            sn = tf * c;
            phx = apq.x / rr;
            phy = apq.y / rr;
          }
        }
        P4[lane] = make_float4(c, sn, phx, phy);
        PI[lane] = make_int2(p, q < n ? q : -1);
      }
      __syncwarp();
      // columns: A <- A J, Q <- Q J;  J = [[c, s], [-s e^{-i phi}, c e^{-i phi}]]
      for (int idx = lane; idx < half * n; idx += 32) {
        const int k = idx / n, i = idx % n;
        const int2 pq = PI[k];
        if (pq.y < 0) continue;
        const float4 r4 = P4[k];
        const float2 aip = A[i + n * pq.x], aiq = A[i + n * pq.y];
        float2 t = make_float2(r4.z * aiq.x + r4.w * aiq.y, r4.z * aiq.y - r4.w * aiq.x);
        A[i + n * pq.x] = make_float2(r4.x * aip.x - r4.y * t.x, r4.x * aip.y - r4.y * t.y);
        A[i + n * pq.y] = make_float2(r4.y * aip.x + r4.x * t.x, r4.y * aip.y + r4.x * t.y);
        const float2 vip = Q[i + n * pq.x], viq = Q[i + n * pq.y];
        t = make_float2(r4.z * viq.x + r4.w * viq.y, r4.z * viq.y - r4.w * viq.x);
        Q[i + n * pq.x] = make_float2(r4.x * vip.x - r4.y * t.x, r4.x * vip.y - r4.y * t.y);
        Q[i + n * pq.y] = make_float2(r4.y * vip.x + r4.x * t.x, r4.y * vip.y + r4.x * t.y);
      }
      __syncwarp();
      // rows: A <- J^H A
      for (int idx = lane; idx < half * n; idx += 32) {
        const int k = idx / n, jj = idx % n;
        const int2 pq = PI[k];
        if (pq.y < 0) continue;
        const float4 r4 = P4[k];
        const float2 apj = A[pq.x + n * jj], aqj = A[pq.y + n * jj];
        const float2 t = make_float2(r4.z * aqj.x - r4.w * aqj.y, r4.z * aqj.y + r4.w * aqj.x);
        A[pq.x + n * jj] = make_float2(r4.x * apj.x - r4.y * t.x, r4.x * apj.y - r4.y * t.y);
        A[pq.y + n * jj] = make_float2(r4.y * apj.x + r4.x * t.x, r4.y * apj.y + r4.x * t.y);
      }
      __syncwarp();
      if (lane < half) {
        const int2 pq = PI[lane];
        if (pq.y >= 0) {
          A[pq.x + n * pq.x].y = 0.f;   // the diagonal of a Hermitian matrix is real
          A[pq.y + n * pq.y].y = 0.f;
        }
      }
      __syncwarp();
    }
  }
}

// C = op(X) Y for n x n complex FP64 matrices in shared memory (column-major),
// op(X) = X^H if XH; one warp.
template <bool XH>
__device__ void wmatmul(int n, const double2 *X, const double2 *Y, double2 *C, int lane) {
  for (int idx = lane; idx < n * n; idx += 32) {
    const int i = idx % n, jj = idx / n;
    double2 acc = make_double2(0.0, 0.0);
    for (int k = 0; k < n; ++k) {
      if (XH) cfma_cj(acc, X[k + n * i], Y[k + n * jj]);
      else cfma(acc, X[i + n * k], Y[k + n * jj]);
    }
    C[idx] = acc;
  }
  __syncwarp();
}

__global__ void k_heig(int batch, int n, const double2 *__restrict__ A, int64_t stride,
                       double *__restrict__ w, double2 *__restrict__ V, int *err) {
  extern __shared__ double2 sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int mat = blockIdx.x * wpb + wib;
  const int nn = n * n;
  double2 *sA = sm + (size_t)wib * (4 * nn + 3 * 16);
  double2 *sV = sA + nn, *sT = sV + nn, *sT2 = sT + nn;
  double2 *sP = sT2 + nn;   // per pair: (c, s), (ph.x, ph.y), (p, q) packed
  float2 *fA = (float2 *)sT, *fQ = fA + nn;   // the FP32 phase, inside sT
  if (mat >= batch) return;
  const double2 *Am = A + (size_t)mat * stride;
  for (int idx = lane; idx < nn; idx += 32) {
    int i = idx % n, j = idx / n;
    double2 v;
    if (i < j) {                       // averaged upper triangle (wannier.f90:481-486)
      double2 aij = Am[i + n * j], aji = Am[j + n * i];
      v = make_double2(0.5 * (aij.x + aji.x), 0.5 * (aij.y - aji.y));
    } else if (i > j) {
      double2 aij = Am[i + n * j], aji = Am[j + n * i];
      v = make_double2(0.5 * (aji.x + aij.x), -0.5 * (aji.y - aij.y));
    } else {
      v = make_double2(Am[i + n * i].x, 0.0);
    }
    sA[idx] = v;
    fA[idx] = make_float2((float)v.x, (float)v.y);
    fQ[idx] = make_float2(i == j ? 1.f : 0.f, 0.f);
  }
  __syncwarp();
  // 1. FP32 sweeps
  jacobi_f32(n, fA, fQ, (float4 *)sP, (int2 *)((float4 *)sP + 16), lane);
  bool finite = true;
  for (int idx = lane; idx < nn; idx += 32) {
    const float2 q = fQ[idx];
    finite = finite && isfinite(q.x) && isfinite(q.y);
    sV[idx] = make_double2((double)q.x, (double)q.y);
  }
  __syncwarp();
  if (!__all_sync(0xffffffffu, finite)) {   // FP32 overflowed: the FP64 sweeps start from A itself
    for (int idx = lane; idx < nn; idx += 32) sV[idx] = make_double2(idx % n == idx / n ? 1.0 : 0.0, 0.0);
    __syncwarp();
  }
  // 2. Q unitary to FP64 rounding: X <- X (3I - X^H X) / 2, twice
  for (int it = 0; it < 2; ++it) {
    wmatmul<true>(n, sV, sV, sT, lane);
    for (int idx = lane; idx < nn; idx += 32) {
      const double2 t = sT[idx];
      sT[idx] = make_double2((idx % n == idx / n ? 3.0 : 0.0) - t.x, -t.y);
    }
    __syncwarp();
    wmatmul<false>(n, sV, sT, sT2, lane);
    for (int idx = lane; idx < nn; idx += 32) sV[idx] = cscale(sT2[idx], 0.5);
    __syncwarp();
  }
  // 3. B = Q^H A Q, made exactly Hermitian (its rounding is below the FP64 sweeps' floor)
  wmatmul<false>(n, sA, sV, sT, lane);
  wmatmul<true>(n, sV, sT, sA, lane);
  for (int idx = lane; idx < nn; idx += 32) {
    const int i = idx % n, j = idx / n;
    if (i < j) {
      const double2 bij = sA[i + n * j], bji = sA[j + n * i];
      const double2 v = make_double2(0.5 * (bij.x + bji.x), 0.5 * (bij.y - bji.y));
      sA[i + n * j] = v;
      sA[j + n * i] = cconj(v);
    } else if (i == j) {
      sA[idx].y = 0.0;
    }
  }
  __syncwarp();
  // 4. FP64 sweeps on B, accumulating into V = Q
  const int m = n + (n & 1);         // even number of players (dummy = n)
  const int half = m / 2;
  bool converged = false;
  double prev_off = INFINITY;
  for (int sweep = 0; sweep < EIG_MAXSWEEP; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int idx = lane; idx < nn; idx += 32) {
      double2 a = sA[idx];
      double a2 = a.x * a.x + a.y * a.y;
      tot += a2;
      if (idx % n != idx / n) off += a2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    // Converged: the off-diagonal norm is ~7 eps of the matrix norm, or it has
    // reached the FP64 rounding floor (the rotations leave a_pq at rounding
    // level rather than zero, so the floor sits near 1e-31..1e-30 of the total
    // and may not pass the first test): below 1e-26 of the total and no longer
    // falling by 4x per sweep.
    if (off <= 1e-30 * tot || off == 0.0 || (off <= 1e-26 * tot && off > 0.25 * prev_off)) {
      converged = true;
      break;
    }
    prev_off = off;
    for (int r = 0; r < m - 1; ++r) {
      if (lane < half) {
        int p, q;
        rr_pair(r, m, lane, p, q);
        double c = 1.0, s = 0.0, phx = 1.0, phy = 0.0;
        if (q < n) {
          // The rotation angle is computed in FP32 on operands scaled by the
          // power of two of a_pq (GB300's FP64 divide / sqrt are slow); the
          // rotation is then made unitary to FP64 rounding, so it is an exact
          // similarity transform that leaves a_pq ~ 1e-7 of its value.  Later
          // rotations remove that residual; a_pq is not forced to zero.  With
          // |a_qq - a_pp| > 1e30 |a_pq| the rotation is negligible and skipped.
          const double2 apq = sA[p + n * q];
          const double d = sA[q + n * q].x - sA[p + n * p].x;
          const double mx = fmax(fabs(apq.x), fabs(apq.y));
          const int ex = ((__double2hiint(mx) >> 20) & 0x7ff) - 1023;
          if (mx > 0.0 && ex > -1000 && ex < 1000) {
            const double sc = __hiloint2double((1023 - ex) << 20, 0);   // 2^-ex: max |a_pq| -> [1, 2)
            const float ax = (float)(apq.x * sc), ay = (float)(apq.y * sc);
            const double dsc = d * sc;
            const float rr = sqrtf(ax * ax + ay * ay);
            if (fabs(dsc) <= 1e30) {
              const float tau = (float)dsc / (2.f * rr);
              const float tf = fabsf(tau) > 1e18f ? 0.5f / tau
                                                  : (tau >= 0.f ? 1.f : -1.f) / (fabsf(tau) + sqrtf(1.f + tau * tau));
              double px = (double)(ax / rr), py = (double)(ay / rr);
              double cc = (double)rsqrtf(1.f + tf * tf);
              double ss = (double)tf * cc;
              // two Newton steps of 1/sqrt(r2) from 1: |ph| = 1 and c^2 + s^2 = 1 in FP64
              double r2 = px * px + py * py, f = 1.5 - 0.5 * r2;
              f = f * (1.5 - 0.5 * r2 * f * f);
              phx = px * f;
              phy = py * f;
              r2 = cc * cc + ss * ss;
              f = 1.5 - 0.5 * r2;
              f = f * (1.5 - 0.5 * r2 * f * f);
              c = cc * f;
              s = ss * f;
            }
          }
        }
        sP[3 * lane] = make_double2(c, s);
        sP[3 * lane + 1] = make_double2(phx, phy);
        sP[3 * lane + 2] = make_double2((double)p, (double)(q < n ? q : -1));
      }
      __syncwarp();
      // columns: A <- A J, V <- V J;  J = [[c, s], [-s e^{-i phi}, c e^{-i phi}]]
      for (int idx = lane; idx < half * n; idx += 32) {
        int k = idx / n, i = idx % n;
        int q = (int)sP[3 * k + 2].y;
        if (q < 0) continue;
        int p = (int)sP[3 * k + 2].x;
        double c = sP[3 * k].x, s = sP[3 * k].y;
        double2 phc = make_double2(sP[3 * k + 1].x, -sP[3 * k + 1].y);
        double2 aip = sA[i + n * p], aiq = sA[i + n * q];
        double2 t = cmul(phc, aiq);
        sA[i + n * p] = make_double2(c * aip.x - s * t.x, c * aip.y - s * t.y);
        sA[i + n * q] = make_double2(s * aip.x + c * t.x, s * aip.y + c * t.y);
        double2 vip = sV[i + n * p], viq = sV[i + n * q];
        t = cmul(phc, viq);
        sV[i + n * p] = make_double2(c * vip.x - s * t.x, c * vip.y - s * t.y);
        sV[i + n * q] = make_double2(s * vip.x + c * t.x, s * vip.y + c * t.y);
      }
      __syncwarp();
      // rows: A <- J^H A
      for (int idx = lane; idx < half * n; idx += 32) {
        int k = idx / n, j = idx % n;
        int q = (int)sP[3 * k + 2].y;
        if (q < 0) continue;
        int p = (int)sP[3 * k + 2].x;
        double c = sP[3 * k].x, s = sP[3 * k].y;
        double2 ph = sP[3 * k + 1];
        double2 apj = sA[p + n * j], aqj = sA[q + n * j];
        double2 t = cmul(ph, aqj);
        sA[p + n * j] = make_double2(c * apj.x - s * t.x, c * apj.y - s * t.y);
        sA[q + n * j] = make_double2(s * apj.x + c * t.x, s * apj.y + c * t.y);
      }
      __syncwarp();
      if (lane < half) {
        int q = (int)sP[3 * lane + 2].y;
        if (q >= 0) {
          int p = (int)sP[3 * lane + 2].x;
          sA[p + n * p].y = 0.0;   // the diagonal of a Hermitian matrix is real
          sA[q + n * q].y = 0.0;
        }
      }
      __syncwarp();
    }
  }
  if (!converged && lane == 0) atomicOr(err, DERR_EIG);
  // sort ascending by rank (ties by index), write eigenvalues and columns
  for (int i = lane; i < n; i += 32) {
    double di = sA[i + n * i].x;
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      double dj = sA[j + n * j].x;
      rank += (dj < di) || (dj == di && j < i);
    }
    w[(size_t)mat * n + rank] = di;
    for (int c = 0; c < n; ++c) V[(size_t)mat * nn + c + n * rank] = sV[c + n * i];
  }
}

void launch_heig(int batch, int n, const double2 *A, int64_t stride, double *w, double2 *V,
                 int *err, cudaStream_t st) {
  if (batch <= 0) return;
  int wpb = n <= 8 ? 4 : n <= 16 ? 2 : 1;
  size_t smem = (size_t)wpb * (4 * n * n + 3 * 16) * sizeof(double2);   // 67 KB at most (n = 32)
  // once per process: changing a kernel attribute can wait for the device's queued work
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(k_heig, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
  });
  k_heig<<<(batch + wpb - 1) / wpb, 32 * wpb, smem, st>>>(batch, n, A, stride, w, V, err);
}

// ============================================================ electrons
// el_wann post-processing (wannier.f90:499-520): energies (eV, + scissor),
// evecs(k,b,:) = eigenvector b, velocities by Feynman-Hellmann.
__global__ void k_el_post(int nk, int nw, const double *w, const double2 *V, const double2 *C,
                          int64_t ldc, int with_vel, const double *scissor, double *energies_f,
                          double *vel_f, double2 *evecs_f, double *ens_i) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nk * nw) return;
  int k = idx / nw, b = idx % nw;
  const size_t nn = (size_t)nw * nw;
  double e = w[(size_t)k * nw + b] * Ryd2eV;
  if (scissor) e += scissor[b];
  if (energies_f) energies_f[k + (int64_t)nk * b] = e;
  if (ens_i) ens_i[(size_t)k * nw + b] = e;
  const double2 *Vk = V + (size_t)k * nn;
  if (evecs_f)
    for (int c = 0; c < nw; ++c) evecs_f[k + (int64_t)nk * (b + (int64_t)nw * c)] = Vk[c + nw * b];
  if (with_vel && vel_f) {
    for (int p = 0; p < 3; ++p) {
      const double2 *dH = C + (int64_t)k * ldc + (size_t)(1 + p) * nn;
      double2 acc = make_double2(0.0, 0.0);
      for (int r = 0; r < nw; ++r) {
        double2 mv = make_double2(0.0, 0.0);
        for (int c = 0; c < nw; ++c) cfma(mv, dH[r + nw * c], Vk[c + nw * b]);
        cfma_cj(acc, Vk[r + nw * b], mv);
      }
      vel_f[k + (int64_t)nk * (b + (int64_t)nw * p)] = acc.x * Ryd2radTHz;
    }
  }
}

void launch_el_post(int nk, int nw, const double *w, const double2 *V, const double2 *C,
                    int64_t ldc, int with_vel, const double *scissor, double *energies_f,
                    double *vel_f, double2 *evecs_f, double *ens_i, cudaStream_t st) {
  int n = nk * nw;
  if (n == 0) return;
  k_el_post<<<(n + 127) / 128, 128, 0, st>>>(nk, nw, w, V, C, ldc, with_vel, scissor, energies_f,
                                             vel_f, evecs_f, ens_i);
}

// ============================================================= phonons
// D(q) assembly with Wigner-Seitz wrapping (wannier.f90:631-665), mass
// normalisation (:716-729).  One block per q.  The wrapped phase sum of each
// (atom pair, WS cell), sum_w e^{2 pi i q.(R + w N_c)} / (deg * nwrap), is
// formed once into shared memory (chunks of DB_CHUNK cells) and then each
// thread contracts it with D(R) for its matrix elements.
constexpr int DB_CHUNK = 64;

__global__ void __launch_bounds__(128) k_dbuild(int nq, const int *qp, int m1, int m2, int m3, int L,
                                                const double2 *roots, const double *qv, PhTerms t, int with_vel,
                                                double2 *Dq, double2 *dDq) {
  extern __shared__ double2 dsm[];   // [npair][DB_CHUNK] phase sums
  const int q = blockIdx.x;
  const int nb = t.nb, nwsq = t.nwsq, npair = t.npair;
  const int mesh[3] = {m1, m2, m3};
  const int ne = nb * nb;
  // each thread owns up to DB_U matrix elements (nb <= 32 gives <= 1024 elements)
  constexpr int DB_U = 8;
  // without velocities and for nb^2 <= blockDim / 2, the cells of each chunk are
  // split over nsl thread slices per element; the slices are added in order at the end
  const int nsl = (!with_vel && 2 * ne <= (int)blockDim.x) ? (int)blockDim.x / ne : 1;
  double2 acc[DB_U], dacc[DB_U][3];
  for (int u = 0; u < DB_U; ++u) {
    acc[u] = make_double2(0.0, 0.0);
    for (int p = 0; p < 3; ++p) dacc[u][p] = make_double2(0.0, 0.0);
  }
  for (int c0 = 0; c0 < nwsq; c0 += DB_CHUNK) {
    const int nc = min(DB_CHUNK, nwsq - c0);
    __syncthreads();
    for (int w = threadIdx.x; w < npair * nc; w += blockDim.x) {
      const int pair = w / nc, iuc = c0 + w % nc;
      const int en = t.pair_off[pair] + iuc;     // entries are (pair, cell) in cell order
      double2 cs = make_double2(0.0, 0.0);
      for (int wv = t.ent_woff[en]; wv < t.ent_woff[en + 1]; ++wv) {
        const int *R = t.wrapR + 3 * wv;
        double2 ph;
        if (qp) {
          ph = roots[phase_index(qp[q], mesh, L, R[0], R[1], R[2])];
        } else {
          double dot = qv[q] * (double)R[0];
          dot += qv[q + nq] * (double)R[1];
          dot += qv[q + 2 * nq] * (double)R[2];
          sincos(TWOPI * dot, &ph.y, &ph.x);
        }
        cs.x += ph.x;
        cs.y += ph.y;
      }
      const double rden = t.ent_rden[en];
      dsm[pair * DB_CHUNK + (iuc - c0)] = make_double2(cs.x * rden, cs.y * rden);
    }
    __syncthreads();
    if (nsl > 1) {   // small nb: thread = (element, slice of the chunk's cells), 4-FMA complex MACs
      if (threadIdx.x < nsl * ne) {
        const int e = threadIdx.x % ne, sl = threadIdx.x / ne;
        const int a = e % nb, b = e / nb;
        const int pair = (a / 3) + t.nat * (b / 3);
        const double2 *Dp = t.D + (int64_t)nwsq * (a + (int64_t)nb * b);
        double ar = acc[0].x, ai = acc[0].y;
        for (int k = sl; k < nc; k += nsl) {
          const double2 ph = dsm[pair * DB_CHUNK + k], dv = Dp[c0 + k];
          ar = fma(ph.x, dv.x, ar);
          ar = fma(-ph.y, dv.y, ar);
          ai = fma(ph.x, dv.y, ai);
          ai = fma(ph.y, dv.x, ai);
        }
        acc[0] = make_double2(ar, ai);
      }
      continue;
    }
#pragma unroll
    for (int u = 0; u < DB_U; ++u) {
      const int e = threadIdx.x + u * blockDim.x;
      if (e >= ne) break;
      const int a = e % nb, b = e / nb;
      const int pair = (a / 3) + t.nat * (b / 3);
      for (int k = 0; k < nc; ++k) {
        const int iuc = c0 + k;
        const double2 term = cmul(dsm[pair * DB_CHUNK + k], t.D[iuc + (int64_t)nwsq * (a + (int64_t)nb * b)]);
        acc[u] = cadd(acc[u], term);
        if (with_vel)
          for (int p = 0; p < 3; ++p) {
            const double rc = t.rcart[iuc + (int64_t)nwsq * p];
            dacc[u][p] = cadd(dacc[u][p], make_double2(-rc * term.y, rc * term.x));
          }
      }
    }
  }
  if (nsl > 1) {
    __syncthreads();
    double2 *part = dsm;   // [nsl][ne] slice sums (nsl * ne <= blockDim = 128 entries)
    if (threadIdx.x < nsl * ne) part[threadIdx.x] = acc[0];
    __syncthreads();
    if (threadIdx.x < ne) {
      const int e = threadIdx.x, a = e % nb, b = e / nb;
      double2 sum = part[e];
      for (int sl = 1; sl < nsl; ++sl) sum = cadd(sum, part[sl * ne + e]);
      const double massnorm = 1.0 / sqrt(t.masses[a / 3] * t.masses[b / 3]) * Ryd2amu;
      Dq[(size_t)q * ne + e] = cscale(sum, massnorm);
    }
    return;
  }
#pragma unroll
  for (int u = 0; u < DB_U; ++u) {
    const int e = threadIdx.x + u * blockDim.x;
    if (e >= ne) break;
    const int a = e % nb, b = e / nb;
    const double massnorm = 1.0 / sqrt(t.masses[a / 3] * t.masses[b / 3]) * Ryd2amu;
    Dq[(size_t)q * ne + e] = cscale(acc[u], massnorm);
    if (with_vel)
      for (int p = 0; p < 3; ++p) dDq[((size_t)q * 3 + p) * ne + e] = cscale(dacc[u][p], massnorm);
  }
}

void launch_dbuild(int nq, const int *qp, const int mesh[3], int L, const double2 *roots,
                   const double *qv, const PhTerms &t, int with_vel, double2 *Dq, double2 *dDq,
                   cudaStream_t st) {
  if (nq <= 0) return;
  // phase sums [npair][DB_CHUNK], reused for the slice sums (<= 128 entries)
  const size_t smem = (size_t)std::max(t.npair * DB_CHUNK, 128) * sizeof(double2);
  // once per process: changing a kernel attribute can wait for the device's queued work
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(k_dbuild, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
  });
  k_dbuild<<<nq, 128, smem, st>>>(nq, qp, mesh ? mesh[0] : 1, mesh ? mesh[1] : 1, mesh ? mesh[2] : 1, L, roots, qv,
                                  t, with_vel, Dq, dDq);
}

// ph_wann post-processing (wannier.f90:740-780)
__global__ void k_ph_post(int nq, int nb, const int *qp, const double *qv, const double *w,
                          const double2 *V, const double2 *dDq, int with_vel,
                          const double *masses, double *energies_f, double2 *evecs_f,
                          double *vel_f, double *om_i, double2 *u_i, float2 *u_f, int *err) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nq * nb) return;
  int q = idx / nb, s = idx % nb;
  const size_t nn = (size_t)nb * nb;
  double o2 = w[(size_t)q * nb + s];
  double e = sqrt(fabs(o2));
  if (o2 < 0.0 || signbit(o2)) e = -e;          // sign(sqrt(abs(w)), w)
  const double2 *Vq = V + (size_t)q * nn;
  double vel[3] = {0.0, 0.0, 0.0};
  if (with_vel) {
    for (int p = 0; p < 3; ++p) {
      const double2 *dD = dDq + ((size_t)q * 3 + p) * nn;
      double2 acc = make_double2(0.0, 0.0);
      for (int r = 0; r < nb; ++r) {
        double2 mv = make_double2(0.0, 0.0);
        for (int c = 0; c < nb; ++c) cfma(mv, dD[r + nb * c], Vq[c + nb * s]);
        cfma_cj(acc, Vq[r + nb * s], mv);
      }
      vel[p] = acc.x / (2.0 * e) * Ryd2radTHz;
    }
  }
  e *= Ryd2eV;
  bool gamma = qp ? (qp[q] == 0) : (qv[q] == 0.0 && qv[q + nq] == 0.0 && qv[q + 2 * nq] == 0.0);
  if (gamma) {
    if (s < 3) e = 0.0;
    vel[0] = vel[1] = vel[2] = 0.0;
  }
  if (e < -0.005) atomicOr(err, DERR_NEG_PHONON);
  else if (e < 0.0 && e > -0.005) e = 0.0;
  if (energies_f) energies_f[q + (int64_t)nq * s] = e;
  if (om_i) om_i[(size_t)q * nb + s] = e;
  if (evecs_f)
    for (int c = 0; c < nb; ++c) evecs_f[q + (int64_t)nq * (s + (int64_t)nb * c)] = Vq[c + nb * s];
  if (u_i || u_f)
    for (int c = 0; c < nb; ++c) {
      // u(ip) = ph_evec(ip)/sqrt(mass) (wannier.f90:937-942)
      double2 u = make_double2(Vq[c + nb * s].x / sqrt(masses[c / 3]), Vq[c + nb * s].y / sqrt(masses[c / 3]));
      if (u_i) u_i[((size_t)q * nb + s) * nb + c] = u;
      if (u_f) u_f[((size_t)q * nb + s) * nb + c] = make_float2((float)u.x, (float)u.y);
    }
  if (with_vel && vel_f)
    for (int p = 0; p < 3; ++p) vel_f[q + (int64_t)nq * (s + (int64_t)nb * p)] = vel[p];
}

void launch_ph_post(int nq, int nb, const int *qp, const double *qv, const double *w,
                    const double2 *V, const double2 *dDq, int with_vel, const double *masses,
                    double *energies_f, double2 *evecs_f, double *vel_f, double *om_i,
                    double2 *u_i, float2 *u_f, int *err, cudaStream_t st) {
  int n = nq * nb;
  if (n == 0) return;
  k_ph_post<<<(n + 127) / 128, 128, 0, st>>>(nq, nb, qp, qv, w, V, dDq, with_vel, masses,
                                             energies_f, evecs_f, vel_f, om_i, u_i, u_f, err);
}

// ======================================================= g(Re,Rp) layouts
// epmatwp order (i, j, Re, s, Rp) -> stage-A matrix G[Re][n], n = i + nw*(j + nw*(s + nb*Rp)),
// so that one row of the GEMM output is gmixed(nw,nw,nb,nwsq) of gkRp (wannier.f90:1085).
__global__ void k_permute_gwann(int nw, int nb, int nwsk, int nwsg, const double2 *raw,
                                double2 *G) {
  const int64_t Nn = (int64_t)nw * nw * nb * nwsg;
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= Nn * nwsk) return;
  int64_t re = idx / Nn, n = idx % Nn;
  int64_t nn = (int64_t)nw * nw;
  int64_t ij = n % nn, s = (n / nn) % nb, rp = n / (nn * nb);
  G[idx] = raw[ij + nn * (re + (int64_t)nwsk * (s + (int64_t)nb * rp))];
}

void launch_permute_gwann(int nw, int nb, int nwsk, int nwsg, const double2 *raw, double2 *G,
                          cudaStream_t st) {
  int64_t n = (int64_t)nw * nw * nb * nwsg * nwsk;
  k_permute_gwann<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nw, nb, nwsk, nwsg, raw, G);
}

// ================================================================ gReq
__global__ void k_permute_greq(int nq, int nw, int nb, int nwsk, const double2 *in,
                               double2 *out) {
  int64_t per = (int64_t)nw * nw * nb * nwsk;
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= per * nq) return;
  int64_t q = idx / per, r = idx % per;
  // out (i, j, s, Re) <- in (i, j, Re, s)
  int64_t ij = r % ((int64_t)nw * nw);
  int64_t rest = r / ((int64_t)nw * nw);
  int64_t s = rest % nb, re = rest / nb;
  out[q * per + r] = in[q * per + ij + (int64_t)nw * nw * (re + (int64_t)nwsk * s)];
}

void launch_permute_greq(int nq, int nw, int nb, int nwsk, const double2 *in, double2 *out,
                         cudaStream_t st) {
  int64_t n = (int64_t)nq * nw * nw * nb * nwsk;
  if (n == 0) return;
  k_permute_greq<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nq, nw, nb, nwsk, in, out);
}

// ============================================================= g2 batch
// One warp per vertex: the reference's g2 (wannier.f90:903-1011, non-polar).
__global__ void k_g2_batch(int nv, int nw, int nb, int nws, const double *qv, const int *R,
                           const double *deg, const double2 *ek, const double2 *ekp,
                           const double2 *eq, const double *ph_en, const double *masses,
                           const double2 *gm, const int64_t *gm_index, int64_t gm_stride,
                           const double2 *Lv, double *g2) {
  const int lane = threadIdx.x & 31;
  const int v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (v >= nv) return;
  double en = ph_en[v];
  if (en == 0.0) { if (lane == 0) g2[v] = 0.0; return; }
  const double2 *g = gm + (gm_index[v] - 1) * gm_stride;
  double2 gb = make_double2(0.0, 0.0);
  for (int iws = lane; iws < nws; iws += 32) {
    double2 ukgu = make_double2(0.0, 0.0);
    for (int sp = 0; sp < nb; ++sp) {
      double2 caux = make_double2(0.0, 0.0);
      for (int np = 0; np < nw; ++np) {
        double2 ckp = ekp[v + (int64_t)nv * np];
        for (int mp = 0; mp < nw; ++mp) {
          // overlap(mp,np) = conj(U_k'(np)) * U_k(mp)
          double2 ov = cmul(cconj(ckp), ek[v + (int64_t)nv * mp]);
          cfma(caux, ov, g[np + nw * (mp + (int64_t)nw * (sp + (int64_t)nb * iws))]);
        }
      }
      double2 u = eq[v + (int64_t)nv * sp];
      u = make_double2(u.x / sqrt(masses[sp / 3]), u.y / sqrt(masses[sp / 3]));
      cfma(ukgu, u, caux);
    }
    double dot = qv[v] * (double)R[3 * iws];
    dot += qv[v + nv] * (double)R[3 * iws + 1];
    dot += qv[v + 2 * (int64_t)nv] * (double)R[3 * iws + 2];
    double2 ph;
    sincos(TWOPI * dot, &ph.y, &ph.x);
    ph.x /= deg[iws];
    ph.y /= deg[iws];
    cfma(gb, ph, ukgu);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gb.x += __shfl_xor_sync(0xffffffffu, gb.x, o);
    gb.y += __shfl_xor_sync(0xffffffffu, gb.y, o);
  }
  if (lane == 0) {
    if (Lv) {   // polar: + long_range_prefac(q, u) * dot_product(el_evec_kp, el_evec_k) (wannier.f90:998-1006)
      double2 gl = make_double2(0.0, 0.0), unm = make_double2(0.0, 0.0);
      for (int sp = 0; sp < nb; ++sp) {
        double2 u = eq[v + (int64_t)nv * sp];
        u = make_double2(u.x / sqrt(masses[sp / 3]), u.y / sqrt(masses[sp / 3]));
        cfma(gl, Lv[(size_t)v * nb + sp], u);
      }
      for (int c = 0; c < nw; ++c) cfma_cj(unm, ekp[v + (int64_t)nv * c], ek[v + (int64_t)nv * c]);
      cfma(gb, gl, unm);
    }
    g2[v] = 0.5 * (gb.x * gb.x + gb.y * gb.y) / en * g2unitfactor;
  }
}

void launch_g2_batch(int nv, int nw, int nb, int nws, const double *qv, const int *R,
                     const double *deg, const double2 *ek, const double2 *ekp,
                     const double2 *eq, const double *ph_en, const double *masses,
                     const double2 *gm, const int64_t *gm_index, int64_t gm_stride,
                     const double2 *Lv, double *g2, cudaStream_t st) {
  if (nv <= 0) return;
  k_g2_batch<<<(nv + 3) / 4, 128, 0, st>>>(nv, nw, nb, nws, qv, R, deg, ek, ekp, eq, ph_en,
                                           masses, gm, gm_index, gm_stride, Lv, g2);
}

// ============================================================ q indices
// q = k' - k folded onto the mesh, on integers (vector.f90:86-102 computes the
// same through fractional coordinates and nint).
__global__ void k_kq_index(int m1, int m2, int m3, int nk, const int64_t *k_idx, int nkp,
                           const int64_t *kp_idx, int64_t *q_idx, int *err) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nk * nkp) return;
  int i = (int)(idx % nk), j = (int)(idx / nk);
  int64_t N = (int64_t)m1 * m2 * m3;
  int64_t a = k_idx[i] - 1, b = kp_idx[j] - 1;
  if (a < 0 || a >= N || b < 0 || b >= N) { atomicOr(err, DERR_INDEX); q_idx[idx] = -1; return; }
  int64_t a1 = a % m1, a2 = (a / m1) % m2, a3 = a / ((int64_t)m1 * m2);
  int64_t b1 = b % m1, b2 = (b / m1) % m2, b3 = b / ((int64_t)m1 * m2);
  int64_t q1 = floormod(b1 - a1, m1), q2 = floormod(b2 - a2, m2), q3 = floormod(b3 - a3, m3);
  q_idx[idx] = (q3 * m2 + q2) * m1 + q1 + 1;   // mux_vector base 0 (misc.f90:906)
}

void launch_kq_index(const int mesh[3], int nk, const int64_t *k_idx, int nkp,
                     const int64_t *kp_idx, int64_t *q_idx, int *err, cudaStream_t st) {
  int64_t n = (int64_t)nk * nkp;
  if (n == 0) return;
  k_kq_index<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(mesh[0], mesh[1], mesh[2], nk, k_idx,
                                                          nkp, kp_idx, q_idx, err);
}

// ======================================================= rate pipeline
__global__ void k_window_flags(int N, int nw, const double *ens, double enref, double fsthick,
                               int *flag) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  int in = 0;
  for (int b = 0; b < nw; ++b) in |= fabs(ens[(size_t)p * nw + b] - enref) <= fsthick;
  flag[p] = in;     // apply_energy_window, electron.f90:613-621
}

void launch_window_flags(int N, int nw, const double *ens, double enref, double fsthick,
                         int *flag, cudaStream_t st) {
  k_window_flags<<<(N + 255) / 256, 256, 0, st>>>(N, nw, ens, enref, fsthick, flag);
}

__global__ void k_state_flags(int nwv, int nw, const int *widx, const double *ens, double enref,
                              double fsthick, int *flag, int *nin_k) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nwv) return;
  int p = widx[i], c = 0;
  for (int m = 0; m < nw; ++m) {
    int f = fabs(ens[(size_t)p * nw + m] - enref) <= fsthick;
    flag[(size_t)i * nw + m] = f;
    c += f;
  }
  nin_k[i] = c;
}

void launch_state_flags(int nwv, int nw, const int *widx, const double *ens, double enref,
                        double fsthick, int *flag, int *nin_k, cudaStream_t st) {
  k_state_flags<<<(nwv + 255) / 256, 256, 0, st>>>(nwv, nw, widx, ens, enref, fsthick, flag,
                                                    nin_k);
}

__global__ void k_iota(int n, int *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i;
}
void launch_iota(int n, int *out, cudaStream_t st) {
  if (n > 0) k_iota<<<(n + 255) / 256, 256, 0, st>>>(n, out);
}

// Stage A rotation over the initial band (the U_k half of wannier.f90:960-978),
// with the k-half of the Rp phase, conj(e^{2 pi i k.Rp})/phwsdeg(Rp), folded in
// so that the Rp Fourier of all states is one GEMM against e^{2 pi i k'.Rp}.
__global__ void k_rotate_states_fp64(int j0, int j1, int i0, const int *st_code, int nw, int nb,
                                     int nws, const int *widx, const double2 *U,
                                     const double2 *gk, int64_t ldgk, int m1, int m2, int m3,
                                     int L, const double2 *roots, const int *Rq,
                                     const double *degq, double2 *B, int64_t ldb) {
  const int j = j0 + blockIdx.y;
  const int rp = blockIdx.x;
  if (j >= j1) return;
  const int code = st_code[j];
  const int i = code / nw, m = code % nw;
  const int p = widx[i];
  const int mesh[3] = {m1, m2, m3};
  double2 ph = roots[phase_index(p, mesh, L, Rq[3 * rp], Rq[3 * rp + 1], Rq[3 * rp + 2])];
  ph = make_double2(ph.x / degq[rp], -ph.y / degq[rp]);
  const double2 *Uk = U + ((size_t)p * nw + m) * nw;
  const double2 *g = gk + (int64_t)(i - i0) * ldgk;
  const int ncol = nw * nb;
  for (int c = threadIdx.x; c < ncol; c += blockDim.x) {
    int np = c % nw, s = c / nw;
    double2 acc = make_double2(0.0, 0.0);
    for (int mp = 0; mp < nw; ++mp)
      cfma(acc, Uk[mp], g[np + nw * (mp + (int64_t)nw * (s + (int64_t)nb * rp))]);
    B[(int64_t)rp * ldb + (int64_t)(j - j0) * ncol + c] = cmul(ph, acc);
  }
}

void launch_rotate_states_fp64(int j0, int j1, int i0, const int *st_code, int nw, int nb,
                               int nws, const int *widx, const double2 *U, const double2 *gk,
                               int64_t ldgk, const int mesh[3], int L, const double2 *roots,
                               const int *Rq, const double *degq, double2 *B, int64_t ldb,
                               cudaStream_t st) {
  if (j1 <= j0) return;
  dim3 grid(nws, j1 - j0);
  k_rotate_states_fp64<<<grid, 64, 0, st>>>(j0, j1, i0, st_code, nw, nb, nws, widx, U, gk, ldgk,
                                            mesh[0], mesh[1], mesh[2], L, roots, Rq, degq, B, ldb);
}

__global__ void k_bose(int n, const double *om, double T, double *bose) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double e = om[i];
  // Bose = 1/expm1(e/kB/T) (misc.f90:992-999), zero for zero-energy phonons (interactions.f90:2287)
  bose[i] = (e != 0.0) ? 1.0 / expm1(e / kB / T) : 0.0;
}

void launch_bose(int N, int nb, const double *om, double T, double *bose, cudaStream_t st) {
  int n = N * nb;
  k_bose<<<(n + 255) / 256, 256, 0, st>>>(n, om, T, bose);
}

// ----------------------------------------------------------- deltas
__device__ inline double fermi(double e, double mu, double T) {
  return 1.0 / (exp((e - mu) / kB / T) + 1.0);     // misc.f90:1001-1009
}

// delta_fn_triang, delta.f90:790-881 (ik 0-based window index, ib 0-based)
__device__ double delta_triang(double e, int ik, int ib, const RateParams &rp, const EpiData &d) {
  double acc = 0.0;
  int num = d.scount[ik];
  for (int itk = 0; itk < num; ++itk) {
    int it = d.smap[((size_t)ik * d.maxc + itk) * 2] - 1;
    int iv = d.smap[((size_t)ik * d.maxc + itk) * 2 + 1];
    const double *ev = d.sevals + (((size_t)it * rp.nw + ib) * 3);
    double e1 = ev[0], e2 = ev[1], e3 = ev[2];
    bool c1 = e <= e1, c2 = e1 < e && e <= e2, c3 = e2 < e && e <= e3, c4 = e3 < e;
    if (c1 || c4) continue;
    double E12 = (e - e2) / (e1 - e2), E21 = (e - e1) / (e2 - e1), E13 = (e - e3) / (e1 - e3);
    double E31 = (e - e1) / (e3 - e1), E23 = (e - e3) / (e2 - e3), E32 = (e - e2) / (e3 - e2);
    double tmp = 0.0;
    if (iv == 1) tmp = c2 ? E21 * (E12 + E13) / (e3 - e1) : (c3 ? E23 * E13 / (e3 - e1) : 0.0);
    else if (iv == 2) tmp = c2 ? E21 * E21 / (e3 - e1) : (c3 ? E23 * E23 / (e3 - e1) : 0.0);
    else if (iv == 3) tmp = c2 ? E21 * E31 / (e3 - e1) : (c3 ? E23 * (E31 + E32) / (e3 - e1) : 0.0);
    acc += tmp;
  }
  if (acc < 1.0e-12) acc = 0.0;
  return acc / (double)(2 * (int64_t)rp.N);
}

// delta_fn_tetra, delta.f90:61-225
__device__ double delta_tetra(double e, int ik, int ib, const RateParams &rp, const EpiData &d) {
  double acc = 0.0, tmp = 0.0;
  int num = d.scount[ik];
  for (int itk = 0; itk < num; ++itk) {
    int it = d.smap[((size_t)ik * d.maxc + itk) * 2] - 1;
    int iv = d.smap[((size_t)ik * d.maxc + itk) * 2 + 1];
    const double *ev = d.sevals + (((size_t)it * rp.nw + ib) * 4);
    double e1 = ev[0], e2 = ev[1], e3 = ev[2], e4 = ev[3];
    double e1e = e1 - e, e2e = e2 - e, e3e = e3 - e, e4e = e4 - e;
    double e21 = e2 - e1, e31 = e3 - e1, e41 = e4 - e1, e32 = e3 - e2, e42 = e4 - e2, e43 = e4 - e3;
    bool c1 = e1 <= e && e <= e2, c2 = e2 <= e && e <= e3, c3 = e3 <= e && e <= e4;
    if (e < e1 || e > e4) continue;
    switch (iv) {
      case 1:
        if (c1) { tmp = (e2e / e21 + e3e / e31 + e4e / e41) * (e1e * e1e) / e41 / e31 / e21; if (e1 == e2) tmp = 0.0; }
        else if (c2) {
          tmp = -0.5 * (e3e / (e31 * e31) * (e3e * e2e / e42 / e32 + e4e * e1e / e41 / e42 + e3e * e1e / e32 / e41) +
                        e4e / (e41 * e41) * (e4e * e1e / e42 / e31 + e4e * e2e / e42 / e32 + e3e * e1e / e31 / e32));
          if (e2 == e3) tmp = -0.5 * (e4e * e1e / e41 / e42 + e1e / e41 + e4e / (e41 * e41) * (e4e * e1e / e42 / e31 + e4e / e42 + e1e / e31));
        } else if (c3) { tmp = (e4e * e4e * e4e) / (e41 * e41) / e42 / e43; if (e3 == e4) tmp = (e4e * e4e) / (e41 * e41) / e42; }
        break;
      case 2:
        if (c1) { tmp = -(e1e * e1e * e1e) / (e21 * e21) / e31 / e41; if (e1 == e2) tmp = 0.0; }
        else if (c2) {
          tmp = -0.5 * (e3e / (e32 * e32) * (e3e * e2e / e42 / e31 + e4e * e2e / e42 / e41 + e3e * e1e / e31 / e41) +
                        e4e / (e42 * e42) * (e3e * e2e / e32 / e31 + e4e * e1e / e41 / e31 + e4e * e2e / e32 / e41));
          if (e2 == e3) tmp = -0.5 * (0.0 + e4e / e42 / e41 + 0.0 + e4e / (e42 * e42) * (0.0 + e4e * e1e / e41 / e31 + 1.0));
        } else if (c3) { tmp = (e4e * e4e * e4e) / e41 / (e42 * e42) / e43; if (e3 == e4) tmp = 0.0; }
        break;
      case 3:
        if (c1) { tmp = -(e1e * e1e * e1e) / e21 / (e31 * e31) / e41; if (e1 == e2) tmp = 0.0; }
        else if (c2) {
          tmp = 0.5 * (e2e / (e32 * e32) * (e3e * e2e / e42 / e31 + e4e * e2e / e42 / e41 + e3e * e1e / e31 / e41) +
                       e1e / (e31 * e31) * (e3e * e2e / e42 / e32 + e4e * e1e / e41 / e42 + e3e * e1e / e32 / e41));
          if (e2 == e3) tmp = 0.5 * (0.0 + e4e / e42 / e41 + e1e / e31 / e41 + e1e / (e31 * e31) * (0.0 + e4e * e1e / e41 / e42 + e1e / e41));
        } else if (c3) { tmp = (e4e * e4e * e4e) / e41 / e42 / (e43 * e43); if (e3 == e4) tmp = 0.0; }
        break;
      case 4:
        if (c1) { tmp = -(e1e * e1e * e1e) / e21 / e31 / (e41 * e41); if (e1 == e2) tmp = 0.0; }
        else if (c2) {
          tmp = 0.5 * (e2e / (e42 * e42) * (e3e * e2e / e32 / e31 + e4e * e1e / e41 / e31 + e4e * e2e / e32 / e41) +
                       e1e / (e41 * e41) * (e4e * e1e / e42 / e31 + e4e * e2e / e42 / e32 + e3e * e1e / e31 / e32));
          if (e2 == e3) tmp = 0.5 * (0.0 + e1e / (e41 * e41) * (e4e * e1e / e42 / e31 + e4e / e42 + e1e / e31));
        } else if (c3) { tmp = -(e3e / e43 + e2e / e42 + e1e / e41) * (e4e * e4e) / e41 / e42 / e43; if (e3 == e4) tmp = 0.0; }
        break;
    }
    if (e1 == e2 && e1 == e3 && e1 == e4 && e == e1) tmp = 0.25;
    acc += tmp;
  }
  if (acc < 1.0e-12) acc = 0.0;
  return acc / (double)(6 * (int64_t)rp.N);
}

__device__ inline double delta_eval(double e, int ikp, int n, double eps_kn, const RateParams &rp,
                                    const EpiData &d) {
  if (rp.delta_kind == 0) {
    double x = (e - eps_kn) / rp.sigma;
    return (1.0 / sqrt(TWOPI)) / rp.sigma * exp(-0.5 * x * x) * rp.inv_nk;
  }
  if (rp.delta_kind == 1) return delta_triang(e, ikp, n, rp, d);
  return delta_tetra(e, ikp, n, rp, d);
}

// Per (k', initial state) epilogue: the k' rotation, the phonon mix, |g|^2
// (wannier.f90:937-1009), X+- (interactions.f90:2278-2332, 2353) and the
// per-pair partial of the RTA rate (interactions.f90:3012-3034).  With the
// phonon side requested, also Y of the same vertex (interactions.f90:1857-1870,
// 1897: the (k, m, k + q, n, s) vertex of phonon state (q, s) is the (k, m, k', n,
// s) vertex here, q = k' - k) added into the phonon state's rate.
// Gv(x) returns the complex Rp-Fourier sum G(n' + nw*s') of the pair.
template <typename GV>
__device__ void pair_epilogue(int ip, int j, GV Gv, const RateParams &rp, const EpiData &d,
                              double &out) {
  const int nw = rp.nw, nb = rp.nb;
  const int code = d.st_code[j];
  const int i = code / nw, m = code % nw;
  const int p = d.sidx[i], pp = d.widx[ip];
  const int iw = d.swin ? d.swin[i] : i;   // the state's k in the window (simplices)
  const double E = d.ens[(size_t)p * nw + m];
  int a1 = p % rp.mesh[0], a2 = (p / rp.mesh[0]) % rp.mesh[1], a3 = p / (rp.mesh[0] * rp.mesh[1]);
  int b1 = pp % rp.mesh[0], b2 = (pp / rp.mesh[0]) % rp.mesh[1], b3 = pp / (rp.mesh[0] * rp.mesh[1]);
  int q = (int)(floormod(b1 - a1, rp.mesh[0]) +
                rp.mesh[0] * (floormod(b2 - a2, rp.mesh[1]) + rp.mesh[1] * floormod(b3 - a3, rp.mesh[2])));
  double acc = 0.0;
  int rank_n = 0;
  const bool ph = d.phr || d.yv;
  const double fermi1 = ph ? fermi(E, rp.chempot, rp.T) : 0.0;
  for (int n = 0; n < nw; ++n) {
    double eps = d.ens[(size_t)pp * nw + n];
    if (fabs(eps - rp.enref) > rp.fsthick) continue;
    const double2 *Ukp = d.U + ((size_t)pp * nw + n) * nw;
    double2 h[32];
    for (int s = 0; s < nb; ++s) {
      double2 a = make_double2(0.0, 0.0);
      for (int np = 0; np < nw; ++np) cfma_cj(a, Ukp[np], Gv(np + nw * s));
      h[s] = a;
    }
    double2 unm = make_double2(0.0, 0.0);   // dot_product(el_evec_kp, el_evec_k), polar crystals
    if (d.glp) {
      const double2 *Uk = d.U + ((size_t)p * nw + m) * nw;
      for (int c = 0; c < nw; ++c) cfma_cj(unm, Ukp[c], Uk[c]);
    }
    for (int s = 0; s < nb; ++s) {
      double om = d.om[(size_t)q * nb + s];
      double2 gsum = make_double2(0.0, 0.0);
      const double2 *u = d.u + ((size_t)q * nb + s) * nb;
      for (int sp = 0; sp < nb; ++sp) cfma(gsum, u[sp], h[sp]);
      if (d.glp) cfma(gsum, d.glp[(size_t)q * nb + s], unm);   // long-range term (wannier.f90:998-1006)
      double g2 = (om == 0.0) ? 0.0 : 0.5 * (gsum.x * gsum.x + gsum.y * gsum.y) / om * g2unitfactor;
      double bose = d.bose[(size_t)q * nb + s];
      double xp = 0.0, xm = 0.0, y = 0.0;
      if (om >= 0.5e-3) {
        double fp = fermi(E + om, rp.chempot, rp.T);
        double fm = fermi(E - om, rp.chempot, rp.T);
        double dp = delta_eval(E + om, ip, n, eps, rp, d);
        double dm = delta_eval(E - om, ip, n, eps, rp, d);
        xp = rp.const_tp * (g2 * (bose + fp) * dp);
        xm = rp.const_tp * (g2 * (1.0 + bose - fm) * dm);
        if (ph) {
          // Y: delta(E' - omega) at the initial electron (k, m), interactions.f90:1862
          const double invboseplus1 = 1.0 / (1.0 + bose);
          const double dy = delta_eval(eps - om, iw, m, E, rp, d);
          y = rp.const_tp * (g2 * (fermi1 * (1.0 - fp) * invboseplus1) * dy);
          if (d.phr && y != 0.0) atomicAdd(d.phr + q + (size_t)rp.N * s, d.ph_scale * y);
        }
      }
      acc += xp + xm;
      if (d.g2) {
        int64_t off = (int64_t)j * d.per_state + ((int64_t)d.cum[ip] + rank_n) * nb + s;
        if (off < d.cap) {
          d.g2[off] = g2;
          if (d.xp) d.xp[off] = xp;
          if (d.xm) d.xm[off] = xm;
          if (d.yv) d.yv[off] = y;
        }
      }
    }
    rank_n++;
  }
  out = acc;
}

// Block-deterministic partial: threads along k' for one state, then a fixed
// order compensated (Neumaier) sum by thread 0.
__device__ void block_partial(double v, double *partial, int j, int nblk) {
  __shared__ double sv[128];
  sv[threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0, c = 0.0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      double x = sv[t], tt = s + x;
      c += (fabs(s) >= fabs(x)) ? (s - tt) + x : (x - tt) + s;
      s = tt;
    }
    partial[(size_t)j * nblk + blockIdx.x] = s + c;
  }
}

__global__ void __launch_bounds__(128) k_epilogue_fp64(int nwv, int j0, const double2 *C,
                                                       int64_t ldc, RateParams rp, EpiData d,
                                                       double *partial, int nblk) {
  const int ip = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = j0 + blockIdx.y;
  const int ncol = rp.nw * rp.nb;
  double v = 0.0;
  if (ip < nwv) {
    const double2 *row = C + (int64_t)ip * ldc + (int64_t)(j - j0) * ncol;
    pair_epilogue(ip, j, [&](int x) { return row[x]; }, rp, d, v);
  }
  block_partial(v, partial, j, nblk);
}

void launch_epilogue_fp64(int nwv, int j0, int j1, const double2 *C, int64_t ldc,
                          const RateParams &rp, const EpiData &d, double *partial, int nblk,
                          cudaStream_t st) {
  if (j1 <= j0) return;
  dim3 grid(nblk, j1 - j0);
  k_epilogue_fp64<<<grid, 128, 0, st>>>(nwv, j0, C, ldc, rp, d, partial, nblk);
}

__global__ void __launch_bounds__(128) k_epilogue_fp32(int nwv, int j0, const float *Cr,
                                                       const float *Ci, int64_t ldc,
                                                       RateParams rp, EpiData d,
                                                       double *partial, int nblk) {
  const int ip = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = j0 + blockIdx.y;
  const int ncol = rp.nw * rp.nb;
  double v = 0.0;
  if (ip < nwv) {
    const int64_t base = (int64_t)ip * ldc + (int64_t)(j - j0) * ncol;
    pair_epilogue(ip, j, [&](int x) { return make_double2((double)Cr[base + x], (double)Ci[base + x]); },
                  rp, d, v);
  }
  block_partial(v, partial, j, nblk);
}

void launch_epilogue_fp32(int nwv, int j0, int j1, const float *Cr, const float *Ci,
                          int64_t ldc, const RateParams &rp, const EpiData &d, double *partial,
                          int nblk, cudaStream_t st) {
  if (j1 <= j0) return;
  dim3 grid(nblk, j1 - j0);
  k_epilogue_fp32<<<grid, 128, 0, st>>>(nwv, j0, Cr, Ci, ldc, rp, d, partial, nblk);
}

// rates(ik, m) = compensated sum of the block partials in block order
__global__ void k_rate_final(int nst, int nblk, const double *partial, const int *st_code, int nw,
                             int N, double *rates_f) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nst) return;
  double s = 0.0, c = 0.0;
  for (int b = 0; b < nblk; ++b) {
    double x = partial[(size_t)j * nblk + b], t = s + x;
    c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  int code = st_code[j];
  rates_f[(code / nw) + (int64_t)N * (code % nw)] = s + c;
}

void launch_rate_final(int nst, int nblk, const double *partial, const int *st_code, int nw,
                       int N, double *rates_f, cudaStream_t st) {
  if (nst <= 0) return;
  k_rate_final<<<(nst + 127) / 128, 128, 0, st>>>(nst, nblk, partial, st_code, nw, N, rates_f);
}

// ------------------------------------------ degenerate-subspace averaging
// The gauge fixing of plot_along_path (wannier.f90:1332-1384, the same loops
// in test/check_interactions_symmetries.f90:330-384) on a |g|^2 vertex list in
// the electron side's order (state j, final state f = (k', n), branch s),
// FP64.  Three passes in the reference's order, each over groups of one index
// with the others fixed: branches s of q = k' - k (phonon energies), initial
// bands m of each k, final bands n of each k' (electron energies); a member's
// partners are those with |E - E'| < thres.  Mode 0 restates the reference's
// loops literally, in place: member a becomes the mean, summed in member
// order, of its partners' values as they are at that moment (so a later member
// sees its predecessors' new values); mode 1 takes every mean from the values
// before the pass.  One thread per group set; groups of a pass are disjoint.
constexpr int DEG_MAXG = 64;

__device__ void deg_group(int mode, double thres, int c, double *v, int64_t st, const double *e) {
  double tmp[DEG_MAXG];
  if (mode == 1)
    for (int a = 0; a < c; ++a) tmp[a] = v[a * st];
  for (int a = 0; a < c; ++a) {
    int cnt = 0;
    double aux = 0.0;
    for (int b = 0; b < c; ++b)
      if (fabs(e[a] - e[b]) < thres) {
        ++cnt;
        aux += mode == 0 ? v[b * st] : tmp[b];
      }
    v[a * st] = aux / (double)cnt;
  }
}

// window bands of mesh point p in band order: their count, bands in `band`
__device__ __forceinline__ int window_bands(const double *ens, int p, int nw, double enref, double fsthick, int *band,
                                            double *e) {
  int c = 0;
  for (int n = 0; n < nw; ++n) {
    const double x = ens[(size_t)p * nw + n];
    if (fabs(x - enref) <= fsthick) {
      band[c] = n;
      e[c] = x;
      ++c;
    }
  }
  return c;
}

struct DegList {
  double *g2;
  const int *st_code, *arow, *widx, *cum, *first_state;
  const double *ens, *om;
  int nst, nA, nwv, nw, nb, mesh[3];
  int64_t per;          // entries per state: nin * nb
  double enref, fsthick, thres;
  int mode;
};

// pass 1: branches, per (state, k' row)
__global__ void k_deg_branches(DegList L) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)L.nst * L.nwv) return;
  const int j = (int)(t / L.nwv), b = (int)(t % L.nwv);
  const int p = L.arow[L.st_code[j] / L.nw], pp = L.widx[b];
  const int a1 = p % L.mesh[0], a2 = (p / L.mesh[0]) % L.mesh[1], a3 = p / (L.mesh[0] * L.mesh[1]);
  const int b1 = pp % L.mesh[0], b2 = (pp / L.mesh[0]) % L.mesh[1], b3 = pp / (L.mesh[0] * L.mesh[1]);
  const int q = (int)(floormod(b1 - a1, L.mesh[0]) +
                      L.mesh[0] * (floormod(b2 - a2, L.mesh[1]) + L.mesh[1] * floormod(b3 - a3, L.mesh[2])));
  double e[DEG_MAXG];
  for (int s = 0; s < L.nb; ++s) e[s] = L.om[(size_t)q * L.nb + s];
  const int nf = L.cum[b + 1] - L.cum[b];
  for (int r = 0; r < nf; ++r)
    deg_group(L.mode, L.thres, L.nb, L.g2 + (int64_t)j * L.per + (int64_t)(L.cum[b] + r) * L.nb, 1, e);
}

// pass 2: initial bands, per (initial k row, final state); the states of one
// k row are consecutive, in band order
__global__ void k_deg_initial(DegList L, int nin) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)L.nA * nin) return;
  const int a = (int)(t / nin), f = (int)(t % nin);
  const int j0 = L.first_state[a], c = L.first_state[a + 1] - j0;
  if (c <= 0) return;
  const int p = L.arow[a];
  double e[DEG_MAXG];
  for (int i = 0; i < c; ++i) e[i] = L.ens[(size_t)p * L.nw + L.st_code[j0 + i] % L.nw];
  for (int s = 0; s < L.nb; ++s)
    deg_group(L.mode, L.thres, c, L.g2 + (int64_t)j0 * L.per + (int64_t)f * L.nb + s, L.per, e);
}

// pass 3: final bands, per (state, k' row)
__global__ void k_deg_final(DegList L) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)L.nst * L.nwv) return;
  const int j = (int)(t / L.nwv), b = (int)(t % L.nwv);
  int band[DEG_MAXG];
  double e[DEG_MAXG];
  const int c = window_bands(L.ens, L.widx[b], L.nw, L.enref, L.fsthick, band, e);
  for (int s = 0; s < L.nb; ++s)
    deg_group(L.mode, L.thres, c, L.g2 + (int64_t)j * L.per + (int64_t)L.cum[b] * L.nb + s, L.nb, e);
}

int launch_degenerate_average(double *g2, int64_t per, int nin, const int *st_code, const int *arow, const int *widx,
                              const int *cum, const int *first_state, const double *ens, const double *om, int nst,
                              int nA, int nwv, int nw, int nb, const int mesh[3], double enref, double fsthick,
                              double thres, int mode, cudaStream_t st) {
  if (nw > DEG_MAXG || nb > DEG_MAXG) return 1;
  DegList L{g2, st_code, arow, widx, cum, first_state, ens, om, nst, nA, nwv, nw, nb, {mesh[0], mesh[1], mesh[2]},
            per, enref, fsthick, thres, mode};
  const int64_t n1 = (int64_t)nst * nwv, n2 = (int64_t)nA * nin;
  if (n1 > 0) k_deg_branches<<<(unsigned)((n1 + 127) / 128), 128, 0, st>>>(L);
  if (n2 > 0) k_deg_initial<<<(unsigned)((n2 + 127) / 128), 128, 0, st>>>(L, nin);
  if (n1 > 0) k_deg_final<<<(unsigned)((n1 + 127) / 128), 128, 0, st>>>(L);
  return 0;
}

}  // namespace ephg
