// ephg_polar.cu - the long-range dipole terms of polar crystals on the device:
// dyn_nonanalytic (wannier.f90:784-901) and long_range_prefac (:1013-1071).
//
// For a box vector G and g = G + q, with per-atom phases p_a = e^{i g.tau_a}
// and z_a(j) = sum_i g_i born(i, j, a), the G + q term of dyn_nonanalytic is
//   D(3a+i, 3b+j) += f(g) z_a(i) z_b(j) p_a conj(p_b),   f = e^{-qeq/4alph}/qeq,
// a rank-one update f w w^H with w(3a+i) = p_a z_a(i), and long_range_prefac is
//   sum_c L(c) u(c),  L(3a+i) = i fac sum_g f(g) conj(p_a) z_a(i).
// One block per q: the box vectors that pass the cut are compacted, in the
// reference's loop order, into shared memory 128 at a time, then each thread
// sums its matrix elements over them in that order (deterministic sums).  For
// q on the mesh (first cell) only the box vectors that can pass the cut for
// some q of the cell are tested; the others never contribute.
#include <mutex>

#include "ephg_common.cuh"
#include "ephg_kernels.cuh"

namespace ephg {

constexpr double BOHR2NM = 0.052917721092;   // params.f90:53
constexpr int PL_CHUNK = 128;   // box vectors tested per pass = threads per block

__device__ inline double geg(const double *eps, const double g[3]) {   // dot_product(g, matmul(epsilon, g))
  double acc = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) acc += g[i] * (eps[i] * g[0] + eps[i + 3] * g[1] + eps[i + 6] * g[2]);
  return acc;
}

// Shared-memory entry of a box vector that passed the cut: f, qeq, g[3], then
// p_a (re, im) per atom, then z (nb values).
__device__ inline int pl_entry_size(int nat) { return 5 + 2 * nat + 3 * nat; }

// mode 0: the G + q terms (Dq / dDq / Lq); mode 1: the q-independent term (Da).
// NU: matrix + vector elements per thread (nb^2 + nb <= NU * PL_CHUNK); VEL: dDq.
// G / M: the box vectors to test (all of them, or those that can pass the cut
// for some q of the first cell, for mesh q).
template <int NU, bool VEL>
__global__ void __launch_bounds__(PL_CHUNK) k_polar(PolarDev P, const double *G, int M, int nq, const int *qp, int m1,
                                                    int m2, int m3, const double *qv, int mode, double2 *Dq,
                                                    double2 *dDq, double2 *Lq, double2 *Da) {
  extern __shared__ double psm[];
  __shared__ int wcount[PL_CHUNK / 32];
  const int q = blockIdx.x;
  const int nat = P.nat, nb = P.nb, ne = nb * nb;
  const int esz = pl_entry_size(nat);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double qc[3] = {0.0, 0.0, 0.0};
  if (mode == 0) {
    double qf[3];
    if (qp) {
      const int p = qp[q];
      qf[0] = (double)(p % m1) / m1;
      qf[1] = (double)((p / m1) % m2) / m2;
      qf[2] = (double)(p / (m1 * m2)) / m3;
    } else {
      qf[0] = qv[q];
      qf[1] = qv[q + nq];
      qf[2] = qv[q + 2 * nq];
    }
    for (int d = 0; d < 3; ++d)   // matmul(reclattvecs, q) * bohr2nm
      qc[d] = (P.rec[d] * qf[0] + P.rec[d + 3] * qf[1] + P.rec[d + 6] * qf[2]) * BOHR2NM;
  }
  const bool want_d = mode == 1 || Dq, want_dd = VEL && mode == 0 && dDq, want_l = mode == 0 && Lq;
  double2 acc[NU], dacc[VEL ? NU : 1][3];
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    acc[u] = make_double2(0.0, 0.0);
    if (VEL)
#pragma unroll
      for (int x = 0; x < 3; ++x) dacc[u][x] = make_double2(0.0, 0.0);
  }
  for (int c0 = 0; c0 < M; c0 += PL_CHUNK) {
    // ---- test up to PL_CHUNK box vectors, compact the passing ones in order
    bool pass = false;
    double g[3], qeq = 0.0;
    const int gi = c0 + tid;
    if (gi < M) {
      for (int d = 0; d < 3; ++d) g[d] = G[3 * gi + d] + qc[d];
      qeq = geg(P.eps, g);
      pass = qeq > 0.0 && qeq / P.alph / 4.0 < P.gmax;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, pass);
    __syncthreads();   // the previous chunk's entries are no longer read
    if (lane == 0) wcount[warp] = __popc(bal);
    __syncthreads();
    int n = 0, off = 0;
    for (int w = 0; w < PL_CHUNK / 32; ++w) {
      if (w < warp) off += wcount[w];
      n += wcount[w];
    }
    off += __popc(bal & ((1u << lane) - 1u));
    if (pass) {
      double *e = psm + (size_t)off * esz;
      e[0] = exp(-qeq / P.alph / 4.0) / qeq;
      e[1] = qeq;
      e[2] = g[0];
      e[3] = g[1];
      e[4] = g[2];
      for (int a = 0; a < nat; ++a) {
        const double arg = g[0] * P.tau[3 * a] + g[1] * P.tau[3 * a + 1] + g[2] * P.tau[3 * a + 2];
        double s, c;
        sincos(arg, &s, &c);
        e[5 + 2 * a] = c;
        e[6 + 2 * a] = s;
        for (int j = 0; j < 3; ++j) {
          const double *Z = P.born + 3 * j + 9 * a;
          e[5 + 2 * nat + 3 * a + j] = g[0] * Z[0] + g[1] * Z[1] + g[2] * Z[2];
        }
      }
    }
    __syncthreads();
    // ---- each thread adds the chunk's terms into its elements, in order
#pragma unroll
    for (int u = 0; u < NU; ++u) {
      const int el = tid + u * PL_CHUNK;
      if (el < ne && want_d) {
        const int i = el % nb, j = el / nb, a = i / 3, b = j / 3;
        if (mode == 1 && a != b) continue;
        for (int k = 0; k < n; ++k) {
          const double *e = psm + (size_t)k * esz;
          const double f = e[0];
          const double *z = e + 5 + 2 * nat;
          const double2 pa = make_double2(e[5 + 2 * a], e[6 + 2 * a]);
          if (mode == 1) {
            // dyn_l(3a+i, 3a+j) -= f z_a(i) fnat_a(j), fnat_a(j) = sum_c z_c(j) e^{i g.(tau_a - tau_c)}
            double2 fn = make_double2(0.0, 0.0);
            for (int c = 0; c < nat; ++c) {
              const double2 pc = make_double2(e[5 + 2 * c], e[6 + 2 * c]);
              const double zc = z[3 * c + j % 3];
              fn.x += zc * (pa.x * pc.x + pa.y * pc.y);   // z * pa * conj(pc)
              fn.y += zc * (pa.y * pc.x - pa.x * pc.y);
            }
            const double t = f * z[i];
            acc[u].x -= t * fn.x;
            acc[u].y -= t * fn.y;
          } else {
            const double2 pb = make_double2(e[5 + 2 * b], e[6 + 2 * b]);
            const double2 fq = make_double2(f * (pa.x * pb.x + pa.y * pb.y), f * (pa.y * pb.x - pa.x * pb.y));
            const double zz = z[i] * z[j];
            acc[u].x += fq.x * zz;
            acc[u].y += fq.y * zz;
            if (VEL && want_dd) {
              const double qeqk = e[1];
              const double *gk = e + 2;
              const double dgc = 0.25 / P.alph + 1.0 / qeqk;
              const int ip = i % 3, jp = j % 3;
#pragma unroll
              for (int x = 0; x < 3; ++x) {
                const double dgeg = (P.eps[x] + P.eps[3 * x]) * gk[0] + (P.eps[x + 3] + P.eps[3 * x + 1]) * gk[1] +
                                    (P.eps[x + 6] + P.eps[3 * x + 2]) * gk[2];
                const double rr = P.tau[3 * a + x] - P.tau[3 * b + x];
                const double re = z[j] * P.born[x + 3 * ip + 9 * a] + z[i] * P.born[x + 3 * jp + 9 * b] -
                                  zz * dgc * dgeg;
                const double im = zz * rr;   // (re + i im) * facq
                dacc[u][x].x += fq.x * re - fq.y * im;
                dacc[u][x].y += fq.x * im + fq.y * re;
              }
            }
          }
        }
      } else if (el >= ne && el < ne + nb && want_l) {
        const int c = el - ne, a = c / 3;
        for (int k = 0; k < n; ++k) {   // f conj(p_a) z(c)
          const double *e = psm + (size_t)k * esz;
          const double t = e[0] * e[5 + 2 * nat + c];
          acc[u].x += t * e[5 + 2 * a];
          acc[u].y -= t * e[6 + 2 * a];
        }
      }
    }
  }
  // ---- outputs
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    const int el = tid + u * PL_CHUNK;
    if (el < ne) {
      const int i = el % nb, j = el / nb;
      if (mode == 1) {
        Da[el] = acc[u];
        continue;
      }
      const double mn = 1.0 / sqrt(P.masses[i / 3] * P.masses[j / 3]) * Ryd2amu;
      if (Dq) {
        double2 d = acc[u];
        if (P.Da) d = cadd(d, P.Da[el]);
        double2 &o = Dq[(size_t)q * ne + el];
        o = cadd(o, cscale(d, P.fac * mn));
      }
      if (VEL && want_dd)
        for (int x = 0; x < 3; ++x) {
          double2 &o = dDq[((size_t)q * 3 + x) * ne + el];
          o = cadd(o, cscale(dacc[u][x], P.fac * BOHR2NM * mn));
        }
    } else if (el < ne + nb && want_l) {
      Lq[(size_t)q * nb + (el - ne)] = make_double2(-P.fac * acc[u].y, P.fac * acc[u].x);   // i fac * acc
    }
  }
}

static size_t polar_smem(int nat) { return (size_t)PL_CHUNK * (5 + 5 * nat) * sizeof(double); }

template <int NU, bool VEL>
static void polar_run(const PolarDev &P, const double *G, int M, int nq, const int *qp, const int mesh[3],
                      const double *qv, int mode, double2 *Dq, double2 *dDq, double2 *Lq, double2 *Da,
                      cudaStream_t st) {
  // once per process: changing a kernel attribute can wait for the device's queued work
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_polar<NU, VEL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
  });
  k_polar<NU, VEL><<<nq, PL_CHUNK, polar_smem(P.nat), st>>>(P, G, M, nq, qp, mesh ? mesh[0] : 1, mesh ? mesh[1] : 1,
                                                            mesh ? mesh[2] : 1, qv, mode, Dq, dDq, Lq, Da);
}

template <bool VEL>
static void polar_dispatch(const PolarDev &P, const double *G, int M, int nq, const int *qp, const int mesh[3],
                           const double *qv, int mode, double2 *Dq, double2 *dDq, double2 *Lq, double2 *Da,
                           cudaStream_t st) {
  const int nel = P.nb * P.nb + P.nb;   // matrix + vector elements
  if (nel <= PL_CHUNK) polar_run<1, VEL>(P, G, M, nq, qp, mesh, qv, mode, Dq, dDq, Lq, Da, st);
  else if (nel <= 3 * PL_CHUNK) polar_run<3, VEL>(P, G, M, nq, qp, mesh, qv, mode, Dq, dDq, Lq, Da, st);
  else polar_run<9, VEL>(P, G, M, nq, qp, mesh, qv, mode, Dq, dDq, Lq, Da, st);
}

void launch_polar_q(const PolarDev &P, int nq, const int *qp, const int mesh[3], const double *qv, double2 *Dq,
                    double2 *dDq, double2 *Lq, cudaStream_t st) {
  if (nq <= 0 || (!Dq && !dDq && !Lq)) return;
  // mesh q lie in the first cell: the box vectors that can pass the cut there suffice
  const double *G = qp ? P.Gcell : P.G;
  const int M = qp ? P.Mcell : P.M;
  if (dDq) polar_dispatch<true>(P, G, M, nq, qp, mesh, qv, 0, Dq, dDq, Lq, nullptr, st);
  else polar_dispatch<false>(P, G, M, nq, qp, mesh, qv, 0, Dq, nullptr, Lq, nullptr, st);
}

void launch_polar_da(const PolarDev &P, double2 *Da, cudaStream_t st) {
  PolarDev Pa = P;
  Pa.Da = nullptr;
  polar_dispatch<false>(Pa, P.G, P.M, 1, nullptr, nullptr, nullptr, 1, nullptr, nullptr, nullptr, Da, st);
}

__global__ void k_glprefac(int nq, int nb, const double2 *Lq, const double2 *u, double2 *glp, float2 *glpf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;   // (q, s)
  if (i >= nq * nb) return;
  const int q = i / nb;
  double2 acc = make_double2(0.0, 0.0);
  for (int c = 0; c < nb; ++c) cfma(acc, Lq[(size_t)q * nb + c], u[(size_t)i * nb + c]);
  glp[i] = acc;
  if (glpf) glpf[i] = make_float2((float)acc.x, (float)acc.y);
}

void launch_glprefac(int nq, int nb, const double2 *Lq, const double2 *u, double2 *glp, float2 *glpf,
                     cudaStream_t st) {
  if (nq <= 0) return;
  k_glprefac<<<(nq * nb + 255) / 256, 256, 0, st>>>(nq, nb, Lq, u, glp, glpf);
}

}  // namespace ephg
