// ephg_sym.cu - crystal symmetry and the irreducible wedge of a mesh.
//
//  - crystal_symmetry: the space-group operations (W, t) of a crystal, x' = W x + t
//    in crystal coordinates, what spg_get_dataset gives calculate_symmetries
//    (symmetry.f90:66-110): the lattice point group by its metric, then for
//    each lattice operation the translations that map the basis onto itself
//    atom type by atom type, both within symprec (Cartesian length).
//  - mesh_qrotations: calculate_symmetries' post-processing for a mesh
//    (symmetry.f90:134-212): reciprocal-space rotations M W M^-1 (M = A^T A),
//    doubled by time reversal, without the rotations that do not map the mesh
//    onto itself or that repeat an earlier one.  Returned as the integer
//    matrices K_ij = mesh_i Q_ij / mesh_j acting on mesh coordinates.
//  - k_sym_rep: the orbit representative of every mesh point, the smallest
//    muxed index of its orbit.  find_irred_wedge (symmetry.f90:303-452) walks
//    the (window) points in index order and opens a new irreducible point at
//    the first point of each orbit, so its irreducible points are exactly the
//    points that are their own representative.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ephg_common.cuh"
#include "ephg_sym.cuh"

namespace ephg {

static void matmul3(const double *a, const double *b, double *c) {   // column-major 3x3
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) c[i + 3 * j] = a[i] * b[3 * j] + a[i + 3] * b[3 * j + 1] + a[i + 6] * b[3 * j + 2];
}

static bool inv3(const double *a, double *b) {
  const double det = a[0] * (a[4] * a[8] - a[7] * a[5]) - a[3] * (a[1] * a[8] - a[7] * a[2]) +
                     a[6] * (a[1] * a[5] - a[4] * a[2]);
  if (det == 0.0) return false;
  b[0] = (a[4] * a[8] - a[7] * a[5]) / det;
  b[3] = -(a[3] * a[8] - a[6] * a[5]) / det;
  b[6] = (a[3] * a[7] - a[6] * a[4]) / det;
  b[1] = -(a[1] * a[8] - a[7] * a[2]) / det;
  b[4] = (a[0] * a[8] - a[6] * a[2]) / det;
  b[7] = -(a[0] * a[7] - a[6] * a[1]) / det;
  b[2] = (a[1] * a[5] - a[4] * a[2]) / det;
  b[5] = -(a[0] * a[5] - a[3] * a[2]) / det;
  b[8] = (a[0] * a[4] - a[3] * a[1]) / det;
  return true;
}

int crystal_symmetry(const double A[9], int nat, const double *basis, const int64_t *types, double symprec,
                     std::vector<SymOp> &ops) {
  ops.clear();
  if (nat < 1 || !(symprec > 0)) return 1;
  double G[9];   // metric A^T A
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      G[i + 3 * j] = A[3 * i] * A[3 * j] + A[3 * i + 1] * A[3 * j + 1] + A[3 * i + 2] * A[3 * j + 2];
  double len[3];
  for (int i = 0; i < 3; ++i) len[i] = sqrt(G[4 * i]);
  // Cartesian distance of the nearest image of a crystal-coordinate difference
  auto cdist = [&](const double *d) {
    double best = INFINITY;
    for (int n0 = -1; n0 <= 1; ++n0)
      for (int n1 = -1; n1 <= 1; ++n1)
        for (int n2 = -1; n2 <= 1; ++n2) {
          const double e[3] = {d[0] - std::round(d[0]) + n0, d[1] - std::round(d[1]) + n1, d[2] - std::round(d[2]) + n2};
          double c2 = 0.0;
          for (int r = 0; r < 3; ++r) {
            const double x = A[r] * e[0] + A[r + 3] * e[1] + A[r + 6] * e[2];
            c2 += x * x;
          }
          best = std::min(best, c2);
        }
    return sqrt(best);
  };
  int W[9];
  for (int code = 0; code < 1953125; ++code) {   // entries in [-2, 2]
    int c = code;
    for (int k = 0; k < 9; ++k) {
      W[k] = c % 5 - 2;
      c /= 5;
    }
    const int det = W[0] * (W[4] * W[8] - W[7] * W[5]) - W[3] * (W[1] * W[8] - W[7] * W[2]) +
                    W[6] * (W[1] * W[5] - W[4] * W[2]);
    if (det != 1 && det != -1) continue;
    // lattice operation: W^T G W = G within the tolerance of lengths symprec
    bool lat = true;
    for (int i = 0; i < 3 && lat; ++i)
      for (int j = 0; j < 3 && lat; ++j) {
        double v = 0.0;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) v += W[a + 3 * i] * G[a + 3 * b] * W[b + 3 * j];
        lat = fabs(v - G[i + 3 * j]) <= 2.0 * symprec * (len[i] + len[j]);
      }
    if (!lat) continue;
    // translations mapping atom 0 onto an atom of its type, checked on all atoms
    double wb0[3];
    for (int r = 0; r < 3; ++r) wb0[r] = W[r] * basis[0] + W[r + 3] * basis[1] + W[r + 6] * basis[2];
    for (int a1 = 0; a1 < nat; ++a1) {
      if (types[a1] != types[0]) continue;
      double t[3];
      for (int r = 0; r < 3; ++r) {
        t[r] = basis[3 * a1 + r] - wb0[r];
        t[r] -= std::floor(t[r]);
        if (t[r] >= 1.0 - 1e-12) t[r] = 0.0;
      }
      bool ok = true;
      for (int a = 0; a < nat && ok; ++a) {
        double x[3];
        for (int r = 0; r < 3; ++r)
          x[r] = W[r] * basis[3 * a] + W[r + 3] * basis[3 * a + 1] + W[r + 6] * basis[3 * a + 2] + t[r];
        bool found = false;
        for (int b = 0; b < nat && !found; ++b) {
          if (types[b] != types[a]) continue;
          const double d[3] = {x[0] - basis[3 * b], x[1] - basis[3 * b + 1], x[2] - basis[3 * b + 2]};
          found = cdist(d) <= symprec;
        }
        ok = found;
      }
      if (!ok) continue;
      bool dup = false;   // the same (W, t) from another atom of the type
      for (const SymOp &o : ops) {
        if (!std::equal(o.W, o.W + 9, W)) continue;
        const double d[3] = {o.t[0] - t[0], o.t[1] - t[1], o.t[2] - t[2]};
        if (cdist(d) <= symprec) dup = true;
      }
      if (dup) continue;
      SymOp op;
      std::copy(W, W + 9, op.W);
      std::copy(t, t + 3, op.t);
      ops.push_back(op);
    }
  }
  // identity first, then a fixed order
  std::stable_sort(ops.begin(), ops.end(), [](const SymOp &a, const SymOp &b) {
    const int ia = a.W[0] == 1 && a.W[4] == 1 && a.W[8] == 1 && a.W[1] == 0 && a.W[2] == 0 && a.W[3] == 0 &&
                   a.W[5] == 0 && a.W[6] == 0 && a.W[7] == 0;
    const int ib = b.W[0] == 1 && b.W[4] == 1 && b.W[8] == 1 && b.W[1] == 0 && b.W[2] == 0 && b.W[3] == 0 &&
                   b.W[5] == 0 && b.W[6] == 0 && b.W[7] == 0;
    return ia > ib;
  });
  return ops.empty() ? 1 : 0;
}

int mesh_qrotations(const double A[9], int nsymm, const int64_t *rot, const int mesh[3], std::vector<int> &K,
                    const char **why) {
  K.clear();
  double G[9], Gi[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      G[i + 3 * j] = A[3 * i] * A[3 * j] + A[3 * i + 1] * A[3 * j + 1] + A[3 * i + 2] * A[3 * j + 2];
  if (!inv3(G, Gi)) {
    *why = "singular lattice";
    return 1;
  }
  // Q = M W M^-1 (symmetry.f90:146-153), then time reversal -Q (:157-159)
  std::vector<int> Q;   // integer reciprocal rotations, 9 per operation
  for (int s = 0; s < 2 * nsymm; ++s) {
    double Wd[9], T[9], Qd[9];
    for (int k = 0; k < 9; ++k) Wd[k] = (double)rot[9 * (s % nsymm) + k];
    matmul3(G, Wd, T);
    matmul3(T, Gi, Qd);
    int q[9];
    for (int k = 0; k < 9; ++k) {
      const double v = s < nsymm ? Qd[k] : -Qd[k];
      q[k] = (int)std::lround(v);
      if (fabs(v - q[k]) > 1e-6) {
        *why = "a rotation is not a symmetry of the lattice";
        return 1;
      }
    }
    Q.insert(Q.end(), q, q + 9);
  }
  // drop rotations that do not map the mesh onto itself (:162-169) and repeated
  // rotations (:174-183).  K_ij = mesh_i Q_ij / mesh_j must be an integer: the
  // image mesh * Q (v / mesh) of every mesh point is then a mesh point.
  std::vector<int> keep;
  for (int s = 0; s < 2 * nsymm; ++s) {
    bool ok = true;   // (a mesh dimension of 1 has only the coordinate 0: its column never acts)
    for (int i = 0; i < 3 && ok; ++i)
      for (int j = 0; j < 3 && ok; ++j) ok = mesh[j] == 1 || ((int64_t)mesh[i] * Q[9 * s + i + 3 * j]) % mesh[j] == 0;
    if (!ok) continue;
    bool dup = false;
    for (int r : keep) dup = dup || std::equal(Q.begin() + 9 * r, Q.begin() + 9 * r + 9, Q.begin() + 9 * s);
    if (dup) continue;
    keep.push_back(s);
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i)
        K.push_back(mesh[j] == 1 ? 0 : (int)((int64_t)mesh[i] * Q[9 * s + i + 3 * j] / mesh[j]));
  }
  return 0;
}

// rep[p] = the smallest muxed index of p's orbit under the K matrices
__global__ void k_sym_rep(int N, int m0, int m1, int m2, int nops, const int *K, int *rep) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  const int v0 = p % m0, v1 = (p / m0) % m1, v2 = p / (m0 * m1);
  int best = p;
  for (int s = 0; s < nops; ++s) {
    const int *k = K + 9 * s;   // column-major: image_i = sum_j K_ij v_j
    const int64_t a = (int64_t)k[0] * v0 + (int64_t)k[3] * v1 + (int64_t)k[6] * v2;
    const int64_t b = (int64_t)k[1] * v0 + (int64_t)k[4] * v1 + (int64_t)k[7] * v2;
    const int64_t c = (int64_t)k[2] * v0 + (int64_t)k[5] * v1 + (int64_t)k[8] * v2;
    const int img = (int)(floormod(a, m0) + m0 * (floormod(b, m1) + m1 * floormod(c, m2)));
    best = min(best, img);
  }
  rep[p] = best;
}

void launch_sym_rep(int N, const int mesh[3], int nops, const int *K, int *rep, cudaStream_t st) {
  if (N <= 0) return;
  k_sym_rep<<<(N + 255) / 256, 256, 0, st>>>(N, mesh[0], mesh[1], mesh[2], nops, K, rep);
}

// energies of every mesh point replaced by those of its representative
__global__ void k_map_ens(int N, int nw, const int *rep, const double *ens, double *ens_m) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)N * nw) return;
  const int p = (int)(i / nw), b = (int)(i % nw);
  ens_m[i] = ens[(size_t)rep[p] * nw + b];
}

void launch_map_ens(int N, int nw, const int *rep, const double *ens, double *ens_m, cudaStream_t st) {
  if (N <= 0) return;
  k_map_ens<<<(unsigned)(((int64_t)N * nw + 255) / 256), 256, 0, st>>>(N, nw, rep, ens, ens_m);
}

// A-row flags: window point i is irreducible when it is its own representative
__global__ void k_irred_flags(int nwv, const int *widx, const int *rep, int *flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nwv) flag[i] = rep[widx[i]] == widx[i];
}

void launch_irred_flags(int nwv, const int *widx, const int *rep, int *flag, cudaStream_t st) {
  if (nwv <= 0) return;
  k_irred_flags<<<(nwv + 255) / 256, 256, 0, st>>>(nwv, widx, rep, flag);
}

}  // namespace ephg
