// ephg_sym.cuh - crystal symmetry and the irreducible wedge (internal interface).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace ephg {

// One space-group operation x' = W x + t, crystal coordinates; W column-major.
struct SymOp {
  int W[9];
  double t[3];
};

// The space-group operations of a crystal (A: lattice vectors as columns;
// basis (3, nat) crystal coordinates; types per atom).  Returns 0, or 1 when
// the input is invalid.  The identity comes first.
int crystal_symmetry(const double A[9], int nat, const double *basis, const int64_t *types, double symprec,
                     std::vector<SymOp> &ops);

// The reciprocal-space rotations of a mesh from nsymm real-space rotations
// rot (3,3,nsymm) column-major: with time reversal, without the rotations
// incompatible with the mesh or repeated; as integer matrices K (9 per
// rotation, column-major) on mesh coordinates.  Returns 0, or 1 with *why.
int mesh_qrotations(const double A[9], int nsymm, const int64_t *rot, const int mesh[3], std::vector<int> &K,
                    const char **why);

void launch_sym_rep(int N, const int mesh[3], int nops, const int *K, int *rep, cudaStream_t st);
void launch_map_ens(int N, int nw, const int *rep, const double *ens, double *ens_m, cudaStream_t st);
void launch_irred_flags(int nwv, const int *widx, const int *rep, int *flag, cudaStream_t st);

}  // namespace ephg
