// ephg_common.cuh - shared definitions of the sm_103a e-ph vertex library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace ephg {

// ---- constants: src/params.f90:27-57 (same expressions, same doubles) ----
constexpr double qe = 1.602176634e-19;
constexpr double me = 9.1093837015e-31;
constexpr double amu = 1.66053906660e-27;
constexpr double hbar = 1.05457172647e-22;
constexpr double hbar_eVps = hbar / qe;
constexpr double kB = 1.380649e-23 / qe;
constexpr double Hartree2radTHz = 27.2116 * qe / hbar;
constexpr double Ryd2radTHz = 0.5 * Hartree2radTHz;
constexpr double Ryd2eV = 0.5 * 27.2116;
constexpr double Ryd2amu = 2.0 * me / amu;
constexpr double g2unitfactor = Ryd2eV * Ryd2eV * Ryd2eV * Ryd2amu;  // wannier.f90:923
// pi is formed at run time as 4*atan(1) exactly like params.f90; see pi_ref().

// device error word bits (set by kernels, read back by the host)
enum : int {
  DERR_EIG = 1,        // Jacobi did not converge
  DERR_NEG_PHONON = 2, // omega < -5 meV (wannier.f90:774-776)
  DERR_INDEX = 4,      // index check failed
  DERR_TIMEOUT = 8,    // bounded wait gave up
};

// ---- complex helpers (double2 / float2) ----
__host__ __device__ inline double2 cmk(double x, double y) { return make_double2(x, y); }
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ inline double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// acc += a * b
__host__ __device__ inline void cfma(double2 &acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}
// acc += conj(a) * b
__host__ __device__ inline void cfma_cj(double2 &acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, fma(a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(-a.y, b.x, acc.y));
}
__host__ __device__ inline void cfmaf(float2 &acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
  acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
}
__host__ __device__ inline void cfmaf_cj(float2 &acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, fmaf(a.y, b.y, acc.x));
  acc.y = fmaf(a.x, b.y, fmaf(-a.y, b.x, acc.y));
}

__host__ __device__ inline int64_t floormod(int64_t a, int64_t n) {
  int64_t r = a % n;
  return r < 0 ? r + n : r;
}

// Rate-request parameters as seen by the kernels.
struct RateParams {
  int mesh[3];
  int N;                 // mesh points
  int nw, nb;
  double enref, fsthick, chempot, T;
  int delta_kind;
  double sigma;
  double inv_nk;
  double const_tp;       // 2*pi/hbar_eVps
};

}  // namespace ephg
