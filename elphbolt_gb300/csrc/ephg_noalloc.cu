// ephg_noalloc.cu - electron interpolation that allocates no device memory.
//
// Some callers cannot allocate device memory at the point where they need the
// electrons: a host code that hands the library buffers it already owns (for
// example arrays kept on the device by OpenACC or CUDA Fortran, or system
// memory the GPU reaches through the Grace C2C link), a process whose memory
// budget is fixed by another framework's pool, or a time-critical loop in which
// cudaMalloc's implicit synchronisation is not acceptable.  For them
// ephg_el_wann_noalloc runs the same kernels as ephg_el_wann on caller-owned
// inputs and outputs, with its scratch (the phase matrix, the batch of H(k)
// matrices and the eigensolver output) in one fixed file-scope device array.
//
// The array is part of the library image: every GPU that loads the library
// holds its EPHG_NOALLOC_SCRATCH_BYTES until the process exits.  Host code may
// not use the array's name as a device address (in host code it names a host
// stand-in); its device address comes from cudaGetSymbolAddress with the
// handle's device current.  The first call on a device looks it up (set-up);
// every later call made while the handle's stream is not capturing looks it up
// again, so that a primary context re-created after cudaDeviceReset (by this
// code or another library in the process) never sees a stale address.
#include <mutex>

#include "ephg_handle.cuh"

namespace {

constexpr size_t SCRATCH_BYTES = (size_t)EPHG_NOALLOC_SCRATCH_BYTES;
__device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
void *g_scratch_addr[MAX_DEVICES];   // device address of the array, per device
std::mutex g_scratch_mu;

// The array's device address on device `dev` (current): looked up on the
// first call and again on every call with `refresh` set (the stream is not
// capturing), else the address of the last lookup.
int scratch_address(int dev, bool refresh, unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (dev < 0 || dev >= MAX_DEVICES) return ephg::api_fail(EPHG_ERR_CUDA, "el_wann_noalloc: device %d out of range", dev);
  if (!g_scratch_addr[dev] || refresh) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return ephg::api_fail(EPHG_ERR_CUDA, "el_wann_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = (unsigned char *)g_scratch_addr[dev];
  return EPHG_OK;
}

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Bytes of scratch that nk k-points need: phase matrix (nk, nwsk), H(k)
// batch (nk, nw, nw), eigenvalues (nk, nw), eigenvectors (nk, nw, nw).
size_t scratch_bytes(int64_t nk, int nw, int nwsk) {
  const size_t nn = (size_t)nw * nw;
  return align256((size_t)nk * nwsk * sizeof(double2)) + align256((size_t)nk * nn * sizeof(double2)) +
         align256((size_t)nk * nw * sizeof(double)) + align256((size_t)nk * nn * sizeof(double2));
}

}  // namespace

extern "C" int ephg_el_wann_noalloc(ephg_handle *h, int64_t nk, const double *kvecs, double *energies,
                                    double *evecs) {
  using namespace ephg;
  if (!h || nk < 0 || (nk > 0 && (!kvecs || !energies))) return api_fail(EPHG_ERR_ARG, "el_wann_noalloc: bad arguments");
  if (nk == 0) return EPHG_OK;
  const int nw = h->nw, nwsk = h->nwsk;
  const size_t need = scratch_bytes(nk, nw, nwsk);
  if (need > SCRATCH_BYTES) {
    int64_t nmax = 0;
    while (scratch_bytes(nmax + 1, nw, nwsk) <= SCRATCH_BYTES) ++nmax;
    return api_fail(EPHG_ERR_ARG,
                    "el_wann_noalloc: %lld k-points need %zu bytes of scratch, more than the fixed %zu; "
                    "call with at most %lld k-points (nw = %d, nwsk = %d)",
                    (long long)nk, need, SCRATCH_BYTES, (long long)nmax, nw, nwsk);
  }
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess || cur != h->device)
    return api_fail(EPHG_ERR_ARG, "el_wann_noalloc: the handle's device (%d) must be current (is %d)", h->device, cur);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->st, &cap) != cudaSuccess)
    return api_fail(EPHG_ERR_CUDA, "el_wann_noalloc: cudaStreamIsCapturing failed");
  unsigned char *base = nullptr;
  int rc = scratch_address(h->device, cap == cudaStreamCaptureStatusNone, &base);
  if (rc) return rc;
  // Every scratch region is written in full before it is read, so nothing has
  // to be cleared between calls.
  const size_t nn = (size_t)nw * nw;
  double2 *P = (double2 *)base;
  double2 *C = (double2 *)(base + align256((size_t)nk * nwsk * sizeof(double2)));
  double *w = (double *)((unsigned char *)C + align256((size_t)nk * nn * sizeof(double2)));
  double2 *V = (double2 *)((unsigned char *)w + align256((size_t)nk * nw * sizeof(double)));
  cudaStream_t st = h->st;
  launch_phase_frac((int)nk, kvecs, nwsk, h->Rk, h->degk, P, nwsk, st);
  launch_zgemm((int)nk, (int)nn, nwsk, P, nwsk, h->Hext, 4 * (int64_t)nn, C, nn, st);
  launch_heig((int)nk, nw, C, nn, w, V, h->err, st);
  launch_el_post((int)nk, nw, w, V, nullptr, 0, 0, nullptr, energies, nullptr, (double2 *)evecs, nullptr, st);
  h->launches += 4;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return api_fail(EPHG_ERR_CUDA, "el_wann_noalloc launch: %s", cudaGetErrorString(e));
  return api_check_err(h);   // synchronises the handle's stream
}
