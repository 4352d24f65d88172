// ephg_api.cu - the C ABI (include/ephg.h): handle, uploads and the
// orchestration of the e-ph vertex path on one GPU and one CUDA stream.
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ephg.h"
#include "ephg_kernels.cuh"
#include "ephg_tc.cuh"
#include "ephg_ws.cuh"
#include "ephg_handle.cuh"
#include "ephg_sym.cuh"

using namespace ephg;

#define fail ephg::api_fail

static thread_local std::string g_err;

int ephg::api_fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(EPHG_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,                \
                  cudaGetErrorString(e_));                                                \
  } while (0)

#define CKL()                                                                             \
  do {                                                                                    \
    cudaError_t e_ = cudaGetLastError();                                                  \
    if (e_ != cudaSuccess)                                                                \
      return fail(EPHG_ERR_CUDA, "%s:%d launch: %s", __FILE__, __LINE__,                   \
                  cudaGetErrorString(e_));                                                \
  } while (0)

namespace {

int gcd_i(int a, int b) { return b == 0 ? a : gcd_i(b, a % b); }
int lcm3(const int m[3]) {
  int l = m[0];
  l = l / gcd_i(l, m[1]) * m[1];
  l = l / gcd_i(l, m[2]) * m[2];
  return l;
}

// ws_wrapping_vectors (wannier.f90:532-582), q independent: evaluated once per
// (R, atom pair) at create time instead of once per q.
std::vector<int> ws_wrap(const double lvec[9], const double vl[3], double eps) {
  int iv0[3];
  double wl[3];
  for (int i = 0; i < 3; ++i) {
    iv0[i] = (int)std::trunc(vl[i]);
    wl[i] = vl[i] - (double)iv0[i];
  }
  double d = 1.79769313486231570815e308;
  auto norm = [&](int i, int j, int k) {
    double v[3] = {wl[0] + i, wl[1] + j, wl[2] + k}, wc[3];
    for (int r = 0; r < 3; ++r) wc[r] = lvec[r] * v[0] + lvec[r + 3] * v[1] + lvec[r + 6] * v[2];
    return std::sqrt(wc[0] * wc[0] + wc[1] * wc[1] + wc[2] * wc[2]);
  };
  for (int k = -3; k <= 3; ++k)
    for (int j = -3; j <= 3; ++j)
      for (int i = -3; i <= 3; ++i) {
        double nr = norm(i, j, k);
        if (std::fabs(nr - d) < eps) {
        } else if (nr < d) d = nr;
      }
  std::vector<int> out;
  for (int k = -3; k <= 3; ++k)
    for (int j = -3; j <= 3; ++j)
      for (int i = -3; i <= 3; ++i)
        if (std::fabs(norm(i, j, k) - d) < eps) {
          out.push_back(i - iv0[0]);
          out.push_back(j - iv0[1]);
          out.push_back(k - iv0[2]);
        }
  return out;
}

}  // namespace


static int read_err(ephg_handle *h, int *word) {
  CK(cudaMemcpyAsync(word, h->err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMemsetAsync(h->err, 0, sizeof(int), h->st));
  return EPHG_OK;
}

int ephg::api_check_err(ephg_handle *h) {
  int w = 0;
  int rc = read_err(h, &w);
  if (rc) return rc;
  if (w & DERR_NEG_PHONON) return fail(EPHG_ERR_NEG_PHONON, "Large negative phonon energy found!");
  if (w & DERR_EIG) return fail(EPHG_ERR_EIG, "Jacobi eigensolver did not converge");
  if (w & DERR_INDEX) return fail(EPHG_ERR_INDEX, "device index check failed");
  if (w & DERR_TIMEOUT) return fail(EPHG_ERR_TIMEOUT, "bounded device wait gave up");
  return EPHG_OK;
}

// workspace failures carry their own message
#define WSFAIL(rc) fail((rc), "%s", h->ws.msg.c_str())

// Small host arrays (tables built on the host, caller arrays of a few MB) reach
// the device through one pinned staging buffer of the library instead of the
// driver's staging of pageable memory, whose occasional page pinning cost
// handle creation ~15 ms every few calls.  Arrays above kStageMax are copied
// directly (the caller's pinned arrays stay asynchronous).
constexpr size_t kStageMax = (size_t)64 << 20;
static int staged_copy(void *dst, const void *src, size_t bytes, cudaStream_t st) {
  static std::mutex mu;
  static void *stage = nullptr;
  static size_t cap = 0;
  std::lock_guard<std::mutex> lk(mu);
  if (cap < bytes) {
    if (stage) cudaFreeHost(stage);
    stage = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes, (size_t)8 << 20);
    if (cudaMallocHost(&stage, want) != cudaSuccess) {
      cudaGetLastError();
      stage = nullptr;
      CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));   // no pinned memory: the plain path
      return EPHG_OK;
    }
    cap = want;
  }
  memcpy(stage, src, bytes);
  CK(cudaMemcpyAsync(dst, stage, bytes, cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));   // the staging buffer is free again for the next copy
  return EPHG_OK;
}

template <typename T>
// n elements from the library pool on st, copied from src; the bytes are added to *acc
static int upload(T **dst, const T *src, size_t n, cudaStream_t st, int64_t *acc = nullptr) {
  const size_t b = std::max<size_t>(n, 1) * sizeof(T);
  CK(pool_alloc((void **)dst, b, st));
  if (acc) *acc += (int64_t)b;
  if (n && n * sizeof(T) <= kStageMax) return staged_copy(*dst, src, n * sizeof(T), st);
  if (n) CK(cudaMemcpyAsync(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice, st));
  return EPHG_OK;
}

extern "C" {

const char *ephg_last_error(void) { return g_err.c_str(); }

int ephg_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int ephg_trim_memory(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(EPHG_ERR_CUDA, "trim_memory: no device");
  cudaMemPool_t pool = lib_pool(dev);
  if (!pool) return fail(EPHG_ERR_CUDA, "trim_memory: no memory pool");
  CK(cudaDeviceSynchronize());   // frees still queued on streams reach the pool first
  CK(cudaMemPoolTrimTo(pool, 0));
  return EPHG_OK;
}

int ephg_destroy(ephg_handle *h) {
  if (!h) return EPHG_OK;
  void *ptrs[] = {h->Rk, h->Rq, h->Rg, h->degk, h->degq, h->degg, h->Hext, h->Hbox, h->Dbox, h->graw, h->G64,
                  h->masses, h->pair_off, h->ent_iuc, h->ent_woff, h->wrapR, h->ent_rden,
                  h->rcartq, h->D, h->err, h->kposk, h->kposq, h->polar_G, h->polar_Gcell,
                  h->polar_born, h->polar_tau, h->polar_Da};
  // stream-ordered frees back to the library pool, which keeps the memory
  // mapped for the next handle
  for (void *p : ptrs)
    if (p) cudaFreeAsync(p, h->st);
  h->ws.release();
  tc::free_split(h->split, h->st);
  cudaStreamSynchronize(h->st);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return EPHG_OK;
}

int ephg_create(const ephg_wannier_desc *d, ephg_handle **out) {
  if (!d || !out) return fail(EPHG_ERR_ARG, "null argument");
  *out = nullptr;
  if (ephg_device_count() <= 0) return fail(EPHG_ERR_CUDA, "no CUDA device visible");
  if (d->numwannbands < 1 || d->numwannbands > 32)
    return fail(EPHG_ERR_ARG, "numwannbands must be in [1, 32]");
  if (d->numbranches != 3 * d->numatoms || d->numbranches > 32)
    return fail(EPHG_ERR_ARG, "numbranches must be 3*numatoms <= 32");
  if (d->nwsg != d->nwsq)
    return fail(EPHG_ERR_ARG, "nwsg must equal nwsq (the vertex Fourier uses rcells_q, wannier.f90:947)");
  for (int64_t i = 0; i < 3 * d->nwsq; ++i)
    if (d->rcells_g[i] != d->rcells_q[i])
      return fail(EPHG_ERR_ARG, "rcells_g must equal rcells_q (wannier.f90:947-951,988-990)");
  for (int64_t i = 0; i < d->nwsq; ++i)
    if (d->gwsdeg[i] != d->phwsdeg[i]) return fail(EPHG_ERR_ARG, "gwsdeg must equal phwsdeg");
  for (int i = 0; i < 3; ++i)
    if (d->coarse_qmesh[i] <= 0) return fail(EPHG_ERR_ARG, "Bad input(s) in wannier.");
  ephg_handle *h = new ephg_handle();
  int rc = EPHG_OK;
  auto bail = [&](int r) {
    ephg_destroy(h);
    return r;
  };
  if (cudaGetDevice(&h->device) != cudaSuccess) return bail(fail(EPHG_ERR_CUDA, "cudaGetDevice"));
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(EPHG_ERR_CUDA, "cudaStreamCreate"));
  h->ws.st = h->st;
  h->nw = (int)d->numwannbands;
  h->nb = (int)d->numbranches;
  h->nwsk = (int)d->nwsk;
  h->nwsq = (int)d->nwsq;
  h->nwsg = (int)d->nwsg;
  h->nat = (int)d->numatoms;
  for (int i = 0; i < 3; ++i) h->cq[i] = (int)d->coarse_qmesh[i];
  for (int i = 0; i < 9; ++i) h->lattvecs[i] = d->lattvecs[i];
  h->masses_h.assign(d->masses, d->masses + h->nat);
  h->basis_h.assign(d->basis, d->basis + 3 * h->nat);
  const int nw = h->nw, nb = h->nb, nwsk = h->nwsk, nwsq = h->nwsq;
  h->Nn = (int64_t)nw * nw * nb * nwsq;
  // R lists as (n,3) int rows and degeneracies as doubles
  auto rows = [](const int64_t *r, int n) {
    std::vector<int> v(3 * (size_t)n);
    for (int i = 0; i < n; ++i)
      for (int c = 0; c < 3; ++c) v[3 * i + c] = (int)r[i + (int64_t)n * c];
    return v;
  };
  std::vector<int> rk = rows(d->rcells_k, nwsk), rq = rows(d->rcells_q, nwsq), rg = rows(d->rcells_g, nwsq);
  std::vector<double> dk(d->elwsdeg, d->elwsdeg + nwsk), dq(d->phwsdeg, d->phwsdeg + nwsq),
      dg(d->gwsdeg, d->gwsdeg + nwsq);
  if ((rc = upload(&h->Rk, rk.data(), rk.size(), h->st, &h->resident_bytes)) || (rc = upload(&h->Rq, rq.data(), rq.size(), h->st, &h->resident_bytes)) ||
      (rc = upload(&h->Rg, rg.data(), rg.size(), h->st, &h->resident_bytes)) || (rc = upload(&h->degk, dk.data(), dk.size(), h->st, &h->resident_bytes)) ||
      (rc = upload(&h->degq, dq.data(), dq.size(), h->st, &h->resident_bytes)) || (rc = upload(&h->degg, dg.data(), dg.size(), h->st, &h->resident_bytes)) ||
      (rc = upload(&h->masses, d->masses, (size_t)h->nat, h->st, &h->resident_bytes)))
    return bail(rc);
  // H(Re) with the velocity companions i*rcart*H (wannier.f90:466-478)
  {
    const size_t nn = (size_t)nw * nw;
    std::vector<double2> hx((size_t)nwsk * 4 * nn);
    for (int r = 0; r < nwsk; ++r) {
      double R[3] = {(double)rk[3 * r], (double)rk[3 * r + 1], (double)rk[3 * r + 2]}, rc3[3];
      for (int i = 0; i < 3; ++i)
        rc3[i] = h->lattvecs[i] * R[0] + h->lattvecs[i + 3] * R[1] + h->lattvecs[i + 6] * R[2];
      for (size_t e = 0; e < nn; ++e) {
        size_t ib = e % nw, jb = e / nw;
        const double *src = d->Hwann + 2 * (r + (size_t)nwsk * (ib + (size_t)nw * jb));
        double2 v = make_double2(src[0], src[1]);
        hx[(size_t)r * 4 * nn + e] = v;
        for (int p = 0; p < 3; ++p)
          hx[(size_t)r * 4 * nn + (1 + p) * nn + e] = make_double2(-rc3[p] * v.y, rc3[p] * v.x);
      }
    }
    if ((rc = upload(&h->Hext, hx.data(), hx.size(), h->st, &h->resident_bytes))) return bail(rc);
    // H(Re) / deg(Re) on the box of Re coordinates, for the mesh Fourier sums
    int hi[3];
    for (int c = 0; c < 3; ++c) {
      h->hlo[c] = hi[c] = nwsk > 0 ? rk[c] : 0;
      for (int r = 0; r < nwsk; ++r) {
        h->hlo[c] = std::min(h->hlo[c], rk[3 * r + c]);
        hi[c] = std::max(hi[c], rk[3 * r + c]);
      }
      h->hext[c] = hi[c] - h->hlo[c] + 1;
    }
    const size_t nbox = (size_t)h->hext[0] * h->hext[1] * h->hext[2];
    if (nbox > ((size_t)1 << 22)) return bail(fail(EPHG_ERR_ARG, "Re cells span too large a box"));
    std::vector<double2> hb(nbox * nn, make_double2(0.0, 0.0));
    for (int r = 0; r < nwsk; ++r) {
      const size_t cell = ((size_t)(rk[3 * r] - h->hlo[0]) * h->hext[1] + (rk[3 * r + 1] - h->hlo[1])) * h->hext[2] +
                          (rk[3 * r + 2] - h->hlo[2]);
      for (size_t e = 0; e < nn; ++e) {
        const double2 v = hx[(size_t)r * 4 * nn + e];
        hb[cell * nn + e] = make_double2(v.x / dk[r], v.y / dk[r]);
      }
    }
    if ((rc = upload(&h->Hbox, hb.data(), hb.size(), h->st, &h->resident_bytes))) return bail(rc);
  }
  // g(Re,Rp): raw epmatwp order and the stage-A layout
  {
    size_t n = (size_t)nw * nw * nwsk * nb * nwsq;
    if ((rc = upload(&h->graw, (const double2 *)d->gwann, n, h->st, &h->resident_bytes))) return bail(rc);
    if (pool_alloc((void **)&h->G64, n * sizeof(double2), h->st) != cudaSuccess)
      return bail(fail(EPHG_ERR_NOMEM, "device allocation of g(Re,Rp), %zu bytes", n * 16));
    h->resident_bytes += (int64_t)(n * sizeof(double2));
    launch_permute_gwann(nw, nb, nwsk, nwsq, h->graw, h->G64, h->st);
  }
  // phonon terms: for each atom pair and WS cell, the shortest wraps
  {
    std::vector<int> pair_off(h->nat * h->nat + 1, 0), ent_iuc, ent_woff(1, 0), wrapR;
    std::vector<double> ent_rden;
    for (int jat = 0; jat < h->nat; ++jat)
      for (int iat = 0; iat < h->nat; ++iat) {
        int pair = iat + h->nat * jat;
        pair_off[pair] = (int)ent_iuc.size();
        for (int iuc = 0; iuc < nwsq; ++iuc) {
          double dist[3];
          for (int c = 0; c < 3; ++c)
            dist[c] = ((double)rq[3 * iuc + c] - d->basis[c + 3 * iat] + d->basis[c + 3 * jat]) /
                      (double)h->cq[c];
          std::vector<int> w = ws_wrap(h->lattvecs, dist, 1.0e-6);
          int nwrap = (int)w.size() / 3;
          ent_iuc.push_back(iuc);
          ent_rden.push_back(1.0 / (double)(d->phwsdeg[iuc] * nwrap));
          for (int iw = 0; iw < nwrap; ++iw)
            for (int c = 0; c < 3; ++c) wrapR.push_back(rq[3 * iuc + c] + w[3 * iw + c] * h->cq[c]);
          ent_woff.push_back((int)wrapR.size() / 3);
        }
      }
    // pair_off must be monotone over the pair index order used by the kernel
    {
      std::vector<int> off(h->nat * h->nat + 1);
      int cur = 0;
      for (int p = 0; p < h->nat * h->nat; ++p) {
        off[p] = cur;
        cur += nwsq;
      }
      off[h->nat * h->nat] = cur;
      // entries were appended in jat-major order, identical to pair = iat + nat*jat
      pair_off = off;
    }
    std::vector<double> rcq((size_t)nwsq * 3);
    for (int r = 0; r < nwsq; ++r)
      for (int i = 0; i < 3; ++i)
        rcq[r + (size_t)nwsq * i] = h->lattvecs[i] * rq[3 * r] + h->lattvecs[i + 3] * rq[3 * r + 1] +
                                    h->lattvecs[i + 6] * rq[3 * r + 2];
    if ((rc = upload(&h->pair_off, pair_off.data(), pair_off.size(), h->st, &h->resident_bytes)) ||
        (rc = upload(&h->ent_iuc, ent_iuc.data(), ent_iuc.size(), h->st, &h->resident_bytes)) ||
        (rc = upload(&h->ent_woff, ent_woff.data(), ent_woff.size(), h->st, &h->resident_bytes)) ||
        (rc = upload(&h->wrapR, wrapR.data(), wrapR.size(), h->st, &h->resident_bytes)) ||
        (rc = upload(&h->ent_rden, ent_rden.data(), ent_rden.size(), h->st, &h->resident_bytes)) ||
        (rc = upload(&h->rcartq, rcq.data(), rcq.size(), h->st, &h->resident_bytes)) ||
        (rc = upload(&h->D, (const double2 *)d->Dphwann, (size_t)nwsq * nb * nb, h->st, &h->resident_bytes)))
      return bail(rc);
    // D(q) on a mesh as one Fourier sum per element over the wrapped vectors R':
    // X_ab(R') = massnorm_ab sum of rden D(iuc)_ab over the (pair(a, b), iuc)
    // entries whose wraps include R' (k_dbuild's sum, regrouped)
    {
      const int ne = nb * nb;
      int lo3[3] = {0, 0, 0}, hi3[3] = {0, 0, 0};
      const int nwr = (int)(wrapR.size() / 3);
      for (int c = 0; c < 3; ++c) {
        lo3[c] = hi3[c] = nwr > 0 ? wrapR[c] : 0;
        for (int i = 0; i < nwr; ++i) {
          lo3[c] = std::min(lo3[c], wrapR[3 * i + c]);
          hi3[c] = std::max(hi3[c], wrapR[3 * i + c]);
        }
        h->dlo[c] = lo3[c];
        h->dext[c] = hi3[c] - lo3[c] + 1;
      }
      const size_t nbox = (size_t)h->dext[0] * h->dext[1] * h->dext[2];
      if (nbox > ((size_t)1 << 22)) return bail(fail(EPHG_ERR_ARG, "phonon cells span too large a box"));
      std::vector<double2> xb(nbox * ne, make_double2(0.0, 0.0));
      const double2 *Dw = (const double2 *)d->Dphwann;
      for (int e = 0; e < ne; ++e) {
        const int a = e % nb, b = e / nb;
        const int pair = (a / 3) + h->nat * (b / 3);
        const double massnorm = 1.0 / std::sqrt(d->masses[a / 3] * d->masses[b / 3]) * Ryd2amu;
        for (int iuc = 0; iuc < nwsq; ++iuc) {
          const int en = pair * nwsq + iuc;   // entries (pair, cell) in cell order
          const double2 dv = Dw[iuc + (size_t)nwsq * (a + (size_t)nb * b)];
          const double f = ent_rden[en] * massnorm;
          for (int wv = ent_woff[en]; wv < ent_woff[en + 1]; ++wv) {
            const size_t cell =
                ((size_t)(wrapR[3 * wv] - lo3[0]) * h->dext[1] + (wrapR[3 * wv + 1] - lo3[1])) * h->dext[2] +
                (wrapR[3 * wv + 2] - lo3[2]);
            xb[cell * ne + e].x += f * dv.x;
            xb[cell * ne + e].y += f * dv.y;
          }
        }
      }
      if ((rc = upload(&h->Dbox, xb.data(), xb.size(), h->st, &h->resident_bytes))) return bail(rc);
    }
    h->terms.npair = h->nat * h->nat;
    h->terms.pair_off = h->pair_off;
    h->terms.ent_iuc = h->ent_iuc;
    h->terms.ent_woff = h->ent_woff;
    h->terms.wrapR = h->wrapR;
    h->terms.ent_rden = h->ent_rden;
    h->terms.D = h->D;
    h->terms.rcart = h->rcartq;
    h->terms.masses = h->masses;
    h->terms.nwsq = nwsq;
    h->terms.nb = nb;
    h->terms.nat = h->nat;
  }
  // contraction order of the split form: cells by decreasing |R| (ties by index),
  // so that the decaying Wannier-space terms are summed smallest first
  {
    auto order = [&](const std::vector<int> &r, int n) {
      std::vector<double> len(n);
      for (int i = 0; i < n; ++i) {
        double c[3];
        for (int d = 0; d < 3; ++d)
          c[d] = h->lattvecs[d] * r[3 * i] + h->lattvecs[d + 3] * r[3 * i + 1] + h->lattvecs[d + 6] * r[3 * i + 2];
        len[i] = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      }
      std::vector<int> idx(n), pos(n);
      for (int i = 0; i < n; ++i) idx[i] = i;
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return len[a] > len[b]; });
      for (int p = 0; p < n; ++p) pos[idx[p]] = p;
      return pos;
    };
    std::vector<int> pk = order(rk, nwsk), pq = order(rq, nwsq);
    if ((rc = upload(&h->kposk, pk.data(), pk.size(), h->st, &h->resident_bytes)) || (rc = upload(&h->kposq, pq.data(), pq.size(), h->st, &h->resident_bytes)))
      return bail(rc);
  }
  if (pool_alloc((void **)&h->err, sizeof(int), h->st) != cudaSuccess)
    return bail(fail(EPHG_ERR_CUDA, "device allocation of the error word"));
  if (cudaMemsetAsync(h->err, 0, sizeof(int), h->st) != cudaSuccess) return bail(fail(EPHG_ERR_CUDA, "memset"));
  if (cudaStreamSynchronize(h->st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return bail(fail(EPHG_ERR_CUDA, "create: %s", cudaGetErrorString(cudaGetLastError())));
  *out = h;
  return EPHG_OK;
}

// ------------------------------------------------------------- polar
// The crystal fields of a polar crystal (crys%polar, epsilon, born;
// crystal.f90:45-49) and what the long-range terms derive from them:
// reciprocal vectors and volume (crystal.f90:282-293), the Cartesian basis in
// bohr, the box of reciprocal-lattice vectors and the q-independent part of
// dyn_nonanalytic (wannier.f90:843-867), formed once.
int ephg_set_polar(ephg_handle *h, const double *epsilon, const double *born) {
  if (!h) return fail(EPHG_ERR_ARG, "set_polar: bad arguments");
  if (epsilon && !born) return fail(EPHG_ERR_ARG, "set_polar: born effective charges are required");
  for (void *p : {(void *)h->polar_G, (void *)h->polar_Gcell, (void *)h->polar_born, (void *)h->polar_tau,
                  (void *)h->polar_Da})
    if (p) cudaFreeAsync(p, h->st);
  CK(cudaStreamSynchronize(h->st));
  h->polar_G = h->polar_Gcell = h->polar_born = h->polar_tau = nullptr;
  h->polar_Da = nullptr;
  h->polar_on = false;
  if (!epsilon) return EPHG_OK;   // non-polar
  const double bohr2nm = 0.052917721092, pi = 4.0 * atan(1.0), twopi = 2.0 * pi;   // params.f90
  const int nat = h->nat, nb = h->nb;
  const double *a = h->lattvecs;
  ephg::PolarDev P;
  for (int i = 0; i < 3; ++i) {
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    P.rec[0 + 3 * i] = a[1 + 3 * j] * a[2 + 3 * k] - a[2 + 3 * j] * a[1 + 3 * k];
    P.rec[1 + 3 * i] = a[2 + 3 * j] * a[0 + 3 * k] - a[0 + 3 * j] * a[2 + 3 * k];
    P.rec[2 + 3 * i] = a[0 + 3 * j] * a[1 + 3 * k] - a[1 + 3 * j] * a[0 + 3 * k];
  }
  const double vol = fabs(a[0] * P.rec[0] + a[1] * P.rec[1] + a[2] * P.rec[2]);
  for (double &r : P.rec) r *= twopi / vol;
  const double a1 = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double tpiba = twopi / a1 * bohr2nm;
  P.alph = tpiba * tpiba;
  P.gmax = 14.0;
  P.fac = 8.0 * pi / (vol / (bohr2nm * bohr2nm * bohr2nm));
  for (int i = 0; i < 9; ++i) P.eps[i] = epsilon[i];
  std::vector<double> G, tau(3 * (size_t)nat);
  for (int m1 = -h->cq[0]; m1 <= h->cq[0]; ++m1)
    for (int m2 = -h->cq[1]; m2 <= h->cq[1]; ++m2)
      for (int m3 = -h->cq[2]; m3 <= h->cq[2]; ++m3)
        for (int d = 0; d < 3; ++d) G.push_back((m1 * P.rec[d] + m2 * P.rec[d + 3] + m3 * P.rec[d + 6]) * bohr2nm);
  for (int at = 0; at < nat; ++at)
    for (int d = 0; d < 3; ++d) {
      const double *b = &h->basis_h[3 * (size_t)at];
      tau[3 * at + d] = (a[d] * b[0] + a[d + 3] * b[1] + a[d + 6] * b[2]) / bohr2nm;
    }
  // The box vectors that can pass the cut qeq < 4 alph gmax for some q of the
  // first cell (the mesh q): qeq >= lmin |G + q|^2 >= lmin (|G| - qmax)^2, with
  // lmin a Gershgorin lower bound of the symmetric part of epsilon and qmax the
  // longest corner of the cell.  Without a positive bound nothing is dropped.
  double lmin = INFINITY, qmax = 0.0;
  for (int i = 0; i < 3; ++i) {
    double off = 0.0;
    for (int j = 0; j < 3; ++j)
      if (j != i) off += fabs(0.5 * (epsilon[i + 3 * j] + epsilon[j + 3 * i]));
    lmin = std::min(lmin, epsilon[i + 3 * i] - off);
  }
  for (int c = 0; c < 8; ++c) {
    double v[3];
    for (int d = 0; d < 3; ++d)
      v[d] = ((c & 1) * P.rec[d] + ((c >> 1) & 1) * P.rec[d + 3] + ((c >> 2) & 1) * P.rec[d + 6]) * bohr2nm;
    qmax = std::max(qmax, sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
  }
  std::vector<double> Gc;
  const double rcut = lmin > 0.0 ? sqrt(4.0 * P.alph * P.gmax / lmin) * (1.0 + 1e-9) + qmax : INFINITY;
  for (size_t i = 0; i < G.size(); i += 3) {
    const double n = sqrt(G[i] * G[i] + G[i + 1] * G[i + 1] + G[i + 2] * G[i + 2]);
    if (n < rcut) Gc.insert(Gc.end(), {G[i], G[i + 1], G[i + 2]});
  }
  P.nat = nat;
  P.nb = nb;
  P.M = (int)(G.size() / 3);
  P.Mcell = (int)(Gc.size() / 3);
  P.masses = h->masses;
  int rc;
  if ((rc = upload(&h->polar_G, G.data(), G.size(), h->st)) ||
      (rc = upload(&h->polar_Gcell, Gc.data(), Gc.size(), h->st)) ||
      (rc = upload(&h->polar_born, born, 9 * (size_t)nat, h->st)) ||
      (rc = upload(&h->polar_tau, tau.data(), tau.size(), h->st)))
    return rc;
  CK(pool_alloc((void **)&h->polar_Da, (size_t)nb * nb * sizeof(double2), h->st));
  P.G = h->polar_G;
  P.Gcell = h->polar_Gcell;
  P.born = h->polar_born;
  P.tau = h->polar_tau;
  launch_polar_da(P, h->polar_Da, h->st);
  CKL();
  CK(cudaStreamSynchronize(h->st));
  P.Da = h->polar_Da;
  h->polar = P;
  h->polar_on = true;
  return EPHG_OK;
}

// ------------------------------------------------------------- symmetry
int ephg_crystal_symmetry(const double *lattvecs, int64_t natoms, const double *basis, const int64_t *atomtypes,
                          double symprec, int64_t maxops, int64_t *nops, int64_t *rotations, double *translations) {
  if (!lattvecs || natoms < 1 || !basis || !atomtypes || !nops || (maxops > 0 && !rotations))
    return fail(EPHG_ERR_ARG, "crystal_symmetry: bad arguments");
  std::vector<ephg::SymOp> ops;
  if (ephg::crystal_symmetry(lattvecs, (int)natoms, basis, atomtypes, symprec, ops))
    return fail(EPHG_ERR_ARG, "crystal_symmetry: no symmetry found (symprec must be > 0)");
  *nops = (int64_t)ops.size();
  if ((int64_t)ops.size() > maxops)
    return fail(EPHG_ERR_ARG, "crystal_symmetry: %lld operations, room for %lld", (long long)ops.size(),
                (long long)maxops);
  for (size_t o = 0; o < ops.size(); ++o) {
    for (int k = 0; k < 9; ++k) rotations[9 * o + k] = ops[o].W[k];
    if (translations)
      for (int d = 0; d < 3; ++d) translations[3 * o + d] = ops[o].t[d];
  }
  return EPHG_OK;
}

int ephg_set_symmetry(ephg_handle *h, int64_t nsymm, const int64_t *rotations) {
  if (!h || nsymm < 0 || (nsymm > 0 && !rotations) || nsymm > 192)
    return fail(EPHG_ERR_ARG, "set_symmetry: bad arguments");
  h->sym_rot.assign(rotations, rotations + 9 * nsymm);
  if (nsymm > 0) {   // every rotation must be a lattice symmetry (an integer reciprocal rotation)
    const int m1[3] = {1, 1, 1};
    std::vector<int> K;
    const char *why = "";
    if (ephg::mesh_qrotations(h->lattvecs, (int)nsymm, rotations, m1, K, &why)) {
      h->sym_rot.clear();
      return fail(EPHG_ERR_ARG, "set_symmetry: %s", why);
    }
  }
  return EPHG_OK;
}

int ephg_irred_wedge(const double *lattvecs, int64_t nsymm, const int64_t *rotations, const int64_t mesh[3],
                     int64_t nk, const int64_t *indexlist, int64_t *nirred, int64_t *indexlist_irred, int64_t *nequiv,
                     int64_t *fbz2ibz) {
  if (!lattvecs || nsymm < 0 || (nsymm > 0 && !rotations) || !mesh || !nirred || !indexlist_irred)
    return fail(EPHG_ERR_ARG, "irred_wedge: bad arguments");
  for (int i = 0; i < 3; ++i)
    if (mesh[i] <= 0 || mesh[i] > 1024) return fail(EPHG_ERR_ARG, "irred_wedge: bad mesh");
  const int m[3] = {(int)mesh[0], (int)mesh[1], (int)mesh[2]};
  const int64_t N = mesh[0] * mesh[1] * mesh[2];
  const int64_t n = indexlist ? nk : N;
  std::vector<int> K;
  const char *why = "";
  if (nsymm > 0 && ephg::mesh_qrotations(lattvecs, (int)nsymm, rotations, m, K, &why))
    return fail(EPHG_ERR_ARG, "irred_wedge: %s", why);
  const int nops = (int)(K.size() / 9);
  // points of the list by muxed index (0-based); -1 outside it
  std::vector<int64_t> pos(N, -1);
  for (int64_t i = 0; i < n; ++i) {
    const int64_t p = indexlist ? indexlist[i] - 1 : i;
    if (p < 0 || p >= N) return fail(EPHG_ERR_ARG, "irred_wedge: index out of range");
    if (i > 0 && indexlist && indexlist[i] <= indexlist[i - 1])
      return fail(EPHG_ERR_ARG, "irred_wedge: indexlist must be sorted ascending");
    pos[p] = i;
  }
  // find_irred_wedge (symmetry.f90:303-452): the first point of each orbit, in list order
  std::vector<int64_t> rep(n);
  int64_t nir = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t p = indexlist ? indexlist[i] - 1 : i;
    const int v0 = (int)(p % m[0]), v1 = (int)((p / m[0]) % m[1]), v2 = (int)(p / ((int64_t)m[0] * m[1]));
    int64_t best = p;
    for (int s = 0; s < nops; ++s) {
      const int *k = &K[9 * s];
      const int64_t a = floormod((int64_t)k[0] * v0 + (int64_t)k[3] * v1 + (int64_t)k[6] * v2, m[0]);
      const int64_t b = floormod((int64_t)k[1] * v0 + (int64_t)k[4] * v1 + (int64_t)k[7] * v2, m[1]);
      const int64_t c = floormod((int64_t)k[2] * v0 + (int64_t)k[5] * v1 + (int64_t)k[8] * v2, m[2]);
      const int64_t img = a + m[0] * (b + m[1] * c);
      if (pos[img] < 0) return fail(EPHG_ERR_ARG, "Severe error: Could not find irreducible wedge.");
      best = std::min(best, img);
    }
    rep[i] = pos[best];
  }
  std::vector<int64_t> ibz_of(n, -1);
  for (int64_t i = 0; i < n; ++i)
    if (rep[i] == i) {
      ibz_of[i] = nir;
      indexlist_irred[nir] = indexlist ? indexlist[i] : i + 1;
      if (nequiv) nequiv[nir] = 0;
      ++nir;
    }
  for (int64_t i = 0; i < n; ++i) {
    const int64_t r = ibz_of[rep[i]];
    if (nequiv) nequiv[r]++;
    if (fbz2ibz) fbz2ibz[i] = r + 1;
  }
  *nirred = nir;
  return EPHG_OK;
}

// ------------------------------------------------------------- el_wann
int ephg_el_wann(ephg_handle *h, int64_t nk, const double *kvecs, double *energies,
                 double *velocities, double *evecs, const double *scissor) {
  if (!h || nk < 0 || (nk > 0 && (!kvecs || !energies)))
    return fail(EPHG_ERR_ARG, "el_wann: bad arguments");
  if (velocities && !evecs)
    return fail(EPHG_ERR_ARG, "In el_wann, velocity is present but not eigenvecs.");
  if (nk == 0) return EPHG_OK;
  const int nw = h->nw, nwsk = h->nwsk;
  const size_t nn = (size_t)nw * nw;
  const int with_vel = velocities != nullptr;
  const int ncol = with_vel ? 4 * (int)nn : (int)nn;
  double *kv, *w, *ens, *vel, *sc = nullptr;
  double2 *P, *C, *V, *ev;
  int rc;
  if ((rc = wsget(h->ws, "el_kv", (size_t)nk * 3, &kv)) || (rc = wsget(h->ws, "el_P", (size_t)nk * nwsk, &P)) ||
      (rc = wsget(h->ws, "el_C", (size_t)nk * ncol, &C)) || (rc = wsget(h->ws, "el_w", (size_t)nk * nw, &w)) ||
      (rc = wsget(h->ws, "el_V", (size_t)nk * nn, &V)) || (rc = wsget(h->ws, "el_e", (size_t)nk * nw, &ens)) ||
      (rc = wsget(h->ws, "el_vel", with_vel ? (size_t)nk * nw * 3 : 1, &vel)) ||
      (rc = wsget(h->ws, "el_ev", evecs ? (size_t)nk * nn : 1, &ev)))
    return WSFAIL(rc);
  if (scissor) {
    if ((rc = wsget(h->ws, "el_sc", (size_t)nw, &sc))) return WSFAIL(rc);
    CK(cudaMemcpyAsync(sc, scissor, nw * sizeof(double), cudaMemcpyHostToDevice, h->st));
  }
  CK(cudaMemcpyAsync(kv, kvecs, (size_t)nk * 3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
  launch_phase_frac((int)nk, kv, nwsk, h->Rk, h->degk, P, nwsk, h->st);
  launch_zgemm((int)nk, ncol, nwsk, P, nwsk, h->Hext, 4 * (int64_t)nn, C, ncol, h->st);
  launch_heig((int)nk, nw, C, ncol, w, V, h->err, h->st);
  launch_el_post((int)nk, nw, w, V, C, ncol, with_vel, sc, ens, with_vel ? vel : nullptr,
                 evecs ? ev : nullptr, nullptr, h->st);
  h->launches += 4;
  CKL();
  CK(cudaMemcpyAsync(energies, ens, (size_t)nk * nw * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (evecs) CK(cudaMemcpyAsync(evecs, ev, (size_t)nk * nn * sizeof(double2), cudaMemcpyDeviceToHost, h->st));
  if (with_vel) CK(cudaMemcpyAsync(velocities, vel, (size_t)nk * nw * 3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  return ephg::api_check_err(h);
}

// ------------------------------------------------------------- ph_wann
int ephg_ph_wann(ephg_handle *h, int64_t nq, const double *qvecs, double *energies,
                 double *evecs, double *velocities) {
  if (!h || nq < 0 || (nq > 0 && (!qvecs || !energies)))
    return fail(EPHG_ERR_ARG, "ph_wann: bad arguments");
  if (velocities && !evecs)
    return fail(EPHG_ERR_ARG, "In ph_wann, velocity is present but not eigenvecs.");
  if (nq == 0) return EPHG_OK;
  const int nb = h->nb;
  const size_t nn = (size_t)nb * nb;
  const int with_vel = velocities != nullptr;
  double *qv, *w, *ens, *vel;
  double2 *Dq, *dDq, *V, *ev;
  int rc;
  if ((rc = wsget(h->ws, "ph_qv", (size_t)nq * 3, &qv)) || (rc = wsget(h->ws, "ph_D", (size_t)nq * nn, &Dq)) ||
      (rc = wsget(h->ws, "ph_dD", with_vel ? (size_t)nq * 3 * nn : 1, &dDq)) ||
      (rc = wsget(h->ws, "ph_w", (size_t)nq * nb, &w)) || (rc = wsget(h->ws, "ph_V", (size_t)nq * nn, &V)) ||
      (rc = wsget(h->ws, "ph_e", (size_t)nq * nb, &ens)) ||
      (rc = wsget(h->ws, "ph_vel", with_vel ? (size_t)nq * nb * 3 : 1, &vel)) ||
      (rc = wsget(h->ws, "ph_ev", evecs ? (size_t)nq * nn : 1, &ev)))
    return WSFAIL(rc);
  CK(cudaMemcpyAsync(qv, qvecs, (size_t)nq * 3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
  launch_dbuild((int)nq, nullptr, nullptr, 1, nullptr, qv, h->terms, with_vel, Dq, dDq, h->st);
  if (h->polar_on)   // non-analytic correction (wannier.f90:684-705)
    launch_polar_q(h->polar, (int)nq, nullptr, nullptr, qv, Dq, with_vel ? dDq : nullptr, nullptr, h->st);
  launch_heig((int)nq, nb, Dq, nn, w, V, h->err, h->st);
  launch_ph_post((int)nq, nb, nullptr, qv, w, V, dDq, with_vel, h->masses, ens,
                 evecs ? ev : nullptr, with_vel ? vel : nullptr, nullptr, nullptr, nullptr, h->err,
                 h->st);
  h->launches += 3;
  CKL();
  CK(cudaMemcpyAsync(energies, ens, (size_t)nq * nb * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (evecs) CK(cudaMemcpyAsync(evecs, ev, (size_t)nq * nn * sizeof(double2), cudaMemcpyDeviceToHost, h->st));
  if (with_vel) CK(cudaMemcpyAsync(velocities, vel, (size_t)nq * nb * 3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  return ephg::api_check_err(h);
}

// ---------------------------------------------------------------- gkRp
int ephg_gkRp(ephg_handle *h, int64_t nk, const double *kvecs, double *gmixed) {
  if (!h || nk < 0 || (nk > 0 && (!kvecs || !gmixed))) return fail(EPHG_ERR_ARG, "gkRp: bad arguments");
  if (nk == 0) return EPHG_OK;
  const int nwsk = h->nwsk;
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nk, (int64_t)(1u << 30) / (h->Nn * 16)));
  double *kv;
  double2 *P, *C;
  int rc;
  if ((rc = wsget(h->ws, "gk_kv", (size_t)chunk * 3, &kv)) || (rc = wsget(h->ws, "gk_P", (size_t)chunk * nwsk, &P)) ||
      (rc = wsget(h->ws, "gk_C", (size_t)chunk * h->Nn, &C)))
    return WSFAIL(rc);
  std::vector<double> kc((size_t)chunk * 3);
  for (int64_t k0 = 0; k0 < nk; k0 += chunk) {
    int64_t n = std::min(chunk, nk - k0);
    for (int c = 0; c < 3; ++c)
      for (int64_t i = 0; i < n; ++i) kc[i + n * c] = kvecs[(k0 + i) + nk * c];
    CK(cudaMemcpyAsync(kv, kc.data(), (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    launch_phase_frac((int)n, kv, nwsk, h->Rk, h->degk, P, nwsk, h->st);
    launch_zgemm((int)n, (int)h->Nn, nwsk, P, nwsk, h->G64, h->Nn, C, h->Nn, h->st);
    h->launches += 2;
    CKL();
    CK(cudaMemcpyAsync(gmixed + 2 * k0 * h->Nn, C, (size_t)n * h->Nn * sizeof(double2),
                       cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  return ephg::api_check_err(h);
}

// ---------------------------------------------------------------- gReq
int ephg_gReq(ephg_handle *h, int64_t nq, const double *qvecs, double *gmixed) {
  if (!h || nq < 0 || (nq > 0 && (!qvecs || !gmixed))) return fail(EPHG_ERR_ARG, "gReq: bad arguments");
  if (nq == 0) return EPHG_OK;
  const int nw = h->nw, nb = h->nb, nwsk = h->nwsk, nwsg = h->nwsg;
  const int64_t per = (int64_t)nw * nw * nb * nwsk;
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nq, (int64_t)(1u << 30) / (per * 16)));
  double *qv;
  double2 *P, *C, *O;
  int rc;
  if ((rc = wsget(h->ws, "gq_qv", (size_t)chunk * 3, &qv)) || (rc = wsget(h->ws, "gq_P", (size_t)chunk * nwsg, &P)) ||
      (rc = wsget(h->ws, "gq_C", (size_t)chunk * per, &C)) || (rc = wsget(h->ws, "gq_O", (size_t)chunk * per, &O)))
    return WSFAIL(rc);
  std::vector<double> qc((size_t)chunk * 3);
  for (int64_t q0 = 0; q0 < nq; q0 += chunk) {
    int64_t n = std::min(chunk, nq - q0);
    for (int c = 0; c < 3; ++c)
      for (int64_t i = 0; i < n; ++i) qc[i + n * c] = qvecs[(q0 + i) + nq * c];
    CK(cudaMemcpyAsync(qv, qc.data(), (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    // sum_Rp e^{2 pi i q.Rp}/gwsdeg * g(i,j,Re,s,Rp): rows of the raw array are Rp
    launch_phase_frac((int)n, qv, nwsg, h->Rg, h->degg, P, nwsg, h->st);
    launch_zgemm((int)n, (int)per, nwsg, P, nwsg, h->graw, per, C, per, h->st);
    launch_permute_greq((int)n, nw, nb, nwsk, C, O, h->st);
    h->launches += 3;
    CKL();
    CK(cudaMemcpyAsync(gmixed + 2 * q0 * per, O, (size_t)n * per * sizeof(double2),
                       cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  return ephg::api_check_err(h);
}

// ------------------------------------------------------------------ g2
int ephg_g2(ephg_handle *h, int64_t wannspace, int64_t nv, const double *kvecs,
            const double *qvecs, const double *el_evec_k, const double *el_evec_kp,
            const double *ph_evec_q, const double *ph_en, int64_t ngm, const double *gmixed,
            const int64_t *gm_index, double *g2_out) {
  if (!h || nv < 0) return fail(EPHG_ERR_ARG, "g2: bad arguments");
  if (wannspace != EPHG_WANNSPACE_EL && wannspace != EPHG_WANNSPACE_PH)
    return fail(EPHG_ERR_ARG, "Invalid value of wannspace in call to g2_epw. Exiting.");
  if (nv == 0) return EPHG_OK;
  for (int64_t v = 0; v < nv; ++v)
    if (gm_index[v] < 1 || gm_index[v] > ngm) return fail(EPHG_ERR_ARG, "g2: gm_index out of range");
  const int nw = h->nw, nb = h->nb;
  const int nws = wannspace == EPHG_WANNSPACE_PH ? h->nwsg : h->nwsk;
  const int64_t gstride = (int64_t)nw * nw * nb * nws;
  double *qv, *en, *out;
  double2 *ek, *ekp, *eq, *gm;
  int64_t *gi;
  int rc;
  if ((rc = wsget(h->ws, "g2_qv", (size_t)nv * 3, &qv)) || (rc = wsget(h->ws, "g2_en", (size_t)nv, &en)) ||
      (rc = wsget(h->ws, "g2_out", (size_t)nv, &out)) || (rc = wsget(h->ws, "g2_ek", (size_t)nv * nw, &ek)) ||
      (rc = wsget(h->ws, "g2_ekp", (size_t)nv * nw, &ekp)) || (rc = wsget(h->ws, "g2_eq", (size_t)nv * nb, &eq)) ||
      (rc = wsget(h->ws, "g2_gm", (size_t)ngm * gstride, &gm)) || (rc = wsget(h->ws, "g2_gi", (size_t)nv, &gi)))
    return WSFAIL(rc);
  const double *kq = wannspace == EPHG_WANNSPACE_PH ? qvecs : kvecs;
  CK(cudaMemcpyAsync(qv, kq, (size_t)nv * 3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(en, ph_en, (size_t)nv * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(ek, el_evec_k, (size_t)nv * nw * sizeof(double2), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(ekp, el_evec_kp, (size_t)nv * nw * sizeof(double2), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(eq, ph_evec_q, (size_t)nv * nb * sizeof(double2), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(gm, gmixed, (size_t)ngm * gstride * sizeof(double2), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(gi, gm_index, (size_t)nv * sizeof(int64_t), cudaMemcpyHostToDevice, h->st));
  const int *R = wannspace == EPHG_WANNSPACE_PH ? h->Rq : h->Rk;
  const double *deg = wannspace == EPHG_WANNSPACE_PH ? h->degq : h->degk;
  double2 *Lv = nullptr;
  if (h->polar_on) {   // the long-range term of each vertex's q (wannier.f90:998-1006)
    double *qp = qv;
    if (wannspace != EPHG_WANNSPACE_PH) {
      if ((rc = wsget(h->ws, "g2_qp", (size_t)nv * 3, &qp))) return WSFAIL(rc);
      CK(cudaMemcpyAsync(qp, qvecs, (size_t)nv * 3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    }
    if ((rc = wsget(h->ws, "g2_L", (size_t)nv * nb, &Lv))) return WSFAIL(rc);
    launch_polar_q(h->polar, (int)nv, nullptr, nullptr, qp, nullptr, nullptr, Lv, h->st);
    h->launches += 1;
  }
  launch_g2_batch((int)nv, nw, nb, nws, qv, R, deg, ek, ekp, eq, en, h->masses, gm, gi, gstride,
                  Lv, out, h->st);
  h->launches += 1;
  CKL();
  CK(cudaMemcpyAsync(g2_out, out, (size_t)nv * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  return ephg::api_check_err(h);
}

// ------------------------------------------------------------ kq index
int ephg_kq_index(ephg_handle *h, const int64_t mesh[3], int64_t nk, const int64_t *k_idx,
                  int64_t nkp, const int64_t *kp_idx, int64_t *q_idx) {
  if (!h || !mesh || nk < 0 || nkp < 0) return fail(EPHG_ERR_ARG, "kq_index: bad arguments");
  for (int i = 0; i < 3; ++i)
    if (mesh[i] <= 0) return fail(EPHG_ERR_ARG, "kq_index: bad mesh");
  if (nk == 0 || nkp == 0) return EPHG_OK;
  int m[3] = {(int)mesh[0], (int)mesh[1], (int)mesh[2]};
  int64_t *a, *b, *q;
  int rc;
  if ((rc = wsget(h->ws, "kq_a", (size_t)nk, &a)) || (rc = wsget(h->ws, "kq_b", (size_t)nkp, &b)) ||
      (rc = wsget(h->ws, "kq_q", (size_t)nk * nkp, &q)))
    return WSFAIL(rc);
  CK(cudaMemcpyAsync(a, k_idx, nk * sizeof(int64_t), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(b, kp_idx, nkp * sizeof(int64_t), cudaMemcpyHostToDevice, h->st));
  launch_kq_index(m, (int)nk, a, (int)nkp, b, q, h->err, h->st);
  h->launches += 1;
  CKL();
  CK(cudaMemcpyAsync(q_idx, q, (size_t)nk * nkp * sizeof(int64_t), cudaMemcpyDeviceToHost, h->st));
  return ephg::api_check_err(h);
}

}  // extern "C"

// ------------------------------------------------------------- rates
namespace {

// form_triangles / form_tetrahedra_3d + fill (delta.f90:494-646,648-788) on the
// host: integer set-up of the simplices of the window mesh, uploaded once per
// request.  Output layouts: map (nwv, maxc, 2), count (nwv), evals (ns, nw, nv).
void build_simplices(int kind, const int mesh[3], const std::vector<int> &widx,
                     const std::vector<double> &ens_w, int nw, std::vector<int> &map,
                     std::vector<int> &count, std::vector<double> &sev, int &nsimplex, int &maxc,
                     int &nv) {
  const int nk = (int)widx.size();
  const int per = kind == 1 ? 2 : 6;
  nv = kind == 1 ? 3 : 4;
  maxc = kind == 1 ? 6 : 24;
  nsimplex = per * nk;
  static const int tri[2][3] = {{1, 2, 3}, {1, 3, 4}};
  static const int tet[6][4] = {{1, 2, 3, 6}, {1, 3, 5, 6}, {3, 5, 6, 7}, {3, 6, 7, 8}, {3, 4, 6, 8}, {2, 3, 4, 6}};
  std::vector<int> simplex((size_t)nsimplex * nv, 0);
  map.assign((size_t)nk * maxc * 2, 0);
  count.assign(nk, 0);
  // widx is sorted ascending (0-based mesh index) = indexlist - 1
  auto find = [&](int mux1) -> int {   // binsearch (misc.f90:738), 1-based or -1
    auto it = std::lower_bound(widx.begin(), widx.end(), mux1 - 1);
    if (it != widx.end() && *it == mux1 - 1) return (int)(it - widx.begin()) + 1;
    return -1;
  };
  int cnt = 1;
  for (int ik = 0; ik < nk; ++ik) {
    int p = widx[ik];
    int i = p % mesh[0] + 1, j = (p / mesh[0]) % mesh[1] + 1, k = p / (mesh[0] * mesh[1]) + 1;
    int ip1 = i == mesh[0] ? 1 : i + 1, jp1 = j == mesh[1] ? 1 : j + 1, kp1 = k == mesh[2] ? 1 : k + 1;
    int sc[8][3] = {{i, j, k}, {ip1, j, k}, {i, jp1, k}, {ip1, jp1, k},
                    {i, j, kp1}, {ip1, j, kp1}, {i, jp1, kp1}, {ip1, jp1, kp1}};
    for (int tk = 0; tk < per; ++tk) {
      for (int tl = 0; tl < nv; ++tl) {
        int a = (kind == 1 ? tri[tk][tl] : tet[tk][tl]) - 1;
        int mux = ((sc[a][2] - 1) * mesh[1] + (sc[a][1] - 1)) * mesh[0] + sc[a][0];
        int tmp = find(mux);
        simplex[(size_t)(cnt - 1) * nv + tl] = tmp;
        if (tmp > 0) {
          int c = ++count[tmp - 1];
          map[((size_t)(tmp - 1) * maxc + (c - 1)) * 2] = cnt;
          map[((size_t)(tmp - 1) * maxc + (c - 1)) * 2 + 1] = tl + 1;
        }
      }
      cnt++;
    }
  }
  sev.assign((size_t)nsimplex * nw * nv, 0.0);
  for (int it = 0; it < nsimplex; ++it) {
    for (int iv = 0; iv < nv; ++iv) {
      int aux = simplex[(size_t)it * nv + iv];
      if (aux > 0)
        for (int ib = 0; ib < nw; ++ib) sev[((size_t)it * nw + ib) * nv + iv] = ens_w[(size_t)(aux - 1) * nw + ib];
    }
    for (int ib = 0; ib < nw; ++ib) std::sort(&sev[((size_t)it * nw + ib) * nv], &sev[((size_t)it * nw + ib) * nv] + nv);
  }
}

struct EvTimer {
  cudaEvent_t e[6];
  EvTimer() { for (auto &x : e) cudaEventCreate(&x); }
  ~EvTimer() { for (auto &x : e) cudaEventDestroy(x); }
};

}  // namespace


// the device error word of an execution view: read, clear, translate
static int check_err_view(const ExecView &x) {
  int w = 0;
  CK(cudaMemcpyAsync(&w, x.err, sizeof(int), cudaMemcpyDeviceToHost, x.st));
  CK(cudaStreamSynchronize(x.st));
  CK(cudaMemsetAsync(x.err, 0, sizeof(int), x.st));
  if (w & DERR_NEG_PHONON) return fail(EPHG_ERR_NEG_PHONON, "Large negative phonon energy found!");
  if (w & DERR_EIG) return fail(EPHG_ERR_EIG, "Jacobi eigensolver did not converge");
  if (w & DERR_INDEX) return fail(EPHG_ERR_INDEX, "device index check failed");
  if (w & DERR_TIMEOUT) return fail(EPHG_ERR_TIMEOUT, "bounded device wait gave up");
  return EPHG_OK;
}

#define WSFAILX(rc) fail((rc), "%s", x.ws->msg.c_str())

static_assert(ephg::MAX_SETS == EPHG_MAX_SETS, "parameter-set bound of the C interface");

int ephg::check_sets(int64_t n, const ephg_rate_request *reqs) {
  if (n < 1 || n > MAX_SETS) return fail(EPHG_ERR_ARG, "el_rates_sets: nsets must be 1..%d", MAX_SETS);
  const ephg_rate_request &a = reqs[0];
  for (int64_t p = 0; p < n; ++p) {
    const ephg_rate_request &b = reqs[p];
    if (b.mesh[0] != a.mesh[0] || b.mesh[1] != a.mesh[1] || b.mesh[2] != a.mesh[2] || b.enref != a.enref ||
        b.fsthick != a.fsthick || b.delta_kind != a.delta_kind || b.precision != a.precision)
      return fail(EPHG_ERR_ARG, "el_rates_sets: set %lld differs from set 0 in more than T, sigma and chempot",
                  (long long)p);
    if (!(b.T > 0)) return fail(EPHG_ERR_ARG, "el_rates_sets: T must be > 0 (set %lld)", (long long)p);
    if (b.delta_kind == 0 && !(b.sigma > 0))
      return fail(EPHG_ERR_ARG, "el_rates_sets: sigma must be > 0 (set %lld)", (long long)p);
  }
  return EPHG_OK;
}

int ephg::el_rates_view(ephg_handle *h, const ExecView &x, const ephg_rate_request *req, double *rates,
                        int64_t *indexlist, ephg_rate_stats *stats, double *g2, double *xplus, double *xminus,
                        int64_t cap, const PhOut *ph, const DegAvgReq *avg, const SetsOut *sets) {
  if (!h || !req || (!ph && !avg && (!rates || !indexlist)) || (ph && !ph->rates_phe) || (avg && (ph || !avg->g2)))
    return fail(EPHG_ERR_ARG, "el_rates: bad arguments");
  if (sets) {
    if (ph || avg || g2 || sets->reqs != req || !sets->rates) return fail(EPHG_ERR_ARG, "el_rates_sets: bad arguments");
    int rc0 = check_sets(sets->n, sets->reqs);
    if (rc0) return rc0;
    for (int p = 0; p < sets->n; ++p)
      if (!sets->rates[p]) return fail(EPHG_ERR_ARG, "el_rates_sets: rates[%d] is NULL", p);
  }
  const int nsets = sets ? sets->n : 1;
  for (int i = 0; i < 3; ++i)
    if (req->mesh[i] <= 0) return fail(EPHG_ERR_ARG, "el_rates: bad mesh");
  if (req->delta_kind < 0 || req->delta_kind > 2) return fail(EPHG_ERR_ARG, "el_rates: bad delta_kind");
  if (req->delta_kind == 0 && !(req->sigma > 0)) return fail(EPHG_ERR_ARG, "el_rates: sigma must be > 0");
  if (!(req->T > 0)) return fail(EPHG_ERR_ARG, "el_rates: T must be > 0");
  if (req->precision != EPHG_PREC_FP64 && req->precision != EPHG_PREC_SPLIT_TF32)
    return fail(EPHG_ERR_ARG, "el_rates: bad precision");
  const int64_t N64 = req->mesh[0] * req->mesh[1] * req->mesh[2];
  if (N64 > (1 << 24)) return fail(EPHG_ERR_ARG, "el_rates: mesh too large");
  const int N = (int)N64;
  const int mesh[3] = {(int)req->mesh[0], (int)req->mesh[1], (int)req->mesh[2]};
  const int L = lcm3(mesh);
  const int nw = h->nw, nb = h->nb, nwsk = h->nwsk, nwsq = h->nwsq;
  const size_t nn = (size_t)nw * nw;
  const int ncol = nw * nb;   // columns per initial state in stage B
  const bool split = req->precision == EPHG_PREC_SPLIT_TF32;
  cudaStream_t st = x.st;
  int rc;
  int64_t launches0 = (*x.launches);
  EvTimer ev;
  (*x.ta).reset();
  (*x.tb).reset();
  CK(cudaEventRecord(ev.e[0], st));
  // ---- set-up: electrons on the full mesh (el_wann, electron.f90:364) ----
  double2 *roots, *Hk, *V, *Dq, *Vq, *u;
  double *w, *ens, *wq, *om, *bose, *rates_d;
  int *flag, *widx, *nwv_d, *sflag, *iota, *st_code, *nst_d, *nin_k, *cum;
  if ((rc = wsget((*x.ws), "r_roots", (size_t)L, &roots)) || (rc = wsget((*x.ws), "r_Hk", (size_t)N * nn, &Hk)) || (rc = wsget((*x.ws), "r_w", (size_t)N * nw, &w)) ||
      (rc = wsget((*x.ws), "r_V", (size_t)N * nn, &V)) || (rc = wsget((*x.ws), "r_ens", (size_t)N * nw, &ens)) ||
      (rc = wsget((*x.ws), "r_flag", (size_t)N, &flag)) || (rc = wsget((*x.ws), "r_widx", (size_t)N, &widx)) ||
      (rc = wsget((*x.ws), "r_nwv", 4, &nwv_d)) || (rc = wsget((*x.ws), "r_iota", (size_t)N * nw, &iota)) ||
      (rc = wsget((*x.ws), "r_Dq", (size_t)N * nb * nb, &Dq)) || (rc = wsget((*x.ws), "r_wq", (size_t)N * nb, &wq)) ||
      (rc = wsget((*x.ws), "r_Vq", (size_t)N * nb * nb, &Vq)) || (rc = wsget((*x.ws), "r_om", (size_t)N * nb, &om)) ||
      (rc = wsget((*x.ws), "r_u", (size_t)N * nb * nb, &u)) || (rc = wsget((*x.ws), "r_bose", (size_t)N * nb, &bose)) ||
      (rc = wsget((*x.ws), "r_rates", (size_t)N * nw, &rates_d)))
    return WSFAILX(rc);
  launch_roots(L, roots, st);
  {   // H(k) on the whole mesh: the Re sum one dimension at a time
    double2 *t1, *t2;
    if ((rc = wsget((*x.ws), "r_ht1", (size_t)h->hext[0] * h->hext[1] * mesh[2] * nn, &t1)) ||
        (rc = wsget((*x.ws), "r_ht2", (size_t)h->hext[0] * mesh[1] * mesh[2] * nn, &t2)))
      return WSFAILX(rc);
    launch_mesh_fourier(h->Hbox, h->hlo, h->hext, (int)nn, mesh, L, roots, t1, t2, Hk, st);
  }
  launch_heig(N, nw, Hk, nn, w, V, x.err, st);
  launch_el_post(N, nw, w, V, nullptr, 0, 0, nullptr, nullptr, nullptr, nullptr, ens, st);
  // ---- crystal symmetry: every mesh point takes the energies of its orbit's
  // representative, the irreducible point (electron.f90:363-385, 531-546); the
  // eigenvectors stay the point's own (:431-437).  The electron side then
  // starts from the irreducible window points only; the phonon side needs
  // every window k and keeps them all.
  const int nsymm = (int)(h->sym_rot.size() / 9);
  const bool ibz = nsymm > 0 && !ph;
  int *rep = nullptr;
  if (nsymm > 0) {
    std::vector<int> K;
    const char *why = "";
    if (ephg::mesh_qrotations(h->lattvecs, nsymm, h->sym_rot.data(), mesh, K, &why))
      return fail(EPHG_ERR_ARG, "el_rates: %s", why);
    int *Kd;
    double *ens_m;
    if ((rc = wsget((*x.ws), "r_symK", K.size(), &Kd)) || (rc = wsget((*x.ws), "r_rep", (size_t)N, &rep)) ||
        (rc = wsget((*x.ws), "r_ensm", (size_t)N * nw, &ens_m)))
      return WSFAILX(rc);
    CK(cudaMemcpyAsync(Kd, K.data(), K.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    launch_sym_rep(N, mesh, (int)(K.size() / 9), Kd, rep, st);
    launch_map_ens(N, nw, rep, ens, ens_m, st);
    ens = ens_m;
    (*x.launches) += 2;
  }
  // ---- window (apply_energy_window, electron.f90:597-636) ----
  launch_window_flags(N, nw, ens, req->enref, req->fsthick, flag, st);
  launch_iota(N * nw, iota, st);
  size_t tmp_bytes = 0, tb2 = 0, tb3 = 0;
  cub::DeviceSelect::Flagged(nullptr, tmp_bytes, iota, flag, widx, nwv_d, N, st);
  if ((rc = wsget((*x.ws), "r_sflag", (size_t)N * nw, &sflag)) || (rc = wsget((*x.ws), "r_stcode", (size_t)N * nw, &st_code)) ||
      (rc = wsget((*x.ws), "r_nst", 4, &nst_d)) || (rc = wsget((*x.ws), "r_nink", (size_t)N + 1, &nin_k)) ||
      (rc = wsget((*x.ws), "r_cum", (size_t)N + 1, &cum)))
    return WSFAILX(rc);
  cub::DeviceSelect::Flagged(nullptr, tb2, iota, sflag, st_code, nst_d, N * nw, st);
  cub::DeviceScan::ExclusiveSum(nullptr, tb3, nin_k, cum, N + 1, st);
  void *cubtmp;
  if ((rc = x.ws->get("r_cub", std::max(tmp_bytes, std::max(tb2, tb3)), &cubtmp))) return WSFAILX(rc);
  size_t tbytes = std::max(tmp_bytes, std::max(tb2, tb3));
  cub::DeviceSelect::Flagged(cubtmp, tbytes, iota, flag, widx, nwv_d, N, st);
  (*x.launches) += 8;
  CKL();
  int nwv = 0;
  CK(cudaMemcpyAsync(&nwv, nwv_d, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if ((rc = check_err_view(x))) return rc;
  if (nwv == 0) return fail(EPHG_ERR_EMPTY_WINDOW, "No states found within Fermi window.");
  // ---- phonons on the q mesh (phonon.f90:208-214) ----
  {   // D(q) on the whole mesh: the sum over wrapped cells one dimension at a time
    double2 *t1, *t2;
    const size_t ne = (size_t)nb * nb;
    if ((rc = wsget((*x.ws), "r_dt1", (size_t)h->dext[0] * h->dext[1] * mesh[2] * ne, &t1)) ||
        (rc = wsget((*x.ws), "r_dt2", (size_t)h->dext[0] * mesh[1] * mesh[2] * ne, &t2)))
      return WSFAILX(rc);
    launch_mesh_fourier(h->Dbox, h->dlo, h->dext, (int)ne, mesh, L, roots, t1, t2, Dq, st);
  }
  double2 *Lq = nullptr, *glp = nullptr;
  float2 *glpf = nullptr;
  if (h->polar_on) {   // dyn_nonanalytic into D(q) and the long-range vector of every mesh q
    if ((rc = wsget((*x.ws), "r_Lq", (size_t)N * nb, &Lq)) || (rc = wsget((*x.ws), "r_glp", (size_t)N * nb, &glp)) ||
        (split && (rc = wsget((*x.ws), "r_glpf", (size_t)N * nb, &glpf))))
      return WSFAILX(rc);
    launch_polar_q(h->polar, N, iota, mesh, nullptr, Dq, nullptr, Lq, st);
    (*x.launches) += 1;
  }
  launch_heig(N, nb, Dq, (int64_t)nb * nb, wq, Vq, x.err, st);
  float2 *uf = nullptr;
  if (split && (rc = wsget((*x.ws), "r_uf", (size_t)N * nb * nb, &uf))) return WSFAILX(rc);
  launch_ph_post(N, nb, iota, nullptr, wq, Vq, nullptr, 0, h->masses, nullptr, nullptr, nullptr, om,
                 u, uf, x.err, st);
  launch_bose(N, nb, om, req->T, bose, st);
  RateSets rs;
  memset(&rs, 0, sizeof rs);
  rs.n = nsets;
  for (int p = 1; p < nsets; ++p) {   // the other parameter sets' Bose factors
    if ((rc = wsget((*x.ws), ("r_bose" + std::to_string(p)).c_str(), (size_t)N * nb, &rs.bose[p])))
      return WSFAILX(rc);
    launch_bose(N, nb, om, sets->reqs[p].T, rs.bose[p], st);
    (*x.launches) += 1;
  }
  if (h->polar_on) {   // long_range_prefac(q, u_s) for every (q, s)
    launch_glprefac(N, nb, Lq, u, glp, glpf, st);
    (*x.launches) += 1;
  }
  // ---- final states: window bands of the window k' (their ranks, cum) ----
  launch_state_flags(nwv, nw, widx, ens, req->enref, req->fsthick, sflag, nin_k, st);
  CK(cudaMemsetAsync(nin_k + nwv, 0, sizeof(int), st));
  tbytes = std::max(tmp_bytes, std::max(tb2, tb3));
  cub::DeviceScan::ExclusiveSum(cubtmp, tbytes, nin_k, cum, nwv + 1, st);
  std::vector<int> widx_h(nwv), code_h;
  CK(cudaMemcpyAsync(widx_h.data(), widx, nwv * sizeof(int), cudaMemcpyDeviceToHost, st));
  // ---- A-rows: the k of the initial states, the window points or, with
  // crystal symmetry, the irreducible ones (IBZ blocks, find_irred_wedge with
  // blocks, electron.f90:553-577), in window order ----
  int nA = nwv;
  const int *arow = widx;
  int *awin = nullptr;
  std::vector<int> arow_h;
  if (ibz) {
    std::vector<int> rep_h(N);
    CK(cudaMemcpyAsync(rep_h.data(), rep, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<int> awin_h;
    for (int i = 0; i < nwv; ++i)
      if (rep_h[widx_h[i]] == widx_h[i]) {
        awin_h.push_back(i);
        arow_h.push_back(widx_h[i]);
      }
    nA = (int)arow_h.size();
    int *arow_d, *ninA;
    if ((rc = wsget((*x.ws), "r_arow", (size_t)nA, &arow_d)) || (rc = wsget((*x.ws), "r_awin", (size_t)nA, &awin)) ||
        (rc = wsget((*x.ws), "r_ninA", (size_t)nA, &ninA)))
      return WSFAILX(rc);
    CK(cudaMemcpyAsync(arow_d, arow_h.data(), (size_t)nA * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(awin, awin_h.data(), (size_t)nA * sizeof(int), cudaMemcpyHostToDevice, st));
    arow = arow_d;
    launch_state_flags(nA, nw, arow, ens, req->enref, req->fsthick, sflag, ninA, st);
  }
  // ---- initial states (demux_state order, interactions.f90:2169-2191) ----
  tbytes = std::max(tmp_bytes, std::max(tb2, tb3));
  cub::DeviceSelect::Flagged(cubtmp, tbytes, iota, sflag, st_code, nst_d, nA * nw, st);
  (*x.launches) += 7;
  CKL();
  int nst = 0, nin = 0;
  CK(cudaMemcpyAsync(&nst, nst_d, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&nin, cum + nwv, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if ((rc = check_err_view(x))) return rc;
  if (!ibz) arow_h = widx_h;
  code_h.resize(nst);
  CK(cudaMemcpyAsync(code_h.data(), st_code, nst * sizeof(int), cudaMemcpyDeviceToHost, st));
  // simplices for triangle / tetrahedron deltas
  EpiData ed;
  memset(&ed, 0, sizeof ed);
  if (req->delta_kind != 0) {
    std::vector<double> ens_all((size_t)N * nw), ens_w((size_t)nwv * nw);
    CK(cudaMemcpyAsync(ens_all.data(), ens, (size_t)N * nw * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int i = 0; i < nwv; ++i)
      for (int b = 0; b < nw; ++b) ens_w[(size_t)i * nw + b] = ens_all[(size_t)widx_h[i] * nw + b];
    std::vector<int> map, count;
    std::vector<double> sev;
    int ns, maxc, nvx;
    build_simplices((int)req->delta_kind, mesh, widx_h, ens_w, nw, map, count, sev, ns, maxc, nvx);
    int *dmap, *dcount;
    double *dsev;
    if ((rc = wsget((*x.ws), "r_smap", map.size(), &dmap)) || (rc = wsget((*x.ws), "r_scount", count.size(), &dcount)) ||
        (rc = wsget((*x.ws), "r_sev", sev.size(), &dsev)))
      return WSFAILX(rc);
    CK(cudaMemcpyAsync(dmap, map.data(), map.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dcount, count.data(), count.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dsev, sev.data(), sev.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    ed.smap = dmap;
    ed.scount = dcount;
    ed.sevals = dsev;
    ed.nsimplex = ns;
    ed.maxc = maxc;
    ed.nvx = nvx;
  }
  CK(cudaStreamSynchronize(st));
  std::vector<int> first_state(nA + 1, nst);
  for (int j = nst - 1; j >= 0; --j) first_state[code_h[j] / nw] = j;
  for (int i = nA - 1; i >= 0; --i)
    if (first_state[i] > first_state[i + 1]) first_state[i] = first_state[i + 1];
  if (avg) {   // degenerate-subspace averaging of the caller's vertex list, no contraction
    const int64_t per = (int64_t)nin * nb, vtot = (int64_t)nst * per;
    if (avg->nv != vtot)
      return fail(EPHG_ERR_ARG, "g2_average_degenerate: the list has %lld entries, the request's vertex list %lld",
                  (long long)avg->nv, (long long)vtot);
    double *g2d;
    int *fsd;
    if ((rc = wsget((*x.ws), "r_vg2", (size_t)vtot, &g2d)) || (rc = wsget((*x.ws), "r_fsd", (size_t)nA + 1, &fsd)))
      return WSFAILX(rc);
    CK(cudaMemcpyAsync(g2d, avg->g2, (size_t)vtot * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(fsd, first_state.data(), (size_t)(nA + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    if (launch_degenerate_average(g2d, per, nin, st_code, arow, widx, cum, fsd, ens, om, nst, nA, nwv, nw, nb, mesh,
                                  req->enref, req->fsthick, avg->thres, avg->mode, st))
      return fail(EPHG_ERR_ARG, "g2_average_degenerate: nw and nb must be <= 64");
    (*x.launches) += 3;
    CKL();
    CK(cudaMemcpyAsync(avg->g2, g2d, (size_t)vtot * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (indexlist)
      for (int i = 0; i < nA; ++i) indexlist[i] = (int64_t)arow_h[i] + 1;
    if ((rc = check_err_view(x))) return rc;
    if (stats) {
      memset(stats, 0, sizeof *stats);
      stats->nwv = nA;
      stats->nstates_inwindow = nin;
      stats->nstates = nst;
      stats->vertices = vtot;
      stats->pairs = (int64_t)nst * nwv;
    }
    return EPHG_OK;
  }
  CK(cudaEventRecord(ev.e[1], st));
  x.yield();   // serving: hand the GPU to a smaller request before the contractions
  // ---- stage A: g(k,Rp) for window k, rotation over m, k-half of the Rp phase ----
  const int64_t ldb = (int64_t)ncol * nst;
  const int64_t Nn = h->Nn;
  RateParams rp;
  for (int i = 0; i < 3; ++i) rp.mesh[i] = mesh[i];
  rp.N = N;
  rp.nw = nw;
  rp.nb = nb;
  rp.enref = req->enref;
  rp.fsthick = req->fsthick;
  rp.chempot = req->chempot;
  rp.T = req->T;
  rp.delta_kind = (int)req->delta_kind;
  rp.sigma = req->sigma;
  rp.inv_nk = 1.0 / (double)N;
  rp.const_tp = 2.0 * 3.141592653589793 / hbar_eVps;
  ed.widx = widx;
  ed.sidx = arow;
  ed.swin = awin;
  ed.st_code = st_code;
  ed.cum = cum;
  ed.ens = ens;
  ed.U = V;
  ed.om = om;
  ed.u = u;
  ed.uf = uf;
  ed.bose = bose;
  ed.glp = glp;
  ed.glpf = glpf;
  ed.per_state = (int64_t)nin * nb;
  double *g2d = nullptr, *xpd = nullptr, *xmd = nullptr, *yd = nullptr, *phr = nullptr;
  int64_t vtot = (int64_t)nst * nin * nb;
  int64_t vcap = std::min<int64_t>(cap, vtot);
  const bool want_y = ph && ph->y;
  const bool lists = (g2 || want_y) && vcap > 0;
  if (lists) {
    if ((rc = wsget((*x.ws), "r_vg2", (size_t)vcap, &g2d)) || (rc = wsget((*x.ws), "r_vxp", (size_t)vcap, &xpd)) ||
        (rc = wsget((*x.ws), "r_vxm", (size_t)vcap, &xmd)) ||
        (want_y && (rc = wsget((*x.ws), "r_vy", (size_t)vcap, &yd))))
      return WSFAILX(rc);
    ed.g2 = g2d;
    ed.xp = xpd;
    ed.xm = xmd;
    ed.yv = yd;
    ed.cap = vcap;
  }
  if (ph) {
    // the phonon states' rates, summed by the epilogues' atomics (ibzq 'Y' + ph-e rates)
    if ((rc = wsget((*x.ws), "r_phr", (size_t)N * nb, &phr))) return WSFAILX(rc);
    CK(cudaMemsetAsync(phr, 0, (size_t)N * nb * sizeof(double), st));
    ed.phr = phr;
    ed.ph_scale = ph->spindeg;
  }
  int nblk = (nwv + 127) / 128;                 // k'-row blocks of the rate partials
  const int nblk_max = std::max((nwv + 15) / 16, (nwv + 255) / 256 * 8);
  double *partial;
  if ((rc = wsget((*x.ws), "r_partial", (size_t)nst * nblk_max, &partial))) return WSFAILX(rc);
  rs.rp[0] = rp;
  rs.bose[0] = bose;
  rs.partial[0] = partial;
  for (int p = 1; p < nsets; ++p) {
    rs.rp[p] = rp;
    rs.rp[p].T = sets->reqs[p].T;
    rs.rp[p].sigma = sets->reqs[p].sigma;
    rs.rp[p].chempot = sets->reqs[p].chempot;
    if ((rc = wsget((*x.ws), ("r_partial" + std::to_string(p)).c_str(), (size_t)nst * nblk_max, &rs.partial[p])))
      return WSFAILX(rc);
  }
  if (!split) {
    double2 *Pk, *gk, *B, *Pq, *Cb;
    const int64_t kc = std::max<int64_t>(1, std::min<int64_t>(nA, ((int64_t)1 << 31) / (Nn * 16)));
    const int64_t sc = std::max<int64_t>(1, std::min<int64_t>({(int64_t)nst, (int64_t)32768,
                                                              ((int64_t)1 << 31) / ((int64_t)nwv * ncol * 16)}));
    if ((rc = wsget((*x.ws), "a_Pk", (size_t)kc * nwsk, &Pk)) || (rc = wsget((*x.ws), "a_gk", (size_t)kc * Nn, &gk)) ||
        (rc = wsget((*x.ws), "a_B", (size_t)nwsq * ldb, &B)) || (rc = wsget((*x.ws), "b_Pq", (size_t)nwv * nwsq, &Pq)) ||
        (rc = wsget((*x.ws), "b_C", (size_t)nwv * ncol * sc, &Cb)))
      return WSFAILX(rc);
    for (int64_t i0 = 0; i0 < nA; i0 += kc) {   // stage A over the A-rows
      int n = (int)std::min<int64_t>(kc, nA - i0);
      launch_phase_mesh(n, arow + i0, mesh, L, nwsk, h->Rk, h->degk, 0, roots, Pk, nwsk, st);
      (*x.ta).begin(st);
      launch_zgemm(n, (int)Nn, nwsk, Pk, nwsk, h->G64, Nn, gk, Nn, st);
      (*x.ta).end(st);
      // the rotation writes B columns of states [j0, j1) (grid.y <= 32768 per launch)
      for (int j0 = first_state[i0], j1 = first_state[i0 + n]; j0 < j1; j0 += 32768) {
        int je = std::min(j1, j0 + 32768);
        launch_rotate_states_fp64(j0, je, (int)i0, st_code, nw, nb, nwsq, arow, V, gk, Nn, mesh, L,
                                  roots, h->Rq, h->degq, B + (int64_t)j0 * ncol, ldb, st);
        (*x.launches) += 1;
      }
      (*x.launches) += 2;
    }
    CK(cudaEventRecord(ev.e[2], st));
    // ---- stage B + C: Rp Fourier against e^{2 pi i k'.Rp}, then the epilogue ----
    launch_phase_mesh(nwv, widx, mesh, L, nwsq, h->Rq, nullptr, 0, roots, Pq, nwsq, st);
    (*x.launches) += 1;
    for (int64_t j0 = 0; j0 < nst; j0 += sc) {
      int ns = (int)std::min<int64_t>(sc, nst - j0);
      (*x.tb).begin(st);
      launch_zgemm(nwv, ns * ncol, nwsq, Pq, nwsq, B + j0 * ncol, ldb, Cb, (int64_t)ns * ncol, st);
      (*x.tb).end(st);
      launch_epilogue_fp64(nwv, (int)j0, (int)j0 + ns, Cb, (int64_t)ns * ncol, rp, ed, partial, nblk, st);
      for (int p = 1; p < nsets; ++p) {   // the same GEMM output under the other parameter sets
        EpiData ep = ed;
        ep.bose = rs.bose[p];
        launch_epilogue_fp64(nwv, (int)j0, (int)j0 + ns, Cb, (int64_t)ns * ncol, rs.rp[p], ep, rs.partial[p], nblk,
                             st);
        (*x.launches) += 1;
      }
      (*x.launches) += 2;
    }
  } else {
    rc = tc::split_rates_stage(h->split, *x.ws, st, h->G64, h->nwsk, nwsq, Nn, nw, nb, nwv, nst,
                               mesh, L, roots, widx, arow, nA, st_code, first_state, h->Rk, h->degk, h->kposk,
                               h->Rq, h->degq, h->kposq, V, rp, ed, partial, nblk_max, &nblk,
                               ev.e[2], x.launches, x.ta, x.tb, &h->split_mu, x.chunk_us, x.yield, &x.bm,
                               x.chunk_bytes, nsets > 1 ? &rs : nullptr);
    if (rc) return fail(rc, "split path: %s", tc::last_error());
  }
  CKL();
  CK(cudaMemsetAsync(rates_d, 0, (size_t)N * nw * sizeof(double), st));
  launch_rate_final(nst, nblk, partial, st_code, nw, N, rates_d, st);
  (*x.launches) += 1;
  std::vector<double *> rates_sets(nsets, rates_d);
  for (int p = 1; p < nsets; ++p) {
    if ((rc = wsget((*x.ws), ("r_rates" + std::to_string(p)).c_str(), (size_t)N * nw, &rates_sets[p])))
      return WSFAILX(rc);
    CK(cudaMemsetAsync(rates_sets[p], 0, (size_t)N * nw * sizeof(double), st));
    launch_rate_final(nst, nblk, rs.partial[p], st_code, nw, N, rates_sets[p], st);
    (*x.launches) += 1;
  }
  CK(cudaEventRecord(ev.e[3], st));
  if (rates) CK(cudaMemcpyAsync(rates, rates_d, (size_t)N * nw * sizeof(double), cudaMemcpyDeviceToHost, st));
  for (int p = 1; p < nsets; ++p)
    CK(cudaMemcpyAsync(sets->rates[p], rates_sets[p], (size_t)N * nw * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (ph) CK(cudaMemcpyAsync(ph->rates_phe, phr, (size_t)N * nb * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (indexlist)   // the rows of the rates: the A-rows
    for (int i = 0; i < nA; ++i) indexlist[i] = (int64_t)arow_h[i] + 1;
  if (lists) {
    if (g2) CK(cudaMemcpyAsync(g2, g2d, vcap * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (g2 && xplus) CK(cudaMemcpyAsync(xplus, xpd, vcap * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (g2 && xminus) CK(cudaMemcpyAsync(xminus, xmd, vcap * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (want_y) CK(cudaMemcpyAsync(ph->y, yd, vcap * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  if ((rc = check_err_view(x))) return rc;
  if (stats) {
    float t01 = 0, t12 = 0, t23 = 0, t03 = 0;
    cudaEventElapsedTime(&t01, ev.e[0], ev.e[1]);
    cudaEventElapsedTime(&t12, ev.e[1], ev.e[2]);
    cudaEventElapsedTime(&t23, ev.e[2], ev.e[3]);
    cudaEventElapsedTime(&t03, ev.e[0], ev.e[3]);
    stats->nwv = nA;
    stats->nstates_inwindow = nin;
    stats->nstates = nst;
    stats->vertices = vtot;
    stats->pairs = (int64_t)nst * nwv;
    stats->kernel_launches = (*x.launches) - launches0;
    stats->ms_setup = t01;
    stats->ms_stage_a = t12;
    stats->ms_stage_bc = t23;
    stats->ms_total = t03;
    stats->stage_a_gflop = 8.0 * (double)nA * nwsk * (double)Nn * 1e-9;
    stats->stage_b_gflop = 8.0 * (double)nwv * nwsq * (double)ncol * nst * 1e-9;
    stats->ms_gemm_a = (*x.ta).total_ms();
    stats->ms_gemm_b = (*x.tb).total_ms();
    stats->gemm_a_launches = (*x.ta).n;
    stats->gemm_b_launches = (*x.tb).n;
  }
  return EPHG_OK;
}

extern "C" int ephg_el_rates(ephg_handle *h, const ephg_rate_request *req, double *rates,
                             int64_t *indexlist, ephg_rate_stats *stats, double *g2,
                             double *xplus, double *xminus, int64_t cap) {
  if (!h) return fail(EPHG_ERR_ARG, "el_rates: bad arguments");
  const ExecView x{h->st, h->err, &h->ws, &h->timer_a, &h->timer_b, &h->launches};
  return el_rates_view(h, x, req, rates, indexlist, stats, g2, xplus, xminus, cap);
}

extern "C" int ephg_el_rates_sets(ephg_handle *h, int64_t nsets, const ephg_rate_request *reqs, double *const *rates,
                                  int64_t *indexlist, ephg_rate_stats *stats) {
  if (!h || !reqs || !rates || !indexlist) return fail(EPHG_ERR_ARG, "el_rates_sets: bad arguments");
  int rc = check_sets(nsets, reqs);
  if (rc) return rc;
  const ExecView x{h->st, h->err, &h->ws, &h->timer_a, &h->timer_b, &h->launches};
  const SetsOut so{(int)nsets, reqs, rates};
  return el_rates_view(h, x, &reqs[0], rates[0], indexlist, stats, nullptr, nullptr, nullptr, 0, nullptr, nullptr,
                       &so);
}

extern "C" int ephg_g2_average_degenerate(ephg_handle *h, const ephg_rate_request *req, int64_t mode, double thres,
                                          int64_t nv, double *g2) {
  if (!h || !req || !g2 || nv < 0) return fail(EPHG_ERR_ARG, "g2_average_degenerate: bad arguments");
  if (mode != EPHG_DEGAVG_REFERENCE && mode != EPHG_DEGAVG_MEAN)
    return fail(EPHG_ERR_ARG, "g2_average_degenerate: bad mode");
  const ExecView x{h->st, h->err, &h->ws, &h->timer_a, &h->timer_b, &h->launches};
  const DegAvgReq avg{g2, nv, (int)mode, thres > 0 ? thres : 1.0e-6};
  return el_rates_view(h, x, req, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, nullptr, &avg);
}

extern "C" int ephg_ph_rates(ephg_handle *h, const ephg_rate_request *req, int64_t spindeg, double *rates_phe,
                             double *el_rates, int64_t *indexlist, ephg_rate_stats *stats, double *g2, double *y,
                             int64_t cap) {
  if (!h || !rates_phe) return fail(EPHG_ERR_ARG, "ph_rates: bad arguments");
  // "spindeg can be 1 or 2.", electron.f90:164-166
  if (spindeg < 1 || spindeg > 2) return fail(EPHG_ERR_ARG, "ph_rates: spindeg must be 1 or 2");
  const ExecView x{h->st, h->err, &h->ws, &h->timer_a, &h->timer_b, &h->launches};
  const PhOut ph{rates_phe, y, (double)spindeg};
  return el_rates_view(h, x, req, el_rates, indexlist, stats, g2, nullptr, nullptr, cap, &ph);
}
