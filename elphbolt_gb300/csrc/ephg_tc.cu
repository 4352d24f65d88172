// ephg_tc.cu - split-FP32 (3xTF32) tcgen05 contractions of the rate pipeline.
//
// The two Fourier contractions of the e-ph vertex path are complex GEMMs:
//   stage A  g(k,Rp)[n]      = sum_Re  e^{2 pi i k.Re}/deg(Re) g(Re,Rp)[n]      (gkRp)
//   stage B  G(k',state)[c]  = sum_Rp  e^{2 pi i k'.Rp}  B(state)[Rp][c]        (g2's Rp sum)
// Each runs here on the 5th-generation tensor cores as a persistent,
// warp-specialised kernel: one thread issues TMA loads of K-major TF32 operand
// planes into 64B-swizzled shared memory, one thread issues tcgen05.mma into
// four TMEM accumulators (main and correction, real and imaginary: all 512
// columns), and the epilogue warps drain TMEM with tcgen05.ld.  Stage A writes
// its FP32 result to HBM; for nw = 8, nb = 6 and the Gaussian delta stage B is
// fused with the rate epilogue (k_stageB_fused86) and its result never leaves
// the SM.  Every complex operand X is stored as four planes
// (hi_re, hi_im, lo_re, lo_im) with hi = tf32(X) and lo = tf32(X - hi); each
// real product uses hi*hi + hi*lo + lo*hi (the "3xTF32" split), FP32
// accumulation.  -Im*Im terms use the instruction descriptor's negate-A bit.
//
// Accuracy.  The tensor core's FP32 accumulation truncates toward zero, so a
// long chain of MMAs into one accumulator drifts low (measured: -6e-6 relative
// on a 279-term complex dot product with the largest terms first).  Two
// measures keep the chain short: the hi*lo + lo*hi correction products go to
// their own accumulators (2^-11 smaller, so their truncation is negligible), the
// two chains being added in the CUDA cores with round-to-nearest; the
// contraction index is ordered by decreasing |R|, i.e. by increasing size of
// the decaying Wannier-space terms, so the main accumulator is small while most
// truncations happen; and the last K block (the nearest cells, the largest
// terms) is accumulated in the short correction chain.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <condition_variable>
#include <mutex>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>

#include "../../include/ephg_debug.h"
#include "ephg_gate.cuh"
#include "ephg_tc.cuh"

namespace ephg {
namespace tc {

static thread_local std::string g_msg;
const char *last_error() { return g_msg.c_str(); }

static int tfail(int code, const char *m) {
  g_msg = m;
  return code;
}

#define TCK(call)                                                                   \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      g_msg = std::string(#call ": ") + cudaGetErrorString(e_);                     \
      return 2;                                                                     \
    }                                                                               \
  } while (0)

// ----------------------------------------------------------------- tiling
constexpr int BM = 128;          // tile rows (UMMA M)
constexpr int BN = 128;          // tile columns per accumulator (UMMA N)
constexpr int BK = 16;           // K per stage: 16 fp32 = 64 B rows, SWIZZLE_64B
constexpr int STAGES = 3;
constexpr int PLANE_BYTES = BM * BK * 4;              // 8 KB (A and B tiles alike)
constexpr int STAGE_BYTES = 8 * PLANE_BYTES;          // 4 A planes + 4 B planes
constexpr int TMEM_COLS = 512;                        // main re, main im, corr re, corr im (128 each)
constexpr int GEMM_EPI_WARPS = 4;                     // one per TMEM lane quadrant
constexpr int GEMM_THREADS = 64 + 32 * GEMM_EPI_WARPS; // TMA warp, MMA warp, epilogue warps
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr long long WAIT_CYCLES = 4000000000LL;       // ~2 s at 2 GHz

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after `limit` SM cycles, records DERR_TIMEOUT and
// returns false.
__device__ __forceinline__ bool mbar_wait_limit(uint64_t *bar, uint32_t parity, int *err, long long limit) {
  if (mbar_try(bar, parity)) return true;
  long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (clock64() - t0 > limit) {
      atomicOr(err, DERR_TIMEOUT);
      return false;
    }
  }
  return true;
}

// The kernels' waits: ~2 s.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err) {
  return mbar_wait_limit(bar, parity, err, WAIT_CYCLES);
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0,
                                            int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

// Same with an L2 cache policy (the phase operand, reused by every n-tile, is
// kept with evict_last so that the streaming output does not push it out).
__device__ __forceinline__ void tma_load_2d_hint(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1,
                                                 uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%3, "
      "%4}], [%2], %5;" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "l"(policy)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// SMEM matrix descriptor: K-major, SWIZZLE_64B (atom = 8 rows x 64 B, SBO = 512 B).
__device__ __forceinline__ uint64_t sdesc(const void *p) {
  uint64_t a = smem_u32(p);
  uint64_t d = (a >> 4) & 0x3FFFull;        // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;          // stride byte offset: 8-row groups 512 B apart
  d |= (uint64_t)1 << 46;                   // descriptor version (sm_100 family)
  d |= (uint64_t)4 << 61;                   // layout: SWIZZLE_64B
  return d;
}

// Instruction descriptor, kind::tf32: D f32, A/B tf32, K-major, M = 128, N = BN.
__host__ __device__ constexpr uint32_t idesc_tf32(bool negA) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((negA ? 1u : 0u) << 13) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

__host__ __device__ constexpr uint32_t idesc_tf32_n(bool negA, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((negA ? 1u : 0u) << 13) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ---- 2-CTA cluster helpers (operand tiles multicast to both CTAs of a pair)
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// TMA load written to the same shared-memory offset of every CTA in mask, each
// CTA's mbarrier at the offset of bar receiving the bytes it got
__device__ __forceinline__ void tma_load_2d_mc(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1,
                                               uint16_t mask) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster [%0], [%1, {%3, "
      "%4}], [%2], %5;" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "h"(mask)
      : "memory");
}

// commit: arrive on the mbarrier at bar's offset in every CTA of mask when the MMAs retire
__device__ __forceinline__ void umma_commit_mc(uint64_t *bar, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"(mask)
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// -------------------------------------------------------- the GEMM kernel
struct GemmArgs {
  int mtiles, ntiles, nkb;   // tile counts, K blocks of BK
  int t0, t1;                // tiles [t0, t1) of this launch
  int64_t Astride, Bstride;  // rows between consecutive planes of the A / B stacks
  int64_t Aoff, Boff;        // first row of the operand inside plane 0
  float *Cr, *Ci;            // [Mp][ldc] outputs
  int64_t ldc;
  int *err;
  int ileave;                // 1: outputs interleaved by 32 rows in groups of 4 columns: (r, c) at
                             //    (r / 32) ldc 32 + (c / 4) 128 + (r % 32) 4 + c % 4 (ldc a multiple of 4)
};

// One output tile as the three roles see it: operand maps, first A / B row of
// plane 0, K blocks, and the tile's first output element.
struct TileJob {
  const CUtensorMap *tA, *tB;
  int arow, brow, nkb;
  int Astride, Bstride;
  float *Cr, *Ci;
  int64_t ldc;
  int ileave;
};

__host__ __device__ __forceinline__ TileJob tile_job(const CUtensorMap *tA, const CUtensorMap *tB, const GemmArgs &g,
                                                     int t) {
  const int mt = t % g.mtiles, nt = t / g.mtiles;
  TileJob j;
  j.tA = tA;
  j.tB = tB;
  j.arow = (int)(g.Aoff + (int64_t)mt * BM);
  j.brow = (int)(g.Boff + (int64_t)nt * BN);
  j.nkb = g.nkb;
  j.Astride = (int)g.Astride;
  j.Bstride = (int)g.Bstride;
  const int64_t off = g.ileave ? ((int64_t)mt * (BM / 32) * g.ldc + (int64_t)nt * BN) * 32
                               : (int64_t)mt * BM * g.ldc + (int64_t)nt * BN;
  j.Cr = g.Cr + off;
  j.Ci = g.Ci + off;
  j.ldc = g.ldc;
  j.ileave = g.ileave;
  return j;
}

// A single GEMM: its maps are kernel parameters.
struct OneGemm {
  const CUtensorMap *tA, *tB;
  const GemmArgs *g;
  static constexpr bool kGlobalMaps = false;
  __device__ __forceinline__ TileJob operator()(int t) const { return tile_job(tA, tB, *g, t); }
};

// A group of GEMMs of different requests, shapes and operands in one launch:
// problem p owns tiles [tile0, tile0 + mtiles * ntiles) of the launch's tile
// space; its maps sit in global memory beside its shape.
struct GroupProblem {   // 64-byte aligned: CUtensorMap is
  CUtensorMap tA, tB;
  GemmArgs g;
  int tile0;
};

struct GroupGemm {
  const GroupProblem *tab;
  int np;
  static constexpr bool kGlobalMaps = true;
  __host__ __device__ __forceinline__ TileJob operator()(int t) const {
    int lo = 0, hi = np - 1;   // last problem with tile0 <= t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
#ifdef __CUDA_ARCH__
      const int t0 = __ldg(&tab[mid].tile0);
#else
      const int t0 = tab[mid].tile0;
#endif
      if (t0 <= t) lo = mid; else hi = mid - 1;
    }
    const GroupProblem *q = tab + lo;
    return tile_job(&q->tA, &q->tB, q->g, t - q->tile0);
  }
};

// Warp-specialised 3xTF32 complex GEMM over the tiles [t0, t1) of a tile
// space, strided by the grid: warp 0 lane 0 issues TMA loads, warp 1 lane 0
// the MMAs, the GEMM_EPI_WARPS warps after them drain TMEM (with more than
// four, each lane quadrant's columns are split between its warps; four
// measured fastest).  Every wait is bounded (err).
template <class Jobs>
__device__ __forceinline__ void cgemm_body(const Jobs &jobs, int t0, int t1, int *err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + STAGES * STAGE_BYTES);
  uint64_t *empty = full + STAGES;
  uint64_t *tfull = empty + STAGES;
  uint64_t *tempty = tfull + 2;
  uint64_t *drain = tempty + 2;
  uint32_t *tslot = (uint32_t *)(drain + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 32 * GEMM_EPI_WARPS);
    }
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {   // ---- TMA producer
      uint64_t keep;
      asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(keep));
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      const CUtensorMap *seen = nullptr;
      for (int t = t0 + blockIdx.x; t < t1 && ok; t += gridDim.x) {
        const TileJob j = jobs(t);
        if (Jobs::kGlobalMaps && j.tA != seen) {
          // maps in global memory, written before the launch: order the tensor-map
          // proxy's reads of them after those writes
          asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(j.tA) : "memory");
          asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(j.tB) : "memory");
          seen = j.tA;
        }
        for (int kb = 0; kb < j.nkb; ++kb) {
          if (!mbar_wait(&empty[stage], phase ^ 1, err)) { ok = false; break; }
          uint8_t *sb = smem + stage * STAGE_BYTES;
          mbar_expect_tx(&full[stage], STAGE_BYTES);
#pragma unroll
          for (int p = 0; p < 4; ++p)
            tma_load_2d_hint(sb + p * PLANE_BYTES, j.tA, &full[stage], kb * BK, p * j.Astride + j.arow, keep);
#pragma unroll
          for (int p = 0; p < 4; ++p)
            tma_load_2d(sb + (4 + p) * PLANE_BYTES, j.tB, &full[stage], kb * BK, p * j.Bstride + j.brow);
          if (++stage == STAGES) { stage = 0; phase ^= 1; }
        }
      }
      // drain: wait until every issued stage has landed before the CTA can exit
      for (int s = 0; s < STAGES; ++s) mbar_wait(&empty[stage], phase ^ 1, err), stage = (stage + 1) % STAGES,
                                         phase ^= (stage == 0);
    }
  } else if (warp == 1) {
    if (lane == 0) {   // ---- MMA issuer
      constexpr uint32_t IDP = idesc_tf32(false), IDN = idesc_tf32(true);
      int stage = 0;
      uint32_t phase = 0;
      int it = 0;
      bool ok = true;
      const uint32_t mr = tmem, mi = tmem + BN, cr = tmem + 2 * BN, ci = tmem + 3 * BN;
      for (int t = t0 + blockIdx.x; t < t1 && ok; t += gridDim.x, ++it) {
        const int nkb = jobs(t).nkb;
        if (!mbar_wait(&tempty[0], (it & 1) ^ 1, err)) { ok = false; break; }
        tc_fence_after();
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&full[stage], phase, err)) { ok = false; break; }
          tc_fence_after();
          uint8_t *sb = smem + stage * STAGE_BYTES;
#pragma unroll
          for (int ks = 0; ks < BK / 8; ++ks) {
            const int off = ks * 32;   // 8 tf32 = 32 B along K inside the swizzle atom
            const uint64_t Ahr = sdesc(sb + 0 * PLANE_BYTES + off), Ahi = sdesc(sb + 1 * PLANE_BYTES + off);
            const uint64_t Alr = sdesc(sb + 2 * PLANE_BYTES + off), Ali = sdesc(sb + 3 * PLANE_BYTES + off);
            const uint64_t Bhr = sdesc(sb + 4 * PLANE_BYTES + off), Bhi = sdesc(sb + 5 * PLANE_BYTES + off);
            const uint64_t Blr = sdesc(sb + 6 * PLANE_BYTES + off), Bli = sdesc(sb + 7 * PLANE_BYTES + off);
            const uint32_t acc = (kb == 0 && ks == 0) ? 0u : 1u;
            // corrections: hi*lo + lo*hi
            umma(cr, Ahr, Blr, IDP, acc);
            umma(cr, Alr, Bhr, IDP, 1);
            umma(cr, Ahi, Bli, IDN, 1);
            umma(cr, Ali, Bhi, IDN, 1);
            umma(ci, Ahr, Bli, IDP, acc);
            umma(ci, Alr, Bhi, IDP, 1);
            umma(ci, Ahi, Blr, IDP, 1);
            umma(ci, Ali, Bhr, IDP, 1);
            // main: Re = Ar Br - Ai Bi, Im = Ar Bi + Ai Br (hi parts).  The last K
            // block holds the nearest cells, the largest terms: they go to the
            // short correction chain instead of the long main chain.
            const bool nearblk = (kb == nkb - 1) && nkb > 1;
            const uint32_t dr = nearblk ? cr : mr, di = nearblk ? ci : mi;
            const uint32_t am = nearblk ? 1u : acc;
            umma(dr, Ahr, Bhr, IDP, am);
            umma(dr, Ahi, Bhi, IDN, 1);
            umma(di, Ahr, Bhi, IDP, am);
            umma(di, Ahi, Bhr, IDP, 1);
          }
          umma_commit(&empty[stage]);     // frees the smem stage when these MMAs retire
          if (++stage == STAGES) { stage = 0; phase ^= 1; }
        }
        if (ok) umma_commit(&tfull[0]);   // accumulators ready for the epilogue
      }
      // a wait gave up: let the MMAs already issued retire before TMEM is freed
      if (!ok) {
        umma_commit(drain);
        mbar_wait(drain, 0, err);
      }
    }
  } else {   // ---- epilogue: warp w drains TMEM lane quadrant w % 4, column block (w - 2) / 4
    const int quad = warp & 3;
    constexpr int CW = BN / (GEMM_EPI_WARPS / 4);
    const int cbeg = ((warp - 2) >> 2) * CW;
    const int row = quad * 32 + lane;
    int it = 0;
    for (int t = t0 + blockIdx.x; t < t1; t += gridDim.x, ++it) {
      const TileJob j = jobs(t);
      if (!mbar_wait(&tfull[0], it & 1, err)) break;
      tc_fence_after();
      const uint32_t tr = tmem + ((uint32_t)(quad * 32) << 16);
      // row-major: the row's 16 columns as float4 stores; interleaved: each group of
      // 4 columns of the warp's 32 rows is 512 consecutive bytes (one float4 per lane)
      float *cr = j.ileave ? j.Cr + (int64_t)quad * j.ldc * 32 + 4 * lane : j.Cr + (int64_t)row * j.ldc;
      float *ci = j.ileave ? j.Ci + (int64_t)quad * j.ldc * 32 + 4 * lane : j.Ci + (int64_t)row * j.ldc;
#pragma unroll 1
      for (int c0 = cbeg; c0 < cbeg + CW; c0 += 16) {
        uint32_t ar[16], ai[16], br[16], bi[16];
        tmem_ld16_nowait(tr + c0, ar);            // four loads in flight, one wait
        tmem_ld16_nowait(tr + BN + c0, ai);
        tmem_ld16_nowait(tr + 2 * BN + c0, br);
        tmem_ld16_nowait(tr + 3 * BN + c0, bi);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        float vr[16], vi[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          vr[q] = __uint_as_float(ar[q]) + __uint_as_float(br[q]);
          vi[q] = __uint_as_float(ai[q]) + __uint_as_float(bi[q]);
        }
        // streaming stores: the output is read once, later, by another kernel
        if (j.ileave) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            __stcs((float4 *)(cr + (int64_t)(c0 + 4 * q) * 32),
                   make_float4(vr[4 * q], vr[4 * q + 1], vr[4 * q + 2], vr[4 * q + 3]));
            __stcs((float4 *)(ci + (int64_t)(c0 + 4 * q) * 32),
                   make_float4(vi[4 * q], vi[4 * q + 1], vi[4 * q + 2], vi[4 * q + 3]));
          }
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            __stcs((float4 *)(cr + c0 + 4 * q), make_float4(vr[4 * q], vr[4 * q + 1], vr[4 * q + 2], vr[4 * q + 3]));
            __stcs((float4 *)(ci + c0 + 4 * q), make_float4(vi[4 * q], vi[4 * q + 1], vi[4 * q + 2], vi[4 * q + 3]));
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&tempty[0]);
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

__global__ void __launch_bounds__(GEMM_THREADS, 1)
    k_cgemm_3xtf32(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, GemmArgs g) {
  cgemm_body(OneGemm{&tA, &tB, &g}, g.t0, g.t1, g.err);
}

// The grouped form: the GEMMs of many rate requests in one persistent launch.
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    k_cgemm_group(const GroupProblem *tab, int np, int t0, int t1, int *err) {
  cgemm_body(GroupGemm{tab, np}, t0, t1, err);
}

// -------------------------------------------------------- tensor maps
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {   // thread-safe one-time initialisation
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000)p;
    return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
  }();
  return fn;
}

// 2D map over a stack of K-major fp32 planes: (Kp, rows), box (box_k, box_rows);
// box_k = 16 (64 B rows) uses the 64B swizzle, box_k = 8 (32 B rows) the 32B swizzle.
static int make_map(CUtensorMap *m, const float *base, int Kp, int64_t rows, int box_rows = 128, int box_k = BK) {
  auto fn = encode_fn();
  if (!fn) return tfail(2, "cuTensorMapEncodeTiled unavailable");
  if (((uintptr_t)base & 15) || (Kp % box_k) || (box_k != 8 && box_k != 16))
    return tfail(1, "operand planes misaligned");
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * 4};
  cuuint32_t box[2] = {(cuuint32_t)box_k, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)base, dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, box_k == 16 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return tfail(2, "cuTensorMapEncodeTiled failed");
  return 0;
}

static int num_sms() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// ------------------------------------------------------ grouped launches
// The GEMMs of rate requests running concurrently (one host thread and stream
// each) are gathered into rounds: a member that reaches a GEMM submits it and
// blocks; when every active member has submitted, the last one launches the
// round's problems as one k_cgemm_group launch on the batcher's stream (after
// each member's stream reached its submit), and each member's stream waits for
// that launch before its next kernel.  Members are active only inside the
// split form's generic contraction stages; anywhere else they do not hold a
// round back.
class GemmBatcher {
 public:
  explicit GemmBatcher(int n)
      : ready_(n, nullptr), gate_(n, [this](std::vector<std::pair<int, Pend>> &r) { return launch_round(r); }) {
    cudaStreamCreateWithFlags(&gst_, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&done_, cudaEventDisableTiming);
    for (auto &e : ready_) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    for (int r = 0; r < kRing; ++r) cudaEventCreateWithFlags(&slot_ev_[r], cudaEventDisableTiming);
    cudaMallocHost((void **)&htab_, sizeof(GroupProblem) * (size_t)kRing * n);
    cudaMalloc((void **)&dtab_, sizeof(GroupProblem) * (size_t)kRing * n);
    cudaMalloc((void **)&derr_, sizeof(int));
    cudaMemset(derr_, 0, sizeof(int));
    cap_ = n;
    ok_ = htab_ && dtab_ && derr_ && gst_;
  }
  ~GemmBatcher() {
    if (gst_) cudaStreamSynchronize(gst_);
    if (htab_) cudaFreeHost(htab_);
    if (dtab_) cudaFree(dtab_);
    if (derr_) cudaFree(derr_);
    for (auto &e : ready_) cudaEventDestroy(e);
    for (int r = 0; r < kRing; ++r) cudaEventDestroy(slot_ev_[r]);
    cudaEventDestroy(done_);
    if (gst_) cudaStreamDestroy(gst_);
  }
  bool ok() const { return ok_; }
  void activate(int id) { gate_.activate(id); }
  void deactivate(int id) { gate_.deactivate(id); }
  int submit(int id, const GroupProblem &p, cudaStream_t st) {
    if (cudaEventRecord(ready_[id], st) != cudaSuccess) return tfail(2, "batch: event record failed");
    return gate_.submit(id, Pend{st, p});
  }
  // device word of the grouped launches' bounded waits (read after the members finished)
  int device_error() {
    int w = 0;
    cudaStreamSynchronize(gst_);
    cudaMemcpy(&w, derr_, sizeof(int), cudaMemcpyDeviceToHost);
    return w;
  }
  void stats(int64_t *launches, int64_t *problems, int64_t *tiles, int64_t *max_group) const {
    *launches = launches_;
    *problems = problems_;
    *tiles = tiles_;
    *max_group = max_group_;
  }

 private:
  static constexpr int kRing = 8;
  struct Pend {
    cudaStream_t st;
    GroupProblem p;
  };
  // one round (under the gate's lock): table upload, the grouped launch, and the
  // members' streams made to wait for it
  int launch_round(std::vector<std::pair<int, Pend>> &pend) {
    // heaviest tiles (most K blocks) first: the strided tile order then ends on light tiles
    std::stable_sort(pend.begin(), pend.end(),
                     [](const std::pair<int, Pend> &a, const std::pair<int, Pend> &b) {
                       return a.second.p.g.nkb > b.second.p.g.nkb;
                     });
    const int np = (int)pend.size();
    const int slot = (int)(nround_++ % kRing);
    GroupProblem *h = htab_ + (size_t)slot * cap_, *d = dtab_ + (size_t)slot * cap_;
    cudaEventSynchronize(slot_ev_[slot]);   // the copy that last read this staging slot has run
    int64_t T = 0;
    for (int i = 0; i < np; ++i) {
      h[i] = pend[i].second.p;
      h[i].tile0 = (int)T;
      T += (int64_t)h[i].g.mtiles * h[i].g.ntiles;
    }
    int rc = 0;
    if (T > INT32_MAX) rc = tfail(1, "batch: too many tiles in one round");
    for (int i = 0; i < np && !rc; ++i)
      if (cudaStreamWaitEvent(gst_, ready_[pend[i].first], 0) != cudaSuccess)
        rc = tfail(2, "batch: stream wait failed");
    if (!rc && cudaMemcpyAsync(d, h, sizeof(GroupProblem) * np, cudaMemcpyHostToDevice, gst_) != cudaSuccess)
      rc = tfail(2, "batch: problem table upload failed");
    if (!rc) {
      cudaEventRecord(slot_ev_[slot], gst_);
      const int grid = (int)std::min<int64_t>(T, num_sms());
      k_cgemm_group<<<grid, GEMM_THREADS, SMEM_BYTES, gst_>>>(d, np, 0, (int)T, derr_);
      if (cudaGetLastError() != cudaSuccess) rc = tfail(2, "batch: grouped GEMM launch failed");
    }
    if (!rc && cudaEventRecord(done_, gst_) != cudaSuccess) rc = tfail(2, "batch: event record failed");
    for (auto &q : pend)
      if (!rc && cudaStreamWaitEvent(q.second.st, done_, 0) != cudaSuccess) rc = tfail(2, "batch: stream wait failed");
    ++launches_;
    problems_ += np;
    tiles_ += T;
    max_group_ = std::max<int64_t>(max_group_, np);
    return rc;
  }
  std::vector<cudaEvent_t> ready_;
  int cap_ = 0;
  uint64_t nround_ = 0;
  cudaStream_t gst_ = nullptr;
  cudaEvent_t done_ = nullptr, slot_ev_[kRing] = {};
  GroupProblem *htab_ = nullptr, *dtab_ = nullptr;
  int *derr_ = nullptr;
  bool ok_ = false;
  int64_t launches_ = 0, problems_ = 0, tiles_ = 0, max_group_ = 0;
  RoundGate<Pend> gate_;   // last: its callback uses the members above
};

GemmBatcher *batcher_create(int nmembers) {
  if (nmembers <= 0) return nullptr;
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(k_cgemm_group, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  });
  GemmBatcher *b = new GemmBatcher(nmembers);
  if (!b->ok()) {
    delete b;
    return nullptr;
  }
  return b;
}
void batcher_destroy(GemmBatcher *b) { delete b; }
void batcher_activate(const BatchMember &m) { if (m.gb) m.gb->activate(m.id); }
void batcher_deactivate(const BatchMember &m) { if (m.gb) m.gb->deactivate(m.id); }
int batcher_device_error(GemmBatcher *b) { return b ? b->device_error() : 0; }
void batcher_stats(const GemmBatcher *b, int64_t *launches, int64_t *problems, int64_t *tiles, int64_t *max_group) {
  b->stats(launches, problems, tiles, max_group);
}

// C[Mp][ldc] (re, im planes) = A x B^T.  A: planes of Astride rows, rows
// [Aoff, Aoff + Mp) of each; B: planes of Bstride rows, rows [Boff, Boff + Np).
// With a batch member the GEMM joins its batcher's next grouped launch.
static int cgemm(const float *Ap, int64_t Astride, int64_t Aoff, int Mp, const float *Bp, int64_t Bstride,
                 int64_t Boff, int Np, int Kp, float *Cr, float *Ci, int64_t ldc, int *err, cudaStream_t st,
                 int chunk_us = 0, const Yield &yield = Yield(), const BatchMember *bm = nullptr, int ileave = 0) {
  if (Mp % BM || Np % BN || Kp % BK || Mp <= 0 || Np <= 0) return tfail(1, "cgemm: shapes not tile multiples");
  if (4 * Astride > INT32_MAX || 4 * Bstride > INT32_MAX) return tfail(1, "cgemm: operand too tall for TMA coords");
  if (bm && bm->gb) {
    GroupProblem p;
    memset(&p, 0, sizeof p);
    int rc;
    if ((rc = make_map(&p.tA, Ap, Kp, 4 * Astride)) || (rc = make_map(&p.tB, Bp, Kp, 4 * Bstride))) return rc;
    p.g.mtiles = Mp / BM;
    p.g.ntiles = Np / BN;
    p.g.nkb = Kp / BK;
    p.g.Astride = Astride;
    p.g.Bstride = Bstride;
    p.g.Aoff = Aoff;
    p.g.Boff = Boff;
    p.g.Cr = Cr;
    p.g.Ci = Ci;
    p.g.ldc = ldc;
    p.g.err = err;
    p.g.ileave = ileave;
    return bm->gb->submit(bm->id, p, st);
  }
  CUtensorMap ta, tb;
  int rc;
  if ((rc = make_map(&ta, Ap, Kp, 4 * Astride)) || (rc = make_map(&tb, Bp, Kp, 4 * Bstride))) return rc;
  // once per process: changing a kernel attribute can wait for the device's queued work
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(k_cgemm_3xtf32, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  });
  GemmArgs g;
  g.mtiles = Mp / BM;
  g.ntiles = Np / BN;
  g.nkb = Kp / BK;
  g.Astride = Astride;
  g.Bstride = Bstride;
  g.Aoff = Aoff;
  g.Boff = Boff;
  g.Cr = Cr;
  g.Ci = Ci;
  g.ldc = ldc;
  g.err = err;
  g.ileave = ileave;
  int tiles = g.mtiles * g.ntiles;
  int grid = std::min(tiles, num_sms());
  // chunk_us > 0: launches of about that length (a tile is ~0.4 us per 16 K positions) so
  // that other streams' kernels get the SMs between them
  const int per_cta = chunk_us > 0 ? std::max(1, (int)((int64_t)chunk_us * 16 * 5 / 2 / std::max(1, Kp))) : 0;
  const int step = per_cta > 0 ? grid * per_cta : tiles;
  for (int t0 = 0; t0 < tiles; t0 += step) {
    if (t0 > 0) yield();
    g.t0 = t0;
    g.t1 = std::min(tiles, t0 + step);
    k_cgemm_3xtf32<<<grid, GEMM_THREADS, SMEM_BYTES, st>>>(ta, tb, g);
    TCK(cudaGetLastError());
  }
  return 0;
}

// ------------------------------------------------------ operand planes
__device__ __forceinline__ float tf32_round(float x) {
  uint32_t u = __float_as_uint(x);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;   // inf / nan untouched
  u += 0x0FFFu + ((u >> 13) & 1u);
  return __uint_as_float(u & 0xFFFFE000u);
}

// hi = tf32(x), lo = tf32(x - hi), from a double
__device__ __forceinline__ void split2(double x, float &hi, float &lo) {
  hi = tf32_round((float)x);
  lo = tf32_round((float)(x - (double)hi));
}

__device__ __forceinline__ void put4(float *P, int64_t plane, int64_t idx, double2 v) {
  float hr, lr, hi, li;
  split2(v.x, hr, lr);
  split2(v.y, hi, li);
  P[0 * plane + idx] = hr;
  P[1 * plane + idx] = hi;
  P[2 * plane + idx] = lr;
  P[3 * plane + idx] = li;
}

// Six-plane form of an operand for the stacked complex MMA (two N-halves):
// (-hi_im, hi_re, hi_im, -lo_im, lo_re, lo_im), so that [re; im] and [-im; re]
// are each two adjacent planes.
__device__ __forceinline__ void put6(float *P, int64_t plane, int64_t idx, double2 v) {
  float hr, lr, hi, li;
  split2(v.x, hr, lr);
  split2(v.y, hi, li);
  P[0 * plane + idx] = -hi;
  P[1 * plane + idx] = hr;
  P[2 * plane + idx] = hi;
  P[3 * plane + idx] = -li;
  P[4 * plane + idx] = lr;
  P[5 * plane + idx] = li;
}

// The stage-A operand of the fused nw = 8, nb = 6 path: column
// c = m' + 8 (kp + KpB (n' + 8 s')) holds g(Re, Rp = kinvB[kp])[n', m', s'], so
// that a 128-column tile is 16 contraction positions x 8 initial bands of one
// (n', s'); K position of Re = kposA[Re].  Six planes [6][NA][KpA].
__global__ void k_gplanes_a6(int nwsk, int64_t Nn, const double2 *G, const int *kposA, const int *kinvB, int KpB,
                             float *P, int64_t NA, int KpA) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= NA * nwsk) return;
  const int64_t c = idx / nwsk;
  const int re = (int)(idx % nwsk);
  const int mp = (int)(c & 7);
  const int64_t rest = c >> 3;
  const int kp = (int)(rest % KpB), ns = (int)(rest / KpB);
  const int np = ns & 7, sp = ns >> 3;
  const int rp = kinvB[kp];
  const double2 v = rp >= 0 ? G[(int64_t)re * Nn + np + 8 * (mp + 8 * (sp + 6 * (int64_t)rp))] : make_double2(0.0, 0.0);
  put6(P, NA * KpA, c * KpA + kposA[re], v);
}

__device__ inline int phase_idx(int p, int m1, int m2, int m3, int L, int r1, int r2, int r3) {
  int v1 = p % m1, v2 = (p / m1) % m2, v3 = p / (m1 * m2);
  int64_t t = (int64_t)v1 * r1 * (L / m1) + (int64_t)v2 * r2 * (L / m2) + (int64_t)v3 * r3 * (L / m3);
  t %= L;
  if (t < 0) t += L;
  return (int)t;
}

// A planes of e^{2 pi i k.R} (/ deg) for the rows k = rowp[0..nrows): [4][Mp][Kp]
// (column of cell r = kpos[r]: the contraction order, far cells first)
__global__ void k_phase_planes(int nrows, const int *rowp, int m1, int m2, int m3, int L, int nR, const int *R,
                               const double *deg, const int *kpos, const double2 *roots, float *P, int Mp, int Kp) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nrows * nR) return;
  int row = (int)(idx / nR), r = (int)(idx % nR);
  double2 v = roots[phase_idx(rowp[row], m1, m2, m3, L, R[3 * r], R[3 * r + 1], R[3 * r + 2])];
  if (deg) v = make_double2(v.x / deg[r], v.y / deg[r]);
  put4(P, (int64_t)Mp * Kp, (int64_t)row * Kp + kpos[r], v);
}

// B planes of the stage-A matrix: G64[Re][n] -> planes [4][Np][Kp] (transposed,
// column of Re = kpos[Re], or Re itself when kpos is null)
__global__ void k_gplanes(int64_t Nn, int nwsk, const double2 *G, const int *kpos, float *P, int64_t Np, int Kp) {
  __shared__ double2 tile[32][33];
  int64_t n0 = (int64_t)blockIdx.x * 32;
  int r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int re = r0 + i;
    int64_t n = n0 + threadIdx.x;
    tile[i][threadIdx.x] = (re < nwsk && n < Nn) ? G[(int64_t)re * Nn + n] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int64_t n = n0 + i;
    int re = r0 + threadIdx.x;
    if (n < Nn && re < nwsk) put4(P, Np * Kp, n * Kp + (kpos ? kpos[re] : re), tile[threadIdx.x][i]);
  }
}

// Rotation over the initial band + k-half of the Rp phase, split into the B
// planes of stage B: Bp[4][Np2][Kp2], column c = (j - j0)*ncol + n' + nw*s'.
__global__ void k_rotate_planes(int j0, int j1, int i0, const int *st_code, int nw, int nb, int nws,
                                const int *widx, const double2 *U, const float *gr, const float *gi, int64_t ldg,
                                int m1, int m2, int m3, int L, const double2 *roots, const int *Rq,
                                const double *degq, const int *kpos, float *Bp, int64_t Np2, int Kp2, int jbase) {
  const int j = j0 + blockIdx.y;
  if (j >= j1) return;
  const int code = st_code[j];
  const int i = code / nw, m = code % nw;
  const int p = widx[i];
  const double2 *Uk = U + ((size_t)p * nw + m) * nw;
  const int ncol = nw * nb;
  const int64_t grow = (int64_t)(i - i0) * ldg;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ncol * nws; e += gridDim.x * blockDim.x) {
    const int rp = e % nws, c = e / nws;
    const int np = c % nw, s = c / nw;
    double2 ph = roots[phase_idx(p, m1, m2, m3, L, Rq[3 * rp], Rq[3 * rp + 1], Rq[3 * rp + 2])];
    ph = make_double2(ph.x / degq[rp], -ph.y / degq[rp]);
    double2 acc = make_double2(0.0, 0.0);
    for (int mp = 0; mp < nw; ++mp) {
      int64_t off = grow + np + nw * (mp + (int64_t)nw * (s + (int64_t)nb * rp));
      cfma(acc, Uk[mp], make_double2((double)gr[off], (double)gi[off]));
    }
    const int64_t col = (int64_t)(j - jbase) * ncol + c;
    put4(Bp, Np2 * Kp2, col * Kp2 + kpos[rp], cmul(ph, acc));
  }
  // the K padding [nws, Kp2) of the state's rows: zero (the workspace holds
  // whatever an earlier request left there, and 0 x NaN is NaN)
  const int npad = Kp2 - nws;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ncol * npad; e += gridDim.x * blockDim.x) {
    const int64_t col = (int64_t)(j - jbase) * ncol + e / npad;
    put4(Bp, Np2 * Kp2, col * Kp2 + nws + e % npad, make_double2(0.0, 0.0));
  }
}

// Stage-A rotation, one block per window k: the block loads g(k,Rp) for KT
// contraction positions at a time (coalesced rows of nw*nw values per mode),
// rotates over the initial band for every in-window state of k, applies the
// k-half of the Rp phase and writes KT consecutive K positions of each operand
// row, so that both the reads and the split-plane writes are whole sectors.
// Modes are taken sch at a time so that the staged g fits shared memory for
// any nb.  kinv[kp] = Rp cell at contraction position kp (-1 for padding).
constexpr int ROT_KT = 8;
static_assert(ROT_KT == 8, "k_rotate_k writes 8 K positions as two float4 per plane");
constexpr int ROT_SMEM = 160 * 1024;
constexpr int ROT_SMEM_TARGET = 72 * 1024;

// shared memory of k_rotate_k for sch modes per pass and nsk <= nw states per row
static size_t rotate_k_smem(int nw, int sch) {
  return ((sizeof(float2) * ROT_KT * nw * nw * sch + 15) & ~(size_t)15) + sizeof(float2) * (nw * nw + ROT_KT);
}

__global__ void __launch_bounds__(256) k_rotate_k(int i0, const int *first_state, int nw, int nb, int sch,
                                                  const int *st_code, const int *widx, const double2 *U,
                                                  const float *gr, const float *gi, int64_t ldg, int m1, int m2,
                                                  int m3, int L, const double2 *roots, const int *Rq,
                                                  const double *degq, const int *kinv, int Kp2, float *Bp,
                                                  int64_t Np2) {
  extern __shared__ unsigned char rsm[];
  const int i = i0 + blockIdx.x;
  const int j0 = first_state[i], j1 = first_state[i + 1];
  const int nsk = j1 - j0;
  if (nsk <= 0) return;
  const int p = widx[i];
  const int per = nw * nw * nb, ncol = nw * nb, nn = nw * nw;
  float2 *sg = (float2 *)rsm;                                   // [ROT_KT][nw * nw * sch]
  float2 *sU = (float2 *)(rsm + ((sizeof(float2) * ROT_KT * nn * sch + 15) & ~(size_t)15));  // [nsk][nw]
  float2 *sph = sU + nsk * nw;                                  // [ROT_KT]
  for (int t = threadIdx.x; t < nsk * nw; t += blockDim.x) {
    int js = t / nw, mp = t % nw;
    int m = st_code[j0 + js] % nw;
    double2 u = U[((size_t)p * nw + m) * nw + mp];
    sU[t] = make_float2((float)u.x, (float)u.y);
  }
  const int64_t grow = (int64_t)(i - i0) * ldg;
  const int64_t plane = Np2 * Kp2;
  for (int s0 = 0; s0 < nb; s0 += sch) {
    const int ns = min(sch, nb - s0), pc = nn * ns, nc = nw * ns;
    for (int kp0 = 0; kp0 < Kp2; kp0 += ROT_KT) {
      __syncthreads();
      // 16-byte loads (4 consecutive values; every row offset is a multiple of 4),
      // four of them in flight per thread before the shared stores
      const int pc4 = pc >> 2, tot = ROT_KT * pc4;
      for (int t0 = threadIdx.x; t0 < tot; t0 += 4 * blockDim.x) {
        float4 a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * blockDim.x;
          a[u] = b[u] = make_float4(0.f, 0.f, 0.f, 0.f);
          if (t < tot) {
            const int kk = t / pc4, e = 4 * (t - kk * pc4);
            const int rp = kinv[kp0 + kk];
            if (rp >= 0) {
              const int64_t off = grow + (int64_t)rp * per + nn * s0 + e;
              a[u] = __ldg((const float4 *)(gr + off));
              b[u] = __ldg((const float4 *)(gi + off));
            }
          }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * blockDim.x;
          if (t < tot) {
            float4 *dst = (float4 *)(sg + 4 * t);
            dst[0] = make_float4(a[u].x, b[u].x, a[u].y, b[u].y);
            dst[1] = make_float4(a[u].z, b[u].z, a[u].w, b[u].w);
          }
        }
      }
      if (threadIdx.x < ROT_KT) {
        int rp = kinv[kp0 + threadIdx.x];
        float2 ph = make_float2(0.f, 0.f);
        if (rp >= 0) {
          double2 r = roots[phase_idx(p, m1, m2, m3, L, Rq[3 * rp], Rq[3 * rp + 1], Rq[3 * rp + 2])];
          ph = make_float2((float)(r.x / degq[rp]), (float)(-r.y / degq[rp]));
        }
        sph[threadIdx.x] = ph;
      }
      __syncthreads();
      // a thread forms the ROT_KT positions of one operand row: lanes walk
      // consecutive bands n' (conflict-free shared reads) and each writes whole
      // 32-byte sectors of the four planes
      for (int o = threadIdx.x; o < nsk * nc; o += blockDim.x) {
        const int c = o % nc, js = o / nc;
        const int np = c % nw, s = c / nw;
        float2 acc[ROT_KT];
#pragma unroll
        for (int kk = 0; kk < ROT_KT; ++kk) acc[kk] = make_float2(0.f, 0.f);
        const float2 *g = sg + np + nn * s;
        const float2 *u = sU + js * nw;
        for (int mp = 0; mp < nw; ++mp) {
          const float2 um = u[mp];
#pragma unroll
          for (int kk = 0; kk < ROT_KT; ++kk) cfmaf(acc[kk], um, g[kk * pc + nw * mp]);
        }
        float pl[4][ROT_KT];
#pragma unroll
        for (int kk = 0; kk < ROT_KT; ++kk) {
          const float2 ph = sph[kk];
          float hr, lr, hi, li;
          split2((double)(ph.x * acc[kk].x - ph.y * acc[kk].y), hr, lr);
          split2((double)(ph.x * acc[kk].y + ph.y * acc[kk].x), hi, li);
          pl[0][kk] = hr;
          pl[1][kk] = hi;
          pl[2][kk] = lr;
          pl[3][kk] = li;
        }
        const int64_t col = (int64_t)(j0 + js) * ncol + np + nw * (s0 + s);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float4 *dst = (float4 *)(Bp + q * plane + col * Kp2 + kp0);
          dst[0] = make_float4(pl[q][0], pl[q][1], pl[q][2], pl[q][3]);
          dst[1] = make_float4(pl[q][4], pl[q][5], pl[q][6], pl[q][7]);
        }
      }
    }
  }
}

__global__ void k_kinv(int n, const int *kpos, int *kinv) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) kinv[kpos[r]] = r;
}

// -------------------------------------------- split-form rate epilogue
struct QTab {
  const float *cx;     // [q][s]: const_tp * g2unitfactor / (2 omega) if omega >= 0.5 meV else 0
  const float *bose;   // [q][s]
  const float4 *wv;    // [q][s]: omega / sigma as a double-float, e^(omega / kT) (wv_pack)
};


__global__ void k_to_f2(int64_t n, const double2 *a, float2 *b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

// Occupation factor of the phonon-side Y, f(x) (1 - f(x + y)) / (1 + n(y)) with
// x = (E - mu)/kT, y = omega/kT (interactions.f90:1838-1839, 1866), in FP32
// from exponentials taken in FP64: 1 - f(x + y) = 1 / (1 + e^-x e^-y),
// 1 / (1 + n) = 1 - e^-y and e^-y = n / (1 + n).  No exponent argument is
// rounded to FP32, so the exponentially small tails away from mu keep their
// relative accuracy.  YOcc holds the per-state part.
struct YOcc {
  float f1;    // f(x)
  float emx;   // e^-x, finite
};
__device__ __forceinline__ YOcc y_occ(double E, double chempot, double kT) {
  const double ex = exp(-(E - chempot) / kT);
  YOcc o;
  o.f1 = (float)(1.0 / (1.0 + 1.0 / ex));
  o.emx = (float)fmin(ex, 3.0e38);
  return o;
}
// Y / (|g|^2 cx delta) of one vertex, bose = n(y): f1 * ib / (1 + emx e^-y)
__device__ __forceinline__ float y_factor(const YOcc &o, float bose) {
  const float ib = 1.0f / (1.0f + bose);
  return o.f1 * ib / (1.0f + o.emx * (bose * ib));
}

// ---- occupation and delta factors of one vertex, split epilogues ----
// The exponents of the Gaussian and of the Fermi factors reach tens to hundreds
// in the tails, where an FP32 argument's rounding (6e-8 relative) becomes a
// relative error of the exponential as large as the argument times 6e-8.  So
// every argument is carried as a double-float (hi + lo, |lo| <= ulp(hi) / 2,
// Dekker / Knuth error-free transformations), the exponential is taken of the
// hi part with the accurate expf and corrected by (1 + lo); the result is
// then accurate to a few FP32 ulps whatever the argument.
struct F2 {
  float hi, lo;
};
__host__ __device__ __forceinline__ F2 f2_of(double x) {
  const float h = (float)x;
  return F2{h, (float)(x - (double)h)};
}
// a + b exactly as hi + lo (Knuth's two-sum)
__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return F2{s, e};
}
// (a + b) for double-floats, to about 2^-44 relative
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  F2 s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return s;
}
// t^2 / 2 for a double-float t (the hi product's rounding error by FMA)
__device__ __forceinline__ F2 f2_half_sq(F2 t) {
  const float p = __fmul_rn(t.hi, t.hi);
  const float e = __fmaf_rn(t.hi, t.hi, -p);
  return F2{0.5f * p, 0.5f * __fmaf_rn(2.0f * t.hi, t.lo, e)};
}
// a b for double-floats, to about 2^-46 relative (the hi product's error by FMA)
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p)));
  const float s = __fadd_rn(p, e);
  return F2{s, __fadd_rn(e, __fsub_rn(p, s))};
}
// e^(hi + lo)
__device__ __forceinline__ float f2_exp(F2 a) { return __fmul_rn(expf(a.hi), __fadd_rn(1.0f, a.lo)); }

// The phonon side's Gaussian factors are formed scaled by 2^64
// (e^(64 ln 2 - t^2/2)), so that its sums keep the tails down to e^-131 in
// FP32's range; the electron side's X+- use unscaled ones.
constexpr float LN2X64_HI = 44.361419677734375f, LN2X64_LO = -1.2189786957605975e-07f;
constexpr float TWO_M64 = 5.421010862427522e-20f;   // 2^-64, exact
constexpr double TWO_M64D = 5.421010862427522e-20;

// Per-mode inputs: w = omega / sigma as a double-float and e^(omega / kT)
// (from FP64, clamped to FP32's range).
__host__ __device__ __forceinline__ float4 wv_pack(double w, double v) {
  const F2 a = f2_of(w);
  return make_float4(a.hi, a.lo, (float)fmin(exp(v), 3.0e38), 0.f);
}

struct VtxF {
  float ap, am;   // n + f(E + omega), n + 1 - f(E - omega)
  float dp;       // delta(E' - E - omega) (= the phonon side's delta(E' - omega - E)), x 2^64 if SHIFT
  float dm;       // delta(E' - E + omega), x 2^64 if SHIFT
};
// dn = (E - E') / sigma (double-float); ex = e^x, emx = e^-x with x = (E -
// mu) / kT (FP64 exponentials, clamped to FP32's range); wv (wv_pack) of the
// mode; bose = n(omega); dnorm = 1 / (sigma sqrt(2 pi) N_k).  The Fermi
// factors need no exponential here: f(E + omega) = 1 / (1 + e^x e^v), and
// 1 + n - f(E - omega) = n + 1 / (1 + e^-x e^v), which has no cancellation
// when f(E - omega) is close to 1.
template <bool SHIFT>
__device__ __forceinline__ VtxF vtx_factors(F2 dn, float ex, float emx, float4 wv, float bose, float dnorm) {
  VtxF r;
  const F2 w{wv.x, wv.y};
  const F2 tp = f2_add(dn, w), tm = f2_add(dn, F2{-w.hi, -w.lo});
  const F2 ap = f2_half_sq(tp), am = f2_half_sq(tm);
  if (SHIFT) {
    const F2 sh{LN2X64_HI, LN2X64_LO};
    r.dp = __fmul_rn(dnorm, f2_exp(f2_add(sh, F2{-ap.hi, -ap.lo})));
    r.dm = __fmul_rn(dnorm, f2_exp(f2_add(sh, F2{-am.hi, -am.lo})));
  } else {
    r.dp = __fmul_rn(dnorm, f2_exp(F2{-ap.hi, -ap.lo}));
    r.dm = __fmul_rn(dnorm, f2_exp(F2{-am.hi, -am.lo}));
  }
  r.ap = __fadd_rn(bose, __frcp_rn(__fmaf_rn(ex, wv.z, 1.0f)));
  r.am = __fadd_rn(bose, __frcp_rn(__fmaf_rn(emx, wv.z, 1.0f)));
  return r;
}
// X+ + X- of one vertex: |g|^2 cx (n + f) delta+ + |g|^2 cx (n + 1 - f) delta-.
// Every rounding is explicit, so that the fused kernel's parameter sets and a
// lone request form the same bits from the same inputs.
__device__ __forceinline__ float vtx_x(float g2c, const VtxF &f, float &xp, float &xm) {
  xp = __fmul_rn(__fmul_rn(g2c, f.ap), f.dp);
  xm = __fmul_rn(__fmul_rn(g2c, f.am), f.dm);
  return __fadd_rn(xp, xm);
}

__global__ void k_qtab(int n, const double *om, const double *bose, double sigma, double kT, double const_tp,
                       float *cx, float *bs, float4 *wv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double o = om[i];
  cx[i] = (o >= 0.5e-3) ? (float)(const_tp * 0.5 * g2unitfactor / o) : 0.0f;
  bs[i] = (float)bose[i];
  wv[i] = wv_pack(o / sigma, o / kT);
}

// One thread per (k', initial state): G(n',s') from the FP32 GEMM output, the
// U_k' and phonon rotations in FP32, the Gaussian delta and occupations from
// FP64 energy differences scaled to O(1) before rounding, X+- and the pair sum.
__global__ void __launch_bounds__(128) k_epilogue_split(int nwv, int j0, const float *Cr, const float *Ci,
                                                        int64_t ldc, RateParams rp, EpiData d, QTab qt,
                                                        double *partial, int nblk) {
  const int ip = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = j0 + blockIdx.y;
  const int nw = rp.nw, nb = rp.nb, ncol = nw * nb;
  double v = 0.0;
  if (ip < nwv) {
    const int code = d.st_code[j];
    const int i = code / nw, m = code % nw;
    const int p = d.sidx[i], pp = d.widx[ip];
    const double E = d.ens[(size_t)p * nw + m];
    const float ex = (float)fmin(exp((E - rp.chempot) / (kB * rp.T)), 3.0e38);
    const double inv_sig = 1.0 / rp.sigma;
    const float dnorm = (float)((1.0 / sqrt(2.0 * 3.141592653589793)) / rp.sigma * rp.inv_nk);
    int a1 = p % rp.mesh[0], a2 = (p / rp.mesh[0]) % rp.mesh[1], a3 = p / (rp.mesh[0] * rp.mesh[1]);
    int b1 = pp % rp.mesh[0], b2 = (pp / rp.mesh[0]) % rp.mesh[1], b3 = pp / (rp.mesh[0] * rp.mesh[1]);
    const int q = (int)(floormod(b1 - a1, rp.mesh[0]) +
                        rp.mesh[0] * (floormod(b2 - a2, rp.mesh[1]) + rp.mesh[1] * floormod(b3 - a3, rp.mesh[2])));
    const int64_t base = (int64_t)ip * ldc + (int64_t)(j - j0) * ncol;
    const bool ph = d.phr || d.yv;
    const YOcc yo = y_occ(E, rp.chempot, kB * rp.T);   // also e^-x of the Fermi factors
    float acc = 0.0f;
    int rank_n = 0;
    for (int n = 0; n < nw; ++n) {
      const double eps = d.ens[(size_t)pp * nw + n];
      if (fabs(eps - rp.enref) > rp.fsthick) continue;
      const float2 *Ukp = d.Uf + ((size_t)pp * nw + n) * nw;
      float2 h[32];
      for (int s = 0; s < nb; ++s) {
        float2 a = make_float2(0.f, 0.f);
        for (int np = 0; np < nw; ++np) {
          int64_t o = base + np + nw * s;
          cfmaf_cj(a, Ukp[np], make_float2(Cr[o], Ci[o]));
        }
        h[s] = a;
      }
      float2 unm = make_float2(0.f, 0.f);   // <U_k'[n]|U_k[m]>, polar crystals
      if (d.glpf) {
        const float2 *Uk = d.Uf + ((size_t)p * nw + m) * nw;
        for (int c = 0; c < nw; ++c) cfmaf_cj(unm, Ukp[c], Uk[c]);
      }
      const F2 dn = f2_of((E - eps) * inv_sig);
      for (int s = 0; s < nb; ++s) {
        const int qs = q * nb + s;
        const float2 *u = d.uf + (size_t)qs * nb;
        float2 g = make_float2(0.f, 0.f);
        for (int sp = 0; sp < nb; ++sp) cfmaf(g, u[sp], h[sp]);
        if (d.glpf) cfmaf(g, d.glpf[qs], unm);   // long-range term (wannier.f90:998-1006)
        const float g2c = (g.x * g.x + g.y * g.y) * qt.cx[qs];
        const VtxF f = vtx_factors<true>(dn, ex, yo.emx, qt.wv[qs], qt.bose[qs], dnorm);
        const float xp = g2c * f.ap * (f.dp * TWO_M64);
        const float xm = g2c * f.am * (f.dm * TWO_M64);
        acc += xp + xm;
        // Y, scaled by 2^64: the Gaussian is even, so delta(E' - omega - E) is dp
        const float y = ph ? g2c * f.dp * y_factor(yo, qt.bose[qs]) : 0.f;
        if (d.phr && y != 0.f) atomicAdd(d.phr + q + (size_t)rp.N * s, d.ph_scale * TWO_M64D * (double)y);
        if (d.g2) {
          int64_t off = (int64_t)j * d.per_state + ((int64_t)d.cum[ip] + rank_n) * nb + s;
          if (off < d.cap) {
            const double om = d.om[qs];
            d.g2[off] = (om == 0.0) ? 0.0 : 0.5 * (double)(g.x * g.x + g.y * g.y) / om * g2unitfactor;
            d.xp[off] = xp;
            d.xm[off] = xm;
            if (d.yv) d.yv[off] = TWO_M64D * (double)y;
          }
        }
      }
      rank_n++;
    }
    v = (double)acc;
  }
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

// Split-form epilogue, one block per 128 consecutive k' rows and a set of
// states: for each state the block stages the rows' 48 complex Rp sums in
// shared memory with coalesced loads, then each thread forms its (k', state)
// pair exactly as k_epilogue_split does.  Block partials are reduced in a fixed
// order (deterministic).
constexpr int EPI_ROWS = 128;

// NW, NB: band and mode counts fixed at compile time (the per-thread arrays then
// live in registers), or 0 to read them from rp.
template <int NW, int NB>
__global__ void __launch_bounds__(EPI_ROWS) k_epilogue_split2(int nwv, int j0, int jend, int spb, const float *Cr,
                                                              const float *Ci, int64_t ldc, RateParams rp,
                                                              EpiData d, QTab qt, double *partial, int nblk) {
  extern __shared__ float esm[];
  const int nw = NW ? NW : rp.nw, nb = NB ? NB : rp.nb, ncol = nw * nb, ld = ncol + 1;
  constexpr int AW = NW ? NW : 32, AB = NB ? NB : 32;
  float *sr = esm, *si = esm + EPI_ROWS * ld;
  __shared__ double wsum[EPI_ROWS / 32];
  const int row = threadIdx.x;
  const int ip0 = blockIdx.x * EPI_ROWS, ip = ip0 + row;
  const bool live = ip < nwv;
  // row-level data, loaded once for all states of the block
  int pp = 0, b1 = 0, b2 = 0, b3 = 0;
  if (live) {
    pp = d.widx[ip];
    b1 = pp % rp.mesh[0];
    b2 = (pp / rp.mesh[0]) % rp.mesh[1];
    b3 = pp / (rp.mesh[0] * rp.mesh[1]);
  }
  const double inv_sig = 1.0 / rp.sigma;
  const float dnorm = (float)((1.0 / sqrt(2.0 * 3.141592653589793)) / rp.sigma * rp.inv_nk);
  const int jb0 = j0 + blockIdx.y * spb;
  const int jb1 = min(jend, jb0 + spb);
  for (int j = jb0; j < jb1; ++j) {
    __syncthreads();
    const int64_t cbase = (int64_t)(j - j0) * ncol;
    if ((ncol & 3) == 0) {
      // 16-byte streaming loads, four rows' worth in flight per thread before
      // the shared stores (rows < Mp exist in the chunk; ldc and the state's
      // column offset are multiples of 4)
      const int nc4 = ncol >> 2, tot = EPI_ROWS * nc4;
      for (int t0 = threadIdx.x; t0 < tot; t0 += 4 * EPI_ROWS) {
        float4 a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * EPI_ROWS;
          if (t < tot) {
            const int r = t / nc4, c4 = t - r * nc4;
            const int64_t o = (int64_t)(ip0 + r) * ldc + cbase + 4 * c4;
            a[u] = __ldcs((const float4 *)(Cr + o));
            b[u] = __ldcs((const float4 *)(Ci + o));
          }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + u * EPI_ROWS;
          if (t < tot) {
            const int r = t / nc4, c = 4 * (t - r * nc4);
            float *dr = sr + r * ld + c, *di = si + r * ld + c;
            dr[0] = a[u].x, dr[1] = a[u].y, dr[2] = a[u].z, dr[3] = a[u].w;
            di[0] = b[u].x, di[1] = b[u].y, di[2] = b[u].z, di[3] = b[u].w;
          }
        }
      }
    } else {
      for (int t = threadIdx.x; t < EPI_ROWS * ncol; t += EPI_ROWS) {
        const int r = t / ncol, c = t % ncol;
        const int64_t o = (int64_t)(ip0 + r) * ldc + cbase + c;    // rows < Mp exist in the chunk
        sr[r * ld + c] = Cr[o];
        si[r * ld + c] = Ci[o];
      }
    }
    __syncthreads();
    double v = 0.0;
    if (live) {
      const int code = d.st_code[j];
      const int i = code / nw, m = code % nw;
      const int p = d.sidx[i];
      const double E = d.ens[(size_t)p * nw + m];
      const float ex = (float)fmin(exp((E - rp.chempot) / (kB * rp.T)), 3.0e38);
      const int a1 = p % rp.mesh[0], a2 = (p / rp.mesh[0]) % rp.mesh[1], a3 = p / (rp.mesh[0] * rp.mesh[1]);
      const int q = (int)(floormod(b1 - a1, rp.mesh[0]) +
                          rp.mesh[0] * (floormod(b2 - a2, rp.mesh[1]) + rp.mesh[1] * floormod(b3 - a3, rp.mesh[2])));
      const float *gr = sr + row * ld, *gi = si + row * ld;
      const bool ph = d.phr || d.yv;
      const YOcc yo = y_occ(E, rp.chempot, kB * rp.T);   // also e^-x of the Fermi factors
      float acc = 0.0f;
      int rank_n = 0;
      for (int n = 0; n < nw; ++n) {
        const double eps = d.ens[(size_t)pp * nw + n];
        if (fabs(eps - rp.enref) > rp.fsthick) continue;
        const float2 *Ukp = d.Uf + ((size_t)pp * nw + n) * nw;
        float2 uk[AW];
#pragma unroll
        for (int np = 0; np < AW; ++np)
          if (np < nw) uk[np] = Ukp[np];
        float2 unm = make_float2(0.f, 0.f);   // <U_k'[n]|U_k[m]>, polar crystals
        if (d.glpf) {
          const float2 *Uk = d.Uf + ((size_t)p * nw + m) * nw;
#pragma unroll
          for (int c = 0; c < AW; ++c)
            if (c < nw) cfmaf_cj(unm, uk[c], Uk[c]);
        }
        float2 h[AB];
#pragma unroll
        for (int s = 0; s < AB; ++s) {
          if (s >= nb) break;
          float2 a = make_float2(0.f, 0.f);
#pragma unroll
          for (int np = 0; np < AW; ++np)
            if (np < nw) cfmaf_cj(a, uk[np], make_float2(gr[np + nw * s], gi[np + nw * s]));
          h[s] = a;
        }
        const F2 dn = f2_of((E - eps) * inv_sig);
#pragma unroll
        for (int s = 0; s < AB; ++s) {
          if (s >= nb) break;
          const int qs = q * nb + s;
          const float2 *u = d.uf + (size_t)qs * nb;
          float2 g = make_float2(0.f, 0.f);
#pragma unroll
          for (int sp = 0; sp < AB; ++sp)
            if (sp < nb) cfmaf(g, u[sp], h[sp]);
          if (d.glpf) cfmaf(g, d.glpf[qs], unm);   // long-range term (wannier.f90:998-1006)
          const float g2c = (g.x * g.x + g.y * g.y) * qt.cx[qs];
          const VtxF f = vtx_factors<true>(dn, ex, yo.emx, qt.wv[qs], qt.bose[qs], dnorm);
          const float xp = g2c * f.ap * (f.dp * TWO_M64);
          const float xm = g2c * f.am * (f.dm * TWO_M64);
          acc += xp + xm;
          // Y, scaled by 2^64: the Gaussian is even, so delta(E' - omega - E) is dp
          const float y = ph ? g2c * f.dp * y_factor(yo, qt.bose[qs]) : 0.f;
          if (d.phr && y != 0.f) atomicAdd(d.phr + q + (size_t)rp.N * s, d.ph_scale * TWO_M64D * (double)y);
          if (d.g2) {
            int64_t off = (int64_t)j * d.per_state + ((int64_t)d.cum[ip] + rank_n) * nb + s;
            if (off < d.cap) {
              const double om = d.om[qs];
              d.g2[off] = (om == 0.0) ? 0.0 : 0.5 * (double)(g.x * g.x + g.y * g.y) / om * g2unitfactor;
              d.xp[off] = xp;
              d.xm[off] = xm;
              if (d.yv) d.yv[off] = TWO_M64D * (double)y;
            }
          }
        }
        rank_n++;
      }
      v = (double)acc;
    }
    // fixed-order block reduction: warp shuffle tree, then the 4 warp sums in order
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double sacc = 0.0;
      for (int w = 0; w < EPI_ROWS / 32; ++w) sacc += wsum[w];
      partial[(size_t)j * nblk + blockIdx.x] = sacc;
    }
  }
}

// Generic-shape split epilogue without shared-memory staging: one thread per
// (k' row, state), EPI_ROWS consecutive rows of one state per block.  A thread
// reads its row's nw x nb complex Rp sums straight from the GEMM output, which
// the GEMM wrote interleaved by 32 rows in 4-column groups (GemmArgs::ileave):
// each float4 load of a warp is 512 consecutive bytes.  NW bands fixed
// at compile time (the band and mode arrays then live in registers), nb <= EPR_NB.
constexpr int EPR_NB = 18;

template <int NW, int NB>
__global__ void __launch_bounds__(EPI_ROWS, NW * NB <= 96 ? 4 : 3) k_epilogue_rows(int nwv, int j0, const float *Cr, const float *Ci,
                                                            int64_t ldc, RateParams rp, EpiData d, QTab qt,
                                                            double *partial, int nblk) {
  static_assert(NW % 4 == 0, "16-byte row loads");
  __shared__ double wsum[EPI_ROWS / 32];
  const int ip = blockIdx.x * EPI_ROWS + threadIdx.x;
  const int j = j0 + blockIdx.y;
  const int nb = rp.nb, ncol = NW * nb;
  double v = 0.0;
  if (ip < nwv) {
    const int code = d.st_code[j];
    const int i = code / NW, m = code % NW;
    const int p = d.sidx[i], pp = d.widx[ip];
    const double E = d.ens[(size_t)p * NW + m];
    const float ex = (float)fmin(exp((E - rp.chempot) / (kB * rp.T)), 3.0e38);
    const double inv_sig = 1.0 / rp.sigma;
    const float dnorm = (float)((1.0 / sqrt(2.0 * 3.141592653589793)) / rp.sigma * rp.inv_nk);
    const int a1 = p % rp.mesh[0], a2 = (p / rp.mesh[0]) % rp.mesh[1], a3 = p / (rp.mesh[0] * rp.mesh[1]);
    const int b1 = pp % rp.mesh[0], b2 = (pp / rp.mesh[0]) % rp.mesh[1], b3 = pp / (rp.mesh[0] * rp.mesh[1]);
    const int q = (int)(floormod(b1 - a1, rp.mesh[0]) +
                        rp.mesh[0] * (floormod(b2 - a2, rp.mesh[1]) + rp.mesh[1] * floormod(b3 - a3, rp.mesh[2])));
    // the GEMM output interleaved by 32 rows in groups of 4 columns: columns c..c+3
    // (c % 4 = 0) of this row are the float4 at rr + 32 c, so that a warp's 32 rows
    // read 512 consecutive bytes per group
    const int64_t base = ((int64_t)(ip >> 5) * ldc + (int64_t)(j - j0) * ncol) * 32 + 4 * (ip & 31);
    const float *rr = Cr + base, *ri = Ci + base;
    const bool ph = d.phr || d.yv;
    const YOcc yo = y_occ(E, rp.chempot, kB * rp.T);   // also e^-x of the Fermi factors
    float acc = 0.0f;
    int rank_n = 0;
    for (int n = 0; n < NW; ++n) {
      const double eps = d.ens[(size_t)pp * NW + n];
      if (fabs(eps - rp.enref) > rp.fsthick) continue;
      const float2 *Ukp = d.Uf + ((size_t)pp * NW + n) * NW;
      float2 uk[NW];
#pragma unroll
      for (int c = 0; c < NW; ++c) uk[c] = Ukp[c];
      float2 unm = make_float2(0.f, 0.f);   // <U_k'[n]|U_k[m]>, polar crystals
      if (d.glpf) {
        const float2 *Uk = d.Uf + ((size_t)p * NW + m) * NW;
#pragma unroll
        for (int c = 0; c < NW; ++c) cfmaf_cj(unm, uk[c], Uk[c]);
      }
      float2 h[NB];
#pragma unroll
      for (int s = 0; s < NB; ++s) {
        if (s >= nb) break;
        float2 a = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < NW; c += 4) {
          const float4 xr = __ldg((const float4 *)(rr + 32 * (c + NW * s)));
          const float4 xi = __ldg((const float4 *)(ri + 32 * (c + NW * s)));
          cfmaf_cj(a, uk[c], make_float2(xr.x, xi.x));
          cfmaf_cj(a, uk[c + 1], make_float2(xr.y, xi.y));
          cfmaf_cj(a, uk[c + 2], make_float2(xr.z, xi.z));
          cfmaf_cj(a, uk[c + 3], make_float2(xr.w, xi.w));
        }
        h[s] = a;
      }
      const F2 dn = f2_of((E - eps) * inv_sig);
#pragma unroll
      for (int s = 0; s < NB; ++s) {
        if (s >= nb) break;
        const int qs = q * nb + s;
        const float2 *u = d.uf + (size_t)qs * nb;
        float2 g = make_float2(0.f, 0.f);
#pragma unroll
        for (int sp = 0; sp < NB; ++sp)
          if (sp < nb) cfmaf(g, u[sp], h[sp]);
        if (d.glpf) cfmaf(g, d.glpf[qs], unm);   // long-range term (wannier.f90:998-1006)
        const float g2c = (g.x * g.x + g.y * g.y) * qt.cx[qs];
        const VtxF f = vtx_factors<true>(dn, ex, yo.emx, qt.wv[qs], qt.bose[qs], dnorm);
        const float xp = g2c * f.ap * (f.dp * TWO_M64);
        const float xm = g2c * f.am * (f.dm * TWO_M64);
        acc += xp + xm;
        // Y, scaled by 2^64: the Gaussian is even, so delta(E' - omega - E) is dp
        const float y = ph ? g2c * f.dp * y_factor(yo, qt.bose[qs]) : 0.f;
        if (d.phr && y != 0.f) atomicAdd(d.phr + q + (size_t)rp.N * s, d.ph_scale * TWO_M64D * (double)y);
        if (d.g2) {
          int64_t off = (int64_t)j * d.per_state + ((int64_t)d.cum[ip] + rank_n) * nb + s;
          if (off < d.cap) {
            const double om = d.om[qs];
            d.g2[off] = (om == 0.0) ? 0.0 : 0.5 * (double)(g.x * g.x + g.y * g.y) / om * g2unitfactor;
            d.xp[off] = xp;
            d.xm[off] = xm;
            if (d.yv) d.yv[off] = TWO_M64D * (double)y;
          }
        }
      }
      rank_n++;
    }
    v = (double)acc;
  }
  // fixed-order block reduction: warp shuffle tree, then the warp sums in order
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sacc = 0.0;
    for (int w = 0; w < EPI_ROWS / 32; ++w) sacc += wsum[w];
    partial[(size_t)j * nblk + blockIdx.x] = sacc;
  }
}

// ------------------------------------- stage B fused with the rate epilogue
// For nw = 8, nb = 6 and the Gaussian delta the Rp-Fourier GEMM and the rate
// epilogue run as one persistent kernel, so that the 48 complex Rp sums of a
// (k', state) pair never leave the SM.  A tile is 128 window k' rows (TMEM
// lanes) x 2 whole initial states (96 columns = 2 x 48 of (n', s')).  The
// state operand is stored as six planes (-hi_im, hi_re, hi_im, -lo_im, lo_re,
// lo_im), so that each complex product is two MMAs of N = 192 over adjacent
// planes; the main and correction accumulators (real | imaginary, 192 columns
// each) start at TMEM columns 0 and 256.  Warp roles: warp 0 lane 0 issues TMA, warp 1 lane 0 issues
// tcgen05.mma, warps 2..9 are the epilogue: warp w drains TMEM lane quadrant
// w % 4 for state slot (w - 2) / 4 of the tile.  A drain reads the state's 48
// columns 8 at a time and forms h(n, s') = sum_n' conj(U_k'[n][n']) G(n', s')
// for the first two window bands of its k' row in registers (further bands, rare,
// are finished while the accumulators are still held), releases TMEM, and then
// forms the vertices while the MMAs of the next tile run.  Each warp reduces its
// 32 rows' rate contributions in a fixed order and writes one partial per
// (state, 32-row block): partial[j][mt * 4 + quadrant].
constexpr int FBN = 96;                                   // state-operand rows per tile (2 states)
constexpr int F_BPLANE = FBN * BK * 4;                    // 6 KB
constexpr int F_STAGE = 4 * PLANE_BYTES + 6 * F_BPLANE;   // 68 KB
constexpr int F_STAGES = 3;
constexpr int F_THREADS = 320;                            // 10 warps
constexpr int F_EPI_THREADS = 256;
constexpr int F_SMEM = F_STAGES * F_STAGE + 1024 + 256;

// Field-major tables of the fused epilogue.  Window k' rows are nearly
// consecutive mesh points, so the 32 rows of a warp read nearly consecutive
// entries of each table (a few cache lines per load instead of 32).
struct StateRec {      // per initial state j
  double E;            // eV
  float ex;            // e^x, x = (E - mu) / kT (FP64 exponential, clamped); e^-x is yo.emx
  int apack;           // mesh coordinates of k: a1 | a2 << 10 | a3 << 20
  YOcc yo;             // per-state part of the phonon-side occupation factor
  int urow;            // p * 8 + m: the state's U_k row in the fp32 eigenvector table
};

// The row and q tables are blocked by 32: entry (i, field) sits at
// ((i >> 5) * nfields + field) * 32 + (i & 31), so a warp's 32 rows read
// consecutive words of each field and the field offsets are constants.
struct FusedTabs {
  const int4 *row;         // [MpB] (mesh index, window-band mask, first final-state rank, packed coordinates)
  const StateRec *state;   // [nst]
  const float4 *U4;        // row-blocked, fields n * 4 + h: U_k'[n][2h], U_k'[n][2h + 1] (fp32 complex)
  const double *ensw;      // row-blocked, fields n: window-k' band energies
  const float4 *rec;       // q-blocked, fields s * 5 + f: u[s][0..1], u[s][2..3], u[s][4..5], (cx, bose, -, -),
                           // (w as a double-float, e^(omega / kT): wv_pack)
  const float2 *glb;       // polar crystals: q-blocked, fields s: long_range_prefac(q, u_s) (else null)
  int MpB, N;
};

__host__ __device__ __forceinline__ int64_t blk32(int64_t i, int nf, int f) {
  return ((i >> 5) * nf + f) * 32 + (i & 31);
}

struct FusedArgs {
  int mtiles, ntiles, nkb;
  int bands;                  // m-bands of the tile walk (fb_tile)
  int t0, t1;                 // tile pairs [t0, t1) of this launch
  int64_t Astride, Bstride;   // rows between planes of the phase / state operand stacks
  int nwv, nst;
  int *err;
  double *partial;
  int nblk;
};

// Sets 1..n-1 of a merged request (RateSets) in the fused kernel's layouts.
struct FusedSets {
  int n;                           // 1: the request alone
  float isg_hi[MAX_SETS], isg_lo[MAX_SETS];   // 1 / sigma_p as a double-float
  float dnorm[MAX_SETS];           // 1 / (sigma_p sqrt(2 pi) N_k)
  const float2 *occ;               // [(p - 1) * nst + j]: (e^x, e^-x), x = (E_j - mu_p) / kT_p, as StateRec / YOcc
  const float4 *mode;              // set p at (p - 1) * mode_stride, q-blocked, fields s:
  int64_t mode_stride;             //   (w = omega / sigma_p as a double-float, e^(omega / kT_p), n_p(omega))
  double *partial[MAX_SETS];
};

__global__ void k_fused_set_tabs(int nst, int N, const StateRec *srec, double chempot, double kT, const float *bs,
                                 const float4 *wv, float2 *occ, float4 *mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nst) {
    const double E = srec[i].E;
    occ[i] = make_float2((float)fmin(exp((E - chempot) / kT), 3.0e38), y_occ(E, chempot, kT).emx);
  }
  if (i < N * 6) {
    const float4 w = wv[i];
    mode[blk32(i / 6, 6, i % 6)] = make_float4(w.x, w.y, w.z, bs[i]);
  }
}

__global__ void k_fused_rows(int nwv, int MpB, const int *widx, const double *ens, const float2 *Uf, const int *cum,
                             double enref, double fsthick, int m0, int m1, int4 *row, float4 *U4, double *ensw) {
  const int ip = blockIdx.x * blockDim.x + threadIdx.x;
  if (ip >= MpB) return;
  if (ip >= nwv) {
    row[ip] = make_int4(0, 0, 0, 0);
    for (int n = 0; n < 8; ++n) {
      ensw[blk32(ip, 8, n)] = 0.0;
      for (int h = 0; h < 4; ++h) U4[blk32(ip, 32, n * 4 + h)] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return;
  }
  const int pp = widx[ip];
  int wmask = 0;
  for (int n = 0; n < 8; ++n) {
    const double e = ens[(size_t)pp * 8 + n];
    ensw[blk32(ip, 8, n)] = e;
    wmask |= (fabs(e - enref) <= fsthick) << n;
    for (int h = 0; h < 4; ++h) {
      const float2 a = Uf[((size_t)pp * 8 + n) * 8 + 2 * h], b = Uf[((size_t)pp * 8 + n) * 8 + 2 * h + 1];
      U4[blk32(ip, 32, n * 4 + h)] = make_float4(a.x, a.y, b.x, b.y);
    }
  }
  const int b1 = pp % m0, b2 = (pp / m0) % m1, b3 = pp / (m0 * m1);
  row[ip] = make_int4(pp, wmask, cum ? cum[ip] : 0, b1 | (b2 << 10) | (b3 << 20));
}

__global__ void k_fused_states(int nst, const int *st_code, const int *widx, const double *ens, double chempot,
                               double kT, int m0, int m1, StateRec *out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nst) return;
  const int code = st_code[j];
  const int p = widx[code >> 3];
  StateRec r;
  r.E = ens[(size_t)p * 8 + (code & 7)];
  r.ex = (float)fmin(exp((r.E - chempot) / kT), 3.0e38);
  r.yo = y_occ(r.E, chempot, kT);
  r.urow = p * 8 + (code & 7);
  const int a1 = p % m0, a2 = (p / m0) % m1, a3 = p / (m0 * m1);
  r.apack = a1 | (a2 << 10) | (a3 << 20);
  out[j] = r;
}

__global__ void k_fused_recs(int N, const float2 *uf, const float *cx, const float *bs, const float4 *wv,
                             float4 *rec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;   // (q, s) = (i / 6, i % 6)
  if (i >= N * 6) return;
  const int q = i / 6, s = i % 6;
  const float2 *u = uf + (size_t)i * 6;
  rec[blk32(q, 30, s * 5 + 0)] = make_float4(u[0].x, u[0].y, u[1].x, u[1].y);
  rec[blk32(q, 30, s * 5 + 1)] = make_float4(u[2].x, u[2].y, u[3].x, u[3].y);
  rec[blk32(q, 30, s * 5 + 2)] = make_float4(u[4].x, u[4].y, u[5].x, u[5].y);
  rec[blk32(q, 30, s * 5 + 3)] = make_float4(cx[i], bs[i], 0.f, 0.f);
  rec[blk32(q, 30, s * 5 + 4)] = wv[i];
}

__global__ void k_fused_glp(int N, const float2 *glpf, float2 *glb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;   // (q, s)
  if (i >= N * 6) return;
  glb[blk32(i / 6, 6, i % 6)] = glpf[i];
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t *r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

// 8 complex columns at c0 (main + correction combined); the main and correction
// accumulators start at TMEM columns 0 and 256, their imaginary halves IM later
template <int IM>
__device__ __forceinline__ void fused_load_one(uint32_t tr, int c0, float *gre, float *gim) {
  uint32_t a[8], b[8], c[8], e[8];
  tmem_ld8_nowait(tr + c0, a);
  tmem_ld8_nowait(tr + IM + c0, b);
  tmem_ld8_nowait(tr + 256 + c0, c);
  tmem_ld8_nowait(tr + 256 + IM + c0, e);
  tmem_wait_ld();
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    gre[i] = __uint_as_float(a[i]) + __uint_as_float(c[i]);
    gim[i] = __uint_as_float(b[i]) + __uint_as_float(e[i]);
  }
}

// U_k' row n of this lane's k' row (ub = the lane's entry of field 0)
__device__ __forceinline__ void load_urow(const float4 *ub, int n, float2 *u) {
  const float4 *un = ub + n * 128;
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    const float4 t = __ldg(un + h * 32);
    u[2 * h] = make_float2(t.x, t.y);
    u[2 * h + 1] = make_float2(t.z, t.w);
  }
}

// h(s') = sum_n' conj(u[n']) G(n', s') from the 8 loaded columns of s'
__device__ __forceinline__ float2 hrot(const float2 *u, const float *gre, const float *gim) {
  float2 a = make_float2(0.f, 0.f);
#pragma unroll
  for (int np = 0; np < 8; ++np) cfmaf_cj(a, u[np], make_float2(gre[np], gim[np]));
  return a;
}

// the six vertices (s) of one (k', n) final state for one initial state; returns X+ + X-
// rec = the lane's entry of field 0 of q's block: fields 32 float4 apart.
// dn = (E - E_n') / sigma as a double-float, ex = e^((E - mu) / kT).
// PH: also ys[s] += |g|^2 cx delta * 2^64, the n-dependent part of Y; its
// occupation factor depends on the initial state and the mode only and is
// applied once per pair (y_factor).
// POLAR: g += long_range_prefac(q, u_s) * <U_k'[n]|U_k[m]> (glb = the lane's
// entry of field 0 of q's block of the prefactor table, unm the overlap).
// OUT: also g2o[s] = |g|^2 cx of the six vertices (the parameter sets reuse them).
template <bool PH, bool POLAR, bool OUT = false>
__device__ __forceinline__ float fused_vertices(const float2 *h, const float4 *rec, F2 dn, float ex,
                                                float dnorm, const EpiData &d, int64_t voff, int q,
                                                const YOcc &yo, float *ys, const float2 *glb, float2 unm,
                                                float *g2o = nullptr) {
  float acc = 0.f;
#pragma unroll
  for (int s = 0; s < 6; ++s) {
    const float4 u01 = __ldg(rec + (5 * s) * 32), u23 = __ldg(rec + (5 * s + 1) * 32),
                 u45 = __ldg(rec + (5 * s + 2) * 32), sc = __ldg(rec + (5 * s + 3) * 32),
                 wv = __ldg(rec + (5 * s + 4) * 32);
    float2 g = make_float2(0.f, 0.f);
    cfmaf(g, make_float2(u01.x, u01.y), h[0]);
    cfmaf(g, make_float2(u01.z, u01.w), h[1]);
    cfmaf(g, make_float2(u23.x, u23.y), h[2]);
    cfmaf(g, make_float2(u23.z, u23.w), h[3]);
    cfmaf(g, make_float2(u45.x, u45.y), h[4]);
    cfmaf(g, make_float2(u45.z, u45.w), h[5]);
    if (POLAR) cfmaf(g, __ldg(glb + s * 32), unm);
    // sc = (cx, bose, -, -)
    const float g2c = __fmul_rn(__fmaf_rn(g.x, g.x, __fmul_rn(g.y, g.y)), sc.x);
    if (OUT) g2o[s] = g2c;
    // PH: the Gaussians x 2^64 (the phonon side's sums keep their tails)
    const VtxF f = vtx_factors<PH>(dn, ex, yo.emx, wv, sc.y, dnorm);
    float xp, xm;
    if (PH) {
      xp = g2c * f.ap * (f.dp * TWO_M64);
      xm = g2c * f.am * (f.dm * TWO_M64);
      acc += xp + xm;
    } else {
      acc = __fadd_rn(acc, vtx_x(g2c, f, xp, xm));
    }
    if (PH) ys[s] = fmaf(g2c, f.dp, ys[s]);   // the Gaussian is even: delta(E' - omega - E) is dp (x 2^64)
    if (d.g2) {
      const int64_t off = voff + s;
      if (off < d.cap) {
        const double om = d.om[(size_t)q * 6 + s];
        d.g2[off] = (om == 0.0) ? 0.0 : 0.5 * (double)(g.x * g.x + g.y * g.y) / om * g2unitfactor;
        d.xp[off] = xp;
        d.xm[off] = xm;
        if (PH && d.yv) d.yv[off] = TWO_M64D * (double)((g2c * f.dp) * y_factor(yo, sc.y));
      }
    }
  }
  return acc;
}

// The electron side's X+ + X- of one (k', n) final state under another
// parameter set, from the six |g|^2 cx of fused_vertices<..., OUT>: that set's
// dn, e^x, e^-x, dnorm and mode factors (mrec = the lane's entry of field 0 of
// q's block of the set's mode table: (w, e^v, bose)), vertex factors as there.
__device__ __forceinline__ float fused_set_band(const float *g2c, const float4 *mrec, F2 dn, float ex, float emx,
                                                float dnorm) {
  float acc = 0.f;
#pragma unroll
  for (int s = 0; s < 6; ++s) {
    const float4 wb = __ldg(mrec + s * 32);
    const VtxF f = vtx_factors<false>(dn, ex, emx, wb, wb.w, dnorm);
    float xp, xm;
    acc = __fadd_rn(acc, vtx_x(g2c[s], f, xp, xm));
  }
  return acc;
}

// Tile order of the fused kernels.  Tile t of mpairs x ntiles (m-tile pair,
// n-tile) walks the m-pairs in `bands` bands, each band over every n-tile
// before the next band starts, so that only a band's phase tiles have to stay
// in L2 while the streamed operand (stage B: the state operand; stage A: the
// g(Re,Rp) planes) passes: it is read `bands` times from DRAM, the phase planes
// once.  fused_bands picks the count from the phase planes' size.
__device__ __forceinline__ void fb_tile(int t, int mpairs, int ntiles, int bands, int &mp, int &nt) {
  const int m0 = (mpairs + bands - 1) / bands;
  const int band = t / (m0 * ntiles);
  const int r = t - band * m0 * ntiles;
  const int sz = min(m0, mpairs - band * m0);
  mp = band * m0 + r % sz;
  nt = r / sz;
}
// One band per 32 MB of phase planes (at most 4): measured at 24^3 (54 MB of
// planes) 46.8 / 14.8 / 15.7 / 18.2 GB of stage-B DRAM reads for 1 / 2 / 3 / 4
// bands; at 12^3 (7 MB) one band reads half of what two do.
static inline int fused_bands(int64_t phase_bytes, int mpairs) {
  const int64_t b = (phase_bytes + (32ll << 20) - 1) / (32ll << 20);
  return (int)std::max<int64_t>(1, std::min<int64_t>({b, 4, (int64_t)mpairs}));
}

// PH: the phonon side too (Y of every vertex into the ph-e rate of its (q, s)).
// POLAR: the long-range term of polar crystals in every vertex.
// SETS: the electron side's rates under the parameter sets 1..xs.n-1 as well
// (not with PH); each set's partials are formed in the same order as set 0's.
template <bool PH, bool POLAR, bool SETS>
__global__ void __launch_bounds__(F_THREADS, 1)
    k_stageB_fused86(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, FusedArgs g,
                     FusedTabs tb, RateParams rp, EpiData d, FusedSets xs) {
  static_assert(!(PH && SETS), "parameter sets are an electron-side form");
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + F_STAGES * F_STAGE);
  uint64_t *empty = full + F_STAGES;
  uint64_t *tfull = empty + F_STAGES;
  uint64_t *tempty = tfull + 1;
  uint64_t *drain = tempty + 1;
  uint32_t *tslot = (uint32_t *)(drain + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // CTA pairs (clusters of 2) take m-tiles 2x, 2x + 1 of the same state pair:
  // each loads its own phase tile and multicasts three of the six state-operand
  // planes to both; a stage is refilled once both CTAs' MMAs have read it.
  const uint32_t crank = cluster_rank();
  if (threadIdx.x == 0) {
    for (int s = 0; s < F_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 2);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, F_EPI_THREADS);
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  cluster_sync();   // the peer's barriers are initialised before any multicast or remote arrive
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const int mpairs = g.mtiles >> 1;
  (void)mpairs;
  const int cid = blockIdx.x >> 1, ncl = gridDim.x >> 1;

  if (warp == 0) {
    if (lane == 0) {   // ---- TMA producer
      uint64_t keep;
      asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(keep));
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      for (int t = g.t0 + cid; t < g.t1 && ok; t += ncl) {
        int mp, nt;
        fb_tile(t, mpairs, g.ntiles, g.bands, mp, nt);
        const int mt = 2 * mp + (int)crank;
        for (int kb = 0; kb < g.nkb; ++kb) {
          if (!mbar_wait(&empty[stage], phase ^ 1, g.err)) { ok = false; break; }
          uint8_t *sb = smem + stage * F_STAGE;
          mbar_expect_tx(&full[stage], F_STAGE);
#pragma unroll
          for (int p = 0; p < 4; ++p)
            tma_load_2d_hint(sb + p * PLANE_BYTES, &tA, &full[stage], kb * BK, (int)(p * g.Astride + mt * BM), keep);
#pragma unroll
          for (int p = 3 * (int)crank; p < 3 * (int)crank + 3; ++p)
            tma_load_2d_mc(sb + 4 * PLANE_BYTES + p * F_BPLANE, &tB, &full[stage], kb * BK,
                           (int)(p * g.Bstride + nt * FBN), (uint16_t)3);
          if (++stage == F_STAGES) { stage = 0; phase ^= 1; }
        }
      }
      for (int s = 0; s < F_STAGES; ++s) mbar_wait(&empty[stage], phase ^ 1, g.err), stage = (stage + 1) % F_STAGES,
                                           phase ^= (stage == 0);
    }
  } else if (warp == 1) {
    if (lane == 0) {   // ---- MMA issuer
      // one MMA of N = 192 forms (Ar Br | Ar Bi) from B rows [re; im], the next
      // (-Ai Bi | Ai Br) from [-im; re]: the real and imaginary halves of a
      // complex product land side by side in one 192-column accumulator.
      constexpr uint32_t ID2 = idesc_tf32_n(false, 2 * FBN);
      int stage = 0;
      uint32_t phase = 0;
      int it = 0;
      bool ok = true;
      const uint32_t dm = tmem, dc = tmem + 256;   // main, correction (re | im each)
      for (int t = g.t0 + cid; t < g.t1 && ok; t += ncl, ++it) {
        if (!mbar_wait(tempty, (it & 1) ^ 1, g.err)) { ok = false; break; }
        tc_fence_after();
        for (int kb = 0; kb < g.nkb; ++kb) {
          if (!mbar_wait(&full[stage], phase, g.err)) { ok = false; break; }
          tc_fence_after();
          uint8_t *sb = smem + stage * F_STAGE;
#pragma unroll
          for (int ks = 0; ks < BK / 8; ++ks) {
            const int off = ks * 32;
            const uint64_t Ahr = sdesc(sb + 0 * PLANE_BYTES + off), Ahi = sdesc(sb + 1 * PLANE_BYTES + off);
            const uint64_t Alr = sdesc(sb + 2 * PLANE_BYTES + off), Ali = sdesc(sb + 3 * PLANE_BYTES + off);
            uint8_t *bb = sb + 4 * PLANE_BYTES;
            const uint64_t BhN = sdesc(bb + 0 * F_BPLANE + off), BhP = sdesc(bb + 1 * F_BPLANE + off);
            const uint64_t BlN = sdesc(bb + 3 * F_BPLANE + off), BlP = sdesc(bb + 4 * F_BPLANE + off);
            const uint32_t acc = (kb == 0 && ks == 0) ? 0u : 1u;
            umma(dc, Ahr, BlP, ID2, acc);   // hi x lo
            umma(dc, Ahi, BlN, ID2, 1);
            umma(dc, Alr, BhP, ID2, 1);     // lo x hi
            umma(dc, Ali, BhN, ID2, 1);
            const bool nearblk = (kb == g.nkb - 1) && g.nkb > 1;
            const uint32_t dd = nearblk ? dc : dm;
            umma(dd, Ahr, BhP, ID2, nearblk ? 1u : acc);   // hi x hi
            umma(dd, Ahi, BhN, ID2, 1);
          }
          umma_commit_mc(&empty[stage], (uint16_t)3);
          if (++stage == F_STAGES) { stage = 0; phase ^= 1; }
        }
        if (ok) umma_commit(tfull);
      }
      // a wait gave up: let the MMAs already issued retire before TMEM is freed
      if (!ok) {
        umma_commit(drain);
        mbar_wait(drain, 0, g.err);
      }
    }
  } else {   // ---- epilogue: warps 2..9
    const int quad = warp & 3, slot = (warp - 2) >> 2;
    const uint32_t tr = tmem + ((uint32_t)(quad * 32) << 16);
    // dn = (E - E') / sigma as the double-float product of E - E' and 1 / sigma,
    // formed the same way for the parameter sets (FusedSets)
    const F2 isg = f2_of(1.0 / rp.sigma);
    const float dnorm = (float)((1.0 / sqrt(2.0 * 3.141592653589793)) / rp.sigma * rp.inv_nk);
    const int m0 = rp.mesh[0], m1 = rp.mesh[1], m2 = rp.mesh[2];
    int it = 0;
    for (int t = g.t0 + cid; t < g.t1; t += ncl, ++it) {
      int mp, nt;
      fb_tile(t, mpairs, g.ntiles, g.bands, mp, nt);
      const int mt = 2 * mp + (int)crank;
      // ---- row and state data, before the accumulators are ready
      const int ip = mt * BM + quad * 32 + lane;      // < MpB
      const int j = nt * 2 + slot;                    // warp-uniform
      const bool jvalid = j < g.nst;
      const int4 ri = __ldg(tb.row + ip);             // zero for padding rows: no window band
      unsigned wmask = 0;
      int q = 0;
      double E = 0.0;
      float ex = 0.f;
      YOcc yo{0.f, 0.f};
      const float2 *Uk = nullptr;   // the state's U_k[m] (polar)
      if (jvalid) {
        const StateRec sr = tb.state[j];
        E = sr.E;
        ex = sr.ex;
        yo = sr.yo;
        if (POLAR) Uk = d.Uf + (size_t)sr.urow * 8;
        wmask = (unsigned)ri.y;
        const int a1 = sr.apack & 1023, a2 = (sr.apack >> 10) & 1023, a3 = sr.apack >> 20;
        const int b1 = ri.w & 1023, b2 = (ri.w >> 10) & 1023, b3 = ri.w >> 20;
        q = (int)(floormod(b1 - a1, m0) + m0 * (floormod(b2 - a2, m1) + m1 * floormod(b3 - a3, m2)));
      }
      const int nbw = __popc(wmask);
      const int n0 = nbw > 0 ? __ffs(wmask) - 1 : 0;
      const unsigned rest = wmask & (wmask - 1);
      const int n1 = nbw > 1 ? __ffs(rest) - 1 : 0;
      const float4 *ub = tb.U4 + blk32(ip, 32, 0);
      const double *eb = tb.ensw + blk32(ip, 8, 0);
      const float4 *rq = tb.rec + blk32(q, 30, 0);
      float2 u0[8], u1[8];
      if (nbw > 0) load_urow(ub, n0, u0);
      if (nbw > 1) load_urow(ub, n1, u1);
      const float2 *glb = POLAR ? tb.glb + blk32(q, 6, 0) : nullptr;
      float2 unm0 = make_float2(0.f, 0.f), unm1 = make_float2(0.f, 0.f);
      if (POLAR && nbw > 0) {   // <U_k'[n]|U_k[m]> of the first two window bands
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const float2 uk = __ldg(Uk + c);
          cfmaf_cj(unm0, u0[c], uk);
          if (nbw > 1) cfmaf_cj(unm1, u1[c], uk);
        }
      }
      const int64_t vbase = (nbw > 0 && d.g2) ? (int64_t)j * d.per_state + (int64_t)ri.z * 6 : 0;
      float acc = 0.f;
      float ys[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      float accr[SETS ? MAX_SETS : 1];   // the other sets' sums over the bands after n0, n1
      if (SETS)
        for (int p = 0; p < MAX_SETS; ++p) accr[p] = 0.f;
      if (!mbar_wait(tfull, it & 1, g.err)) break;
      tc_fence_after();
      // ---- drain: h for the first two window bands
      float2 h0[6], h1[6];
#pragma unroll
      for (int sp = 0; sp < 6; ++sp) {
        float gre[8], gim[8];
        __syncwarp();
        fused_load_one<FBN>(tr, slot * 48 + 8 * sp, gre, gim);
        if (nbw > 0) h0[sp] = hrot(u0, gre, gim);
        if (nbw > 1) h1[sp] = hrot(u1, gre, gim);
      }
      // further window bands (rare): finished while the accumulators are held
      const int nbmax = __reduce_max_sync(0xffffffffu, nbw);
      if (nbmax > 2) {
        unsigned left = rest & (rest - 1);   // bands after n0, n1
        for (int b = 2; b < nbmax; ++b) {
          const bool mine = b < nbw;
          const int nb_ = mine ? __ffs(left) - 1 : 0;
          if (mine) left &= left - 1;
          float2 ux[8], hx[6];
          if (mine) load_urow(ub, nb_, ux);
#pragma unroll
          for (int sp = 0; sp < 6; ++sp) {
            float gre[8], gim[8];
            __syncwarp();
            fused_load_one<FBN>(tr, slot * 48 + 8 * sp, gre, gim);
            if (mine) hx[sp] = hrot(ux, gre, gim);
          }
          if (mine) {
            const F2 dn = f2_mul(f2_of(E - __ldg(eb + nb_ * 32)), isg);
            float2 unmx = make_float2(0.f, 0.f);
            if (POLAR)
#pragma unroll
              for (int c = 0; c < 8; ++c) cfmaf_cj(unmx, ux[c], __ldg(Uk + c));
            float g2x[6];
            acc = __fadd_rn(acc, fused_vertices<PH, POLAR, SETS>(hx, rq, dn, ex, dnorm, d, vbase + (int64_t)b * 6, q,
                                                                 yo, ys, glb, unmx, g2x));
            if (SETS) {
              const F2 dd = f2_of(E - __ldg(eb + nb_ * 32));
              for (int p = 1; p < xs.n; ++p) {
                const float2 oc = xs.occ[(size_t)(p - 1) * g.nst + j];
                accr[p] = __fadd_rn(accr[p], fused_set_band(g2x, xs.mode + (p - 1) * xs.mode_stride + blk32(q, 6, 0),
                                                            f2_mul(dd, F2{xs.isg_hi[p], xs.isg_lo[p]}), oc.x, oc.y,
                                                            xs.dnorm[p]));
              }
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(tempty);
      // ---- vertices of the first two bands, overlapping the next tile's MMAs
      float acc01 = 0.f;
      float g2a[SETS ? 6 : 1], g2b[SETS ? 6 : 1];   // |g|^2 cx of the first two bands, for the other sets
      if (nbw > 0) {
        const F2 dn = f2_mul(f2_of(E - __ldg(eb + n0 * 32)), isg);
        acc01 = __fadd_rn(acc01,
                          fused_vertices<PH, POLAR, SETS>(h0, rq, dn, ex, dnorm, d, vbase, q, yo, ys, glb, unm0, g2a));
      }
      if (nbw > 1) {
        const F2 dn = f2_mul(f2_of(E - __ldg(eb + n1 * 32)), isg);
        acc01 = __fadd_rn(acc01, fused_vertices<PH, POLAR, SETS>(h1, rq, dn, ex, dnorm, d, vbase + 6, q, yo, ys,
                                                                  glb, unm1, g2b));
      }
      double v = (double)acc01 + (double)acc;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0 && jvalid) g.partial[(size_t)j * g.nblk + mt * 4 + quad] = v;
      if (SETS) {   // the same sums under the other parameter sets
        const F2 dd0 = f2_of(E - __ldg(eb + n0 * 32)), dd1 = f2_of(E - __ldg(eb + n1 * 32));
        for (int p = 1; p < xs.n; ++p) {
          float a01 = 0.f;
          if (jvalid && nbw > 0) {
            const float2 oc = xs.occ[(size_t)(p - 1) * g.nst + j];
            const F2 isgp{xs.isg_hi[p], xs.isg_lo[p]};
            const float4 *mq = xs.mode + (p - 1) * xs.mode_stride + blk32(q, 6, 0);
            a01 = __fadd_rn(a01, fused_set_band(g2a, mq, f2_mul(dd0, isgp), oc.x, oc.y, xs.dnorm[p]));
            if (nbw > 1) a01 = __fadd_rn(a01, fused_set_band(g2b, mq, f2_mul(dd1, isgp), oc.x, oc.y, xs.dnorm[p]));
          }
          double vp = (double)a01 + (double)accr[p];
          for (int o = 16; o > 0; o >>= 1) vp += __shfl_down_sync(0xffffffffu, vp, o);
          if (lane == 0 && jvalid) xs.partial[p][(size_t)j * g.nblk + mt * 4 + quad] = vp;
        }
      }
      if (PH && jvalid && nbw > 0 && d.phr) {   // this pair's Y into the rates of (q, s), s = 0..5
#pragma unroll
        for (int s = 0; s < 6; ++s) {
          const float y = ys[s] * y_factor(yo, __ldg(rq + (5 * s + 3) * 32).y);   // x 2^64
          if (y != 0.f) atomicAdd(d.phr + q + (size_t)rp.N * s, d.ph_scale * TWO_M64D * (double)y);
        }
      }
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
  cluster_sync();   // no CTA leaves while its peer may still arrive on its barriers
}

// Launch a persistent kernel as clusters of 2 CTAs: as many pairs as can be
// resident at once (at most one CTA per SM), at most `pairs` (work units).
// chunk > 0 splits the work into launches of chunk units per cluster, so that
// kernels of other streams (other requests of the serving loop) get the SMs
// between launches; launch(cfg, t0, t1) issues the launch for units [t0, t1).
template <class F>
static int launch_pairs(const void *kernel, int smem, int64_t pairs, cudaStream_t st, int chunk, const Yield &yield,
                        F launch) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(F_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3((unsigned)(2 * std::max<int64_t>(1, std::min<int64_t>(pairs, num_sms() / 2))));
  int ncl = 0;
  TCK(cudaOccupancyMaxActiveClusters(&ncl, kernel, &cfg));
  if (ncl <= 0) return tfail(2, "no 2-CTA cluster fits on the device");
  const int64_t nc = std::min<int64_t>(pairs, ncl);
  cfg.gridDim = dim3((unsigned)(2 * nc));
  const int64_t step = chunk > 0 ? nc * chunk : pairs;
  for (int64_t t0 = 0; t0 < pairs; t0 += step) {
    if (t0 > 0) yield();
    TCK(launch(cfg, (int)t0, (int)std::min<int64_t>(pairs, t0 + step)));
    TCK(cudaGetLastError());
  }
  return 0;
}

static int stageB_fused86(const float *PB, int MpB, const float *B2, int64_t Np2, int KpB, int nwv, int nst,
                          const RateParams &rp, const EpiData &ed, const FusedTabs &tabs, double *partial, int nblk,
                          int *err, cudaStream_t st, int chunk, const Yield &yield, const FusedSets &xs) {
  if (MpB % BM || Np2 % FBN || KpB % BK) return tfail(1, "stage B: shapes not tile multiples");
  if (4 * (int64_t)MpB > INT32_MAX || 6 * Np2 > INT32_MAX) return tfail(1, "stage B: operand too tall for TMA coords");
  CUtensorMap ta, tb;
  int rc;
  if ((rc = make_map(&ta, PB, KpB, 4 * (int64_t)MpB)) || (rc = make_map(&tb, B2, KpB, 6 * Np2, FBN))) return rc;
  // once per process: changing a kernel attribute can wait for the device's queued work
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(k_stageB_fused86<false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, F_SMEM);
    cudaFuncSetAttribute(k_stageB_fused86<true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, F_SMEM);
    cudaFuncSetAttribute(k_stageB_fused86<false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, F_SMEM);
    cudaFuncSetAttribute(k_stageB_fused86<true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, F_SMEM);
    cudaFuncSetAttribute(k_stageB_fused86<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, F_SMEM);
    cudaFuncSetAttribute(k_stageB_fused86<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, F_SMEM);
  });
  const bool ph = ed.phr || ed.yv, polar = tabs.glb != nullptr, sets = xs.n > 1;
  if (ph && sets) return tfail(1, "stage B: parameter sets are an electron-side form");
  FusedArgs g;
  g.mtiles = MpB / BM;
  g.ntiles = (nst + 1) / 2;
  g.nkb = KpB / BK;
  g.bands = fused_bands(4 * (int64_t)MpB * KpB * 4, g.mtiles / 2);
  g.Astride = MpB;
  g.Bstride = Np2;
  g.nwv = nwv;
  g.nst = nst;
  g.err = err;
  g.partial = partial;
  g.nblk = nblk;
  if ((int64_t)g.ntiles * FBN > Np2) return tfail(1, "stage B: state operand too short");
  if (g.mtiles % 2) return tfail(1, "stage B: row tiles must pair");
  const int64_t pairs = (int64_t)(g.mtiles / 2) * g.ntiles;
  if (pairs > INT32_MAX) return tfail(1, "stage B: too many tiles");
  auto run = [&](auto kernel) {
    return launch_pairs((const void *)kernel, F_SMEM, pairs, st, chunk, yield,
                        [&](cudaLaunchConfig_t &cfg, int t0, int t1) {
                          g.t0 = t0;
                          g.t1 = t1;
                          return cudaLaunchKernelEx(&cfg, kernel, ta, tb, g, tabs, rp, ed, xs);
                        });
  };
  if (sets) return polar ? run(k_stageB_fused86<false, true, true>) : run(k_stageB_fused86<false, false, true>);
  if (polar) return ph ? run(k_stageB_fused86<true, true, false>) : run(k_stageB_fused86<false, true, false>);
  return ph ? run(k_stageB_fused86<true, false, false>) : run(k_stageB_fused86<false, false, false>);
}

// ------------------------------- stage A fused with the initial-band rotation
// For the same nw = 8, nb = 6 path the stage-A contraction g(k,Rp) = sum_Re
// e^{2 pi i k.Re}/deg g(Re,Rp) runs fused with the rotation over the initial
// band and the k-half of the Rp phase, writing the six-plane stage-B state
// operand directly (the FP32 g(k,Rp) of all window k, 10 GB at 24^3, is never
// stored).  A tile is 128 window k rows x 128 columns = 16 contraction
// positions kp x 8 initial bands m' of one (n', s'); a complex product is two
// MMAs of N = 256 over the six-plane operand, the main and correction
// accumulators (real | imaginary) filling TMEM columns 0..255 and 256..511.
// K blocks are 8 wide (32 B rows, 32B swizzle) so that five 40 KB stages fit.
// Epilogue warp w drains lane quadrant w % 4 for the 8 positions of half
// (w - 2) / 4: per window state (k, m) of its row it forms
//   B(state)[n' + 8 s'][kp] = conj(e^{2 pi i k.Rp}) / deg(Rp) sum_m' U_k[m][m'] g(k,Rp)[n', m', s']
// for the first two states in registers, releases TMEM, and writes 32-byte
// sectors of the six planes.
constexpr int A_BK = 8;
constexpr int A_PLANE = BM * A_BK * 4;          // 4 KB
constexpr int A_STAGE = 10 * A_PLANE;           // 4 A planes + 6 B planes
constexpr int A_STAGES = 5;
constexpr int A_SMEM = A_STAGES * A_STAGE + 1024 + 256;

// SMEM matrix descriptor: K-major, SWIZZLE_32B (atom = 8 rows x 32 B, SBO = 256 B).
__device__ __forceinline__ uint64_t sdesc32(const void *p) {
  uint64_t a = smem_u32(p);
  uint64_t d = (a >> 4) & 0x3FFFull;
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(256 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)6 << 61;
  return d;
}

struct FusedAArgs {
  int mtiles, ntiles, nkb, nkp16;   // nkp16: 16-position blocks of the state operand's K
  int bands;                        // m-bands of the tile walk (fb_tile)
  int t0, t1;                        // tile pairs [t0, t1) of this launch
  int64_t Astride, Bstride;          // rows between planes: phase operand, stage-A operand
  int KpB;
  int64_t Np2;                       // rows per plane of the state operand
  float *B2;                         // [6][Np2][KpB] output
  const float2 *phk;                 // conj(e^{2 pi i k.Rp}) / deg(Rp): row-blocked, fields kp (0 at padding)
  int *err;
};

// conj(e^{2 pi i k.Rp}) / deg(Rp) for window row ip and contraction position kp,
// stored row-blocked by 32 (field kp): built once per request (its FP64
// divisions kept out of the GEMM epilogue), read coalesced.
__global__ void k_phase_k_table(int nwv, int Mp, int KpB, const int *widx, const int *kinvB, int m0, int m1, int m2,
                                int L, const int *Rq, const double *degq, const double2 *roots, float2 *phk) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)Mp * KpB) return;
  const int ip = (int)(idx / KpB), kp = (int)(idx % KpB);
  const int rp = kinvB[kp];
  float2 v = make_float2(0.f, 0.f);
  if (ip < nwv && rp >= 0) {
    const double2 r = roots[phase_idx(widx[ip], m0, m1, m2, L, Rq[3 * rp], Rq[3 * rp + 1], Rq[3 * rp + 2])];
    v = make_float2((float)(r.x / degq[rp]), (float)(-r.y / degq[rp]));
  }
  phk[blk32(ip, KpB, kp)] = v;
}

// write the 8 positions of one state row (32-byte sectors of the six planes)
__device__ __forceinline__ void write_state8(const FusedAArgs &g, int64_t row, int kp0, const float2 *o,
                                             const float2 *ph) {
  float v[6][8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const float xr = ph[r].x * o[r].x - ph[r].y * o[r].y, xi = ph[r].x * o[r].y + ph[r].y * o[r].x;
    const float hr = tf32_round(xr), hi = tf32_round(xi);
    const float lr = tf32_round(xr - hr), li = tf32_round(xi - hi);
    v[0][r] = -hi;
    v[1][r] = hr;
    v[2][r] = hi;
    v[3][r] = -li;
    v[4][r] = lr;
    v[5][r] = li;
  }
  const int64_t plane = g.Np2 * g.KpB;
  float *base = g.B2 + row * g.KpB + kp0;
#pragma unroll
  for (int pl = 0; pl < 6; ++pl) {
    float4 *d4 = (float4 *)(base + pl * plane);
    d4[0] = make_float4(v[pl][0], v[pl][1], v[pl][2], v[pl][3]);
    d4[1] = make_float4(v[pl][4], v[pl][5], v[pl][6], v[pl][7]);
  }
}

// rotation over m' of the 8 loaded columns (one position): sum_m' u[m'] G(m')
__device__ __forceinline__ float2 mrot(const float2 *u, const float *gre, const float *gim) {
  float2 a = make_float2(0.f, 0.f);
#pragma unroll
  for (int mp = 0; mp < 8; ++mp) cfmaf(a, u[mp], make_float2(gre[mp], gim[mp]));
  return a;
}

__global__ void __launch_bounds__(F_THREADS, 1)
    k_stageA_fused86(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, FusedAArgs g,
                     FusedTabs tb) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + A_STAGES * A_STAGE);
  uint64_t *empty = full + A_STAGES;
  uint64_t *tfull = empty + A_STAGES;
  uint64_t *tempty = tfull + 1;
  uint64_t *drain = tempty + 1;
  uint32_t *tslot = (uint32_t *)(drain + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // CTA pairs (clusters of 2) take m-tiles 2x, 2x + 1 of the same n-tile: each
  // loads its own phase tile and multicasts three of the six operand planes to
  // both; a stage is refilled once both CTAs' MMAs have read it.
  const uint32_t crank = cluster_rank();
  if (threadIdx.x == 0) {
    for (int s = 0; s < A_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 2);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, F_EPI_THREADS);
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  cluster_sync();   // the peer's barriers are initialised before any multicast or remote arrive
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const int mpairs = g.mtiles >> 1;
  (void)mpairs;
  const int cid = blockIdx.x >> 1, ncl = gridDim.x >> 1;

  if (warp == 0) {
    if (lane == 0) {   // ---- TMA producer
      uint64_t keep;
      asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(keep));
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      for (int t = g.t0 + cid; t < g.t1 && ok; t += ncl) {
        int mp, nt;
        fb_tile(t, mpairs, g.ntiles, g.bands, mp, nt);
        const int mt = 2 * mp + (int)crank;
        for (int kb = 0; kb < g.nkb; ++kb) {
          if (!mbar_wait(&empty[stage], phase ^ 1, g.err)) { ok = false; break; }
          uint8_t *sb = smem + stage * A_STAGE;
          mbar_expect_tx(&full[stage], A_STAGE);
#pragma unroll
          for (int p = 0; p < 4; ++p)
            tma_load_2d_hint(sb + p * A_PLANE, &tA, &full[stage], kb * A_BK, (int)(p * g.Astride + mt * BM), keep);
#pragma unroll
          for (int p = 3 * (int)crank; p < 3 * (int)crank + 3; ++p)
            tma_load_2d_mc(sb + (4 + p) * A_PLANE, &tB, &full[stage], kb * A_BK, (int)(p * g.Bstride + nt * BM),
                           (uint16_t)3);
          if (++stage == A_STAGES) { stage = 0; phase ^= 1; }
        }
      }
      for (int s = 0; s < A_STAGES; ++s) mbar_wait(&empty[stage], phase ^ 1, g.err), stage = (stage + 1) % A_STAGES,
                                           phase ^= (stage == 0);
    }
  } else if (warp == 1) {
    if (lane == 0) {   // ---- MMA issuer
      constexpr uint32_t ID2 = idesc_tf32_n(false, 2 * BM);
      int stage = 0;
      uint32_t phase = 0;
      int it = 0;
      bool ok = true;
      const uint32_t dm = tmem, dc = tmem + 256;
      for (int t = g.t0 + cid; t < g.t1 && ok; t += ncl, ++it) {
        if (!mbar_wait(tempty, (it & 1) ^ 1, g.err)) { ok = false; break; }
        tc_fence_after();
        for (int kb = 0; kb < g.nkb; ++kb) {
          if (!mbar_wait(&full[stage], phase, g.err)) { ok = false; break; }
          tc_fence_after();
          uint8_t *sb = smem + stage * A_STAGE;
          const uint64_t Ahr = sdesc32(sb + 0 * A_PLANE), Ahi = sdesc32(sb + 1 * A_PLANE);
          const uint64_t Alr = sdesc32(sb + 2 * A_PLANE), Ali = sdesc32(sb + 3 * A_PLANE);
          const uint64_t BhN = sdesc32(sb + 4 * A_PLANE), BhP = sdesc32(sb + 5 * A_PLANE);
          const uint64_t BlN = sdesc32(sb + 7 * A_PLANE), BlP = sdesc32(sb + 8 * A_PLANE);
          const uint32_t acc = kb == 0 ? 0u : 1u;
          umma(dc, Ahr, BlP, ID2, acc);   // hi x lo
          umma(dc, Ahi, BlN, ID2, 1);
          umma(dc, Alr, BhP, ID2, 1);     // lo x hi
          umma(dc, Ali, BhN, ID2, 1);
          // the last 16 positions (nearest cells, largest terms) go to the short correction chain
          const bool nearblk = g.nkb > 2 && kb >= g.nkb - 2;
          const uint32_t dd = nearblk ? dc : dm;
          umma(dd, Ahr, BhP, ID2, nearblk ? 1u : acc);   // hi x hi
          umma(dd, Ahi, BhN, ID2, 1);
          umma_commit_mc(&empty[stage], (uint16_t)3);
          if (++stage == A_STAGES) { stage = 0; phase ^= 1; }
        }
        if (ok) umma_commit(tfull);
      }
      // a wait gave up: let the MMAs already issued retire before TMEM is freed
      if (!ok) {
        umma_commit(drain);
        mbar_wait(drain, 0, g.err);
      }
    }
  } else {   // ---- epilogue: warps 2..9
    const int quad = warp & 3, half = (warp - 2) >> 2;
    const uint32_t tr = tmem + ((uint32_t)(quad * 32) << 16);
    int it = 0;
    for (int t = g.t0 + cid; t < g.t1; t += ncl, ++it) {
      int mp, nt;
      fb_tile(t, mpairs, g.ntiles, g.bands, mp, nt);
      const int mt = 2 * mp + (int)crank;
      const int kpb = nt % g.nkp16, ns = nt / g.nkp16;
      const int col0 = (ns & 7) + 8 * (ns >> 3);      // n' + 8 s'
      const int kp0 = kpb * 16 + half * 8;
      const int ip = mt * BM + quad * 32 + lane;
      const int4 ri = __ldg(tb.row + ip);             // padding rows: no window band, no state
      const unsigned wmask = (unsigned)ri.y;
      const int nbw = __popc(wmask);
      const int m0b = nbw > 0 ? __ffs(wmask) - 1 : 0;
      const unsigned rest = wmask & (wmask - 1);
      const int m1b = nbw > 1 ? __ffs(rest) - 1 : 0;
      const float4 *ub = tb.U4 + blk32(ip, 32, 0);
      float2 u0[8], u1[8], ph[8];
      if (nbw > 0) load_urow(ub, m0b, u0);
      if (nbw > 1) load_urow(ub, m1b, u1);
      if (nbw > 0) {
        const float2 *pk = g.phk + blk32(ip, g.KpB, kp0);
#pragma unroll
        for (int r = 0; r < 8; ++r) ph[r] = __ldg(pk + 32 * r);
      }
      if (!mbar_wait(tfull, it & 1, g.err)) break;
      tc_fence_after();
      float2 o0[8], o1[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        float gre[8], gim[8];
        __syncwarp();
        fused_load_one<BM>(tr, 8 * (half * 8 + r), gre, gim);
        if (nbw > 0) o0[r] = mrot(u0, gre, gim);
        if (nbw > 1) o1[r] = mrot(u1, gre, gim);
      }
      // rows with more than two window states (rare): finished while the accumulators are held
      const int nbmax = __reduce_max_sync(0xffffffffu, nbw);
      if (nbmax > 2) {
        unsigned left = rest & (rest - 1);
        for (int b = 2; b < nbmax; ++b) {
          const bool mine = b < nbw;
          const int mb = mine ? __ffs(left) - 1 : 0;
          if (mine) left &= left - 1;
          float2 ux[8], ox[8];
          if (mine) load_urow(ub, mb, ux);
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            float gre[8], gim[8];
            __syncwarp();
            fused_load_one<BM>(tr, 8 * (half * 8 + r), gre, gim);
            if (mine) ox[r] = mrot(ux, gre, gim);
          }
          if (mine) write_state8(g, (int64_t)(ri.z + b) * 48 + col0, kp0, ox, ph);
        }
      }
      tc_fence_before();
      mbar_arrive(tempty);
      if (nbw > 0) write_state8(g, (int64_t)ri.z * 48 + col0, kp0, o0, ph);
      if (nbw > 1) write_state8(g, (int64_t)(ri.z + 1) * 48 + col0, kp0, o1, ph);
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
  cluster_sync();   // no CTA leaves while its peer may still arrive on its barriers
}

static int stageA_fused86(const float *PA, int MpA, const float *GA6, int64_t NA, int KpA, const FusedTabs &tabs,
                          FusedAArgs g, cudaStream_t st, int chunk, const Yield &yield) {
  if (MpA % BM || NA % BM || KpA % A_BK || g.KpB % 16) return tfail(1, "stage A: shapes not tile multiples");
  if (4 * (int64_t)MpA > INT32_MAX || 6 * NA > INT32_MAX) return tfail(1, "stage A: operand too tall for TMA coords");
  CUtensorMap ta, tb;
  int rc;
  if ((rc = make_map(&ta, PA, KpA, 4 * (int64_t)MpA, BM, A_BK)) || (rc = make_map(&tb, GA6, KpA, 6 * NA, BM, A_BK)))
    return rc;
  // once per process: changing a kernel attribute can wait for the device's queued work
  static std::once_flag attr_once;
  std::call_once(attr_once, [] {
    cudaFuncSetAttribute(k_stageA_fused86, cudaFuncAttributeMaxDynamicSharedMemorySize, A_SMEM);
  });
  g.mtiles = MpA / BM;
  g.ntiles = (int)(NA / BM);
  g.nkb = KpA / A_BK;
  g.bands = fused_bands(4 * (int64_t)MpA * KpA * 4, g.mtiles / 2);
  g.nkp16 = g.KpB / 16;
  g.Astride = MpA;
  g.Bstride = NA;
  if ((int64_t)g.nkp16 * 48 != g.ntiles) return tfail(1, "stage A: operand width mismatch");
  if (g.mtiles % 2) return tfail(1, "stage A: row tiles must pair");
  const int64_t pairs = (int64_t)(g.mtiles / 2) * g.ntiles;
  if (pairs > INT32_MAX) return tfail(1, "stage A: too many tiles");
  return launch_pairs((const void *)k_stageA_fused86, A_SMEM, pairs, st, chunk, yield,
                      [&](cudaLaunchConfig_t &cfg, int t0, int t1) {
                        g.t0 = t0;
                        g.t1 = t1;
                        return cudaLaunchKernelEx(&cfg, k_stageA_fused86, ta, tb, g, tabs);
                      });
}

// ------------------------------------------------------------ orchestration
void free_split(SplitOperands &s, cudaStream_t st) {
  if (s.G) cudaFreeAsync(s.G, st);
  if (s.GA6) cudaFreeAsync(s.GA6, st);
  s.G = nullptr;
  s.GA6 = nullptr;
  s.bytes = 0;
}

static inline int64_t rup(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// fp32 copies of the eigenvectors and the per-(q, s) scalars of the epilogues
struct EpiTables {
  float2 *Uf;
  float *cx, *bs;
  float4 *wv;
};

static int epi_tables(Workspace &ws, cudaStream_t st, const double2 *U, const RateParams &rp, const EpiData &ed_in,
                      int64_t *launches, EpiTables *t) {
  const int N = rp.N, nw = rp.nw, nb = rp.nb;
  if (wsget(ws, "tc_Uf", (size_t)N * nw * nw, &t->Uf) || wsget(ws, "tc_cx", (size_t)N * nb, &t->cx) ||
      wsget(ws, "tc_bs", (size_t)N * nb, &t->bs) || wsget(ws, "tc_wv", (size_t)N * nb, &t->wv))
    return tfail(6, ws.msg.c_str());
  k_to_f2<<<(unsigned)(((int64_t)N * nw * nw + 255) / 256), 256, 0, st>>>((int64_t)N * nw * nw, U, t->Uf);
  k_qtab<<<(N * nb + 255) / 256, 256, 0, st>>>(N * nb, ed_in.om, ed_in.bose, rp.sigma, kB * rp.T, rp.const_tp, t->cx,
                                                t->bs, t->wv);
  TCK(cudaGetLastError());
  *launches += 2;
  return 0;
}

// Any nw, nb and delta: stage A as chunked GEMMs + rotation into a four-plane
// state operand, stage B as chunked GEMMs + a separate epilogue.
static int split_rates_generic(SplitOperands &s, Workspace &ws, cudaStream_t st, const double2 *G64, int nwsk,
                               int nwsq, int64_t Nn, int nw, int nb, int nwv, int nst, const int mesh[3], int L,
                               const double2 *roots, const int *widx, const int *arow, int nA, const int *st_code,
                               const std::vector<int> &first_state, const int *Rk, const double *degk,
                               const int *kposA, const int *Rq, const double *degq, const int *kposB, const double2 *U,
                               const RateParams &rp, const EpiData &ed_in, double *partial, int nblk, int *err,
                               cudaEvent_t ev_stage_a, int64_t *launches, LaunchTimer *tA, LaunchTimer *tB,
                               std::mutex *build_mu, int chunk_us, const Yield &yield, const BatchMember *bm,
                               int64_t chunk_bytes, const RateSets *sets) {
  int rc;
  const int KpA = (int)rup(nwsk, BK), KpB = (int)rup(nwsq, BK);
  const int64_t NpA = rup(Nn, BN);
  // g(Re,Rp) planes, built once per handle
  {
  std::lock_guard<std::mutex> build_lock(*build_mu);
  if (!s.G) {
    TCK(pool_alloc((void **)&s.G, (size_t)4 * NpA * KpA * sizeof(float), st));
    s.bytes += (int64_t)4 * NpA * KpA * sizeof(float);
    TCK(cudaMemsetAsync(s.G, 0, (size_t)4 * NpA * KpA * sizeof(float), st));
    dim3 grid((unsigned)((Nn + 31) / 32), (unsigned)((KpA + 31) / 32));
    k_gplanes<<<grid, dim3(32, 8), 0, st>>>(Nn, nwsk, G64, kposA, s.G, NpA, KpA);
    TCK(cudaGetLastError());
    s.Nn = NpA;
    s.Kp = KpA;
    (*launches)++;
    TCK(cudaStreamSynchronize(st));   // complete before other streams may read it
  }
  }
  const int ncol = nw * nb;
  // batched: this request takes part in the grouped launches from here to the end of stage B
  struct ActiveScope {
    const BatchMember *m;
    explicit ActiveScope(const BatchMember *m_) : m(m_) { if (m) batcher_activate(*m); }
    ~ActiveScope() { if (m) batcher_deactivate(*m); }
  } active_scope(bm && bm->gb ? bm : nullptr);
  // stage A over the A-rows in chunks of kc rows (multiple of BM)
  const int64_t kc = std::max<int64_t>(BM, std::min<int64_t>(rup(nA, BM), chunk_bytes / (NpA * 8) / BM * BM));
  const int64_t Np2 = rup((int64_t)nst * ncol, BN);
  float *PA, *CAr, *CAi, *B2;
  if ((rc = wsget(ws, "tc_PA", (size_t)4 * kc * KpA, &PA)) || (rc = wsget(ws, "tc_CAr", (size_t)kc * NpA, &CAr)) ||
      (rc = wsget(ws, "tc_CAi", (size_t)kc * NpA, &CAi)) || (rc = wsget(ws, "tc_B2", (size_t)4 * Np2 * KpB, &B2)))
    return tfail(6, ws.msg.c_str());
  // the rotation writes every K position of every state row; zero the padding rows only
  {
    const int64_t used = (int64_t)nst * ncol;
    for (int pl = 0; pl < 4; ++pl)
      if (Np2 > used)
        TCK(cudaMemsetAsync(B2 + ((int64_t)pl * Np2 + used) * KpB, 0, (size_t)(Np2 - used) * KpB * sizeof(float), st));
  }
  // first state of each A-row, and the Rp cell at each contraction position
  int *fs_d, *kinvB;
  if ((rc = wsget(ws, "tc_fs", (size_t)nA + 1, &fs_d)) || (rc = wsget(ws, "tc_kinv", (size_t)KpB, &kinvB)))
    return tfail(6, ws.msg.c_str());
  TCK(cudaMemcpyAsync(fs_d, first_state.data(), (size_t)(nA + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  TCK(cudaMemsetAsync(kinvB, 0xFF, (size_t)KpB * sizeof(int), st));
  k_kinv<<<(nwsq + 255) / 256, 256, 0, st>>>(nwsq, kposB, kinvB);
  TCK(cudaGetLastError());
  *launches += 1;
  for (int64_t i0 = 0; i0 < nA; i0 += kc) {
    if (i0 > 0) yield();
    const int n = (int)std::min<int64_t>(kc, nA - i0);
    const int Mp = (int)rup(n, BM);
    TCK(cudaMemsetAsync(PA, 0, (size_t)4 * Mp * KpA * sizeof(float), st));
    int64_t ne = (int64_t)n * nwsk;
    k_phase_planes<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(n, arow + i0, mesh[0], mesh[1], mesh[2], L, nwsk, Rk,
                                                                 degk, kposA, roots, PA, Mp, KpA);
    TCK(cudaGetLastError());
    tA->begin(st);
    if ((rc = cgemm(PA, Mp, 0, Mp, s.G, NpA, 0, (int)NpA, KpA, CAr, CAi, NpA, err, st, chunk_us, yield, bm)))
      return rc;
    tA->end(st);
    {
      // modes per pass: as many as keep the staged g within ROT_SMEM_TARGET (three
      // blocks per SM), at least one (up to ROT_SMEM)
      int sch = nb;
      while (sch > 1 && rotate_k_smem(nw, sch) > (size_t)ROT_SMEM_TARGET) --sch;
      const size_t sm = rotate_k_smem(nw, sch);
      if (sm <= (size_t)ROT_SMEM && (nw % 2) == 0) {   // 16-byte staging: nw * nw a multiple of 4
        // once per process: changing a kernel attribute can wait for the device's queued work
        static std::once_flag attr_once;
        std::call_once(attr_once, [] {
          cudaFuncSetAttribute(k_rotate_k, cudaFuncAttributeMaxDynamicSharedMemorySize, ROT_SMEM);
        });
        k_rotate_k<<<n, 256, sm, st>>>((int)i0, fs_d, nw, nb, sch, st_code, arow, U, CAr, CAi, NpA, mesh[0],
                                      mesh[1], mesh[2], L, roots, Rq, degq, kinvB, KpB, B2, Np2);
        TCK(cudaGetLastError());
        (*launches)++;
      } else {   // large nw*nw*nb: one thread per output element
        for (int j0 = first_state[i0], j1 = first_state[i0 + n]; j0 < j1; j0 += 32768) {
          int je = std::min(j1, j0 + 32768);
          dim3 grid(std::max(1, std::min(64, (ncol * nwsq + 255) / 256)), je - j0);
          k_rotate_planes<<<grid, 256, 0, st>>>(j0, je, (int)i0, st_code, nw, nb, nwsq, arow, U, CAr, CAi, NpA,
                                               mesh[0], mesh[1], mesh[2], L, roots, Rq, degq, kposB, B2, Np2, KpB, 0);
          TCK(cudaGetLastError());
          (*launches)++;
        }
      }
    }
    *launches += 3;
  }
  TCK(cudaEventRecord(ev_stage_a, st));
  // stage B: A planes = e^{2 pi i k'.Rp} for the window k'
  const int MpB = (int)rup(nwv, BM);
  float *PB, *CBr, *CBi;
  // states per chunk: a multiple of 8 (8 * 48 = 3 * 128 columns) bounded by chunk_bytes of output
  int64_t sc = chunk_bytes / ((int64_t)MpB * ncol * 8);
  sc = std::max<int64_t>(8, sc / 8 * 8);
  sc = std::min<int64_t>(sc, rup(nst, 8));
  sc = std::min<int64_t>(sc, 32768);
  const int64_t NpC = rup(sc * ncol, BN);
  if ((rc = wsget(ws, "tc_PB", (size_t)4 * MpB * KpB, &PB)) || (rc = wsget(ws, "tc_CBr", (size_t)MpB * NpC, &CBr)) ||
      (rc = wsget(ws, "tc_CBi", (size_t)MpB * NpC, &CBi)))
    return tfail(6, ws.msg.c_str());
  TCK(cudaMemsetAsync(PB, 0, (size_t)4 * MpB * KpB * sizeof(float), st));
  {
    int64_t ne = (int64_t)nwv * nwsq;
    k_phase_planes<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(nwv, widx, mesh[0], mesh[1], mesh[2], L, nwsq, Rq,
                                                                 nullptr, kposB, roots, PB, MpB, KpB);
    TCK(cudaGetLastError());
  }
  EpiTables et;
  if ((rc = epi_tables(ws, st, U, rp, ed_in, launches, &et))) return rc;
  EpiData ed = ed_in;
  ed.Uf = et.Uf;
  QTab qt{et.cx, et.bs, et.wv};
  // the other parameter sets: their mode tables; no vertex lists
  const int nsets = sets ? sets->n : 1;
  QTab qts[MAX_SETS];
  qts[0] = qt;
  if (nsets > 1) {
    const int N = rp.N;
    float *cxp, *bsp;
    float4 *wvp;
    if ((rc = wsget(ws, "tc_scx", (size_t)N * nb, &cxp)) || (rc = wsget(ws, "tc_sbs", (size_t)(nsets - 1) * N * nb, &bsp)) ||
        (rc = wsget(ws, "tc_swv", (size_t)(nsets - 1) * N * nb, &wvp)))
      return tfail(6, ws.msg.c_str());
    for (int p = 1; p < nsets; ++p) {
      const RateParams &r = sets->rp[p];
      float *bs = bsp + (size_t)(p - 1) * N * nb;
      float4 *wv = wvp + (size_t)(p - 1) * N * nb;
      k_qtab<<<(N * nb + 255) / 256, 256, 0, st>>>(N * nb, ed_in.om, sets->bose[p], r.sigma, kB * r.T, r.const_tp,
                                                    cxp, bs, wv);
      TCK(cudaGetLastError());
      *launches += 1;
      qts[p] = QTab{et.cx, bs, wv};
    }
  }
  const RateParams &rp0 = rp;
  double *const partial0 = partial;
  const EpiData eds = ed, eds_in = ed_in;
  // the row epilogue reads the GEMM output interleaved by 32 rows (coalesced), the others row-major
  const bool rows_kernel = rp.delta_kind == 0 && nb <= EPR_NB && (nw == 8 || nw == 16 || nw == 24 || nw == 32);
  for (int64_t j0 = 0; j0 < nst; j0 += sc) {
    const int ns = (int)std::min<int64_t>(sc, nst - j0);
    const int Npc = (int)rup((int64_t)ns * ncol, BN);
    tB->begin(st);
    if (j0 > 0) yield();
    if ((rc = cgemm(PB, MpB, 0, MpB, B2, Np2, j0 * ncol, Npc, KpB, CBr, CBi, NpC, err, st, chunk_us, yield, bm,
                    rows_kernel ? 1 : 0)))
      return rc;
    tB->end(st);
    const size_t esm = (size_t)2 * EPI_ROWS * (ncol + 1) * sizeof(float);
    for (int set = 0; set < nsets; ++set) {   // one epilogue per parameter set over the same GEMM output
    const RateParams &rp = set ? sets->rp[set] : rp0;
    const QTab &qt = qts[set];
    double *partial = set ? sets->partial[set] : partial0;
    EpiData ed = eds, ed_in = eds_in;
    if (set) {
      ed.bose = ed_in.bose = sets->bose[set];
      ed.g2 = ed.xp = ed.xm = ed.yv = ed_in.g2 = ed_in.xp = ed_in.xm = ed_in.yv = nullptr;
      ed.phr = ed_in.phr = nullptr;
    }
    if (rows_kernel) {
      dim3 grid(nblk, ns);
      // NB: the mode arrays' size (6, 12 or 18), the smallest that holds nb
      auto rows = [&](auto kernel) {
        kernel<<<grid, EPI_ROWS, 0, st>>>(nwv, (int)j0, CBr, CBi, NpC, rp, ed, qt, partial, nblk);
      };
      const int nbc = nb <= 6 ? 6 : nb <= 12 ? 12 : 18;
#define EPHG_ROWS_NB(NWV)                                                          \
  (nbc == 6 ? rows(k_epilogue_rows<NWV, 6>) : nbc == 12 ? rows(k_epilogue_rows<NWV, 12>) \
            : rows(k_epilogue_rows<NWV, 18>))
      if (nw == 8)
        EPHG_ROWS_NB(8);
      else if (nw == 16)
        EPHG_ROWS_NB(16);
      else if (nw == 24)
        EPHG_ROWS_NB(24);
      else
        EPHG_ROWS_NB(32);
#undef EPHG_ROWS_NB
      TCK(cudaGetLastError());
    } else if (rp.delta_kind == 0 && esm > 200 * 1024) {
      dim3 grid(nblk, ns);
      k_epilogue_split<<<grid, 128, 0, st>>>(nwv, (int)j0, CBr, CBi, NpC, rp, ed, qt, partial, nblk);
      TCK(cudaGetLastError());
    } else if (rp.delta_kind == 0) {
      const int spb = 16;
      dim3 grid(nblk, (ns + spb - 1) / spb);
      const size_t sm = esm;
      // once per process: changing a kernel attribute can wait for the device's queued work
      static std::once_flag attr_once;
      std::call_once(attr_once, [] {
        cudaFuncSetAttribute(k_epilogue_split2<0, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      });
      k_epilogue_split2<0, 0><<<grid, EPI_ROWS, sm, st>>>(nwv, (int)j0, (int)j0 + ns, spb, CBr, CBi, NpC, rp, ed, qt,
                                                         partial, nblk);
      TCK(cudaGetLastError());
    } else {
      launch_epilogue_fp32(nwv, (int)j0, (int)j0 + ns, CBr, CBi, NpC, rp, ed_in, partial, nblk, st);
    }
    *launches += 1;
    }
    *launches += 1;
  }
  return 0;
}

// The nw = 8, nb = 6 Gaussian-delta path: fused stage A (contraction over Re +
// initial-band rotation + k-half of the Rp phase, writing the six-plane state
// operand) and fused stage B (contraction over Rp + rate epilogue).
static int split_rates_fused86(SplitOperands &s, Workspace &ws, cudaStream_t st, const double2 *G64, int nwsk,
                               int nwsq, int64_t Nn, int nwv, int nst, const int mesh[3], int L, const double2 *roots,
                               const int *widx, const int *arow, int nA, const int *st_code,
                               const std::vector<int> &first_state, const int *Rk, const double *degk,
                               const int *kposA, const int *Rq, const double *degq, const int *kposB, const double2 *U,
                               const RateParams &rp, const EpiData &ed_in, double *partial, int nblk, int *err,
                               cudaEvent_t ev_stage_a, int64_t *launches, LaunchTimer *tA, LaunchTimer *tB,
                               std::mutex *build_mu, int chunk_us, const Yield &yield, const RateSets *sets) {
  int rc;
  const int ncol = 48;
  const int KpA = (int)rup(nwsk, 16), KpB = (int)rup(nwsq, 16);
  const int N = rp.N;
  const int Mp = (int)rup(nwv, 2 * BM);             // window k' rows, whole tile pairs
  const bool own_a = arow != widx;                  // A-rows other than the window (irreducible wedge)
  const int MpA = own_a ? (int)rup(nA, 2 * BM) : Mp;   // stage-A k rows
  const int64_t NA = (int64_t)8 * KpB * ncol;       // stage-A columns (m', kp, n', s')
  // contraction position -> Rp cell
  int *kinvB;
  if ((rc = wsget(ws, "tc_kinv", (size_t)KpB, &kinvB))) return tfail(6, ws.msg.c_str());
  TCK(cudaMemsetAsync(kinvB, 0xFF, (size_t)KpB * sizeof(int), st));
  k_kinv<<<(nwsq + 255) / 256, 256, 0, st>>>(nwsq, kposB, kinvB);
  TCK(cudaGetLastError());
  (*launches)++;
  // stage-A operand, built once per handle
  {
  std::lock_guard<std::mutex> build_lock(*build_mu);
  if (!s.GA6 || s.NA != NA || s.KpA6 != KpA) {
    if (s.GA6) {
      cudaFreeAsync(s.GA6, st);
      s.bytes -= (int64_t)6 * s.NA * s.KpA6 * sizeof(float);
    }
    s.GA6 = nullptr;
    TCK(pool_alloc((void **)&s.GA6, (size_t)6 * NA * KpA * sizeof(float), st));
    s.bytes += (int64_t)6 * NA * KpA * sizeof(float);
    TCK(cudaMemsetAsync(s.GA6, 0, (size_t)6 * NA * KpA * sizeof(float), st));
    const int64_t ne = NA * nwsk;
    k_gplanes_a6<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(nwsk, Nn, G64, kposA, kinvB, KpB, s.GA6, NA, KpA);
    TCK(cudaGetLastError());
    s.NA = NA;
    s.KpA6 = KpA;
    (*launches)++;
    TCK(cudaStreamSynchronize(st));   // complete before other streams may read it
  }
  }
  EpiTables et;
  if ((rc = epi_tables(ws, st, U, rp, ed_in, launches, &et))) return rc;
  // row, state and q tables of the fused epilogues
  int4 *trow;
  StateRec *tst;
  float4 *tU4, *trec;
  double *tens;
  if ((rc = wsget(ws, "tc_frow", (size_t)Mp, &trow)) || (rc = wsget(ws, "tc_fst", (size_t)nst, &tst)) ||
      (rc = wsget(ws, "tc_fU4", (size_t)32 * Mp, &tU4)) || (rc = wsget(ws, "tc_fens", (size_t)8 * Mp, &tens)) ||
      (rc = wsget(ws, "tc_frec", (size_t)30 * rup(N, 32), &trec)))
    return tfail(6, ws.msg.c_str());
  k_fused_rows<<<(Mp + 127) / 128, 128, 0, st>>>(nwv, Mp, widx, ed_in.ens, et.Uf, ed_in.cum, rp.enref, rp.fsthick,
                                                 mesh[0], mesh[1], trow, tU4, tens);
  k_fused_states<<<(nst + 127) / 128, 128, 0, st>>>(nst, st_code, arow, ed_in.ens, rp.chempot, kB * rp.T, mesh[0],
                                                    mesh[1], tst);
  k_fused_recs<<<(N * 6 + 255) / 256, 256, 0, st>>>(N, ed_in.uf, et.cx, et.bs, et.wv, trec);
  TCK(cudaGetLastError());
  *launches += 3;
  float2 *tglb = nullptr;   // polar: long_range_prefac(q, u_s), q-blocked
  if (ed_in.glpf) {
    if ((rc = wsget(ws, "tc_fglb", (size_t)6 * rup(N, 32), &tglb))) return tfail(6, ws.msg.c_str());
    k_fused_glp<<<(N * 6 + 255) / 256, 256, 0, st>>>(N, ed_in.glpf, tglb);
    TCK(cudaGetLastError());
    *launches += 1;
  }
  const FusedTabs tabs{trow, tst, tU4, tens, trec, tglb, Mp, N};
  // the other parameter sets' state and mode tables
  FusedSets xs{};
  xs.n = sets ? sets->n : 1;
  if (xs.n > 1) {
    float2 *occ;
    float4 *mode, *wvp;
    float *cxp, *bsp;
    const int64_t mstride = (int64_t)6 * rup(N, 32);
    if ((rc = wsget(ws, "tc_socc", (size_t)(xs.n - 1) * nst, &occ)) ||
        (rc = wsget(ws, "tc_smode", (size_t)(xs.n - 1) * mstride, &mode)) ||
        (rc = wsget(ws, "tc_scx", (size_t)N * 6, &cxp)) || (rc = wsget(ws, "tc_sbs", (size_t)N * 6, &bsp)) ||
        (rc = wsget(ws, "tc_swv", (size_t)N * 6, &wvp)))
      return tfail(6, ws.msg.c_str());
    for (int p = 1; p < xs.n; ++p) {
      const RateParams &r = sets->rp[p];
      k_qtab<<<(N * 6 + 255) / 256, 256, 0, st>>>(N * 6, ed_in.om, sets->bose[p], r.sigma, kB * r.T, r.const_tp, cxp,
                                                  bsp, wvp);
      k_fused_set_tabs<<<(std::max(nst, N * 6) + 127) / 128, 128, 0, st>>>(
          nst, N, tst, r.chempot, kB * r.T, bsp, wvp, occ + (size_t)(p - 1) * nst, mode + (p - 1) * mstride);
      TCK(cudaGetLastError());
      *launches += 2;
      const F2 isg = f2_of(1.0 / r.sigma);
      xs.isg_hi[p] = isg.hi;
      xs.isg_lo[p] = isg.lo;
      xs.dnorm[p] = (float)((1.0 / sqrt(2.0 * 3.141592653589793)) / r.sigma * r.inv_nk);
      xs.partial[p] = sets->partial[p];
    }
    xs.occ = occ;
    xs.mode = mode;
    xs.mode_stride = mstride;
  }
  // stage A's row tables: the window rows, or the A-rows with their first states
  FusedTabs tabsA = tabs;
  if (own_a) {
    int4 *trowA;
    float4 *tU4A;
    double *tensA;
    int *fsA;
    if ((rc = wsget(ws, "tc_frowA", (size_t)MpA, &trowA)) || (rc = wsget(ws, "tc_fU4A", (size_t)32 * MpA, &tU4A)) ||
        (rc = wsget(ws, "tc_fensA", (size_t)8 * MpA, &tensA)) || (rc = wsget(ws, "tc_fsA", (size_t)nA + 1, &fsA)))
      return tfail(6, ws.msg.c_str());
    TCK(cudaMemcpyAsync(fsA, first_state.data(), (size_t)(nA + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    k_fused_rows<<<(MpA + 127) / 128, 128, 0, st>>>(nA, MpA, arow, ed_in.ens, et.Uf, fsA, rp.enref, rp.fsthick,
                                                    mesh[0], mesh[1], trowA, tU4A, tensA);
    TCK(cudaGetLastError());
    *launches += 1;
    tabsA.row = trowA;
    tabsA.U4 = tU4A;
    tabsA.ensw = tensA;
    tabsA.MpB = MpA;
  }
  // state operand: whole 8-state groups (8 x 48 = 384 rows), six planes; padding rows zero
  const int64_t Np2 = rup(nst, 8) * ncol;
  float *PA, *PB, *B2;
  if ((rc = wsget(ws, "tc_PAf", (size_t)4 * MpA * KpA, &PA)) || (rc = wsget(ws, "tc_PB", (size_t)4 * Mp * KpB, &PB)) ||
      (rc = wsget(ws, "tc_B2", (size_t)6 * Np2 * KpB, &B2)))
    return tfail(6, ws.msg.c_str());
  {
    const int64_t used = (int64_t)nst * ncol;
    for (int pl = 0; pl < 6; ++pl)
      if (Np2 > used)
        TCK(cudaMemsetAsync(B2 + ((int64_t)pl * Np2 + used) * KpB, 0, (size_t)(Np2 - used) * KpB * sizeof(float), st));
  }
  // ---- stage A over the A-rows
  TCK(cudaMemsetAsync(PA, 0, (size_t)4 * MpA * KpA * sizeof(float), st));
  {
    const int64_t ne = (int64_t)nA * nwsk;
    k_phase_planes<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(nA, arow, mesh[0], mesh[1], mesh[2], L, nwsk, Rk,
                                                                 degk, kposA, roots, PA, MpA, KpA);
    TCK(cudaGetLastError());
    (*launches)++;
  }
  float2 *phk;
  if ((rc = wsget(ws, "tc_phk", (size_t)MpA * KpB, &phk))) return tfail(6, ws.msg.c_str());
  {
    const int64_t ne = (int64_t)MpA * KpB;
    k_phase_k_table<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(nA, MpA, KpB, arow, kinvB, mesh[0], mesh[1], mesh[2],
                                                                  L, Rq, degq, roots, phk);
    TCK(cudaGetLastError());
    (*launches)++;
  }
  FusedAArgs ga{};
  ga.KpB = KpB;
  ga.Np2 = Np2;
  ga.B2 = B2;
  ga.phk = phk;
  ga.err = err;
  tA->begin(st);
  if ((rc = stageA_fused86(PA, MpA, s.GA6, NA, KpA, tabsA, ga, st, chunk_us > 0 ? std::max(1, chunk_us / 25) : 0,
                           yield)))
    return rc;
  yield();
  tA->end(st);
  (*launches)++;
  TCK(cudaEventRecord(ev_stage_a, st));
  // ---- stage B: A planes = e^{2 pi i k'.Rp} for the window k'
  TCK(cudaMemsetAsync(PB, 0, (size_t)4 * Mp * KpB * sizeof(float), st));
  {
    const int64_t ne = (int64_t)nwv * nwsq;
    k_phase_planes<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(nwv, widx, mesh[0], mesh[1], mesh[2], L, nwsq, Rq,
                                                                 nullptr, kposB, roots, PB, Mp, KpB);
    TCK(cudaGetLastError());
    (*launches)++;
  }
  EpiData ed = ed_in;
  ed.Uf = et.Uf;
  tB->begin(st);
  if ((rc = stageB_fused86(PB, Mp, B2, Np2, KpB, nwv, nst, rp, ed, tabs, partial, nblk, err, st,
                           chunk_us > 0 ? std::max(1, chunk_us / 13) : 0, yield, xs)))
    return rc;
  tB->end(st);
  (*launches)++;
  return 0;
}

int split_rates_stage(SplitOperands &s, Workspace &ws, cudaStream_t st, const double2 *G64, int nwsk, int nwsq,
                      int64_t Nn, int nw, int nb, int nwv, int nst, const int mesh[3], int L, const double2 *roots,
                      const int *widx, const int *arow, int nA, const int *st_code,
                      const std::vector<int> &first_state, const int *Rk,
                      const double *degk, const int *kposA, const int *Rq, const double *degq, const int *kposB,
                      const double2 *U, const RateParams &rp, const EpiData &ed_in, double *partial, int nblk_max,
                      int *nblk_used, cudaEvent_t ev_stage_a, int64_t *launches, LaunchTimer *tA, LaunchTimer *tB,
                      std::mutex *build_mu, int chunk_us, const Yield &yield, const BatchMember *bm,
                      int64_t chunk_bytes, const RateSets *sets) {
  // The fused path packs mesh coordinates in 10 bits each.
  const bool fast86 = (nw == 8 && nb == 6 && rp.delta_kind == 0 && mesh[0] <= 1024 && mesh[1] <= 1024 &&
                       mesh[2] <= 1024);
  // rate partials per state: one per 32-row block of the fused kernel, one per 128 k' rows otherwise
  const int nblk = fast86 ? (int)(rup(nwv, 2 * BM) / 32) : (nwv + EPI_ROWS - 1) / EPI_ROWS;
  if (nblk > nblk_max) return tfail(1, "rate partial buffer too small");
  *nblk_used = nblk;
  int rc;
  int *err = nullptr;
  // the device error word lives in the workspace; the caller checks its own word afterwards
  if ((rc = wsget(ws, "tc_err", 1, &err))) return tfail(6, ws.msg.c_str());
  TCK(cudaMemsetAsync(err, 0, sizeof(int), st));
  if (fast86) {
    if ((rc = split_rates_fused86(s, ws, st, G64, nwsk, nwsq, Nn, nwv, nst, mesh, L, roots, widx, arow, nA, st_code,
                                  first_state, Rk, degk, kposA, Rq, degq, kposB, U, rp, ed_in, partial, nblk, err,
                                  ev_stage_a, launches, tA, tB, build_mu, chunk_us, yield, sets)))
      return rc;
  } else if ((rc = split_rates_generic(s, ws, st, G64, nwsk, nwsq, Nn, nw, nb, nwv, nst, mesh, L, roots, widx, arow,
                                       nA, st_code, first_state, Rk, degk, kposA, Rq, degq, kposB, U, rp, ed_in,
                                       partial, nblk, err,
                                       ev_stage_a, launches, tA, tB, build_mu, chunk_us, yield, bm,
                                       std::max<int64_t>(chunk_bytes, (int64_t)1 << 24), sets))) {
    return rc;
  }
  int herr = 0;
  TCK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  TCK(cudaStreamSynchronize(st));
  if (herr & DERR_TIMEOUT) return tfail(7, "tcgen05 GEMM: a bounded mbarrier wait gave up");
  return 0;
}
}  // namespace tc
}  // namespace ephg

// ----------------------------------------------------------- test hook
namespace ephg {
namespace tc {
// A (M,K) complex row-major -> planes [4][Mp][Kp]
__global__ void k_planes_rows(int64_t M, int K, const double2 *A, float *P, int64_t Mp, int Kp) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * K) return;
  int64_t r = idx / K;
  int k = (int)(idx % K);
  put4(P, Mp * Kp, r * Kp + k, A[idx]);
}
__global__ void k_join(int64_t M, int64_t N, const float *Cr, const float *Ci, int64_t ldc, double2 *C) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * N) return;
  int64_t r = idx / N, c = idx % N;
  C[idx] = make_double2(Cr[r * ldc + c], Ci[r * ldc + c]);
}

// The give-up path of the tcgen05 kernels' bounded waits, run on its own: one
// CTA of 64 threads.  Warp 1 allocates TMEM as the kernels do; warp 0 lane 0
// waits `limit` cycles on a barrier that no thread arrives on (or, with
// `arrive`, on one it has arrived on itself, which ends at once).  When the
// wait gives up it records DERR_TIMEOUT and, as an MMA issuer whose wait gave
// up, commits to its drain barrier and waits for it (no MMA was issued, so the
// commit arrives at once); then the CTA frees TMEM and returns.  No TMA load
// and no MMA is issued.
__global__ void __launch_bounds__(64) k_wait_probe(long long limit, int arrive, int *err) {
  __shared__ uint64_t bars[2];
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tslot)),
                 "r"(32)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;
  if (warp == 0 && lane == 0) {
    if (arrive) mbar_arrive(&bars[0]);
    if (!mbar_wait_limit(&bars[0], 0, err, limit)) {
      umma_commit(&bars[1]);
      mbar_wait_limit(&bars[1], 0, err, WAIT_CYCLES);
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(32) : "memory");
  }
}
}  // namespace tc
}  // namespace ephg

extern "C" int ephg_debug_wait_timeout(int64_t limit_cycles, int64_t arrive, int *device_err) {
  using namespace ephg;
  using namespace ephg::tc;
  if (limit_cycles < 0 || limit_cycles > WAIT_CYCLES) return tfail(1, "debug_wait_timeout: limit out of range");
  int *err = nullptr;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return tfail(2, "debug_wait_timeout: cudaMalloc failed");
  int rc = 0, herr = 0;
  cudaMemset(err, 0, sizeof(int));
  k_wait_probe<<<1, 64>>>((long long)limit_cycles, arrive ? 1 : 0, err);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (device_err) *device_err = herr;
  if (e != cudaSuccess) rc = tfail(2, cudaGetErrorString(e));
  else if (herr & DERR_TIMEOUT) rc = tfail(7, "debug_wait_timeout: bounded wait gave up");
  return rc;
}

extern "C" int ephg_debug_cgemm(int64_t M, int64_t N, int64_t K, const double *A, const double *B, double *C) {
  using namespace ephg;
  using namespace ephg::tc;
  if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !C) return tfail(1, "debug_cgemm: bad arguments");
  const int64_t Mp = rup(M, BM), Np = rup(N, BN), Kp = rup(K, BK);
  double2 *dA = nullptr, *dB = nullptr, *dC = nullptr;
  float *PA = nullptr, *PB = nullptr, *Cr = nullptr, *Ci = nullptr;
  int *err = nullptr;
  int rc = 0;
  cudaStream_t st = 0;
  auto cleanup = [&]() {
    for (void *p : {(void *)dA, (void *)dB, (void *)dC, (void *)PA, (void *)PB, (void *)Cr, (void *)Ci, (void *)err})
      if (p) cudaFree(p);
  };
  if (cudaMalloc(&dA, M * K * 16) || cudaMalloc(&dB, K * N * 16) || cudaMalloc(&dC, M * N * 16) ||
      cudaMalloc(&PA, 4 * Mp * Kp * 4) || cudaMalloc(&PB, 4 * Np * Kp * 4) || cudaMalloc(&Cr, Mp * Np * 4) ||
      cudaMalloc(&Ci, Mp * Np * 4) || cudaMalloc(&err, 4)) {
    cleanup();
    return tfail(6, "debug_cgemm: cudaMalloc failed");
  }
  cudaMemcpy(dA, A, M * K * 16, cudaMemcpyHostToDevice);
  cudaMemcpy(dB, B, K * N * 16, cudaMemcpyHostToDevice);
  cudaMemset(PA, 0, 4 * Mp * Kp * 4);
  cudaMemset(PB, 0, 4 * Np * Kp * 4);
  cudaMemset(err, 0, 4);
  k_planes_rows<<<(unsigned)((M * K + 255) / 256), 256>>>(M, (int)K, dA, PA, Mp, (int)Kp);
  dim3 grid((unsigned)((N + 31) / 32), (unsigned)((Kp + 31) / 32));
  k_gplanes<<<grid, dim3(32, 8)>>>(N, (int)K, dB, nullptr, PB, Np, (int)Kp);
  rc = cgemm(PA, Mp, 0, (int)Mp, PB, Np, 0, (int)Np, (int)Kp, Cr, Ci, Np, err, st);
  if (!rc) {
    k_join<<<(unsigned)((M * N + 255) / 256), 256>>>(M, N, Cr, Ci, Np, dC);
    cudaError_t e = cudaDeviceSynchronize();
    int herr = 0;
    cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = tfail(2, cudaGetErrorString(e));
    else if (herr) rc = tfail(7, "debug_cgemm: bounded wait gave up");
    else cudaMemcpy(C, dC, M * N * 16, cudaMemcpyDeviceToHost);
  }
  cleanup();
  return rc;
}

extern "C" const char *ephg_debug_last_error(void) { return ephg::tc::last_error(); }

// The grouped GEMM's tile lookup on the host: np problems of mtiles[i] x
// ntiles[i] tiles laid out as the batcher lays them out; every tile of the
// launch is mapped and hits[tile0(i) + mt + mtiles[i] nt] counted.  Returns
// EPHG_ERR_INDEX if a tile maps outside its problem or its rows disagree.
extern "C" int ephg_debug_group_tiles(int np, const int *mtiles, const int *ntiles, int *hits) {
  using namespace ephg::tc;
  if (np <= 0 || !mtiles || !ntiles || !hits) return 1;
  std::vector<GroupProblem> tab(np);
  int64_t T = 0;
  for (int i = 0; i < np; ++i) {
    memset(&tab[i], 0, sizeof(GroupProblem));
    if (mtiles[i] <= 0 || ntiles[i] <= 0) return 1;
    tab[i].g.mtiles = mtiles[i];
    tab[i].g.ntiles = ntiles[i];
    tab[i].g.nkb = 1;
    tab[i].g.Astride = (int64_t)mtiles[i] * BM;
    tab[i].g.Bstride = (int64_t)ntiles[i] * BN;
    tab[i].g.ldc = (int64_t)ntiles[i] * BN;
    tab[i].tile0 = (int)T;
    T += (int64_t)mtiles[i] * ntiles[i];
  }
  if (T > INT32_MAX) return 1;
  const GroupGemm jobs{tab.data(), np};
  for (int t = 0; t < (int)T; ++t) {
    const TileJob j = jobs(t);
    const int64_t p = (const uint8_t *)j.tA - (const uint8_t *)&tab[0].tA;
    if (p < 0 || p % (int64_t)sizeof(GroupProblem)) return EPHG_ERR_INDEX;
    const int i = (int)(p / (int64_t)sizeof(GroupProblem));
    if (i >= np || j.tB != &tab[i].tB || j.arow % BM || j.brow % BN) return EPHG_ERR_INDEX;
    const int mt = j.arow / BM, nt = j.brow / BN;
    if (mt >= mtiles[i] || nt >= ntiles[i] || t - tab[i].tile0 != mt + mtiles[i] * nt) return EPHG_ERR_INDEX;
    if ((int64_t)(j.Cr - (float *)nullptr) != (int64_t)mt * BM * tab[i].g.ldc + (int64_t)nt * BN)
      return EPHG_ERR_INDEX;
    hits[tab[i].tile0 + mt + mtiles[i] * nt]++;
  }
  return EPHG_OK;
}
