// ephg_tc.cuh - split-precision (3xTF32) tensor-core path of the rate pipeline.
#pragma once
#include <atomic>
#include <mutex>
#include <vector>

#include "ephg_kernels.cuh"
#include "ephg_ws.cuh"

namespace ephg {
namespace tc {

// Operand planes of the split form kept resident per handle.
struct SplitOperands {
  float *G = nullptr;      // g(Re,Rp) as K-major TF32 planes [4][Nn][Kpad]: hi_r, hi_i, lo_r, lo_i
  int64_t Nn = 0;
  int Kp = 0;              // padded K (WS cells)
  float *GA6 = nullptr;    // the fused nw = 8, nb = 6 path's stage-A operand: six planes [6][NA][KpA6]
  int64_t NA = 0;
  int KpA6 = 0;
  std::atomic<int64_t> bytes{0};   // device bytes held by G and GA6 (read by the serving loop's budget)
};

// stream-ordered on st (the handle's stream, synchronised by the caller)
void free_split(SplitOperands &s, cudaStream_t st);
const char *last_error();

// Grouped launches of the split form's GEMMs across rate requests that run
// concurrently, one host thread and stream each (the batched form): a member
// that reaches a GEMM waits until every active member has one too, and the
// round's GEMMs run as one persistent launch.  Members are active only inside
// the generic contraction stages.
class GemmBatcher;
struct BatchMember {
  GemmBatcher *gb = nullptr;
  int id = -1;   // 0 .. nmembers - 1: one per concurrently running request
};
GemmBatcher *batcher_create(int nmembers);   // nullptr on failure
void batcher_destroy(GemmBatcher *b);
void batcher_activate(const BatchMember &m);
void batcher_deactivate(const BatchMember &m);
// the device error word of the grouped launches (DERR_TIMEOUT if a bounded wait gave up)
int batcher_device_error(GemmBatcher *b);
void batcher_stats(const GemmBatcher *b, int64_t *launches, int64_t *problems, int64_t *tiles, int64_t *max_group);

// Stage A + B + C of the rate pipeline in the split form: fills the rate
// partials.  widx (nwv) lists the window k' rows of stage B; arow (nA) the
// k-points of the initial states (the A-rows of stage A: the window points, or
// their irreducible wedge), st_code the states as A-row * nw + band and
// first_state (nA + 1) the first state of each A-row.  Fills the rate
// partials [state][k'-block] like the FP64 path, using up to nblk_max k'
// blocks (*nblk_used returns the count).  kposA / kposB give the contraction
// position of each Re / Rp cell (cells ordered far to near).  Records
// ev_stage_a after stage A.  The operand planes kept in s are built once,
// under build_mu and completed before it is released, so that requests on
// other streams may share them.  chunk_us > 0 splits the persistent
// contraction kernels into launches of about that many microseconds, so that
// other streams' kernels get the SMs between them.  bm: the generic path's
// GEMMs join the member's batcher (grouped launches).  chunk_bytes bounds the
// generic path's per-chunk GEMM outputs (stage-A rows, stage-B states).
// Returns 0 or an EPHG_ERR_* code (message in last_error()).
int split_rates_stage(SplitOperands &s, Workspace &ws, cudaStream_t st, const double2 *G64,
                      int nwsk, int nwsq, int64_t Nn, int nw, int nb, int nwv, int nst,
                      const int mesh[3], int L, const double2 *roots, const int *widx,
                      const int *arow, int nA, const int *st_code, const std::vector<int> &first_state,
                      const int *Rk,
                      const double *degk, const int *kposA, const int *Rq, const double *degq,
                      const int *kposB, const double2 *U, const RateParams &rp, const EpiData &ed,
                      double *partial, int nblk_max, int *nblk_used, cudaEvent_t ev_stage_a,
                      int64_t *launches, LaunchTimer *tA, LaunchTimer *tB, std::mutex *build_mu,
                      int chunk_us = 0, const Yield &yield = Yield(), const BatchMember *bm = nullptr,
                      int64_t chunk_bytes = (int64_t)1 << 31, const RateSets *sets = nullptr);

}  // namespace tc
}  // namespace ephg
