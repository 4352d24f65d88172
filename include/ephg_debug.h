/*
 * ephg_debug.h - test hook of the split-precision contraction kernel.
 *
 * Not part of the drop-in surface: no reference procedure corresponds to it.
 * It exposes the 3xTF32 tcgen05 complex GEMM on its own so that tests can
 * check it against an FP64 product on arbitrary shapes.
 */
#ifndef EPHG_DEBUG_H
#define EPHG_DEBUG_H
#include <stdint.h>

#include "ephg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* C (M,N) = A (M,K) x B (K,N), complex, row-major, interleaved (re, im)
 * doubles on the host; computed on the device as a 3xTF32 tcgen05 GEMM with
 * FP32 accumulation.  Returns EPHG_OK or an error code. */
int ephg_debug_cgemm(int64_t M, int64_t N, int64_t K, const double *A, const double *B, double *C);
/* message of the last failure of the hook */
const char *ephg_debug_last_error(void);

/* The give-up path of the tcgen05 kernels' bounded barrier waits, on its own:
 * one CTA allocates TMEM, waits limit_cycles (0 .. ~4e9 SM cycles) on a
 * barrier that nothing arrives on (arrive != 0: one it arrived on itself),
 * records the timeout in its error word, drains its (empty) MMA queue, frees
 * TMEM and returns; no TMA load or MMA is issued.  *device_err (nullable)
 * receives the error word.  Returns EPHG_ERR_TIMEOUT when the wait gave up --
 * what every kernel entry point returns when one of its waits does -- and
 * EPHG_OK when it did not; the CUDA context stays usable either way. */
int ephg_debug_wait_timeout(int64_t limit_cycles, int64_t arrive, int *device_err);

/* The serving loop's slots, queue, admission, GPU hand-over and statistics run
 * against a simulated executor (no GPU): two crystals of 1000 resident bytes
 * each; request i for crystal i % 2 with a cubic mesh meshes[i] needs
 * per_request_bytes * mesh^3 / 1000 bytes and service_ms * (mesh / 8)^3 of
 * simulated device time in four parts with yield points between them; request
 * 0 is submitted 0.2 ms before the others.  Fills *out with the server's
 * statistics, *max_concurrent with the most requests seen in flight at once
 * and lat_ms[i] (nullable) with each request's latency (-1: refused or
 * failed); returns EPHG_ERR_INDEX if a result reached the wrong ticket.
 * temps (nullable): request i's T, which makes it mergeable with the queued
 * requests of its crystal and mesh (ephg_server_set_merge; max_sets in
 * 1..EPHG_MAX_SETS, else the default); a merged run takes one request's
 * simulated time and writes crystal + 1000 T as each request's result. */
int ephg_debug_server_selftest(int nreq, int nslots, double service_ms, int64_t budget, int64_t per_request_bytes,
                               const int64_t *meshes, const double *temps, int max_sets, ephg_server_stats *out,
                               int *max_concurrent, double *lat_ms);

/* The batched form's round logic (the grouped launches' gate) under nmembers
 * host threads, no GPU: members alternate active stretches of 1-4 submissions
 * with random pauses (seeded) and inactive stretches, iters times each.
 * Checks that every submission is launched exactly once, in each member's
 * order, before its submit returns, and that no member stays blocked (60 s).
 * Fills *rounds (launches) and *max_group (most items in one launch);
 * returns EPHG_ERR_INDEX on a broken invariant, EPHG_ERR_TIMEOUT on a
 * deadlock. */
int ephg_debug_batcher_selftest(int nmembers, int iters, uint64_t seed, int64_t *rounds, int64_t *max_group);

/* The grouped GEMM's tile -> (problem, row tile, column tile) lookup, run on
 * the host over np problems of mtiles[i] x ntiles[i] output tiles laid out in
 * one launch's tile space as the batcher lays them out (problem i from tile
 * sum_{j<i} mtiles[j] ntiles[j]); counts each tile's hits in hits[] (sized
 * to the total).  Returns EPHG_ERR_INDEX if a tile maps outside its problem
 * or its operand rows and output offset disagree. */
int ephg_debug_group_tiles(int np, const int *mtiles, const int *ntiles, int *hits);

#ifdef __cplusplus
}
#endif
#endif
