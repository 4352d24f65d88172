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

#ifdef __cplusplus
extern "C" {
#endif

/* C (M,N) = A (M,K) x B (K,N), complex, row-major, interleaved (re, im)
 * doubles on the host; computed on the device as a 3xTF32 tcgen05 GEMM with
 * FP32 accumulation.  Returns EPHG_OK or an error code. */
int ephg_debug_cgemm(int64_t M, int64_t N, int64_t K, const double *A, const double *B, double *C);
/* message of the last failure of the hook */
const char *ephg_debug_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
