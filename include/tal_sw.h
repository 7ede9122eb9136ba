/*
 * tal_sw.h -- C ABI of the GB300 unbanded Smith-Waterman scorer.
 *
 * Drop-in for TAL's PairWiseSW_8 / PairWiseSW_16 / PairWiseSW_32
 * (src/alignment/Smith-Waterman/PairWiseSW*.h): local alignment scores with
 * affine gaps, one score per pair, on one GB300 GPU (sm_103a).  Plain C types
 * only.  Scores equal the reference's getScores on the same inputs.
 */
#ifndef TAL_SW_H
#define TAL_SW_H

#include <stddef.h>
#include <stdint.h>

#include "tal_bsw.h" /* status codes TAL_OK ... */

#ifdef __cplusplus
extern "C" {
#endif

/* SeqPair of the unbanded kernels (PairWiseSW.h:44-49): 12 bytes.  Pair k's
 * sequences lie in the caller's buffer at seqBuf + 2*id*L (seq1, length len1)
 * and seqBuf + (2*id + 1)*L (seq2, length len2), L = the precision's
 * MAX_SEQ_LEN: 128 (8-bit), 1024 (16- and 32-bit), as in
 * PairWiseSW_16.cpp:297,313.  Bytes are compared as they are. */
typedef struct tal_sw_pair {
    int32_t id;
    int16_t len1, len2;
    int32_t score;
} tal_sw_pair;

/* Constructor arguments of PairWiseSW (PairWiseSW.h:86): weights added to a
 * score, so mismatch, open and extend are <= 0 (TAL_EINVAL otherwise: with a
 * positive gap weight the reference's result depends on which other pairs
 * share its SIMD group). */
typedef struct tal_sw_params {
    int32_t w_match, w_mismatch, w_open, w_extend;
} tal_sw_params;

typedef struct tal_sw_ctx *tal_sw_handle;

int tal_sw_create(const tal_sw_params *params, int device, tal_sw_handle *out);
int tal_sw_destroy(tal_sw_handle h);

/* Replaces getScores(pairArray, seqBuf, numPairs, numThreads) of
 * PairWiseSW_8 / _16 / _32 (bits = 8, 16, 32): scores pairs[0, numPairs) on
 * host buffers.  Exact range, else TAL_EDOMAIN (tal_sw_last_bad_pair names
 * the first pair): sequence lengths up to MAX_SEQ_LEN - 4 (the reference
 * writes past its buffers beyond that), the best score and the weights inside
 * the precision's element type. */
int tal_sw_scores(tal_sw_handle h, tal_sw_pair *pairs, const uint8_t *seqBuf, int32_t numPairs,
                  int bits);

/* The same on device buffers (seq_bytes: size of d_seqbuf); synchronous. */
int tal_sw_scores_device(tal_sw_handle h, tal_sw_pair *d_pairs, const uint8_t *d_seqbuf,
                         size_t seq_bytes, int32_t numPairs, int bits);

/* The handle's CUDA stream (a cudaStream_t). */
void *tal_sw_stream(tal_sw_handle h);
const char *tal_sw_last_error(tal_sw_handle h);
int64_t tal_sw_last_bad_pair(tal_sw_handle h);
/* len1 * len2 summed over the last call's pairs (the reference driver's
 * SW_cells, bench-smith-waterman.cpp:117). */
uint64_t tal_sw_last_cells(tal_sw_handle h);

#ifdef __cplusplus
}
#endif

#endif /* TAL_SW_H */
