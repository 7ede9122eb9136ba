/*
 * tal_chain.h -- C ABI of the GB300 anchor chaining DP.
 *
 * Drop-in for TAL's dp_chain::mm_dp_vectorized
 * (src/chaining/parallel_chaining_32_bit.h:104-118 constructor, :216
 * mm_dp_vectorized), the minimap2 chaining step that benchmarks/
 * bench-dp-chaining.cpp times: per read, for every anchor, the best chain
 * score ending there (f), its predecessor (p) and the peak score on that
 * chain (v).  One GB300 GPU (sm_103a), many reads per call.  Plain C types
 * only.  Outputs equal the reference's on the same inputs.
 */
#ifndef TAL_CHAIN_H
#define TAL_CHAIN_H

#include <stddef.h>
#include <stdint.h>

#include "tal_bsw.h" /* status codes TAL_OK ... */

#ifdef __cplusplus
extern "C" {
#endif

/* anchor_t (parallel_chaining_32_bit.h:58-67): 16 bytes.  r: reference
 * position (the 64-bit value orders the anchors and bounds the predecessor
 * window; its low 32 bits enter the score), q: query position, l: anchor
 * length (>= 0).  A read's anchors are sorted by r, as the reference expects
 * (unsorted input is scored exactly as the reference scores it). */
typedef struct tal_anchor {
    uint64_t r;
    int32_t q;
    int32_t l;
} tal_anchor;

/* The eight tunables of dp_chain's constructor, in its order.  The scoring
 * uses bw and max_iter; the others are kept for the interface, as in the
 * reference's 32-bit path. */
typedef struct tal_chain_params {
    int32_t max_dist_x, max_dist_y, bw, max_skip, max_iter;
    float gap_scale;
    int32_t is_cdna, n_segs;
} tal_chain_params;

typedef struct tal_chain_ctx *tal_chain_handle;

int tal_chain_create(const tal_chain_params *params, int device, tal_chain_handle *out);
int tal_chain_destroy(tal_chain_handle h);

/* Replaces mm_dp_vectorized(n, anchors, anchor_r, anchor_q, anchor_l, f, p,
 * v, dr, dq, NULL, NULL) for n_reads reads at once, on host buffers: read k
 * is anchors[offsets[k], offsets[k+1]) and its outputs f, p, v sit at the
 * same indices (p indexes within the read, -1 for none).  dr, dq: the
 * call's distance limits (5000 and 5000 in the reference driver).  Errors:
 * TAL_EINVAL (malformed offsets), TAL_EDOMAIN (a negative anchor length or a
 * read of 2^31 anchors or more; tal_chain_last_bad_read names the read). */
int tal_chain_dp(tal_chain_handle h, const tal_anchor *anchors, const int64_t *offsets,
                 int32_t n_reads, int32_t dr, int32_t dq, uint32_t *f, int32_t *p, int32_t *v);

/* The same on device buffers (d_offsets has n_reads + 1 entries, anchors up
 * to d_offsets[n_reads]); synchronous. */
int tal_chain_dp_device(tal_chain_handle h, const tal_anchor *d_anchors, const int64_t *d_offsets,
                        int32_t n_reads, int32_t dr, int32_t dq, uint32_t *d_f, int32_t *d_p,
                        int32_t *d_v);

/* The handle's CUDA stream (a cudaStream_t). */
void *tal_chain_stream(tal_chain_handle h);
const char *tal_chain_last_error(tal_chain_handle h);
int64_t tal_chain_last_bad_read(tal_chain_handle h);
/* Predecessors scored by the last call: the sum over anchors of i - st. */
uint64_t tal_chain_last_evals(tal_chain_handle h);

#ifdef __cplusplus
}
#endif

#endif /* TAL_CHAIN_H */
