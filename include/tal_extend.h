/*
 * tal_extend.h -- caller-side seed extension on the GB300 banded
 * Smith-Waterman: the step before BandedPairWiseSW::getScores in a BWA-MEM2
 * style aligner (its mem_chain2aln stage, which is not part of TAL), that
 * turns exact-match seeds into SeqPair batches -- a left extension over the
 * reversed sequences before the seed, then a right extension after it whose
 * h0 is the left result -- and the two results into an alignment region.
 * Plain C types only.
 *
 * Per seed (read r of length L, query [qbeg, qbeg + len) matching the
 * reference at [rbeg, rbeg + len)), with the handle's scoring (a = w_match)
 * and the call's band w:
 *   gap(n) = clamp(max((n*a - o_del) / e_del + 1, (n*a - o_ins) / e_ins + 1), 1, 2w)
 *            (integer division)
 *   left, when qbeg > 0: target = reference [max(0, rbeg - qbeg - gap(qbeg)), rbeg)
 *     reversed, query = read [0, qbeg) reversed, h0 = len * a.  Result
 *     (score, qle, tle, gtle, gscore): if gscore <= 0 or gscore <= score -
 *     pen_clip5, the local end: qb = qbeg - qle, rb = rbeg - tle, sc = score;
 *     else the read's start: qb = 0, rb = rbeg - gtle, sc = gscore.
 *     Without a left extension: qb = qbeg, rb = rbeg, sc = len * a.
 *   right, when qbeg + len < L: target = reference [rbeg + len, min(ref_len,
 *     rbeg + len + (L - qbeg - len) + gap(L - qbeg - len))), query = read
 *     [qbeg + len, L), h0 = sc.  If gscore <= 0 or gscore <= score - pen_clip3:
 *     qe = qbeg + len + qle, re = rbeg + len + tle, sc = score; else qe = L,
 *     re = rbeg + len + gtle, sc = gscore.  Without one: qe = qbeg + len,
 *     re = rbeg + len.
 * All left extensions of a call are one batch, all right ones another, both
 * through the plain device launch (8/16-bit routing per pair); with band
 * retries, the pairs that go again form a smaller batch per attempt, on the
 * same windows (the right batch starts after the left one's last attempt).
 * The call uses
 * the handle's stream and buffers: do not run it concurrently with other
 * calls on the same handle.
 */
#ifndef TAL_EXTEND_H
#define TAL_EXTEND_H

#include <stddef.h>
#include <stdint.h>

#include "tal_bsw.h"

#ifdef __cplusplus
extern "C" {
#endif

/* An exact match of read `read`'s bases [qbeg, qbeg + len) to the
 * reference's [rbeg, rbeg + len).  24 bytes. */
typedef struct tal_seed {
    int32_t read;
    int32_t qbeg;
    int64_t rbeg;
    int32_t len;
    int32_t pad_;
} tal_seed;

typedef struct tal_extend_params {
    int32_t w;          /* band of both extensions */
    int32_t pen_clip5;  /* left clipping penalty */
    int32_t pen_clip3;  /* right clipping penalty */
    int32_t band_tries; /* attempts per extension, band w << i (0 or 1: one; BWA-MEM uses 2;
                           at most 8, and w << (band_tries - 1) at most 2^24):
                           an extension is run again with the doubled band while its score
                           changed from the previous attempt's (or it is the first) and its
                           max_off >= (band >> 1) + (band >> 2); the last attempt's result
                           stands */
} tal_extend_params;

/* The region a seed extends to: reference [rb, re), read [qb, qe), its score,
 * and the score after the left extension (the right one's h0).  32 bytes. */
typedef struct tal_region {
    int64_t rb, re;
    int32_t qb, qe;
    int32_t score;
    int32_t left_score;
} tal_region;

/* Extends n_seeds seeds over host buffers: the reference (ref_len bases),
 * the reads back to back (read k = reads[read_off[k], read_off[k+1])), the
 * seeds; writes one region per seed.  Bases 0..3, 4 = N.  Errors:
 * TAL_EINVAL (NULL buffers, negative counts), TAL_EDOMAIN (a seed outside its
 * read or the reference -- tal_bsw_last_bad_pair names it -- or an extension
 * outside the scorer's exact range), TAL_ENOMEM, TAL_ECUDA. */
int tal_bsw_extend_seeds(tal_bsw_handle h, const uint8_t *ref, int64_t ref_len, const uint8_t *reads,
                         const int64_t *read_off, int32_t n_reads, const tal_seed *seeds,
                         int32_t n_seeds, const tal_extend_params *xp, tal_region *out);

#ifdef __cplusplus
}
#endif

#endif /* TAL_EXTEND_H */
