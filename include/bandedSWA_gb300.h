/*
 * bandedSWA_gb300.h -- C++ drop-in for TAL's BandedPairWiseSW
 * (src/alignment/BSW/bandedSWA.h:90-336) on one GB300, over the C ABI in
 * tal_bsw.h.  Header only; link with libtal_bsw.so.
 *
 * Same class name, constructor, method names, argument order and meaning as
 * the reference, and the same SeqPair record (14 x int32, layout checked
 * below), so a caller written against bandedSWA.h (benchmarks/bench-bsw.cpp
 * :213-258, BWA-MEM2's extension step) compiles against this header
 * unchanged.  Where the reference exits the process on failure
 * (bandedSWA.cpp:88-93, 2705-2708), so does this class, after printing the
 * library's reason.
 *
 *   getScores8 / getScores16   (bandedSWA.h:257-262, 285-290): the vector
 *       kernels' outputs, bit for bit, the reference's SIMD grouping
 *       included (see tal_bsw_scores).
 *   scalarBandedSWA / scalarBandedSWAWrapper (bandedSWA.h:124-135): the
 *       reference's scalar path scores pairs one at a time with the scoring
 *       matrix and a z-drop weighted by the gap extension; it equals the
 *       vector kernels' outputs for a pair alone in its group when
 *       e_del = e_ins = 1 and the matrix is the one bench-bsw builds
 *       (bwa_fill_scmat: w_match on the diagonal, -w_mismatch off it, -1 for
 *       N).  Those calls run on the GPU (TAL_BSW_PER_PAIR); any other
 *       parameters are refused with a message, since the GPU does not run the
 *       scalar arithmetic.
 *   SW_cells (bandedSWA.h:116): the DP cells of the calls so far (the
 *       reference declares the counter and never increments it).
 *
 * One instance owns one library handle (a CUDA stream and device buffers);
 * calls on one instance are serialised, separate instances may run at once.
 * numThreads is accepted and ignored (the reference ignores it too).
 */
#ifndef BANDEDSWA_GB300_H
#define BANDEDSWA_GB300_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tal_bsw.h"

/* SeqPair, bandedSWA.h:90-99. */
typedef struct dnaSeqPair {
    int32_t idr, idq, id;
    int32_t len1, len2;
    int32_t h0;
    int seqid, regid;
    int32_t score, tle, gtle, qle;
    int32_t gscore, max_off;
} SeqPair;

static_assert(sizeof(SeqPair) == 56, "SeqPair is 14 x int32");
static_assert(sizeof(SeqPair) == sizeof(tal_seq_pair), "SeqPair matches tal_seq_pair");
static_assert(offsetof(SeqPair, idr) == offsetof(tal_seq_pair, idr), "idr");
static_assert(offsetof(SeqPair, idq) == offsetof(tal_seq_pair, idq), "idq");
static_assert(offsetof(SeqPair, id) == offsetof(tal_seq_pair, id), "id");
static_assert(offsetof(SeqPair, len1) == offsetof(tal_seq_pair, len1), "len1");
static_assert(offsetof(SeqPair, len2) == offsetof(tal_seq_pair, len2), "len2");
static_assert(offsetof(SeqPair, h0) == offsetof(tal_seq_pair, h0), "h0");
static_assert(offsetof(SeqPair, seqid) == offsetof(tal_seq_pair, seqid), "seqid");
static_assert(offsetof(SeqPair, regid) == offsetof(tal_seq_pair, regid), "regid");
static_assert(offsetof(SeqPair, score) == offsetof(tal_seq_pair, score), "score");
static_assert(offsetof(SeqPair, tle) == offsetof(tal_seq_pair, tle), "tle");
static_assert(offsetof(SeqPair, gtle) == offsetof(tal_seq_pair, gtle), "gtle");
static_assert(offsetof(SeqPair, qle) == offsetof(tal_seq_pair, qle), "qle");
static_assert(offsetof(SeqPair, gscore) == offsetof(tal_seq_pair, gscore), "gscore");
static_assert(offsetof(SeqPair, max_off) == offsetof(tal_seq_pair, max_off), "max_off");

class BandedPairWiseSW {
public:
    uint64_t SW_cells;

    BandedPairWiseSW(const int o_del, const int e_del, const int o_ins, const int e_ins,
                     const int zdrop, const int end_bonus, const int8_t *mat_,
                     const int8_t w_match, const int8_t w_mismatch, int numThreads)
        : SW_cells(0), h_(nullptr), e_del_(e_del), e_ins_(e_ins), std_mat_(true) {
        (void)numThreads;
        tal_bsw_params p;
        p.o_del = o_del; p.e_del = e_del; p.o_ins = o_ins; p.e_ins = e_ins;
        p.zdrop = zdrop; p.end_bonus = end_bonus;
        p.w_match = w_match;
        p.w_mismatch = w_mismatch;
        if (tal_bsw_create(&p, -1, &h_) != TAL_OK) {
            fprintf(stderr, "BandedPairWiseSW: parameters out of range or no GB300 device\n");
            exit(EXIT_FAILURE);
        }
        // the scalar path's scoring matrix: the one bench-bsw builds?
        if (mat_) {
            for (int i = 0; i < 5; i++)
                for (int j = 0; j < 5; j++) {
                    const int want = (i == 4 || j == 4) ? -1 : (i == j ? w_match : -w_mismatch);
                    if (mat_[i * 5 + j] != want) std_mat_ = false;
                }
        }
    }
    ~BandedPairWiseSW() {
        if (h_) tal_bsw_destroy(h_);
    }
    BandedPairWiseSW(const BandedPairWiseSW &) = delete;
    BandedPairWiseSW &operator=(const BandedPairWiseSW &) = delete;

    // bandedSWA.h:257-262
    void getScores8(SeqPair *pairArray, uint8_t *seqBufRef, uint8_t *seqBufQer, int32_t numPairs,
                    uint16_t numThreads, int32_t w) {
        (void)numThreads;
        run(pairArray, seqBufRef, seqBufQer, numPairs, w, TAL_BSW_8, "getScores8");
    }
    // bandedSWA.h:285-290
    void getScores16(SeqPair *pairArray, uint8_t *seqBufRef, uint8_t *seqBufQer, int32_t numPairs,
                     uint16_t numThreads, int32_t w) {
        (void)numThreads;
        run(pairArray, seqBufRef, seqBufQer, numPairs, w, TAL_BSW_16, "getScores16");
    }

    // bandedSWA.h:124-128: one pair; returns the score, the rest through the pointers
    int scalarBandedSWA(int qlen, const uint8_t *query, int tlen, const uint8_t *target, int32_t w,
                        int h0, int *_qle, int *_tle, int *_gtle, int *_gscore, int *_max_off) {
        scalar_check("scalarBandedSWA");
        SeqPair p;
        memset(&p, 0, sizeof(p));
        p.len1 = tlen;
        p.len2 = qlen;
        p.h0 = h0;
        run(&p, const_cast<uint8_t *>(target), const_cast<uint8_t *>(query), 1, w,
            TAL_BSW_16 | TAL_BSW_PER_PAIR, "scalarBandedSWA");
        if (_qle) *_qle = p.qle;
        if (_tle) *_tle = p.tle;
        if (_gtle) *_gtle = p.gtle;
        if (_gscore) *_gscore = p.gscore;
        if (_max_off) *_max_off = p.max_off;
        return p.score;
    }
    // bandedSWA.h:130-135 (query = seq2 = len2, target = seq1 = len1, as
    // bandedSWA.cpp:242-260 passes them)
    void scalarBandedSWAWrapper(SeqPair *seqPairArray, uint8_t *seqBufRef, uint8_t *seqBufQer,
                                int numPairs, int nthreads, int32_t w) {
        (void)nthreads;
        scalar_check("scalarBandedSWAWrapper");
        run(seqPairArray, seqBufRef, seqBufQer, numPairs, w, TAL_BSW_16 | TAL_BSW_PER_PAIR,
            "scalarBandedSWAWrapper");
    }

    // The library handle, for the calls of tal_bsw.h this class does not wrap
    // (batched form, device-resident buffers, serving).
    tal_bsw_handle handle() const { return h_; }

private:
    tal_bsw_handle h_;
    int e_del_, e_ins_;
    bool std_mat_;

    void run(SeqPair *pairs, uint8_t *ref, uint8_t *qer, int32_t n, int32_t w, int bits,
             const char *what) {
        const int rc = tal_bsw_scores(h_, reinterpret_cast<tal_seq_pair *>(pairs), ref, qer, n, w, bits);
        if (rc != TAL_OK) {
            fprintf(stderr, "BandedPairWiseSW::%s: status %d: %s (pair %lld)\n", what, rc,
                    tal_bsw_last_error(h_), (long long)tal_bsw_last_bad_pair(h_));
            exit(EXIT_FAILURE);
        }
        SW_cells += tal_bsw_last_cells(h_);
    }
    void scalar_check(const char *what) const {
        if (e_del_ != 1 || e_ins_ != 1 || !std_mat_) {
            fprintf(stderr,
                    "BandedPairWiseSW::%s: the GPU runs the scalar path only where it equals the "
                    "vector kernels (e_del = e_ins = 1, bench-bsw's scoring matrix)\n", what);
            exit(EXIT_FAILURE);
        }
    }
};

#endif /* BANDEDSWA_GB300_H */
