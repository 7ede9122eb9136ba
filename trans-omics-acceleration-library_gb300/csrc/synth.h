// Seeded synthetic seed-extension workloads (host only).  Stand-in for the
// pair files that benchmarks/bench-bsw.cpp:117-169 reads; see synth.cpp.
#ifndef TAL_BSW_SYNTH_H
#define TAL_BSW_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    TAL_SYNTH_LEN_FIXED = 0,      // len2 = len_lo
    TAL_SYNTH_LEN_UNIFORM = 1,    // len2 ~ U[len_lo, len_hi]
    TAL_SYNTH_LEN_LOGNORMAL = 2   // len2 = clip(round(exp(ln median + sigma N(0,1))), lo, hi)
};

typedef struct tal_synth_cfg {
    uint64_t seed;
    int32_t len_dist, len_lo, len_hi;
    double len_median, len_sigma;
    double n_rate;                 // per-base probability of N (4) in the query
    double err_lo, err_hi;         // per-pair error rate ~ U[err_lo, err_hi]
    double sub_frac, ins_frac, del_frac;  // split of the error rate
    int32_t indel_lo, indel_hi;    // indel length ~ U[indel_lo, indel_hi]
    double homopolymer_del_bias;   // > 1: deletions this much likelier inside runs
    int32_t extra_lo, extra_hi;    // len1 = len2 + U[extra_lo, extra_hi]
    int32_t h0_lo, h0_hi;          // h0 ~ U[h0_lo, h0_hi]
    int32_t h0_cap_8bit;           // 1: h0 <= 127 - match * min(len1, len2)
    int32_t match;                 // match score used by h0_cap_8bit
    int32_t w_default;             // band when n_w_choices == 0
    int32_t n_w_choices;           // > 0: band drawn uniformly from w_choices
    int32_t w_choices[8];
} tal_synth_cfg;

// Per-pair lengths, h0 and band for pairs [first, first + count).  Any output
// pointer may be NULL.  nthreads <= 0: all hardware threads.
int tal_synth_plan(const tal_synth_cfg *cfg, int64_t first, int64_t count,
                   int32_t *len1, int32_t *len2, int32_t *h0, int32_t *w,
                   int nthreads);

// Bases of pairs [first, first + count): reference k at ref + ref_off[k],
// query k at qer + qer_off[k], lengths from tal_synth_plan.
int tal_synth_fill(const tal_synth_cfg *cfg, int64_t first, int64_t count,
                   const int32_t *len1, const int32_t *len2,
                   const int64_t *ref_off, const int64_t *qer_off,
                   uint8_t *ref, uint8_t *qer, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
