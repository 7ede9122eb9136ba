// Test infrastructure only: a C entry point around the reference's own
// BandedPairWiseSW, compiled straight from the read-only reference tree by
// oracle/build_ref.sh into oracle/_ref/.  Used to pin the oracle restatement
// (oracle/bsw_oracle.c) and to generate the golden fixtures; never linked into
// the product library.
//
// The reference class is driven exactly the way benchmarks/bench-bsw.cpp:213-253
// drives it: one instance built from (o_del, e_del, o_ins, e_ins, zdrop,
// end_bonus, mat, a, b, 1) with mat from bwa_fill_scmat (bench-bsw.cpp:56-64),
// then getScores8 / getScores16 / scalarBandedSWAWrapper on a SeqPair array.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
// The scratch rows (F16_, H16_, ...) are private members that the reference
// allocates uninitialised and never clears between 32/64-pair groups; the
// "pristine" mode below needs to zero them, so the shim views them as public.
// The class layout is unchanged.
#define private public
#include "bandedSWA.h"
#undef private

// bandedSWA.cpp:43 declares this profiling table extern; bench-bsw.cpp:54
// normally defines it.
uint64_t prof[10][112];

static void fill_scmat(int a, int b, int ambig, int8_t mat[25]) {
    int k = 0;
    for (int i = 0; i < 4; ++i) {
        for (int j = 0; j < 4; ++j) mat[k++] = (i == j) ? a : -b;
        mat[k++] = ambig;
    }
    for (int j = 0; j < 5; ++j) mat[k++] = ambig;
}

extern "C" {

int ref_simd_width8(void) { return SIMD_WIDTH8; }
int ref_simd_width16(void) { return SIMD_WIDTH16; }

// mode: 8 -> getScores8, 16 -> getScores16, 0 -> scalarBandedSWAWrapper.
// pristine != 0 (vector modes only): one call per group of SIMD_WIDTH pairs,
// with the instance's scratch rows zeroed before each group.  The reference
// reads one scratch cell it has not written in the current group (the vertical
// gap row at column ncol, in the tail re-derivation after a band-limited row,
// bandedSWA.cpp:3267-3314), so without this its results can depend on what
// earlier groups or earlier heap users left there.
// pairs: 14 x int32 per pair (the SeqPair layout).  The reference writes
// pairArray[n .. roundUp(n, SIMD_WIDTH)) and reads a few entries further for
// prefetching (bandedSWA.cpp:2013-2018, 2104), so the call runs on a padded,
// zero-filled copy and only [0, n) is copied back.
int ref_bsw_run(int o_del, int e_del, int o_ins, int e_ins, int zdrop,
                int end_bonus, int a, int b, int mode, int32_t *pairs,
                uint8_t *ref, uint8_t *qer, int32_t n, int32_t w, int pristine) {
    int8_t mat[25];
    fill_scmat(a, b, -1, mat);
    BandedPairWiseSW bsw(o_del, e_del, o_ins, e_ins, zdrop, end_bonus, mat,
                         (int8_t)a, (int8_t)b, 1);
    size_t cap = (size_t)n + 256;
    SeqPair *buf = (SeqPair *)calloc(cap, sizeof(SeqPair));
    if (!buf) return -1;
    memcpy(buf, pairs, (size_t)n * sizeof(SeqPair));
    const size_t s8 = (size_t)MAX_SEQ_LEN8 * SIMD_WIDTH8;
    const size_t s16 = (size_t)MAX_SEQ_LEN16 * SIMD_WIDTH16 * sizeof(int16_t);
    if (mode == 0) {
        bsw.scalarBandedSWAWrapper(buf, ref, qer, n, 1, w);
    } else if (!pristine) {
        if (mode == 8) bsw.getScores8(buf, ref, qer, n, 1, w);
        else bsw.getScores16(buf, ref, qer, n, 1, w);
    } else {
        const int W = (mode == 8) ? SIMD_WIDTH8 : SIMD_WIDTH16;
        // each group padded the reference's way, in a private zeroed array
        SeqPair *grp = (SeqPair *)calloc((size_t)W + 256, sizeof(SeqPair));
        if (!grp) { free(buf); return -1; }
        for (int32_t g = 0; g < n; g += W) {
            int32_t k = (n - g < W) ? (n - g) : W;
            memset(grp, 0, ((size_t)W + 256) * sizeof(SeqPair));
            memcpy(grp, buf + g, (size_t)k * sizeof(SeqPair));
            if (mode == 8 && k < W) {
                // getScores8 pads with the last pair of the whole call
                // (bandedSWA.cpp:2017); keep that length for the padding
                for (int l = k; l < W; l++) grp[l].len2 = buf[n - 1].len2;
            }
            memset(bsw.F8_, 0, s8); memset(bsw.H8_, 0, s8); memset(bsw.H8__, 0, s8);
            memset(bsw.F16_, 0, s16); memset(bsw.H16_, 0, s16); memset(bsw.H16__, 0, s16);
            if (mode == 8) bsw.getScores8(grp, ref, qer, k, 1, w);
            else bsw.getScores16(grp, ref, qer, k, 1, w);
            for (int l = 0; l < k; l++) buf[g + l] = grp[l];
        }
        free(grp);
    }
    memcpy(pairs, buf, (size_t)n * sizeof(SeqPair));
    free(buf);
    return 0;
}

}  // extern "C"
