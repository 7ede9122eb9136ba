// Test infrastructure only: C entry points around the reference's own
// unbanded Smith-Waterman classes (src/alignment/Smith-Waterman), compiled
// from the read-only reference tree by oracle/build_ref.sh into oracle/_ref/.
// Used to pin the oracle (oracle/sw_oracle.cpp) and to generate golden
// fixtures; never linked into the product library.
//
// The classes are driven the way benchmarks/bench-smith-waterman.cpp drives
// them: one instance of PairWiseSW_8 / _16 / _32 built from
// (match, mismatch, open, extend), then getScores(pairs, seqBuf, n, 1), with
// pair k's sequences at seqBuf + 2*id*MAX_SEQ_LEN and + (2*id+1)*MAX_SEQ_LEN.
// PairWiseSW.h defines its own __rdtsc, which clashes with the compiler's; the
// recipe includes <immintrin.h> first and renames the header's copy.
#include <immintrin.h>
#define __rdtsc tal_ref_rdtsc
#include "PairWiseSW_16.h"
#include "PairWiseSW_32.h"
#include "PairWiseSW_8.h"

#include <stdlib.h>
#include <string.h>

extern "C" {

int ref_sw_max_len(int bits) {
    return bits == 8 ? MAX_SEQ_LEN_8 : bits == 16 ? MAX_SEQ_LEN_16 : MAX_SEQ_LEN_32;
}

// bits: 8, 16, 32 (vector getScores) or 0 (PairWiseSW::smithWatermanOnePairWrapper,
// which places pair k's sequences by its index, with stride MAX_SEQ_LEN_32).
// pairs: 12-byte SeqPair records; the reference writes entries up to the next
// multiple of its SIMD width, so the call runs on a padded copy and only
// [0, n) is copied back.
int ref_sw_run(int bits, int match, int mismatch, int open, int ext, void *pairs,
               uint8_t *seqbuf, int32_t n) {
    SeqPair *buf = (SeqPair *)calloc((size_t)n + 128, sizeof(SeqPair));
    if (!buf) return -1;
    memcpy(buf, pairs, sizeof(SeqPair) * (size_t)n);
    if (bits == 8) {
        PairWiseSW_8 sw(match, mismatch, open, ext);
        sw.getScores(buf, seqbuf, n, 1);
    } else if (bits == 16) {
        PairWiseSW_16 sw(match, mismatch, open, ext);
        sw.getScores(buf, seqbuf, n, 1);
    } else if (bits == 32) {
        PairWiseSW_32 sw(match, mismatch, open, ext);
        sw.getScores(buf, seqbuf, n, 1);
    } else {
        PairWiseSW sw(match, mismatch, open, ext);
        sw.smithWatermanOnePairWrapper(buf, seqbuf, n, MAX_SEQ_LEN_32);
    }
    memcpy(pairs, buf, sizeof(SeqPair) * (size_t)n);
    free(buf);
    return 0;
}

}  // extern "C"
