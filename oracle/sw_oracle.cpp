// ORACLE -- test infrastructure only.  CPU restatement of the reference's
// unbanded Smith-Waterman scores (src/alignment/Smith-Waterman):
//   PairWiseSW::smithWatermanOnePair                 PairWiseSW.cpp:63-114
//   PairWiseSW_{8,16,32}::smithWatermanInterTaskVectorized
//                                                    PairWiseSW_16.cpp:151-229 (MAIN_CODE :62-76)
// Local alignment with affine gaps, score only.  Per cell (row i of seq1,
// column j of seq2):
//   M = H(i-1, j-1) + (seq1[i] == seq2[j] ? match : mismatch)
//   H = max(M, E, F, 0)                 (E from the left, F from above)
//   E' = max(H + open, E + extend)      (next column)
//   F' = max(F + extend, H + open)      (next row)
// with E = open at the start of each row and F = open, H = 0 on the row above
// the first -- the vector kernels' initialisation, which gives the scalar
// kernel's values (its LOW_INIT_VALUE start makes E(i, 1) = F(1, j) = open as
// well).  Bytes are compared as they are (any code, N included, matches
// itself).  Arithmetic is exact (int64); the reference's 8/16-bit kernels
// agree inside their range.  A pair's sequences lie at seqBuf + 2*id*stride
// (seq1) and seqBuf + (2*id+1)*stride (seq2), as in PairWiseSW_16.cpp:297,313.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

namespace {

struct SwPair {  // PairWiseSW.h:44-49
    int32_t id;
    int16_t len1, len2;
    int32_t score;
};
static_assert(sizeof(SwPair) == 12, "SeqPair of the unbanded kernels is 12 bytes");

int64_t score_pair(const uint8_t *s1, int len1, const uint8_t *s2, int len2, int64_t match,
                   int64_t mismatch, int64_t open, int64_t ext, std::vector<int64_t> &H,
                   std::vector<int64_t> &F) {
    H.assign(len2 + 1, 0);
    F.assign(len2 + 1, open);
    int64_t best = 0;
    for (int i = 0; i < len1; i++) {
        int64_t e = open, hdiag = 0;  // H(i-1, -1) = 0
        for (int j = 0; j < len2; j++) {
            const int64_t m = hdiag + (s1[i] == s2[j] ? match : mismatch);
            const int64_t f = F[j];
            int64_t h = std::max(std::max(m, e), std::max(f, (int64_t)0));
            best = std::max(best, h);
            const int64_t t = h + open;
            e = std::max(t, e + ext);
            F[j] = std::max(f + ext, t);
            hdiag = H[j];
            H[j] = h;
        }
    }
    return best;
}

}  // namespace

extern "C" {

// params: {match, mismatch, open, extend}; scores written into pairs[k].score.
int oracle_sw(const int32_t *params, void *pairs, int64_t n, const uint8_t *seqbuf,
              int64_t stride, int nthreads) {
    if (!params || (!pairs && n) || stride <= 0) return -1;
    SwPair *p = static_cast<SwPair *>(pairs);
    const int64_t a = params[0], b = params[1], o = params[2], e = params[3];
    auto work = [&](int64_t lo, int64_t hi) {
        std::vector<int64_t> H, F;
        for (int64_t k = lo; k < hi; k++) {
            const uint8_t *s1 = seqbuf + 2 * (int64_t)p[k].id * stride;
            const uint8_t *s2 = seqbuf + (2 * (int64_t)p[k].id + 1) * stride;
            p[k].score = (int32_t)score_pair(s1, std::max<int>(p[k].len1, 0), s2,
                                             std::max<int>(p[k].len2, 0), a, b, o, e, H, F);
        }
    };
    const int T = std::max(1, nthreads);
    std::vector<std::thread> th;
    for (int t = 0; t < T; t++) th.emplace_back(work, n * t / T, n * (t + 1) / T);
    for (auto &x : th) x.join();
    return 0;
}

}  // extern "C"
