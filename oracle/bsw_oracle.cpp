// ORACLE — test infrastructure only.  Nothing in the product library links or
// calls this file; tests/, __graft_entry__.smoke() and bench.py's CPU legs load
// it as the test oracle / CPU baseline.
//
// A CPU restatement, written from the reference's algorithm, of TAL's banded
// Smith-Waterman seed extension (src/alignment/BSW/bandedSWA.cpp):
//
//   * oracle_bsw_vector(): the inter-task SIMD kernels getScores16 /
//     getScores8 (AVX-512BW: bandedSWA.cpp:2664-3356 and :1970-2661), restated
//     as a loop over W "lanes" with the element width (int16 / int8, wrapping)
//     and every blend, mask and narrowing scan of the vector code.  W is a
//     parameter: W=32 (16-bit) / W=64 (8-bit) reproduces the reference's
//     grouping of consecutive pairs exactly; W=1 runs every pair on its own.
//   * oracle_bsw_scalar(): scalarBandedSWA / scalarBandedSWAWrapper
//     (bandedSWA.cpp:116-260), which also counts the inner-loop iterations
//     ("ref-cells", the reference's own SW_cells site at bandedSWA.cpp:199).
//
// Parity status: pinned.  tests/test_oracle_pin.py compares this file with the
// reference compiled from source (oracle/build_ref.sh) on seeded inputs of
// every workload shape, and tests/golden/ holds fixtures produced by the
// reference itself.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include <thread>
#include <atomic>
#include <algorithm>

namespace {

// SeqPair, bandedSWA.h:90-99 (14 x int32).
struct Pair {
    int32_t idr, idq, id, len1, len2, h0, seqid, regid;
    int32_t score, tle, gtle, qle, gscore, max_off;
};
static_assert(sizeof(Pair) == 56, "SeqPair is 14 x int32");

struct Params {
    int o_del, e_del, o_ins, e_ins, zdrop, end_bonus, a, b;
};

constexpr int AMBIG = 4;     // bandedSWA.cpp:44
constexpr int DUMMY1 = 99;   // bandedSWA.cpp:45
constexpr int DUMMY2 = 100;  // bandedSWA.cpp:46

// Element-type traits: S is the lane type (int16_t / int8_t), U its unsigned
// twin.  Every arithmetic result is folded back into S, as the epi16/epi8
// instructions do.
template <typename S>
struct Lane {
    typedef typename std::conditional<sizeof(S) == 2, uint16_t, uint8_t>::type U;
    static constexpr int BITS = 8 * (int)sizeof(S);
    static inline S wrap(int x) { return (S)(U)(unsigned)x; }
    static inline U uns(S x) { return (U)x; }
    static inline bool topbit(S x) { return ((U)x >> (BITS - 1)) & 1u; }
    static inline S ones() { return (S)(U)~0u; }
};

template <typename S>
struct Scratch {
    std::vector<S> s1, s2, Hh, Hv, F;
};

// One group of W consecutive pairs: smithWatermanBatchWrapper16/8's per-group
// set-up (bandedSWA.cpp:2787-2904 / 2091-2205) followed by
// smithWaterman512_16/8 (:2962-3356 / :2263-2661).
template <typename S>
void run_group(const Params &P, int W, Pair *p, const uint8_t *ref,
               const uint8_t *qer, int32_t w_call, Scratch<S> &sc) {
    typedef Lane<S> L;
    typedef typename L::U U;
    const bool is16 = sizeof(S) == 2;

    // ---- scores and constants (ctor bandedSWA.cpp:50-68)
    const S w_match = L::wrap((int8_t)P.a);
    const S w_mismatch = L::wrap((int8_t)(P.b * -1));
    const S w_ambig = L::wrap(-1);
    const S e_del = L::wrap(P.e_del), oe_del = L::wrap(P.o_del + P.e_del);
    const S e_ins = L::wrap(P.e_ins), oe_ins = L::wrap(P.o_ins + P.e_ins);
    const S o_del = L::wrap(P.o_del);
    const S zdropv = L::wrap(P.zdrop);

    // max over the scores, int16_t (16-bit wrapper :2779) / int8_t (8-bit :2082)
    S maxsc = 0;
    if (maxsc < (int8_t)P.a) maxsc = L::wrap((int8_t)P.a);
    if (maxsc < (int8_t)(P.b * -1)) maxsc = L::wrap((int8_t)(P.b * -1));
    if (maxsc < -1) maxsc = L::wrap(-1);

    // ---- lengths; nrow/ncol exactly as the wrapper hands them to the kernel
    uint16_t maxLen1 = 0;
    int maxLen2 = 0;
    for (int l = 0; l < W; l++) {
        if (maxLen1 < p[l].len1) maxLen1 = (uint16_t)p[l].len1;
        if (is16) {
            if ((uint16_t)maxLen2 < p[l].len2) maxLen2 = (uint16_t)p[l].len2;
        } else {
            if ((uint8_t)maxLen2 < p[l].len2) maxLen2 = (uint8_t)p[l].len2;
        }
    }
    const int nrow = is16 ? (int)maxLen1 : (int)(uint8_t)maxLen1;
    const int ncol = maxLen2;
    const int wrapRows = (int)maxLen1;  // the wrapper's own loops use uint16 maxLen1

    const size_t colCap = (size_t)std::max(ncol, 1) + 3;
    const size_t rowCap = (size_t)std::max(wrapRows, nrow) + 3;
    sc.s1.assign(rowCap * W, 0);
    sc.Hv.assign(rowCap * W, 0);
    sc.s2.assign(colCap * W, 0);
    sc.Hh.assign(colCap * W, 0);
    sc.F.assign(colCap * W, 0);
    S *s1 = sc.s1.data(), *s2 = sc.s2.data(), *Hh = sc.Hh.data();
    S *Hv = sc.Hv.data(), *F = sc.F.data();
    const S ambv = L::ones();

    std::vector<S> h0(W), qlenb(W);
    std::vector<S> myband(W);
    // SoA transpose of the targets, column-0 values (:2796-2837 / :2101-2139)
    for (int l = 0; l < W; l++) {
        h0[l] = L::wrap((U)p[l].h0);
        const uint8_t *seq1 = ref + (int64_t)p[l].idr;
        for (int k = 0; k < p[l].len1; k++) {
            s1[(size_t)k * W + l] = seq1[k] == AMBIG ? ambv : L::wrap(seq1[k]);
            Hv[(size_t)k * W + l] = 0;
        }
        qlenb[l] = L::wrap((U)(p[l].len2 * maxsc));
    }
    for (int l = 0; l < W; l++)
        for (int k = p[l].len1; k <= wrapRows; k++) {
            s1[(size_t)k * W + l] = DUMMY1;
            Hv[(size_t)k * W + l] = DUMMY1;
        }
    for (int l = 0; l < W; l++) Hv[l] = h0[l];
    {
        std::vector<S> t(W);
        for (int l = 0; l < W; l++) t[l] = L::wrap(h0[l] - o_del);
        for (int k = 1; k < wrapRows; k++)
            for (int l = 0; l < W; l++) {
                t[l] = L::wrap(t[l] - e_del);
                Hv[(size_t)k * W + l] = t[l] > 0 ? t[l] : 0;
            }
    }
    // SoA transpose of the queries, row-0 values (:2839-2879 / :2141-2181)
    for (int l = 0; l < W; l++) {
        const uint8_t *seq2 = qer + (int64_t)p[l].idq;
        for (int k = 0; k < p[l].len2; k++) {
            s2[(size_t)k * W + l] = seq2[k] == AMBIG ? ambv : L::wrap(seq2[k]);
            Hh[(size_t)k * W + l] = 0;
        }
    }
    for (int l = 0; l < W; l++)
        for (int k = p[l].len2; k <= maxLen2; k++) {
            s2[(size_t)k * W + l] = DUMMY2;
            Hh[(size_t)k * W + l] = 0;
        }
    {
        std::vector<S> t(W);
        for (int l = 0; l < W; l++) {
            Hh[l] = h0[l];
            S d = L::wrap(h0[l] - oe_ins);
            t[l] = (h0[l] > oe_ins) ? d : 0;
            Hh[(size_t)W + l] = t[l];
        }
        for (int k = 2; k < maxLen2; k++)
            for (int l = 0; l < W; l++) {
                S d = L::wrap(t[l] - e_ins);
                t[l] = d > 0 ? d : 0;
                Hh[(size_t)k * W + l] = t[l];
            }
    }
    // band clamp per lane (:2882-2904 / :2183-2205); integer division then +1.0
    int32_t bsize = w_call;
    {
        const S eb_ins = L::wrap(P.end_bonus - P.o_ins);
        const S eb_del = L::wrap(P.end_bonus - P.o_del);
        for (int l = 0; l < W; l++) {
            U temp = (U)L::wrap(qlenb[l] + eb_ins);
            double val = temp / P.e_ins + 1.0;
            int mi = (int)val;
            mi = mi > 1 ? mi : 1;
            myband[l] = L::wrap((U)(bsize > mi ? mi : bsize));
        }
        for (int l = 0; l < W; l++) {
            U temp = (U)L::wrap(qlenb[l] + eb_del);
            double val = temp / P.e_del + 1.0;
            int mi = (int)val;
            mi = mi > 1 ? mi : 1;
            int mb = (int)(U)myband[l];
            myband[l] = L::wrap((U)(mb > mi ? mi : mb));
            if (bsize < (int)(U)myband[l]) bsize = (int)(U)myband[l];
        }
    }
    const int32_t w = bsize;

    // ---------------- kernel (smithWaterman512_16 / 512_8) ----------------
    std::vector<S> tlen(W), qlen(W), head(W), tail(W), mlen(W);
    std::vector<S> maxScore(W), x(W), y(W), gscore(W), max_off(W), exit0(W), max_ie(W);
    std::vector<S> e11(W), h10(W), maxRS1(W), y1(W), index(W);
    std::vector<uint8_t> tmpb(W), zl(W);
    int32_t minq = 10000000;
    for (int l = 0; l < W; l++) {
        tlen[l] = L::wrap((U)p[l].len1);
        qlen[l] = L::wrap((U)p[l].len2);
        if (p[l].len2 < minq) minq = p[l].len2;
    }
    minq -= 1;
    for (int l = 0; l < W; l++) {
        tail[l] = qlen[l];
        head[l] = 0;
        U ml = (U)L::wrap(qlen[l] + myband[l]);
        mlen[l] = L::wrap(std::min<U>(ml, (U)tlen[l]));
        maxScore[l] = Hv[l];
        x[l] = y[l] = 0;
        gscore[l] = -1;
        max_off[l] = 0;
        exit0[l] = L::ones();
        max_ie[l] = 0;
    }
    for (int j = 0; j < ncol; j++)
        for (int l = 0; l < W; l++) F[(size_t)j * W + l] = 0;

    auto at = [&](S *a, long idx, int l) -> S & { return a[(size_t)idx * W + l]; };
    auto inCol = [&](long idx) { return idx >= 0 && (size_t)idx < colCap; };

    int beg = 0, end = ncol, nbeg = 0, nend = ncol;
    for (int i = 0; i < nrow; i++) {
        const S i1 = L::wrap(i + 1);
        for (int l = 0; l < W; l++) { e11[l] = 0; maxRS1[l] = 0; y1[l] = 0; }
        beg = nbeg; end = nend;
        if (beg < i - w) beg = i - w;
        if (end > i + w + 1) end = i + w + 1;
        if (end > ncol) end = ncol;
        for (int l = 0; l < W; l++) h10[l] = (beg == 0) ? at(Hv, i + 1, l) : (S)0;

        // per-lane band (:3080-3089)
        bool unchanged = true;
        for (int l = 0; l < W; l++) {
            S ph = head[l], pt = tail[l];
            S c = L::wrap(i - myband[l]);
            head[l] = head[l] > c ? head[l] : c;
            U c2 = (U)L::wrap(i1 + myband[l]);
            U t = std::min<U>((U)tail[l], c2);
            t = std::min<U>(t, (U)qlen[l]);
            tail[l] = (S)t;
            if (head[l] != ph || tail[l] != pt) unchanged = false;
        }
        // trimming (:3091-3112)
        if (!unchanged) {
            for (int lcol = beg; lcol < end; lcol++) {
                const S pj = L::wrap(lcol), jn = L::wrap(lcol + 1);
                bool any = false;
                for (int l = 0; l < W; l++) any |= head[l] > pj;
                if (!any) break;
                for (int l = 0; l < W; l++)
                    if (head[l] > pj || jn > tail[l]) {
                        at(Hh, lcol, l) = 0;
                        at(F, lcol, l) = 0;
                    }
            }
        }
        // row exit status (:3119-3129)
        for (int l = 0; l < W; l++)
            if (i1 > mlen[l] || tail[l] == head[l] || head[l] > tail[l]) exit0[l] = 0;

        // DP row (:3135-3196)
        S j512 = L::wrap(beg);
        int j;
        for (j = beg; j < end; j++) {
            const S pj = j512;
            j512 = L::wrap(j512 + 1);
            for (int l = 0; l < W; l++) {
                const S h00 = at(Hh, j, l), f11 = at(F, j, l);
                const S a1 = at(s1, i, l), a2 = at(s2, j, l);
                S sbt = (a1 == a2) ? w_match : w_mismatch;
                if (L::topbit((S)std::max<U>((U)a1, (U)a2))) sbt = w_ambig;
                S m11 = L::wrap(h00 + sbt);
                if (h00 == 0) m11 = 0;
                S h11 = m11 > e11[l] ? m11 : e11[l];
                h11 = h11 > f11 ? h11 : f11;
                S t = L::wrap(m11 - oe_ins);
                S val = t > 0 ? t : 0;
                S e = L::wrap(e11[l] - e_ins);
                e11[l] = val > e ? val : e;
                t = L::wrap(m11 - oe_del);
                val = t > 0 ? t : 0;
                S f21 = L::wrap(f11 - e_del);
                f21 = val > f21 ? val : f21;

                const bool cmp2 = head[l] > pj;
                const bool mask = (pj > tail[l]) || cmp2;
                S hst = mask ? (S)0 : h10[l];
                if (mask) f21 = 0;

                const S bmax = maxRS1[l];
                S nm = maxRS1[l] > h11 ? maxRS1[l] : h11;
                const bool cmpA = (nm > bmax) || (nm == h11);
                const bool cmp1b = (j512 > tail[l]) || cmp2;
                if (!cmp1b) {
                    if (cmpA) y1[l] = j512;
                    maxRS1[l] = nm;
                }
                at(F, j, l) = f21;
                at(Hh, j, l) = hst;
                h10[l] = h11;

                if (j >= minq) {
                    const bool cq = j512 == qlen[l];
                    S max_gh = gscore[l] > h11 ? gscore[l] : h11;
                    const bool cgh = gscore[l] > h11;
                    S t1 = cgh ? max_ie[l] : i1;
                    t1 = cq ? t1 : max_ie[l];
                    const bool mex0 = L::topbit(exit0[l]);
                    t1 = mex0 ? t1 : max_ie[l];
                    max_gh = mex0 ? max_gh : gscore[l];
                    max_gh = cq ? max_gh : gscore[l];
                    const bool ct = j512 > tail[l];
                    max_gh = ct ? gscore[l] : max_gh;
                    max_ie[l] = ct ? max_ie[l] : t1;
                    gscore[l] = max_gh;
                }
            }
        }
        // last column of the row (:3197-3203); j == max(beg, end) here
        for (int l = 0; l < W; l++) {
            const bool m = (head[l] > j512) || (j512 > tail[l]);
            if (inCol(j)) {
                at(Hh, j, l) = m ? (S)0 : h10[l];
                at(F, j, l) = 0;
            }
        }
        // zero row in every lane ends the group (:3206-3209)
        bool allz = true;
        for (int l = 0; l < W; l++) allz &= maxRS1[l] == 0;
        if (allz) break;
        for (int l = 0; l < W; l++) {
            if (maxRS1[l] == 0) exit0[l] = 0;
            const S bmaxScore = maxScore[l];
            const S sc2 = maxScore[l] > maxRS1[l] ? maxScore[l] : maxRS1[l];
            if (L::topbit(exit0[l])) maxScore[l] = sc2;
            const bool cmp = maxScore[l] > bmaxScore;
            if (cmp) {
                y[l] = y1[l];
                x[l] = i1;
                S ind = L::wrap(y1[l] - i1);
                ind = (ind < 0) ? L::wrap(-ind) : ind;  // abs_epi16 (wrapping)
                max_off[l] = max_off[l] > ind ? max_off[l] : ind;
            }
            // ZSCORE16 / ZSCORE8 (:1868-1881 / :1826-1839): no gap-extend weight
            const S tmpi = L::wrap(i1 - x[l]);
            const S tmpj = L::wrap(y1[l] - y[l]);
            const bool cz = tmpi > tmpj;
            const S score = L::wrap(maxScore[l] - maxRS1[l]);
            const S d = cz ? L::wrap(tmpi - tmpj) : L::wrap(tmpj - tmpi);
            const S t1 = L::wrap(score - d);
            if (t1 > zdropv) exit0[l] = 0;
        }

        // band narrowing (:3235-3260)
        auto allZero = [&](int c) {
            for (int l = 0; l < W; l++)
                if ((at(F, c, l) | at(Hh, c, l)) != 0) return false;
            return true;
        };
        int lc;
        for (lc = beg; lc < end; lc++) {
            if (allZero(lc)) nbeg = lc;
            else break;
        }
        for (lc = end; lc >= beg; lc--)
            if (!allZero(lc)) break;
        nend = lc + 2 < ncol ? lc + 2 : ncol;

        // per-lane head / tail (:3265-3316 / :2571-2621)
        if (is16) { beg = nbeg; end = nend; }
        {
            std::fill(tmpb.begin(), tmpb.end(), 1);
            S l512 = L::wrap(beg);
            for (lc = beg; lc < end; lc++) {
                bool any = false;
                for (int l = 0; l < W; l++) {
                    const S exit1 = (S)(exit0[l] ^ L::ones());
                    zl[l] = ((at(F, lc, l) | at(Hh, lc, l) | exit1) == 0);
                    any |= zl[l];
                }
                if (!any) break;
                l512 = L::wrap(l512 + 1);
                for (int l = 0; l < W; l++) {
                    const bool t = zl[l] && tmpb[l];
                    if (t) head[l] = l512;
                    tmpb[l] = t;
                }
            }
            for (int l = 0; l < W; l++) index[l] = tail[l];
            std::fill(tmpb.begin(), tmpb.end(), 1);
            l512 = L::wrap(end);
            for (lc = end; lc >= beg; lc--) {
                bool any = false;
                for (int l = 0; l < W; l++) {
                    const S exit1 = (S)(exit0[l] ^ L::ones());
                    zl[l] = ((at(F, lc, l) | at(Hh, lc, l) | exit1) == 0);
                    any |= zl[l];
                }
                if (!any) break;
                l512 = L::wrap(l512 - 1);
                for (int l = 0; l < W; l++) {
                    const bool t = zl[l] && tmpb[l];
                    if (t) index[l] = l512;
                    tmpb[l] = t;
                }
            }
            for (int l = 0; l < W; l++) {
                S ix = L::wrap(index[l] + 2);
                tail[l] = ix < qlen[l] ? ix : qlen[l];
            }
        }
    }
    for (int l = 0; l < W; l++) {
        p[l].score = maxScore[l];
        p[l].tle = x[l];
        p[l].qle = y[l];
        p[l].max_off = max_off[l];
        p[l].gscore = gscore[l];
        p[l].gtle = max_ie[l];
    }
}

// Runs [first, last) groups of one batch.  Lanes past n are filled the way
// the reference pads its array (16-bit :2711-2717: len1 = len2 = 0;
// 8-bit :2012-2018: len1 = 0, len2 = last pair's len2), with h0 = 0.
template <typename S>
void run_batch_range(const Params &P, int W, Pair *pairs, int64_t n,
                     const uint8_t *ref, const uint8_t *qer, int32_t w,
                     int64_t g0, int64_t g1) {
    Scratch<S> sc;
    std::vector<Pair> grp(W);
    for (int64_t g = g0; g < g1; g++) {
        int64_t base = g * W;
        for (int l = 0; l < W; l++) {
            int64_t k = base + l;
            if (k < n) {
                grp[l] = pairs[k];
            } else {
                memset(&grp[l], 0, sizeof(Pair));
                grp[l].id = (int32_t)k;
                grp[l].len1 = 0;
                grp[l].len2 = (sizeof(S) == 2) ? 0 : pairs[n - 1].len2;
            }
        }
        run_group<S>(P, W, grp.data(), ref, qer, w, sc);
        for (int l = 0; l < W && base + l < n; l++) {
            Pair &o = pairs[base + l];
            o.score = grp[l].score; o.tle = grp[l].tle; o.gtle = grp[l].gtle;
            o.qle = grp[l].qle; o.gscore = grp[l].gscore; o.max_off = grp[l].max_off;
        }
    }
}

template <typename F>
void parallel_groups(int64_t ngroups, int nthreads, F fn) {
    if (nthreads <= 1 || ngroups < 2) { fn(0, ngroups); return; }
    std::atomic<int64_t> next(0);
    const int64_t chunk = 64;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&]() {
            for (;;) {
                int64_t s = next.fetch_add(chunk);
                if (s >= ngroups) break;
                fn(s, std::min(ngroups, s + chunk));
            }
        });
    for (auto &t : th) t.join();
}

// scalarBandedSWA (bandedSWA.cpp:116-237) for one pair; returns the score and
// adds the inner-loop iterations to *cells.
int scalar_pair(const Params &P, const int8_t *mat, int qlen, const uint8_t *query,
                int tlen, const uint8_t *target, int32_t w, int h0, int *_qle,
                int *_tle, int *_gtle, int *_gscore, int *_max_off,
                uint64_t *cells, std::vector<int32_t> &eh_h,
                std::vector<int32_t> &eh_e, std::vector<int8_t> &qp) {
    const int m5 = 5;
    const int oe_del = P.o_del + P.e_del, oe_ins = P.o_ins + P.e_ins;
    qp.assign((size_t)qlen * m5 + 1, 0);
    eh_h.assign((size_t)qlen + 1, 0);
    eh_e.assign((size_t)qlen + 1, 0);
    for (int k = 0, i = 0; k < m5; ++k) {
        const int8_t *row = &mat[k * m5];
        for (int j = 0; j < qlen; ++j) qp[i++] = row[query[j]];
    }
    eh_h[0] = h0;
    if (qlen >= 1) eh_h[1] = h0 > oe_ins ? h0 - oe_ins : 0;
    for (int j = 2; j <= qlen && eh_h[j - 1] > P.e_ins; ++j) eh_h[j] = eh_h[j - 1] - P.e_ins;
    int mx = 0;
    for (int i = 0; i < m5 * m5; ++i) mx = mx > mat[i] ? mx : mat[i];
    int max_ins = (int)((double)(qlen * mx + P.end_bonus - P.o_ins) / P.e_ins + 1.);
    max_ins = max_ins > 1 ? max_ins : 1;
    w = w < max_ins ? w : max_ins;
    int max_del = (int)((double)(qlen * mx + P.end_bonus - P.o_del) / P.e_del + 1.);
    max_del = max_del > 1 ? max_del : 1;
    w = w < max_del ? w : max_del;
    int max = h0, max_i = -1, max_j = -1, max_ie = -1, gscore = -1, max_off = 0;
    int beg = 0, end = qlen;
    uint64_t c = 0;
    for (int i = 0; i < tlen; ++i) {
        int f = 0, h1, m = 0, mj = -1;
        const int8_t *q = &qp[(size_t)target[i] * qlen];
        if (beg < i - w) beg = i - w;
        if (end > i + w + 1) end = i + w + 1;
        if (end > qlen) end = qlen;
        if (beg == 0) {
            h1 = h0 - (P.o_del + P.e_del * (i + 1));
            if (h1 < 0) h1 = 0;
        } else h1 = 0;
        int j;
        for (j = beg; j < end; ++j) {
            int M = eh_h[j], e = eh_e[j], h, t;
            eh_h[j] = h1;
            M = M ? M + q[j] : 0;
            h = M > e ? M : e;
            h = h > f ? h : f;
            h1 = h;
            mj = m > h ? mj : j;
            m = m > h ? m : h;
            t = M - oe_del; t = t > 0 ? t : 0;
            e -= P.e_del; e = e > t ? e : t;
            eh_e[j] = e;
            t = M - oe_ins; t = t > 0 ? t : 0;
            f -= P.e_ins; f = f > t ? f : t;
        }
        c += (uint64_t)(end > beg ? end - beg : 0);
        eh_h[end] = h1; eh_e[end] = 0;
        if (j == qlen) {
            max_ie = gscore > h1 ? max_ie : i;
            gscore = gscore > h1 ? gscore : h1;
        }
        if (m == 0) break;
        if (m > max) {
            max = m, max_i = i, max_j = mj;
            max_off = max_off > abs(mj - i) ? max_off : abs(mj - i);
        } else if (P.zdrop > 0) {
            if (i - max_i > mj - max_j) {
                if (max - m - ((i - max_i) - (mj - max_j)) * P.e_del > P.zdrop) break;
            } else {
                if (max - m - ((mj - max_j) - (i - max_i)) * P.e_ins > P.zdrop) break;
            }
        }
        for (j = beg; j < end && eh_h[j] == 0 && eh_e[j] == 0; ++j) {}
        beg = j;
        for (j = end; j >= beg && eh_h[j] == 0 && eh_e[j] == 0; --j) {}
        end = j + 2 < qlen ? j + 2 : qlen;
    }
    *cells += c;
    *_qle = max_j + 1; *_tle = max_i + 1; *_gtle = max_ie + 1;
    *_gscore = gscore; *_max_off = max_off;
    return max;
}

// The library's group-coupling detector, restated for testing (the GPU
// kernels compute the same flag, csrc/bsw_couple.cuh).  Scores one pair as
// if alone in its SIMD group -- the oracle's W = 1 path -- and returns a
// non-zero flag unless its outputs provably equal its outputs in ANY group of
// the reference (bandedSWA.cpp:3053-3316, :2355-2621).  A group influences a
// lane only through values it shares: the band [beg, end) of each row, the
// trimming pass, the ranges of the head / tail re-derivation scans and the
// width of its row-0 initialisation (the longest query).  For each, the check
// below bounds the group's value (beg >= i - w, end <= i + w + 1, scans from
// any nbeg' <= nbeg to any nend' <= end + 2, width up to the element limit)
// and verifies that every value in the bound leaves the lane's stored row
// and outputs unchanged; the head and tail the group could hold instead of
// the lane's own are carried as intervals [hlo, hhi], [tlo, thi].
template <typename S>
int detect_pair(const Params &P, Pair *p, const uint8_t *ref, const uint8_t *qer, int32_t w_call) {
    typedef Lane<S> L; typedef typename L::U U;
    const bool is16 = sizeof(S) == 2;
    const int CMAX = is16 ? 32767 : 127;
    const S w_match = L::wrap((int8_t)P.a), w_mismatch = L::wrap((int8_t)(P.b * -1)), w_ambig = L::wrap(-1);
    const S e_del = L::wrap(P.e_del), oe_del = L::wrap(P.o_del + P.e_del);
    const S e_ins = L::wrap(P.e_ins), oe_ins = L::wrap(P.o_ins + P.e_ins), o_del = L::wrap(P.o_del);
    const S zdropv = L::wrap(P.zdrop);
    S maxsc = 0;
    if (maxsc < (int8_t)P.a) maxsc = L::wrap((int8_t)P.a);
    if (maxsc < (int8_t)(P.b * -1)) maxsc = L::wrap((int8_t)(P.b * -1));
    if (maxsc < -1) maxsc = L::wrap(-1);
    const int len1 = p->len1, len2 = p->len2;
    const int nrow = len1, ncol = len2;
    std::vector<S> s1(len1 + 3), s2(len2 + 3), Hh(len2 + 3), Hv(len1 + 3), F(len2 + 3);
    const S ambv = L::ones();
    const S h0 = L::wrap((U)p->h0);
    for (int k = 0; k < len1; k++) { uint8_t b = ref[p->idr + k]; s1[k] = b == AMBIG ? ambv : L::wrap(b); }
    Hv[len1] = DUMMY1; s1[len1] = DUMMY1;
    Hv[0] = h0;
    { S t = L::wrap(h0 - o_del); for (int k = 1; k < len1; k++) { t = L::wrap(t - e_del); Hv[k] = t > 0 ? t : 0; } }
    for (int k = 0; k < len2; k++) { uint8_t b = qer[p->idq + k]; s2[k] = b == AMBIG ? ambv : L::wrap(b); }
    s2[len2] = DUMMY2; Hh[len2] = 0;
    Hh[0] = h0;
    const int v1 = (h0 > oe_ins) ? (int)L::wrap(h0 - oe_ins) : 0;
    { S t = (S)v1; Hh[1] = t;
      for (int k = 2; k < len2; k++) { S dd = L::wrap(t - e_ins); t = dd > 0 ? dd : 0; Hh[k] = t; } }
    // row-0 values are positive exactly at columns 1 <= k < K0 (and at 0 when h0 > 0)
    const int K0 = v1 > 0 ? (v1 - 1) / (int)e_ins + 2 : 1;
    auto initA_pos = [&](int c) { return c == 0 ? h0 > 0 : c == 1 ? v1 > 0 : (c < len2 && c < K0); };
    int32_t bsize = w_call; S myband;
    {
        const S eb_ins = L::wrap(P.end_bonus - P.o_ins), eb_del = L::wrap(P.end_bonus - P.o_del);
        S qlenb = L::wrap((U)(len2 * maxsc));
        U temp = (U)L::wrap(qlenb + eb_ins); double val = temp / P.e_ins + 1.0; int mi = (int)val; mi = mi > 1 ? mi : 1;
        myband = L::wrap((U)(bsize > mi ? mi : bsize));
        temp = (U)L::wrap(qlenb + eb_del); val = temp / P.e_del + 1.0; mi = (int)val; mi = mi > 1 ? mi : 1;
        int mb = (int)(U)myband; myband = L::wrap((U)(mb > mi ? mi : mb));
        if (bsize < (int)(U)myband) bsize = (int)(U)myband;
    }
    const int32_t w = bsize;
    const S tlen = L::wrap((U)len1), qlen = L::wrap((U)len2);
    S head = 0, tail = qlen;
    int hlo = 0, hhi = 0, tlo = (int)qlen, thi = (int)qlen;
    const S mlen = L::wrap(std::min<U>((U)L::wrap(qlen + myband), (U)tlen));
    S maxScore = Hv[0], x = 0, y = 0, gscore = -1, max_off = 0, max_ie = 0; bool ex = true;
    const int minq = len2 - 1;
    int flag = 0;
    int beg = 0, end = ncol, nbeg = 0, nend = ncol;
    int frozenTo = 0, fzMax = -1, fzMin = 1 << 30;
    int maxEnd = -1;             // furthest column written so far
    bool reachedLen2 = false;
    int Fv = 0;
    auto nzA = [&](int c) -> bool { return c >= 0 && c <= len2 && ((Hh[c] | F[c]) != 0); };
    // first column in (a, b] that may be nonzero right of everything written (a >= end)
    auto firstRightNZ = [&](int a, int b) -> int {
        // A's own columns: written ones in (end, maxEnd] are zero; beyond: row-0 values
        int c0 = std::max(a, maxEnd) + 1;
        if (c0 <= b && c0 < len2 && initA_pos(c0)) return c0;
        if (c0 <= b && c0 <= 1 && initA_pos(1) && 1 < len2 && 1 <= b) return 1;
        // column len2 in the group's view
        if (len2 > a && len2 <= b) {
            bool nz = (len2 <= maxEnd ? nzA(len2) : false) || Fv > 0 || (!reachedLen2 && len2 >= 2 && len2 < K0) || (len2 == 1 && !reachedLen2 && v1 > 0);
            if (nz) return len2;
        }
        int c1 = std::max(a, len2) + 1;
        if (c1 <= b && c1 < CMAX && c1 < K0) return c1;
        return -1;
    };
    auto score = [&](int i, int j) -> S {
        const S a1 = s1[i], a2 = s2[j];
        S sbt = (a1 == a2) ? w_match : w_mismatch;
        if (L::topbit((S)std::max<U>((U)a1, (U)a2))) sbt = w_ambig;
        return sbt;
    };
    auto FL = [&](int b, int) { flag |= b; };
    for (int i = 0; i < nrow; i++) {
        const S i1 = L::wrap(i + 1);
        S e11 = 0, maxRS1 = 0, y1 = 0;
        beg = nbeg; end = nend;
        if (beg < i - w) beg = i - w;
        if (end > i + w + 1) end = i + w + 1;
        if (end > ncol) end = ncol;
        for (int c = frozenTo; c < beg; c++) if (nzA(c)) { fzMax = std::max(fzMax, c); fzMin = std::min(fzMin, c); }
        frozenTo = std::max(frozenTo, beg);
        S h10 = (beg == 0) ? Hv[i + 1] : (S)0;
        const S h10init = h10;
        const S ph = head, pt = tail;
        {
            S c = L::wrap(i - myband); head = head > c ? head : c;
            hlo = std::max(hlo, (int)c); hhi = std::max(hhi, (int)c);
            U c2 = (U)L::wrap(i1 + myband);
            U t = std::min<U>((U)tail, c2); t = std::min<U>(t, (U)qlen); tail = (S)t;
            tlo = (int)(S)std::min<U>(std::min<U>((U)(S)tlo, c2), (U)qlen);
            thi = (int)(S)std::min<U>(std::min<U>((U)(S)thi, c2), (U)qlen);
        }
        const bool changed = head != ph || tail != pt;
        const bool wasActive = ex;
        if (i1 > mlen || tail == head || head > tail) ex = false;
        const bool active = wasActive && ex;
        const bool uncH = hlo != hhi;
        const int lo = std::max(0, i - w);
        const int Emax = std::min(i + w + 1, CMAX);
        if (wasActive && !(i1 > mlen) && tlo <= hhi && thi > hlo) FL(1 << 12, i);
        if (active) {
            if (tlo != thi) FL(1 << 14, i);            // tail uncertainty: flagged
            if (uncH && hhi > end) FL(1 << 13, i);
            // old values on [beg, min(end, max(head, hhi))): the masked-left loop (and [head, hhi))
            if (!changed || uncH) {
                for (int c = beg; c < std::min(end, std::max((int)head, hhi)); c++) if (nzA(c)) { FL(1, i); break; }
            }
            if (uncH && beg >= hlo && beg < hhi && h10init != 0) FL(1 << 13, i);
            if (beg > lo) {
                // columns [lo, beg) the group may compute: zero inputs give
                // zero cells, except column 0's stored H_v[i + 1]
                if (fzMax >= lo) FL(2, i);
                else if (lo == 0 && hlo <= 0 && Hv[i + 1] != 0) FL(2, i);
            }
            if (end < Emax) {
                if (end < thi) FL(16, i);  // real cells right of the lane's band
                // stale row-0 values right of everything written, left of Emax
                const int a = std::max(end, tlo);
                int c0 = std::max(a, maxEnd) + 1;
                if (c0 <= std::min(Emax, len2 - 1) && initA_pos(c0)) FL(32, i);
            }
        }
        if (changed) {
            for (int lc = beg; lc < end; lc++) {
                const S pj = L::wrap(lc), jn = L::wrap(lc + 1);
                if (!(head > pj)) break;
                if (head > pj || jn > tail) { Hh[lc] = 0; F[lc] = 0; }
            }
        }
        S j512 = L::wrap(beg);
        int j;
        S f21_tail = 0; bool tail_in = false;
        S oldHhEnd = (end <= len2) ? Hh[end] : 0, oldFEnd = (end <= len2) ? F[end] : 0;
        for (j = beg; j < end; j++) {
            const S pj = j512; j512 = L::wrap(j512 + 1);
            const S h00 = Hh[j], f11 = F[j];
            S sbt = score(i, j);
            S m11 = L::wrap(h00 + sbt); if (h00 == 0) m11 = 0;
            S h11 = m11 > e11 ? m11 : e11; h11 = h11 > f11 ? h11 : f11;
            S t = L::wrap(m11 - oe_ins); S val = t > 0 ? t : 0; S e = L::wrap(e11 - e_ins); e11 = val > e ? val : e;
            t = L::wrap(m11 - oe_del); val = t > 0 ? t : 0; S f21 = L::wrap(f11 - e_del); f21 = val > f21 ? val : f21;
            if (j == tail) { f21_tail = f21; tail_in = true; }
            const bool cmp2 = head > pj; const bool mask = (pj > tail) || cmp2;
            S hst = mask ? (S)0 : h10; if (mask) f21 = 0;
            const S bmax = maxRS1; S nm = maxRS1 > h11 ? maxRS1 : h11;
            const bool cmpA = (nm > bmax) || (nm == h11); const bool cmp1b = (j512 > tail) || cmp2;
            if (!cmp1b) { if (cmpA) y1 = j512; maxRS1 = nm; }
            F[j] = f21; Hh[j] = hst; h10 = h11;
            if (j >= minq) {
                const bool cq = j512 == qlen; S max_gh = gscore > h11 ? gscore : h11; const bool cgh = gscore > h11;
                S t1 = cgh ? max_ie : i1; t1 = cq ? t1 : max_ie; t1 = ex ? t1 : max_ie;
                max_gh = ex ? max_gh : gscore; max_gh = cq ? max_gh : gscore;
                const bool ct = j512 > tail; max_gh = ct ? gscore : max_gh; max_ie = ct ? max_ie : t1; gscore = max_gh;
            }
        }
        if (active) {
            if (tail_in && f21_tail != 0 && (int)tail < Emax) FL(64, i);
            if (end < Emax && end == tail && head <= end && end < len2) {
                S sbt = score(i, end);
                S m11 = L::wrap(oldHhEnd + sbt); if (oldHhEnd == 0) m11 = 0;
                S t = L::wrap(m11 - oe_del); S val = t > 0 ? t : 0; S f21 = L::wrap(oldFEnd - e_del); f21 = val > f21 ? val : f21;
                if (f21 != 0) FL(128, i);
            }
        }
        {   const bool m = (head > j512) || (j512 > tail);
            if (j <= len2) { Hh[j] = m ? (S)0 : h10; F[j] = 0; } }
        maxEnd = std::max(maxEnd, j);
        if (j == len2) {
            reachedLen2 = true;
            const S hv = Hh[len2];
            const int sc = (s1[i] == ambv) ? -1 : (int)w_mismatch;
            int M = hv ? (int)hv + sc : 0;
            int nf = std::max(Fv - (int)e_del, std::max(M - (int)oe_del, 0));
            Fv = (len2 > tail || head > len2) ? 0 : nf;
        }
        if (maxRS1 == 0) { ex = false; break; }
        {
            const S bmaxScore = maxScore; const S sc2 = maxScore > maxRS1 ? maxScore : maxRS1;
            if (ex) maxScore = sc2;
            if (maxScore > bmaxScore) { y = y1; x = i1; S ind = L::wrap(y1 - i1); ind = (ind < 0) ? L::wrap(-ind) : ind; max_off = max_off > ind ? max_off : ind; }
            const S tmpi = L::wrap(i1 - x), tmpj = L::wrap(y1 - y); const bool cz = tmpi > tmpj;
            const S sc = L::wrap(maxScore - maxRS1); const S d = cz ? L::wrap(tmpi - tmpj) : L::wrap(tmpj - tmpi);
            if (L::wrap(sc - d) > zdropv) ex = false;
        }
        int lc;
        for (lc = beg; lc < end; lc++) { if (!nzA(lc)) nbeg = lc; else break; }
        for (lc = end; lc >= beg; lc--) if (nzA(lc)) break;
        nend = lc + 2 < ncol ? lc + 2 : ncol;
        const int sb = is16 ? nbeg : beg, se = is16 ? nend : end;
        S newhead = head; bool runToEnd = false;
        {
            S l512 = L::wrap(sb); bool tb = true; int lc2;
            for (lc2 = sb; lc2 < se; lc2++) { bool z = ex && !nzA(lc2); if (!z) break; l512 = L::wrap(l512 + 1); if (z && tb) newhead = l512; tb = z && tb; }
            runToEnd = ex && (lc2 >= se) && se > sb;
        }
        S index = tail; bool runToBot = false;
        {
            S l512 = L::wrap(se); bool tb = true; int lc2;
            for (lc2 = se; lc2 >= sb; lc2--) { bool z = ex && !nzA(lc2); if (!z) break; l512 = L::wrap(l512 - 1); if (z && tb) index = l512; tb = z && tb; }
            runToBot = ex && lc2 < sb;
        }
        if (ex && i + 1 < nrow) {
            if (runToEnd && !(se <= end && Hh[se] != 0)) FL(256, i);
            if (runToBot) FL(512, i);
            const int los = is16 ? 0 : lo;
            const bool nzsb = nzA(sb);
            int nhlo, nhhi;
            if (nzsb) { nhlo = hlo; nhhi = hhi; } else { nhlo = nhhi = newhead; }
            if (sb > los) {
                int Pl = -1;
                if (is16) { if (fzMin < sb) Pl = std::min(fzMax, sb - 1); }
                else { if (fzMax >= lo) Pl = fzMax; }
                if (nzsb && Pl < sb - 1) { nhlo = std::min(nhlo, sb); nhhi = std::max(nhhi, sb); }
                if (Pl >= 0) { nhlo = std::min({nhlo, hlo, los}); nhhi = std::max({nhhi, hhi, Pl}); }
            }
            const int Smax = is16 ? std::min(Emax + 2, CMAX) : Emax;
            int rlo, rhi;
            if (nzA(se)) { rlo = tlo; rhi = thi; } else { rlo = rhi = index; }
            if (Smax > se) {
                const int Qr = firstRightNZ(std::max(se, end), Smax);
                if (nzA(se)) { rlo = std::min(rlo, se); rhi = std::max(rhi, se); }
                if (Qr >= 0) { rlo = std::min({rlo, tlo, Qr}); rhi = std::max({rhi, thi, Smax - 1}); }
            }
            auto T2 = [&](int r) { int v = r + 2; return v < (int)qlen ? v : (int)qlen; };
            tlo = T2(rlo); thi = T2(rhi);
            hlo = nhlo; hhi = nhhi;
        } else {
            hlo = hhi = newhead;
            { S ix = L::wrap(index + 2); tlo = thi = ix < qlen ? ix : qlen; }
        }
        head = newhead;
        { S ix = L::wrap(index + 2); tail = ix < qlen ? ix : qlen; }
        if (hlo > head) hlo = head; if (hhi < head) hhi = head;
        if (tlo > tail) tlo = tail; if (thi < tail) thi = tail;
        if (!ex) break;
    }
    p->score = maxScore; p->tle = x; p->qle = y; p->max_off = max_off; p->gscore = gscore; p->gtle = max_ie;
    return flag;
}

Params unpack(const int32_t *pp) {
    Params P;
    P.o_del = pp[0]; P.e_del = pp[1]; P.o_ins = pp[2]; P.e_ins = pp[3];
    P.zdrop = pp[4]; P.end_bonus = pp[5]; P.a = pp[6]; P.b = pp[7];
    return P;
}

}  // namespace

extern "C" {

// params: {o_del, e_del, o_ins, e_ins, zdrop, end_bonus, a, b}
// bits: 16 (getScores16) or 8 (getScores8).  W: lanes per group (32 / 64 for
// the reference's own grouping, 1 for pair-at-a-time).  Outputs written into
// pairs[0, n).  Returns 0, or -1 on bad arguments.
int oracle_bsw_vector(const int32_t *params, int bits, int W, int32_t *pairs,
                      int64_t n, const uint8_t *ref, const uint8_t *qer,
                      int32_t w, int nthreads) {
    if (!params || !pairs || n < 0 || W < 1 || (bits != 8 && bits != 16)) return -1;
    if (n == 0) return 0;
    Params P = unpack(params);
    if (P.e_del <= 0 || P.e_ins <= 0) return -1;
    Pair *pp = (Pair *)pairs;
    int64_t ngroups = (n + W - 1) / W;
    parallel_groups(ngroups, nthreads, [&](int64_t g0, int64_t g1) {
        if (bits == 16)
            run_batch_range<int16_t>(P, W, pp, n, ref, qer, w, g0, g1);
        else
            run_batch_range<int8_t>(P, W, pp, n, ref, qer, w, g0, g1);
    });
    return 0;
}

// scalarBandedSWAWrapper (bandedSWA.cpp:242-260) with mat = bwa_fill_scmat(a,
// b, -1) (benchmarks/bench-bsw.cpp:56-64).  cells_out (may be NULL) receives
// the total inner-loop iterations.
int oracle_bsw_scalar(const int32_t *params, int32_t *pairs, int64_t n,
                      const uint8_t *ref, const uint8_t *qer, int32_t w,
                      uint64_t *cells_out, int nthreads) {
    if (!params || !pairs || n < 0) return -1;
    Params P = unpack(params);
    if (P.e_del <= 0 || P.e_ins <= 0) return -1;
    int8_t mat[25];
    {
        int k = 0;
        for (int i = 0; i < 4; ++i) {
            for (int j = 0; j < 4; ++j) mat[k++] = i == j ? P.a : -P.b;
            mat[k++] = -1;
        }
        for (int j = 0; j < 5; ++j) mat[k++] = -1;
    }
    Pair *pp = (Pair *)pairs;
    std::atomic<uint64_t> total(0);
    parallel_groups(n, nthreads, [&](int64_t s, int64_t e) {
        std::vector<int32_t> eh_h, eh_e;
        std::vector<int8_t> qp;
        uint64_t c = 0;
        for (int64_t k = s; k < e; k++) {
            Pair *p = pp + k;
            p->score = scalar_pair(P, mat, p->len2, qer + p->idq, p->len1,
                                   ref + p->idr, w, p->h0, &p->qle, &p->tle,
                                   &p->gtle, &p->gscore, &p->max_off, &c, eh_h,
                                   eh_e, qp);
        }
        total += c;
    });
    if (cells_out) *cells_out = total.load();
    return 0;
}


// The library's group-coupling detector (see detect_pair): every pair scored
// alone; outputs into pairs[0, n), flags[k] != 0 where pair k's outputs may
// depend on its SIMD group.  Returns 0, or -1 on bad arguments.
int oracle_bsw_detect(const int32_t *params, int bits, int32_t *pairs, int64_t n,
                      const uint8_t *ref, const uint8_t *qer, int32_t w, int32_t *flags,
                      int nthreads) {
    if (!params || !pairs || !flags || n < 0 || (bits != 8 && bits != 16)) return -1;
    Params P = unpack(params);
    if (P.e_del <= 0 || P.e_ins <= 0) return -1;
    Pair *pp = (Pair *)pairs;
    parallel_groups(n, nthreads, [&](int64_t s, int64_t e) {
        for (int64_t k = s; k < e; k++)
            flags[k] = bits == 16 ? detect_pair<int16_t>(P, pp + k, ref, qer, w)
                                  : detect_pair<int8_t>(P, pp + k, ref, qer, w);
    });
    return 0;
}

}  // extern "C"
