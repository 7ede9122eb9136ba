// Lane-per-pair banded Smith-Waterman for short pairs (sm_103a).
//
// Each lane scores its own pair, row by row, exactly as the reference scores
// one lane of its SIMD group (smithWaterman512_16 / _8, bandedSWA.cpp
// :2962-3356 / :2263-2661, with the group reduced to that pair; the rare
// outputs that depend on the group are the grouped kernel's, bsw_group.cuh).
// There are no collectives: lanes are independent
// and a lane that finishes a pair takes the next one from the work counter.
// This is the GPU form of the reference's inter-task layout (one pair per SIMD
// lane), without its shared band: every lane walks its own band.
//
// Shared memory per warp, interleaved by lane so that any mix of per-lane
// columns is bank-conflict free:
//   HF[col][lane]      H_h (low 16 bits) | F (high 16 bits), the reference's
//                      scratch rows with their stale values
//   QS[col/8][lane]    eight query base codes, one nibble each; four nibbles
//                      are a byte-permute selector that looks up the four
//                      columns' scores in the row's score table at once
// The target base of each row is read from global memory (one byte per row).
//
// Windowed rows: a row of the reference touches only columns
// [i - w, i + w + 3] (band, its last column, the lazily initialised columns
// ahead of it), so HF and QS may be rings of W >= 2w + 12 columns (a power of
// two; column j lives in slot j & (W - 1)) instead of whole rows, which
// makes the shared memory per pair depend on the band, not on the query
// length.  The one read of the reference below the band -- the 16-bit head
// re-derivation scans from nbeg, which may lag behind the band, over columns
// that left the band rows ago -- is answered from `p`, the first nonzero of
// those frozen columns, recorded as each column leaves the band (a column
// left of the band is never written again).
//
// The inner loop over a row's band is split into the columns left of the
// per-pair head (masked), the clean middle, and the columns at/after the tail,
// so the middle -- nearly every cell -- runs without predicates.
#pragma once

#include "bsw_kernel.cuh"

namespace talbsw {

// win = 0: whole rows of cols_cap + 4 columns; else a ring of win columns.
__host__ __device__ __forceinline__ size_t lane_hf_words(int cols_cap, int win) {
    return (size_t)(win > 0 ? win : cols_cap + 4) * 32;
}
__host__ __device__ __forceinline__ size_t lane_qs_words(int cols_cap, int win) {
    return (size_t)(win > 0 ? win / 8 : (cols_cap + 7) / 8 + 2) * 32;
}
__host__ __device__ __forceinline__ size_t lane_warp_smem_bytes(int cols_cap, int win) {
    return (lane_hf_words(cols_cap, win) + lane_qs_words(cols_cap, win)) * 4;
}

// Smallest ring (a power of two, at least 64 columns) of at least `cols`.
__host__ __device__ __forceinline__ int lane_ring_at_least(long long cols) {
    int W = 64;
    while (W < (1 << 30) && (long long)W < cols) W <<= 1;
    return W;
}

// Smallest ring that holds every column a row with band w touches.
__host__ __device__ __forceinline__ int lane_window_for(long long w) {
    return lane_ring_at_least(2 * w + 12);
}

// The lane kernel's ring for band w: 2w + 12 columns rounded up to a
// multiple of 32 (the lane kernel maps columns to slots by a remainder; the
// G kernel's rings are powers of two).
__host__ __device__ __forceinline__ int lane_ring_exact(long long w) {
    return (int)((2 * w + 12 + 31) & ~31LL);
}

// Score of query code q (0..4) against the row's table, sign-extended.
__device__ __forceinline__ int lane_score1(uint32_t tlo, uint32_t thi, uint32_t q) {
    return prmt_sext(__byte_perm(tlo, thi, q), 0u, 0x8880u);
}

// One cell of the recurrence (bandedSWA.cpp:1883-1906) given its score sb;
// returns H(i, j), updates the horizontal gap e, writes the vertical gap f2.
__device__ __forceinline__ int lane_cell(uint32_t w, int sb, int &e, int &f2, const int oe_ins,
                                         const int e_ins, const int oe_del, const int e_del) {
    const int h00 = (int)(w & 0xffffu);
    const int f = (int)(w >> 16);
    const int M = __viaddmin_s32(h00, sb, h00 << 12);      // h00 ? h00 + S : <= 0
    const int H = __vimax3_s32(M, e, f);
    const int T = __viaddmax_s32_relu(M, -oe_ins, 0);       // max(M - oe_ins, 0)
    e = __viaddmax_s32(e, -e_ins, T);
    f2 = __viaddmax_s32_relu(f, -e_del, M - oe_del);
    return H;
}

// Four consecutive columns j..j+3 of a row (row words w0..w3 at hp[0],
// hp[32], hp[64], hp[96]); qw: their four query codes as a selector.  SYM:
// o_del == o_ins and e_del == e_ins, so the vertical gap reuses max(M - oe, 0).
template <bool SYM>
__device__ __forceinline__ void lane_group4(uint32_t *hp, int j, uint32_t w0, uint32_t w1,
                                            uint32_t w2, uint32_t w3, uint32_t qw, uint32_t tlo,
                                            uint32_t thi, int &e, int &hprev, uint32_t &key,
                                            const int oe_ins, const int e_ins, const int oe_del,
                                            const int e_del) {
    const uint32_t r4 = __byte_perm(tlo, thi, qw);  // four scores, one per byte
    const uint32_t w[4] = {w0, w1, w2, w3};
    int M[4], T[4], f[4], H[4], f2[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int sb = prmt_sext(r4, 0u, 0x8880u + 0x1111u * (uint32_t)k);
        const int h00 = (int)(w[k] & 0xffffu);
        f[k] = (int)(w[k] >> 16);
        M[k] = __viaddmin_s32(h00, sb, h00 << 12);       // h00 ? h00 + S : <= 0
        T[k] = __viaddmax_s32_relu(M[k], -oe_ins, 0);     // max(M - oe_ins, 0)
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        H[k] = __vimax3_s32(M[k], e, f[k]);
        e = __viaddmax_s32(e, -e_ins, T[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (SYM) f2[k] = __viaddmax_s32(f[k], -e_del, T[k]);
        else f2[k] = __viaddmax_s32_relu(f[k], -e_del, M[k] - oe_del);
    }
    hp[0] = __byte_perm((uint32_t)hprev, (uint32_t)f2[0], 0x5410u);
    hp[32] = __byte_perm((uint32_t)H[0], (uint32_t)f2[1], 0x5410u);
    hp[64] = __byte_perm((uint32_t)H[1], (uint32_t)f2[2], 0x5410u);
    hp[96] = __byte_perm((uint32_t)H[2], (uint32_t)f2[3], 0x5410u);
    // the row-max key takes the group's maximum with one past its last
    // column; the row's end resolves it to the last column holding it
    const int m4 = __vimax3_s32(H[0], H[1], imax(H[2], H[3]));
    const uint32_t kg = __byte_perm((uint32_t)(j + 4), (uint32_t)m4, 0x5410u);
    key = kg > key ? kg : key;
    hprev = H[3];
}

// Per-lane pair state.
struct LanePair {
    DevPair *pp;
    const uint8_t *q, *t;
    int pidx, req;
    int fend, p;   // frozen columns [nbeg, fend) seen; p: first nonzero of them, or -1
    int nrow, ncol, i, initc, tnext;
    int head, tail, nbeg, nend;
    int maxScore, x, y, gscore, max_off, max_ie;
    int h0e, v1, wk, bandE, qlenE, mlen, zdropE, sh, msk;
    bool is8;
    unsigned long long ncells;
    Couple cp;  // group-coupling detector state
};

// V bit 0: plain group loop (else explicit prefetch of the next group);
// V bit 1: symmetric gap parameters (o_del == o_ins, e_del == e_ins);
// V bit 2: a ring of any multiple of 8 columns (else a power of two, or
// whole rows).
template <int V>
__global__ void __launch_bounds__(128) bsw_lane_kernel(LaunchArgs A) {
    constexpr bool SYM = (V & 2) != 0;
    constexpr bool EXACT = (V & 4) != 0;
    TALBSW_DYNAMIC_SMEM(smem_raw);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    uint32_t *wsm = reinterpret_cast<uint32_t *>(smem_raw) +
                    (size_t)wib * (lane_hf_words(A.cols_cap, A.win) + lane_qs_words(A.cols_cap, A.win));
    uint32_t *HF = wsm + lane;                                     // column j: HF[slot(j) * 32]
    uint32_t *QS = wsm + lane_hf_words(A.cols_cap, A.win) + lane;  // columns 8q..8q+7: QS[qslot(q) * 32]
    // column j -> ring slot: j mod W (a multiply-high by ceil(2^32 / W),
    // exact for j < 2^16, in a ring of any multiple of 8 columns; a mask in a
    // power-of-two ring; j itself in whole rows).  Query word of column j:
    // slot >> 3 (W is a multiple of 8).
    const uint32_t W = A.win > 0 ? (uint32_t)A.win : 0u;
    const uint32_t wmask = W ? W - 1 : 0xffffffffu;
    const uint32_t mg = EXACT ? (uint32_t)((0x100000000ULL + W - 1) / W) : 0u;
    auto slot = [&](uint32_t j) -> uint32_t {
        if constexpr (EXACT) return j - W * __umulhi(j, mg);
        else return j & wmask;
    };
    auto hf = [&](int j) -> uint32_t & { return HF[slot((uint32_t)j) << 5]; };
    auto qs = [&](int j) -> uint32_t & { return QS[(slot((uint32_t)j) >> 3) << 5]; };
    const KernelParams P = A.P;
    const int oe_ins = P.o_ins + P.e_ins, oe_del = P.o_del + P.e_del;
    const int e_ins = P.e_ins, e_del = P.e_del;

    LanePair s = {};
    bool active = false;
    const bool det = A.flagged != nullptr;  // run the group-coupling detector
    const int nwork = work_count(A);
    const int32_t *order = A.seg ? A.order + A.seg[0] : A.order;
    const int32_t *order_req = A.reqs ? (A.seg ? A.order_req + A.seg[0] : A.order_req) : nullptr;
    auto fail = [&](int flag, int req, int pidx) { report_error(A, req, flag, pidx); };
    // a pair ends (exit, zero row, z-drop, last row): its outputs, or, when the
    // detector flagged it during this row, its place on the flagged list
    auto finish = [&]() {
        active = false;
        if (det && s.cp.flag) {
            flag_pair(A, s.req, s.pidx);
            return;
        }
        if (A.cells) atomicAdd(A.cells, s.ncells);
        s.pp->score = s.maxScore;
        s.pp->tle = s.x;
        s.pp->qle = s.y;
        s.pp->max_off = s.max_off;
        s.pp->gscore = s.gscore;
        s.pp->gtle = s.max_ie;
    };

    // One iteration = one row of this lane's pair; a lane that finishes a pair
    // takes the next one at the top of the next iteration, independently of
    // the other lanes.
    for (;;) {
        if (!active) {
            const int item = atomicAdd(A.work_counter, 1);
            if (item >= nwork) break;
            const int pidx = order ? order[item] : item;
            const int req = order_req ? order_req[item] : -1;
            const PairSrc src = pair_src(A, pidx, req);
            DevPair *pp = src.pp;
            const int len1 = pp->len1, len2 = pp->len2, h0in = pp->h0;
            const int idr = pp->idr, idq = pp->idq;
            const int wcall = src.w;
            bool is8;
            if (src.bits == 8) is8 = true;
            else if (src.bits == 16) is8 = false;
            else is8 = pair_in_range(P, len1, len2, h0in, wcall, true);
            const bool inwin = (long long)idr >= src.ref_lo && (long long)idq >= src.qer_lo &&
                               (long long)idr + len1 <= src.ref_hi && (long long)idq + len2 <= src.qer_hi;
            const bool ok = pair_in_range(P, len1, len2, h0in, wcall, is8) && wcall >= 0 && inwin;
            if (!ok) {
                // outside the exact range of int32 cells: the grouped kernel
                // computes in the element type and takes it
                if (det && inwin && pair_in_group_range(len1, len2, h0in, wcall, is8)) flag_pair(A, req, pidx);
                else fail(ERR_DOMAIN, req, pidx);
                continue;
            }
            if (A.win > 0 ? (2LL * wcall + 12 > A.win && len2 + 4 > A.win) : (len2 > A.cols_cap)) {
                if (det) flag_pair(A, req, pidx);
                else fail(ERR_CAPACITY, req, pidx);
                continue;
            }
            // per-pair constants (smithWatermanBatchWrapper16/8 set-up)
            s.pp = pp;
            s.pidx = pidx;
            s.req = req;
            s.q = src.qer + (idq - src.qer_lo);
            s.t = src.ref + (idr - src.ref_lo);
            s.nrow = len1; s.ncol = len2; s.i = 0; s.initc = 0; s.ncells = 0;
            s.is8 = is8;
            s.sh = is8 ? 24 : 16;
            s.msk = is8 ? 0xff : 0xffff;
            const int sh = s.sh, msk = s.msk;
            s.h0e = wrapS(wrapU(h0in, msk), sh);
            s.v1 = (s.h0e > oe_ins) ? wrapS(s.h0e - oe_ins, sh) : 0;
            int maxsc = 0;  // max(0, a, -b, -1) in the element type (:2779-2782)
            {
                const int av = wrapS((int8_t)P.a, sh), bv = wrapS((int8_t)(-P.b), sh);
                if (maxsc < av) maxsc = av;
                if (maxsc < bv) maxsc = bv;
                if (maxsc < -1) maxsc = -1;
            }
            int myband;  // band clamp (:2882-2904): integer division, then +1
            {
                const int qlen_b = wrapU(len2 * maxsc, msk);
                const int tmp1 = wrapU(qlen_b + wrapS(P.end_bonus - P.o_ins, sh), msk);
                int mi = tmp1 / P.e_ins + 1;
                if (mi < 1) mi = 1;
                myband = wrapU(wcall > mi ? mi : wcall, msk);
                const int tmp2 = wrapU(qlen_b + wrapS(P.end_bonus - P.o_del, sh), msk);
                int md = tmp2 / P.e_del + 1;
                if (md < 1) md = 1;
                myband = wrapU(myband > md ? md : myband, msk);
                s.wk = wcall < myband ? myband : wcall;
            }
            s.qlenE = wrapS(len2, sh);
            s.mlen = wrapS(imin(wrapU(s.qlenE + myband, msk), wrapU(wrapS(len1, sh), msk)), sh);
            s.zdropE = wrapS(P.zdrop, sh);
            s.bandE = wrapS(myband, sh);
            s.head = 0; s.tail = s.qlenE;
            s.maxScore = s.h0e; s.x = 0; s.y = 0; s.gscore = -1; s.max_off = 0; s.max_ie = 0;
            s.nbeg = 0; s.nend = len2;
            s.fend = 0; s.p = -1;
            s.tnext = len1 > 0 ? s.t[0] : 0;
            s.cp.init(s.qlenE, s.v1, e_ins);
            active = true;
        }
        if (s.i >= s.nrow) { finish(); continue; }

        const int sh = s.sh, msk = s.msk;
        const int i = s.i, ncol = s.ncol;
        const int i1 = wrapS(i + 1, sh);
        const int tb = s.tnext;
        if (tb > 4) { fail(ERR_BASE, s.req, s.pidx); active = false; continue; }
        if (i + 1 < s.nrow) s.tnext = s.t[i + 1];
        // columns up to i + wk + 3 can be touched by this row (band end + 2):
        // give them their row-0 values and stage their query selectors now
        {
            const int lim = imin(imax(ncol, 1), i + s.wk + 3);
            bool bad = false;
            for (int k = s.initc; k <= lim; k++) {
                int hv;
                if (k == 0) hv = s.h0e;
                else if (k == 1) hv = s.v1;
                else if (k < ncol) hv = imax(s.v1 - (k - 1) * e_ins, 0);
                else hv = 0;
                hf(k) = (uint32_t)hv;
                if (!(k & 7) && k < ncol) {
                    uint32_t wq = 0;
                    const int m = imin(8, ncol - k);
                    for (int b = 0; b < m; b++) {
                        const uint32_t c = s.q[k + b];
                        bad |= c > 4u;
                        wq |= (c & 7u) << (4 * b);
                    }
                    qs(k) = wq;
                }
            }
            if (lim + 1 > s.initc) s.initc = lim + 1;
            if (bad) { fail(ERR_BASE, s.req, s.pidx); active = false; continue; }
        }
        int beg = s.nbeg, end = s.nend;
        if (beg < i - s.wk) beg = i - s.wk;
        if (end > i + s.wk + 1) end = i + s.wk + 1;
        if (end > ncol) end = ncol;
        // columns that left the band since the last row are frozen: note the
        // first nonzero one at or after nbeg (16-bit head re-derivation)
        if (!s.is8) {
            if (s.p < 0)
                for (int c = imax(s.fend, s.nbeg); c < beg; c++)
                    if (hf(c) != 0u) { s.p = c; break; }
            s.fend = imax(s.fend, beg);
        }
        // H_v[i+1] (:3065-3067): the first column's value, used when beg == 0
        const int hv_next = (i + 1 == s.nrow) ? 99 : imax(wrapS(s.h0e - P.o_del - (i + 1) * P.e_del, sh), 0);
        const int h10init = beg == 0 ? hv_next : 0;
        if (det) {  // columns frozen since the last row: lowest / highest non-zero
            for (int c = s.cp.frozenTo; c < beg; c++)
                if (hf(c) != 0u) s.cp.frozen_nz(c);
            s.cp.frozenTo = imax(s.cp.frozenTo, beg);
        }
        // per-pair band (:3080-3089) and trimming (:3091-3112)
        const int phead = s.head, ptail = s.tail;
        const int head = imax(s.head, wrapS(i - s.bandE, sh));
        int tail;
        {
            int tt = imin(wrapU(s.tail, msk), wrapU(i1 + s.bandE, msk));
            tt = imin(tt, wrapU(s.qlenE, msk));
            tail = wrapS(tt, sh);
        }
        s.head = head;
        s.tail = tail;
        const bool changed = head != phead || tail != ptail;
        bool oldnz_masked = false;  // old entries of [beg, head) seen non-zero (untrimmed rows)
        if (det) {
            s.cp.clamp(wrapS(i - s.bandE, sh), wrapU(i1 + s.bandE, msk), wrapU(s.qlenE, msk), sh, msk);
            const bool stay = !(i1 > s.mlen || tail == head || head > tail);
            s.cp.row_checks(true, i1 > s.mlen, stay, i, s.wk, beg, end, ncol, h10init, hv_next,
                            s.is8 ? 127 : 32767);
            if (stay && s.cp.hlo != s.cp.hhi) {  // uncertain head: [beg, max(head, hhi)) before trimming
                const int hi = s.cp.trim_hi(changed, end, head);
                for (int l = beg; l < hi; l++)
                    if (hf(l) != 0u) { s.cp.flag |= CPL_TRIM; break; }
            }
        }
        if (changed) {
            const int hi = imin(end, head);
            for (int l = beg; l < hi; l++) hf(l) = 0u;
        }
        // row exit status (:3119-3129); outputs freeze once a pair exits
        if (i1 > s.mlen || tail == head || head > tail) { finish(); continue; }

        // score table of the row's target base: byte q of {thi:tlo} is S(t, q)
        // as a signed byte (query code q: 0..3 bases, 4 = N)
        uint32_t tlo;
        {
            const uint32_t mis = (uint32_t)(-P.b) & 0xffu;
            const uint32_t mat = (uint32_t)P.a & 0xffu;
            if (tb >= 4) {
                tlo = 0xffffffffu;
            } else {
                tlo = mis * 0x01010101u;
                tlo = (tlo & ~(0xffu << (8 * tb))) | (mat << (8 * tb));
            }
        }
        const uint32_t thi = 0x000000ffu;
        if (det) {  // F the group could store differently at the tail column and at the band end
            const bool tin = tail >= beg && tail < end;
            int ft = 0, fe = 0;
            if (tin) {
                const uint32_t wv = hf(tail);
                const uint32_t q = (qs(tail) >> (4 * (tail & 7))) & 0xfu;
                ft = Couple::fnext((int)(wv & 0xffffu), (int)(wv >> 16), lane_score1(tlo, thi, q), e_del, oe_del);
            }
            if (end < ncol && end == tail) {
                const uint32_t wv = hf(end);
                const uint32_t q = (qs(end) >> (4 * (end & 7))) & 0xfu;
                fe = Couple::fnext((int)(wv & 0xffffu), (int)(wv >> 16), lane_score1(tlo, thi, q), e_del, oe_del);
            }
            s.cp.f_checks(true, i, s.wk, beg, end, head, tail, ncol, s.is8 ? 127 : 32767, tin, ft, fe);
        }

        // ---- the band [beg, end): masked left part, clean middle, tail part
        int e = 0, hprev = h10init;
        uint32_t key = 0;
        const int jA = imin(imax(beg, head), end);  // columns j < head: masked
        const int jB = imax(imin(end, tail), jA);   // columns j >= tail: not in the max
        if (end > beg) s.ncells += (unsigned long long)(end - beg);
        for (int j = beg; j < jA; j++) {
            const uint32_t w = hf(j);
            oldnz_masked |= w != 0u;
            const uint32_t q = (qs(j) >> (4 * (j & 7))) & 0xfu;
            int f2;
            hprev = lane_cell(w, lane_score1(tlo, thi, q), e, f2, oe_ins, e_ins, oe_del, e_del);
            hf(j) = 0u;  // masked: H and F stored as zero
        }
        {
            int j = jA;
            // single columns up to a multiple of 4
            for (; (j & 3) && j < jB; j++) {
                const uint32_t w = hf(j);
                const uint32_t q = (qs(j) >> (4 * (j & 7))) & 0xfu;
                int f2;
                const int H = lane_cell(w, lane_score1(tlo, thi, q), e, f2, oe_ins, e_ins, oe_del, e_del);
                hf(j) = __byte_perm((uint32_t)hprev, (uint32_t)f2, 0x5410u);
                const uint32_t kk = __byte_perm((uint32_t)(j + 1), (uint32_t)H, 0x5410u);
                key = kk > key ? kk : key;
                hprev = H;
            }
            // groups of four columns: one table lookup for four scores
            if constexpr ((V & 1) == 0) {
                // next group's row words loaded before this group is computed
                if (j + 3 < jB) {
                    uint32_t *hp = &hf(j);
                    uint32_t w0 = hp[0], w1 = hp[32], w2 = hp[64], w3 = hp[96];
                    uint32_t qw = qs(j) >> (4 * (j & 4));
                    for (;;) {
                        const int jn = j + 4;
                        const bool more = jn + 3 < jB;
                        uint32_t n0 = 0, n1 = 0, n2 = 0, n3 = 0, nq = 0;
                        uint32_t *hn = &hf(jn);
                        if (more) {
                            n0 = hn[0]; n1 = hn[32]; n2 = hn[64]; n3 = hn[96];
                            nq = qs(jn) >> (4 * (jn & 4));
                        }
                        lane_group4<SYM>(hp, j, w0, w1, w2, w3, qw, tlo, thi, e, hprev, key,
                                         oe_ins, e_ins, oe_del, e_del);
                        hp = hn;
                        j = jn;
                        if (!more) break;
                        w0 = n0; w1 = n1; w2 = n2; w3 = n3; qw = nq;
                    }
                }
            } else {
                // plain loop over groups; two groups per iteration so that
                // the second group's loads can be issued early
                // the group's slot advances by four (j is a multiple of 4, and
                // so is W: a group never straddles the ring's end)
                uint32_t sj = j + 3 < jB ? slot((uint32_t)j) : 0u;
#pragma unroll 2
                for (; j + 3 < jB; j += 4) {
                    uint32_t *hp = &HF[sj << 5];
                    const uint32_t qw = QS[(sj >> 3) << 5] >> (4 * (j & 4));
                    lane_group4<SYM>(hp, j, hp[0], hp[32], hp[64], hp[96], qw, tlo, thi, e, hprev,
                                     key, oe_ins, e_ins, oe_del, e_del);
                    sj += 4;
                    if constexpr (EXACT) sj = sj >= W ? sj - W : sj;
                    else sj &= wmask;
                }
            }
            for (; j < jB; j++) {
                const uint32_t w = hf(j);
                const uint32_t q = (qs(j) >> (4 * (j & 7))) & 0xfu;
                int f2;
                const int H = lane_cell(w, lane_score1(tlo, thi, q), e, f2, oe_ins, e_ins, oe_del, e_del);
                hf(j) = __byte_perm((uint32_t)hprev, (uint32_t)f2, 0x5410u);
                const uint32_t kk = __byte_perm((uint32_t)(j + 1), (uint32_t)H, 0x5410u);
                key = kk > key ? kk : key;
                hprev = H;
            }
        }
        for (int j = jB; j < end; j++) {
            const uint32_t w = hf(j);
            const uint32_t q = (qs(j) >> (4 * (j & 7))) & 0xfu;
            int f2;
            const int H = lane_cell(w, lane_score1(tlo, thi, q), e, f2, oe_ins, e_ins, oe_del, e_del);
            // j >= tail: not in the row maximum; j > tail: H and F stored as zero
            hf(j) = (j > tail) ? 0u : __byte_perm((uint32_t)hprev, (uint32_t)f2, 0x5410u);
            hprev = H;
        }
        // last column of the row (:3197-3203)
        const bool ran = end > beg;
        {
            const int jl = ran ? end : beg;
            const bool m = (head > jl) || (jl > tail);
            const uint32_t hst = m ? 0u : ((uint32_t)hprev & 0xffffu);
            if (jl <= ncol + 1) hf(jl) = hst;
            if (det) {
                if (!changed && oldnz_masked) s.cp.flag |= CPL_TRIM;  // the group may trim them
                s.cp.stored_last(jl, ncol, (int)hst, tb >= 4 ? -1 : -P.b, head, tail, e_del, oe_del);
            }
        }
        // gscore at the query's last column (:3177-3195): in the band exactly
        // when end == ncol, and then it is column end-1
        if (ran && end == ncol && !(s.qlenE > tail)) {
            s.max_ie = (s.gscore > hprev) ? s.max_ie : i1;
            s.gscore = imax(s.gscore, hprev);
        }
        const int maxRS1 = (int)(key >> 16);
        if (maxRS1 == 0) { finish(); continue; }  // a zero row ends the pair (:3206-3211)
        // y1 = one past the last column holding the row maximum.  A key is one
        // past a single column (which holds the maximum) or one past a group of
        // four (the last of them that holds it); the row's H(c) of a column
        // scored in the clean middle is stored at column c + 1.
        int y1;
        {
            const int k = (int)(key & 0xffffu);
            const int a3 = (int)(hf(k) & 0xffffu);
            const int a2 = (int)(hf(imax(k - 1, 0)) & 0xffffu);
            const int a1 = (int)(hf(imax(k - 2, 0)) & 0xffffu);
            y1 = a3 == maxRS1 ? k : a2 == maxRS1 ? k - 1 : a1 == maxRS1 ? k - 2 : k - 3;
        }
        {   // maximum, its position and max_off (:3213-3226)
            const int bmax = s.maxScore;
            s.maxScore = imax(s.maxScore, maxRS1);
            if (s.maxScore > bmax) {
                s.y = y1;
                s.x = i1;
                int ind = wrapS(y1 - i1, sh);
                if (ind < 0) ind = wrapS(-ind, sh);
                s.max_off = imax(s.max_off, ind);
            }
        }
        {   // z-drop (:3229 -> ZSCORE16 :1868-1881, ZSCORE8 :1826-1839)
            const int tmpi = wrapS(i1 - s.x, sh);
            const int tmpj = wrapS(y1 - s.y, sh);
            const int d = (tmpi > tmpj) ? wrapS(tmpi - tmpj, sh) : wrapS(tmpj - tmpi, sh);
            const int t1 = wrapS(wrapS(s.maxScore - maxRS1, sh) - d, sh);
            if (t1 > s.zdropE) { finish(); continue; }
        }
        {   // band narrowing (:3235-3260)
            int l = beg;
            while (l < end && hf(l) == 0u) l++;
            if (l > beg) {  // nbeg >= beg: no frozen columns at or after it yet
                s.nbeg = l - 1;
                s.fend = s.nbeg;
                s.p = -1;
            }
            l = end;
            while (l >= beg && hf(l) == 0u) l--;
            s.nend = (l + 2 < ncol) ? l + 2 : ncol;
        }
        {   // per-pair head / tail (:3265-3316; 8-bit: the row's own range :2571-2621)
            const int B = s.is8 ? beg : s.nbeg;
            const int E = s.is8 ? end : s.nend;
            bool run_end = false, run_bot = false;
            if (E > B) {
                int l = B;
                bool found = false;
                if (l < beg) {  // frozen columns [nbeg, beg): their first nonzero
                    if (s.p >= 0 && s.p < E) { l = s.p; found = true; }
                    else l = imin(beg, E);
                }
                if (!found) while (l < E && hf(l) == 0u) l++;
                run_end = l == E;
                if (l > B) s.head = wrapS(l, sh);
            }
            int index = s.tail;
            if (E >= B) {
                // a cell with H > 0 left a nonzero in [beg + 1, end], so this
                // scan stops inside the band
                int l = E;
                while (l >= B && hf(l) == 0u) l--;
                run_bot = l < B;
                if (l < beg && W > 0) {  // would have read a ring slot reused since
                    if (det) flag_pair(A, s.req, s.pidx);
                    else fail(ERR_CAPACITY, s.req, s.pidx);
                    active = false;
                    continue;
                }
                if (l != E) index = l;
            }
            const int index0 = index;
            index = wrapS(index + 2, sh);
            s.tail = index < s.qlenE ? index : s.qlenE;
            if (det) {
                const bool last_row = i + 1 >= s.nrow;
                const bool nz_sb = B < beg ? s.p == B : hf(B) != 0u;
                const uint32_t wse = hf(E);
                s.cp.scans(true, last_row, s.is8, i, s.wk, beg, end, B, E, nz_sb, wse != 0u, run_end,
                           (wse & 0xffffu) != 0u, run_bot, s.head, index0, s.qlenE, ncol,
                           s.is8 ? 127 : 32767);
                s.cp.settle(true, last_row, s.head, s.tail);
                if (s.cp.flag) { flag_pair(A, s.req, s.pidx); active = false; continue; }
            }
        }
        s.i = i + 1;
    }
}

}  // namespace talbsw
