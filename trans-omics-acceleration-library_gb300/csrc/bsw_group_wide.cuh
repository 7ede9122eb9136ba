// The reference's SIMD groups, one thread block per group: the kernel of the
// regroup pass (bsw_regroup.cu), which re-scores the groups of flagged pairs.
//
// bsw_group.cuh follows the reference's kernel with one warp per group: lane
// l of the group is thread l, and each thread walks the group's band
// [beg, end) column by column.  That walk is a serial chain of ~60
// instructions per column, so a lone group (the regroup pass re-scores a few
// hundred, spread over the device) advances one column every ~500 cycles and
// a group of 2,000-base pairs takes tens of milliseconds.  Here NW warps
// (wide_warps) share the group: every warp holds all of the group's lanes
// (thread t of each warp is lane t, and t + 32 in 8-bit), and the band is
// cut into NW contiguous column chunks, one per warp.
//
// Per row (bandedSWA.cpp:3080-3316 for 16-bit, :2371-2621 for 8-bit):
//  * the per-lane state (band clamp, head, tail, maxima, exit) is replicated
//    in every warp, so every warp takes the same branches;
//  * the cells: M and F of a column depend only on the row above, E on the
//    columns to its left, E(j + 1) = max(E(j) - e_ins, max(M(j) - oe_ins, 0)).
//    Pass 1: each warp runs that recurrence over its chunk from E = 0 and
//    publishes the E leaving it; E(j) >= 0 throughout, so the E entering
//    chunk k is max(A(k-1), E(k-1) - n(k-1) * e_ins) exactly (max-plus).
//    Pass 2: each warp re-walks its chunk from the true entering E and the
//    previous column's H (from the neighbouring chunk's published values),
//    storing the row exactly as the sequential walk does.  Both passes load
//    the next column's word one column ahead, and score a cell with one byte
//    permute of the row's score table (query selectors stored per column);
//  * every store also records the column's mask of lanes holding a non-zero
//    word (NZ).  The narrowing reads the masks' union; the head / tail scans
//    (each warp a part of the range) take 32 columns per step: a ballot
//    finds the first column where no live lane is zero, a 32 x 32 bit
//    transpose gives every lane its first column where it is not a live zero;
//    a scan's stopping column and each lane's first such column are minima /
//    maxima over the warps' parts, combined through shared memory, as are
//    the row maximum with its last column (a packed key).
// Every value is kept in the element width and wraps as the reference's
// does, as in bsw_group.cuh.
//
// Member mode stops a group once its needed lanes (the flagged pairs) have
// exited: a lane's outputs freeze at its exit, and only the needed lanes'
// outputs are written (the others keep their per-pair results, which the
// detector proved equal to the grouped ones).
#pragma once

#include <climits>

#include "bsw_group.cuh"

namespace talbsw {

// Warps per group: 16 for 16-bit groups (4 / 8 / 16 measured 6.2 / 3.2 / 2.6 ms for
// C2's regroup pass), 8 for 8-bit ones (two lanes per thread need ~160 registers)
template <int SB>
__host__ __device__ constexpr int wide_warps() { return SB == 16 ? 16 : 8; }

// Cross-warp exchange of one block, at the start of its shared memory.
template <int NW>
struct WideX {
    int g;                     // the group this block scores
    int bad;                   // a lane's input is out of range (skip the group)
    int endnz;                 // column `end` holds a non-zero word after the row
    int nzF[NW], nzL[NW];      // first / last column of a warp's chunk holding a non-zero word
    int Z[NW], Zr[NW];         // head / tail scan: first / last column of a warp's part where no live lane is zero
    int Aagg[NW][64];          // E leaving a warp's chunk, the chunk entered with E = 0
    int Elast[NW][64];         // that E, entering the chunk's last column
    int MF[NW][64];            // max(M, F) at the chunk's last column
    unsigned key[NW][64];      // row maximum and its last column: (H << 16) | (j + 1)
    int R[NW][64], Q[NW][64];  // head / tail scan: a lane's first / last non-zero column
    int gscore[64], max_ie[64];
};

// 32 x 32 bit transpose across a warp: thread t holds row t on entry and
// column t on return (bit r of the result = bit t of thread r's row), in
// five exchange steps of halving width (the recursive block transpose).
__device__ __forceinline__ unsigned transpose32(unsigned x, int t) {
    unsigned m = 0x0000ffffu;
    for (int j = 16; j != 0; j >>= 1, m ^= (m << j)) {
        const unsigned y = __shfl_xor_sync(0xffffffffu, x, j);
        x = (t & j) ? (((y >> j) & m) | (x & ~m)) : ((x & m) | ((y << j) & ~m));
    }
    return x;
}

template <int NW>
__host__ __device__ constexpr size_t wide_x_bytes() {
    return (sizeof(WideX<NW>) + 15) & ~(size_t)15;
}

// int16 elements of a block's global slot: whole rows of col_cap columns as
// in group_slot_elems, then the per-column masks of non-zero lanes.
__host__ __device__ inline size_t wide_slot_elems(int col_cap, int bits) {
    const size_t lpt = bits == 8 ? 2 : 1;
    return group_slot_elems(col_cap, bits) + ((size_t)col_cap * 4 * lpt + 32) / 2 + 8;
}

template <int SB, int NW>
__device__ __forceinline__ void group_wide_body(const GroupArgs &A, unsigned char *smem) {
    typedef GE<SB> E;
    constexpr int LPT = SB == 8 ? 2 : 1;  // lanes per thread
    constexpr int W = 32 * LPT;           // lanes per group
    constexpr bool is16 = SB == 16;
    const unsigned full = 0xffffffffu;
    const int t = threadIdx.x & 31;
    const int wp = threadIdx.x >> 5;
    WideX<NW> &X = *reinterpret_cast<WideX<NW> *>(smem);
    uint32_t *const smRows = reinterpret_cast<uint32_t *>(smem + wide_x_bytes<NW>());
    const size_t rows_bytes = A.smem_bytes > wide_x_bytes<NW>() ? A.smem_bytes - wide_x_bytes<NW>() : 0;
    uint32_t *const HFg = reinterpret_cast<uint32_t *>(A.scratch + (size_t)blockIdx.x * A.slot_elems);
    const KernelParams &P = A.P;
    const bool mm = A.members != nullptr;  // member mode
    const int ngroups = mm ? imin(*A.ngroups_dev, A.ngroups_cap) : (A.n + W - 1) / W;

    // scores and constants (bandedSWA.cpp:50-68), wrapped to the element width
    const int w_match = E::ws((int8_t)P.a);
    const int w_mismatch = E::ws((int8_t)(P.b * -1));
    const int e_del = E::ws(P.e_del), oe_del = E::ws(P.o_del + P.e_del);
    const int e_ins = E::ws(P.e_ins), oe_ins = E::ws(P.o_ins + P.e_ins);
    const int o_del = E::ws(P.o_del);
    const int zdropv = E::ws(P.zdrop);
    int maxsc = 0;  // max of the scores (:2779 / :2082)
    if (maxsc < (int8_t)P.a) maxsc = E::ws((int8_t)P.a);
    if (maxsc < (int8_t)(P.b * -1)) maxsc = E::ws((int8_t)(P.b * -1));

    for (;;) {
        __syncthreads();  // the previous group's reads of X and of the rows are done
        if (threadIdx.x == 0) {
            X.g = atomicAdd(A.work_counter, 1);
            X.bad = 0;
        }
        __syncthreads();
        const int g = X.g;
        if (g >= ngroups) break;

        // ---- the group's lanes (as bsw_group.cuh; lanes past n are padded
        // as the reference pads its array)
        int len1[LPT], len2[LPT], h0r[LPT];
        long long idr[LPT], idq[LPT];
        DevPair *pp[LPT];
        long long lidx[LPT];
        bool real[LPT], needl[LPT];
        bool bad = false;
        int gw = A.w, greq = -1, padq = 0;
        DevPair *gpairs = A.pairs;
        const uint8_t *Aref = A.ref, *Aqer = A.qer;
        long long ref_lo = A.ref_lo, ref_hi = A.ref_hi, qer_lo = A.qer_lo, qer_hi = A.qer_hi;
        unsigned long long needm = ~0ull;
        if (mm) {
            const int4 gi = A.ginfo[g];
            gw = gi.x; greq = gi.y; padq = gi.z;
            if (A.need) needm = A.need[g];
            if (greq >= 0) {
                const ReqDesc &d = A.reqs[greq];
                gpairs = d.pairs;
                Aref = d.ref; Aqer = d.qer;
                ref_lo = d.ref_lo; ref_hi = d.ref_hi; qer_lo = d.qer_lo; qer_hi = d.qer_hi;
            }
        }
        auto gerr = [&](int flag, long long k) {  // idempotent: any warp may report
            atomicOr(A.err_flags, flag);
            if (greq >= 0) {
                atomicOr(&A.reqs[greq].err, flag);
                atomicMin(&A.reqs[greq].bad, k);
            } else {
                atomicMin(A.err_index, k);
            }
        };
        for (int u = 0; u < LPT; u++) {
            const int l = t + 32 * u;
            long long k = (long long)g * W + l;
            if (mm) {
                k = A.members[(size_t)g * 64 + l];
                real[u] = k >= 0;
                if (real[u] && greq >= 0) k -= A.reqs[greq].first;
            } else {
                real[u] = k < A.n;
            }
            needl[u] = real[u] && ((needm >> l) & 1ull);
            lidx[u] = k;
            pp[u] = real[u] ? gpairs + k : nullptr;
            if (real[u]) {
                const DevPair &p = *pp[u];
                len1[u] = p.len1; len2[u] = p.len2; h0r[u] = p.h0;
                idr[u] = p.idr; idq[u] = p.idq;
                const int lim = is16 ? 32767 : 127;
                const bool ok = len1[u] >= 0 && len2[u] >= 0 && len1[u] <= lim && len2[u] <= lim &&
                                h0r[u] >= 0 && idr[u] >= ref_lo && idr[u] + len1[u] <= ref_hi &&
                                idq[u] >= qer_lo && idq[u] + len2[u] <= qer_hi &&
                                len2[u] + 3 <= A.col_cap;
                if (!ok) {
                    gerr(ERR_DOMAIN, k);
                    bad = true;
                }
            } else {
                len1[u] = 0;
                len2[u] = is16 ? 0 : (mm ? padq : A.pairs[A.n - 1].len2);
                h0r[u] = 0;
                idr[u] = idq[u] = -1;
            }
        }
        if (__any_sync(full, bad)) continue;  // the same lanes in every warp: uniform

        // ---- lengths as the wrapper hands them to the kernel
        int m1 = 0, m2 = 0, mq = 0x7fffffff;
        for (int u = 0; u < LPT; u++) {
            m1 = imax(m1, len1[u]);
            m2 = imax(m2, len2[u]);
            mq = imin(mq, len2[u]);
        }
        const int maxLen1 = __reduce_max_sync(full, m1);
        const int maxLen2 = __reduce_max_sync(full, m2);
        const int minq = __reduce_min_sync(full, mq) - 1;
        const int nrow = maxLen1, ncol = maxLen2, wrapRows = maxLen1;
        const int colCap = (ncol > 1 ? ncol : 1) + 3;

        // ---- per-lane set-up: band clamp, query bases checked
        int h0[LPT], tlen[LPT], qlen[LPT], myband[LPT], tt1[LPT], tt2[LPT];
        const uint8_t *qp[LPT];
        int bsz = gw;
        for (int u = 0; u < LPT; u++) {
            const int l = t + 32 * u;
            h0[u] = E::ws((int)E::us(h0r[u]));
            tlen[u] = E::ws((int)E::us(len1[u]));
            qlen[u] = E::ws((int)E::us(len2[u]));
            // a padding lane (8-bit) reads the query bytes at the caller's
            // offset 0, as the reference's zeroed SeqPair does
            qp[u] = real[u] ? Aqer + (idq[u] - qer_lo)
                  : (qer_lo <= 0 && len2[u] <= qer_hi) ? Aqer - qer_lo : nullptr;
            // row 0: h0, tt1 = h0 - oe_ins (wrapped), then the reference's chain
            // tt = max(tt - e_ins, 0) below the group's longest query; from
            // column 2 on the chain starts from a value >= 0 and no longer
            // wraps, so column k holds max(tt2 - (k - 2) e_ins, 0)
            tt1[u] = (h0[u] > oe_ins) ? E::ws(h0[u] - oe_ins) : 0;
            tt2[u] = imax(E::ws(tt1[u] - e_ins), 0);
            if (real[u] && qp[u])
                for (int k = wp; k < len2[u]; k += NW)
                    if (qp[u][k] > 4) {
                        gerr(ERR_BASE, lidx[u]);
                        bad = true;
                        break;
                    }
            // band clamp (:2882-2904 / :2183-2205): integer division, then +1.0
            const int qlenb = E::ws(len2[u] * maxsc);
            const int eb_ins = E::ws(P.end_bonus - P.o_ins), eb_del = E::ws(P.end_bonus - P.o_del);
            int temp = (int)E::us(qlenb + eb_ins);
            int mi = temp / P.e_ins + 1;
            mi = mi > 1 ? mi : 1;
            myband[u] = E::ws((int)E::us(gw > mi ? mi : gw));
            temp = (int)E::us(qlenb + eb_del);
            mi = temp / P.e_del + 1;
            mi = mi > 1 ? mi : 1;
            const int mb = (int)E::us(myband[u]);
            myband[u] = E::ws((int)E::us(mb > mi ? mi : mb));
            bsz = imax(bsz, (int)E::us(myband[u]));
            if (wp == 0) {
                X.gscore[l] = -1;
                X.max_ie[l] = 0;
            }
        }
        if (__any_sync(full, bad)) X.bad = 1;  // a base code above 4 in this warp's columns
        __syncthreads();
        if (X.bad) continue;
        const int w = __reduce_max_sync(full, bsz);

        // ---- the group's rows.  Row i touches columns up to i + w + 3 (its
        // band end, the last-column store, the scans' end) and writes none
        // below its band start beg >= i - w, which never decreases.  So the
        // rows live in a ring of WR >= 2w + 8 columns (column c in slot
        // c mod WR) when that is shorter than the query, whole rows when not,
        // and in the block's global slot when neither fits shared memory.
        // Beside them, for every column, the mask of lanes whose (H, F) word
        // is non-zero (NZ), kept current at every store: the narrowing and
        // the head / tail scans read only those masks, so a column that left
        // the band needs no slot once its last store is recorded.
        int WR = 8;
        while (WR < 2 * w + 8) WR <<= 1;
        bool ring = WR < colCap;
        if (!ring) WR = colCap;
        const size_t nz_bytes = (size_t)colCap * 4 * LPT + 32;
        const size_t rows_need = (ring ? (size_t)WR * W * 5 : group_smem_bytes(colCap, SB)) + nz_bytes;
        if (rows_need <= A.skip_upto) continue;             // the first launch scored it
        if (A.defer && rows_need > rows_bytes) continue;  // the second launch will
        uint32_t *HF = smRows;
        if (rows_need > rows_bytes) {
            ring = false;
            WR = colCap;
            HF = HFg;
        }
        const int wm = WR - 1;
        // query selectors: one byte per lane and slot, [slot][lane] like HF
        uint8_t *const Q2 = reinterpret_cast<uint8_t *>(HF + (size_t)WR * W);
        uint32_t *const NZ = reinterpret_cast<uint32_t *>(
            reinterpret_cast<uintptr_t>(Q2 + ((((size_t)WR + 3) & ~(size_t)3) + 8) * W + 15) & ~(uintptr_t)15);
        auto slot = [&](int c) -> int { return ring ? (c & wm) : c; };
        auto HFa = [&](int c, int u) -> uint32_t & { return HF[(size_t)slot(c) * W + t + 32 * u]; };
        auto pack = [](int h, int f) -> uint32_t { return (uint32_t)(uint16_t)h | ((uint32_t)(uint16_t)f << 16); };
        // column k's query selector and row-0 entry, for every lane of this
        // thread.  Selector: 0 for N, 1 + b for base b, 5 for the padding code
        // past the lane's query (DUMMY2, :46) -- the byte of the row's score
        // table (below) that holds S(target base, query code)
        // warp wp initialises the columns k = wp mod NW and loads the query
        // byte of its next one a row ahead (kp, bp), off the row's critical path
        int kp = -1, bp[LPT];
        auto qbyte = [&](int k, int u) -> int { return k < len2[u] && qp[u] ? qp[u][k] : 4; };
        auto init_col = [&](int k) {
            const int sc = slot(k);
            for (int u = 0; u < LPT; u++) {
                const int l = t + 32 * u;
                int sel = 1;
                if (k < len2[u]) {
                    const int b = k == kp ? bp[u] : qbyte(k, u);
                    sel = b == 4 ? 0 : b + 1;
                } else if (k <= maxLen2) {
                    sel = 5;
                }
                Q2[(size_t)sc * W + l] = (uint8_t)sel;
                int hv = 0;
                if (k == 0) hv = h0[u];
                else if (k == 1) hv = tt1[u];
                else if (k < maxLen2) hv = imax(tt2[u] - (k - 2) * e_ins, 0);
                HF[(size_t)sc * W + l] = (uint16_t)hv;
                const unsigned m = __ballot_sync(full, (uint16_t)hv != 0);
                if (t == 0) NZ[(size_t)k * LPT + u] = m;
            }
        };
        int initc = 0;  // next column to initialise

        // ---- the kernel proper (:2962-3356 / :2263-2661)
        int head[LPT], tail[LPT], mlen[LPT], maxScore[LPT], x[LPT], y[LPT];
        int max_off[LPT], exit0[LPT];
        for (int u = 0; u < LPT; u++) {
            tail[u] = qlen[u];
            head[u] = 0;
            const unsigned ml = E::us(qlen[u] + myband[u]);
            mlen[u] = E::ws((int)umin(ml, E::us(tlen[u])));
            maxScore[u] = h0[u];
            x[u] = y[u] = 0;
            max_off[u] = 0;
            exit0[u] = -1;
        }
        auto Hv = [&](int k, int u) -> int {
            if (k == 0) return h0[u];
            if (k < wrapRows) {
                const int v = E::ws(h0[u] - o_del - k * e_del);
                return v > 0 ? v : 0;
            }
            return 99;  // DUMMY1 (:45)
        };
        unsigned long long ncells = 0;
        int tnext[LPT];
        for (int u = 0; u < LPT; u++) tnext[u] = len1[u] > 0 ? Aref[idr[u] - ref_lo] : 0;
        int beg = 0, end = ncol, nbeg = 0, nend = ncol;
        for (int i = 0; i < nrow; i++) {
            const int i1 = E::ws(i + 1);
            int h10[LPT], maxRS1[LPT], y1[LPT], s1[LPT];
            unsigned rkey[LPT];  // this warp's chunk: row maximum key
            uint32_t tlo[LPT], thi[LPT];  // the row's score table (bytes by selector)
            beg = nbeg; end = nend;
            if (beg < i - w) beg = i - w;
            if (end > i + w + 1) end = i + w + 1;
            if (end > ncol) end = ncol;
            bool changed = false;
            for (int u = 0; u < LPT; u++) {
                maxRS1[u] = 0; y1[u] = 0; rkey[u] = 0;
                h10[u] = beg == 0 ? Hv(i + 1, u) : 0;
                if (i < len1[u]) {
                    const int b = tnext[u];  // loaded a row ahead
                    if (i + 1 < len1[u]) tnext[u] = Aref[idr[u] - ref_lo + i + 1];
                    s1[u] = b == 4 ? -1 : E::ws(b);
                    if (b > 4) gerr(ERR_BASE, lidx[u]);
                } else {
                    s1[u] = 99;  // DUMMY1
                }
                // score of the row's target code s1 against each query
                // selector, as the kernel's blends compute it (:1883-1906): match
                // or mismatch, -1 where either side is N (negative code)
                {
                    const uint32_t mt = (uint32_t)(uint8_t)w_match, ms = (uint32_t)(uint8_t)w_mismatch;
                    uint32_t lo = 0xffu | (ms << 8) | (ms << 16) | (ms << 24);  // N, bases 0..2
                    uint32_t hi = ms | (ms << 8) | (ms << 16) | (ms << 24);     // base 3, DUMMY2, -
                    if (s1[u] >= 0 && s1[u] <= 2) lo = (lo & ~(0xffu << (8 * (s1[u] + 1)))) | (mt << (8 * (s1[u] + 1)));
                    else if (s1[u] == 3) hi = (hi & ~0xffu) | mt;
                    if (s1[u] < 0) { lo = 0xffffffffu; hi = 0xffffffffu; }
                    tlo[u] = lo;
                    thi[u] = hi;
                }
                // per-lane band (:3080-3089)
                const int ph = head[u], pt = tail[u];
                const int c = E::ws(i - myband[u]);
                head[u] = head[u] > c ? head[u] : c;
                unsigned tu = umin(E::us(tail[u]), E::us(i1 + myband[u]));
                tu = umin(tu, E::us(qlen[u]));
                tail[u] = E::ws((int)tu);
                changed |= head[u] != ph || tail[u] != pt;
            }
            // columns coming within reach: query codes and row-0 entries.  From
            // row 1 on they lie past the band end, and the ring slots they take
            // belong to columns below the previous row's band start, which no
            // row reads or writes again; so none of this races with the trimming
            const int lim = imin(colCap - 1, i + w + 3);
            const bool ini = initc <= lim;
            if (ini) {
                for (int k = initc + ((wp - initc) & (NW - 1)); k <= lim; k += NW) init_col(k);
                initc = lim + 1;
                const int kn = initc + ((wp - initc) & (NW - 1));
                if (kn < colCap && kn != kp) {
                    kp = kn;
                    for (int u = 0; u < LPT; u++) bp[u] = qbyte(kn, u);
                }
            }
            // trimming (:3091-3112): the sequential pass stops at the first
            // column no lane's head is beyond, so it covers [beg, max head)
            const bool trim = __any_sync(full, changed);
            if (trim) {
                if (i == 0) __syncthreads();  // row 0 may trim columns it has just initialised
                int mh = INT_MIN;
                for (int u = 0; u < LPT; u++) mh = imax(mh, head[u]);
                mh = __reduce_max_sync(full, mh);
                const int hi = imin(end, mh);
                for (int lc = beg + wp; lc < hi; lc += NW) {
                    const int pj = E::ws(lc), jn = E::ws(lc + 1);
                    for (int u = 0; u < LPT; u++)
                        if (head[u] > pj || jn > tail[u]) HFa(lc, u) = 0;
                }
            }
            if (ini || trim) __syncthreads();
            // row exit status (:3119-3129)
            bool need_live = false;
            for (int u = 0; u < LPT; u++) {
                if (i1 > mlen[u] || tail[u] == head[u] || head[u] > tail[u]) exit0[u] = 0;
                need_live |= needl[u] && exit0[u] != 0;
            }
            // every needed lane has exited: its outputs are final
            if (!__any_sync(full, need_live)) break;

            // ---- the DP row (:3135-3196): contiguous chunks of the band
            const int n = end > beg ? end - beg : 0;
            const int cs = (n + NW - 1) / NW;
            const int c0 = beg + imin(n, wp * cs), c1 = beg + imin(n, (wp + 1) * cs);
            auto m11_of = [&](uint32_t sel, int u, int h00) -> int {
                const int sbt = (int)(int8_t)(uint8_t)__byte_perm(tlo[u], thi[u], sel);
                const int m11 = E::ws(h00 + sbt);
                return h00 == 0 ? 0 : m11;
            };
            // pass 1: E over the chunk from 0 (the next column's word and code
            // loaded one column ahead)
            if (c1 > c0) {
                for (int u = 0; u < LPT; u++) {
                    int el = 0;
                    int bi = slot(c0) * W + t + 32 * u;  // element of (column j, lane)
                    uint32_t hfn = HF[bi];
                    uint32_t an = Q2[bi];
                    for (int j = c0; j < c1; j++) {
                        const uint32_t hf = hfn;
                        const uint32_t a2 = an;
                        bi += W;
                        if (ring && bi >= WR * W) bi -= WR * W;
                        if (j + 1 < c1) {
                            hfn = HF[bi];
                            an = Q2[bi];
                        }
                        const int h00 = (int16_t)(hf & 0xffffu), f11 = (int16_t)(hf >> 16);
                        const int m11 = m11_of(a2, u, h00);
                        if (j == c1 - 1) {
                            X.Elast[wp][t + 32 * u] = el;
                            X.MF[wp][t + 32 * u] = imax(m11, f11);
                        }
                        // E >= 0 throughout, so E - e_ins cannot wrap
                        el = __vimax3_s32(E::ws(m11 - oe_ins), 0, el - e_ins);
                    }
                    X.Aagg[wp][t + 32 * u] = el;
                }
            }
            __syncthreads();
            // pass 2: the chunk from its true entering E and H
            int fnz = INT_MAX, lnz = -1;
            if (c1 > c0) {
                int e11[LPT];
                for (int u = 0; u < LPT; u++) {
                    const int l = t + 32 * u;
                    int e = 0, eprev = 0;
                    for (int k = 0; k < wp; k++) {  // chunks before this one are full (cs columns)
                        eprev = e;
                        e = imax(X.Aagg[k][l], e - cs * e_ins);
                    }
                    e11[u] = e;
                    if (wp > 0) {  // H at column c0 - 1: the previous chunk's last column
                        const int el = imax(X.Elast[wp - 1][l], eprev - (cs - 1) * e_ins);
                        h10[u] = imax(X.MF[wp - 1][l], el);
                    }
                }
                uint32_t hfn[LPT], an[LPT];
                int gcol[LPT];  // the query's last column, where gscore is taken (:3178-3195)
                int bj = slot(c0) * W + t;  // element of (column j, lane t)
                for (int u = 0; u < LPT; u++) {
                    hfn[u] = HF[bj + 32 * u];
                    an[u] = Q2[bj + 32 * u];
                    gcol[u] = qlen[u] - 1 >= minq ? qlen[u] - 1 : -1;
                }
                for (int j = c0; j < c1; j++) {
                    // j + 1 <= ncol fits the element width: no wrap
                    const int pj = j;
                    const int jn = j + 1;
                    const int bc = bj;
                    bj += W;
                    if (ring && bj >= WR * W) bj -= WR * W;
                    unsigned nzc = 0;
                    for (int u = 0; u < LPT; u++) {
                        const int l = t + 32 * u;
                        const uint32_t hf = hfn[u];
                        const uint32_t a2 = an[u];
                        if (j + 1 < c1) {  // next column's inputs (never this column's store)
                            hfn[u] = HF[bj + 32 * u];
                            an[u] = Q2[bj + 32 * u];
                        }
                        const int h00 = (int16_t)(hf & 0xffffu), f11 = (int16_t)(hf >> 16);
                        const int m11 = m11_of(a2, u, h00);
                        const int h11 = __vimax3_s32(m11, e11[u], f11);
                        // E and F are >= 0 throughout: E - e_ins, F - e_del cannot wrap
                        e11[u] = __vimax3_s32(E::ws(m11 - oe_ins), 0, e11[u] - e_ins);
                        int f21 = __vimax3_s32(E::ws(m11 - oe_del), 0, f11 - e_del);
                        const bool cmp2 = head[u] > pj;
                        const bool mask = pj > tail[u] || cmp2;
                        const int hst = mask ? 0 : h10[u];
                        if (mask) f21 = 0;
                        // the row maximum and the last column attaining it, as one key
                        // (h11 >= 0 and jn < 2^16: the larger key is the later column of
                        // a tie, as the sequential walk's >= keeps)
                        const unsigned kc = ((unsigned)h11 << 16) | (unsigned)jn;
                        if (!(jn > tail[u] || cmp2)) rkey[u] = kc > rkey[u] ? kc : rkey[u];
                        const uint32_t word = pack(hst, f21);
                        HF[bc + 32 * u] = word;
                        const unsigned m = __ballot_sync(full, word != 0u);
                        if (t == 0) NZ[(size_t)j * LPT + u] = m;
                        nzc |= m;
                        h10[u] = h11;
                        // end-to-end score (:3178-3195), in the query's last column
                        if (j == gcol[u] && exit0[u] < 0 && !(jn > tail[u]) && !(X.gscore[l] > h11)) {
                            X.gscore[l] = h11;
                            X.max_ie[l] = i1;
                        }
                    }
                    if (nzc) {
                        if (fnz == INT_MAX) fnz = j;
                        lnz = j;
                    }
                }
            }
            for (int u = 0; u < LPT; u++)
                X.key[wp][t + 32 * u] = rkey[u];
            if (t == 0) {
                X.nzF[wp] = fnz;
                X.nzL[wp] = lnz;
            }
            // the row's last column (:3197-3203), by the warp holding column end - 1
            const int lw = n > 0 ? (n - 1) / cs : 0;
            if (wp == lw) {
                const int j = beg > end ? beg : end;
                const int j512 = E::ws(j);
                unsigned nzc = 0;
                if (j < colCap) {
                    for (int u = 0; u < LPT; u++) {
                        const bool m = head[u] > j512 || j512 > tail[u];
                        const uint32_t word = pack(m ? 0 : h10[u], 0);
                        HFa(j, u) = word;
                        const unsigned b = __ballot_sync(full, word != 0u);
                        if (t == 0) NZ[(size_t)j * LPT + u] = b;
                        nzc |= b;
                    }
                }
                // column end (== j when end >= beg) after the row, for the narrowing
                if (t == 0) X.endnz = end >= beg && nzc != 0;
            }
            ncells += (unsigned long long)n;
            __syncthreads();

            // row maximum of each lane over the chunks
            for (int u = 0; u < LPT; u++) {
                unsigned kk = 0;
                for (int k = 0; k < NW; k++) {
                    const unsigned v = X.key[k][t + 32 * u];
                    kk = v > kk ? v : kk;
                }
                maxRS1[u] = (int)(kk >> 16);
                y1[u] = (int)(kk & 0xffffu);
            }
            // a zero row in every lane ends the group (:3206-3209)
            bool nzr = false;
            for (int u = 0; u < LPT; u++) nzr |= maxRS1[u] != 0;
            if (!__any_sync(full, nzr)) break;
            for (int u = 0; u < LPT; u++) {
                if (maxRS1[u] == 0) exit0[u] = 0;
                const int bms = maxScore[u];
                const int sc2 = maxScore[u] > maxRS1[u] ? maxScore[u] : maxRS1[u];
                if (exit0[u] < 0) maxScore[u] = sc2;
                if (maxScore[u] > bms) {
                    y[u] = y1[u];
                    x[u] = i1;
                    int ind = E::ws(y1[u] - i1);
                    ind = ind < 0 ? E::ws(-ind) : ind;  // abs (wrapping)
                    max_off[u] = max_off[u] > ind ? max_off[u] : ind;
                }
                // ZSCORE16 / ZSCORE8 (:1868-1881 / :1826-1839)
                const int tmpi = E::ws(i1 - x[u]), tmpj = E::ws(y1[u] - y[u]);
                const int score = E::ws(maxScore[u] - maxRS1[u]);
                const int d = tmpi > tmpj ? E::ws(tmpi - tmpj) : E::ws(tmpj - tmpi);
                if (E::ws(score - d) > zdropv) exit0[u] = 0;
            }
            // band narrowing (:3235-3260): the leading all-zero columns from
            // beg and the last non-zero column at or below end
            {
                int F = INT_MAX, L = -1;
                for (int k = 0; k < NW; k++) {
                    F = imin(F, X.nzF[k]);
                    L = imax(L, X.nzL[k]);
                }
                if (end > beg) {
                    const int f = imin(F, end);
                    if (f > beg) nbeg = f - 1;
                }
                int lc;
                if (end < beg) lc = end;
                else if (X.endnz) lc = end;
                else lc = L >= beg ? L : beg - 1;
                nend = lc + 2 < ncol ? lc + 2 : ncol;
            }
            if (is16) { beg = nbeg; end = nend; }
            // per-lane head / tail (:3265-3316 / :2571-2621): each warp scans a
            // part of the range on the columns' masks and stops where no live
            // lane is zero
            {
                const int B = beg, Ee = end;
                unsigned liveM[LPT];  // lanes still live (a zero there counts)
                for (int u = 0; u < LPT; u++) liveM[u] = __ballot_sync(full, exit0[u] != 0);
                const int mh = Ee > B ? Ee - B : 0;
                const int ch = (mh + NW - 1) / NW;
                const int p0 = B + imin(mh, wp * ch), p1 = B + imin(mh, (wp + 1) * ch);
                // 32 columns per step, thread t holding column cb + t (head scan)
                // or ct - t (tail scan, downwards): a ballot gives the columns
                // where no live lane is zero, and a bit transpose gives each
                // lane (thread) the columns where it is not a live zero
                int Zk = INT_MAX, Rk[LPT];
                for (int u = 0; u < LPT; u++) Rk[u] = INT_MAX;
                for (int cb = p0; cb < p1; cb += 32) {
                    const int c = cb + t;
                    const bool inr = c < p1;
                    unsigned zlive = 0;
                    unsigned ok[LPT];  // lanes that are not a live zero at column c
                    for (int u = 0; u < LPT; u++) {
                        const unsigned nz = inr ? NZ[(size_t)c * LPT + u] : 0u;
                        zlive |= liveM[u] & ~nz;
                        ok[u] = inr ? (~liveM[u] | nz) : 0u;
                    }
                    const unsigned zc = __ballot_sync(full, inr && zlive == 0u);
                    for (int u = 0; u < LPT; u++) {
                        const unsigned x = transpose32(ok[u], t);
                        if (Rk[u] == INT_MAX && x) Rk[u] = cb + __ffs(x) - 1;
                    }
                    if (zc) { Zk = cb + __ffs(zc) - 1; break; }
                }
                const int mt = Ee >= B ? Ee - B + 1 : 0;  // the tail scan includes column Ee
                const int ct = (mt + NW - 1) / NW;
                const int q0 = Ee - imin(mt, wp * ct), q1 = Ee - imin(mt, (wp + 1) * ct);
                int Zrk = INT_MIN, Qk[LPT];
                for (int u = 0; u < LPT; u++) Qk[u] = INT_MIN;
                for (int cb = q0; cb > q1; cb -= 32) {
                    const int c = cb - t;
                    const bool inr = c > q1;
                    unsigned zlive = 0;
                    unsigned ok[LPT];
                    for (int u = 0; u < LPT; u++) {
                        const unsigned nz = inr ? NZ[(size_t)c * LPT + u] : 0u;
                        zlive |= liveM[u] & ~nz;
                        ok[u] = inr ? (~liveM[u] | nz) : 0u;
                    }
                    const unsigned zc = __ballot_sync(full, inr && zlive == 0u);
                    for (int u = 0; u < LPT; u++) {
                        const unsigned x = transpose32(ok[u], t);
                        if (Qk[u] == INT_MIN && x) Qk[u] = cb - (__ffs(x) - 1);
                    }
                    if (zc) { Zrk = cb - (__ffs(zc) - 1); break; }
                }
                for (int u = 0; u < LPT; u++) {
                    X.R[wp][t + 32 * u] = Rk[u];
                    X.Q[wp][t + 32 * u] = Qk[u];
                }
                if (t == 0) {
                    X.Z[wp] = Zk;
                    X.Zr[wp] = Zrk;
                }
                __syncthreads();
                int Z = Ee, Zr = B - 1;
                for (int k = 0; k < NW; k++) {
                    Z = imin(Z, X.Z[k]);
                    Zr = imax(Zr, X.Zr[k]);
                }
                for (int u = 0; u < LPT; u++) {
                    int R = Ee, Q = B - 1;
                    for (int k = 0; k < NW; k++) {
                        R = imin(R, X.R[k][t + 32 * u]);
                        Q = imax(Q, X.Q[k][t + 32 * u]);
                    }
                    // the head: the last column of the lane's leading zero run, up to the scan's stop
                    const int hm = imin(R, Z);
                    if (hm > B) head[u] = E::ws(hm);
                    // the tail: from the top, the same
                    int index = tail[u];
                    const int tm = imax(Q, Zr);
                    if (tm < Ee) index = E::ws(tm);
                    const int ix = E::ws(index + 2);
                    tail[u] = ix < qlen[u] ? ix : qlen[u];
                }
            }
        }
        if (wp == 0) {
            for (int u = 0; u < LPT; u++) {
                if (!needl[u]) continue;
                const int l = t + 32 * u;
                DevPair &p = *pp[u];
                p.score = maxScore[u];
                p.tle = x[u];
                p.qle = y[u];
                p.max_off = max_off[u];
                p.gscore = X.gscore[l];
                p.gtle = X.max_ie[l];
            }
            if (A.cells) {
                int nr = 0;
                for (int u = 0; u < LPT; u++) nr += real[u];
                const int nreal = __reduce_add_sync(full, nr);
                if (t == 0) atomicAdd(A.cells, ncells * (unsigned long long)nreal);
            }
        }
    }
}

template <int SB>
__global__ void __launch_bounds__(32 * wide_warps<SB>(), 1) bsw_group_wide_kernel(GroupArgs A) {
    TALBSW_DYNAMIC_SMEM(smem_w);
    group_wide_body<SB, wide_warps<SB>()>(A, smem_w);
}

}  // namespace talbsw
