// Group-coupling detector of the per-pair kernels.
//
// The reference scores its pairs in SIMD groups of 32 (16-bit) / 64 (8-bit)
// consecutive pairs that share one band [beg, end) per row, one trimming
// pass, the ranges of the head / tail re-derivation scans and the width of
// the row-0 initialisation (the group's longest query) -- bandedSWA.cpp
// :2787-2879 and :3053-3316 (16-bit), :2091-2181 and :2355-2621 (8-bit).  A
// pair's outputs almost never depend on the rest of its group; the per-pair
// kernels score each pair alone and run this detector beside it.  A pair is
// flagged unless its outputs provably equal its outputs in ANY group: for
// every value a group can share with the lane, the detector bounds it
//   beg' in [i - w, beg], end' in [end, i + w + 1], scans from any
//   nbeg' <= nbeg to any nend' <= end' + 2, row-0 width up to the element
//   limit,
// and checks that every value in the bound leaves the lane's stored row
// and its outputs unchanged.  The heads and tails the group could hold
// instead of the lane's own are carried as intervals [hlo, hhi] and
// [tlo, thi].  Flagged pairs are re-scored in their groups by the grouped
// kernel (bsw_group.cuh), so every output equals the reference's.
//
// Two facts keep every check O(1) per row:
//  * right of the band, the only non-zero entries are row-0 values beyond
//    the furthest column ever written (maxEnd): the band only shrinks past
//    columns the narrowing found zero, so written columns in (end, maxEnd]
//    are zero, and a row-0 value h0 - o_ins - k*e_ins is positive exactly
//    for 1 <= k < K0;
//  * left of the band a column never changes once frozen, so the lowest and
//    highest frozen non-zero columns (fzMin, fzMax) answer every question
//    the group's extra columns and lagging scans can ask.
// The CPU restatement of the same rules is oracle_bsw_detect
// (oracle/bsw_oracle.cpp); the tests compare the two flag for flag.
#pragma once

// Included by bsw_kernel.cuh after the element-width helpers it uses
// (imin, imax, wrapS, wrapU); not a stand-alone header.

namespace talbsw {

// Flag reasons (bit set); any non-zero flag sends the pair's group to the
// grouped kernel.
enum : int {
    CPL_TRIM = 1,        // the group may trim (or skip trimming) non-zero old entries
    CPL_LEFT = 2,        // columns left of the band the group may compute are not all zero
    CPL_RIGHT = 16,      // the group may compute real cells right of the band
    CPL_STALE = 32,      // the group may zero row-0 values the lane later reads
    CPL_TAILF = 64,      // the group may trim the tail column before its F is stored
    CPL_ENDF = 128,      // the group may store an F the lane does not at its band end
    CPL_RUNEND = 256,    // the head scan ran past the lane's band
    CPL_RUNBOT = 512,    // the tail scan ran below the lane's band
    CPL_EXIT = 4096,     // the exit decision depends on the group's head / tail
    CPL_HEAD = 8192,     // uncertain head over non-zero cells
    CPL_TAIL = 16384,    // uncertain tail
    CPL_RANGE = 1 << 16, // outside the per-pair kernels' exact range (wrapping values)
    CPL_CAP = 1 << 17    // the pair's rows do not fit the per-pair kernels' shared memory
};

struct Couple {
    int hlo, hhi, tlo, thi;  // heads / tails the group could hold
    int fzMin, fzMax;        // lowest / highest frozen non-zero column
    int frozenTo;            // columns below it have been examined as frozen
    int maxEnd;              // furthest column written by a row
    int Fv;                  // bound of the group's F at column len2
    int K0;                  // row-0 values are positive at columns 1 <= k < K0
    int flag;
    bool reached;            // a row has stored at column len2

    __device__ void init(int qlenE, int v1, int e_ins) {
        hlo = hhi = 0;
        tlo = thi = qlenE;
        fzMin = 1 << 30;
        fzMax = -1;
        frozenTo = 0;
        maxEnd = -1;
        Fv = 0;
        K0 = v1 > 0 ? (v1 - 1) / e_ins + 2 : 1;
        flag = 0;
        reached = false;
    }
    // a frozen column c (examined once, in order) was non-zero
    __device__ void frozen_nz(int c) {
        if (c < fzMin) fzMin = c;
        if (c > fzMax) fzMax = c;
    }
    // the band clamp of a row (bandedSWA.cpp:3080-3089) applied to the intervals
    __device__ void clamp(int hc, int c2u, int qlenU, int sh, int msk) {
        hlo = imax(hlo, hc);
        hhi = imax(hhi, hc);
        tlo = wrapS(imin(imin(wrapU(tlo, msk), c2u), qlenU), sh);
        thi = wrapS(imin(imin(wrapU(thi, msk), c2u), qlenU), sh);
    }
    // the checks that need only the row's scalars, before its cells
    // (active: the lane is still scoring this row; h10init: the row's
    // column-(beg - 1) value, hv_next: H_v[i + 1]); cmax = element limit.
    // Straight-line selects: the lanes of a warp hold different pairs.
    __device__ void row_checks(bool was_active, bool mlen_exit, bool active, int i, int w,
                               int beg, int end, int len2, int h10init, int hv_next, int cmax) {
        int f = 0;
        f |= (was_active && !mlen_exit && tlo <= hhi && thi > hlo) ? CPL_EXIT : 0;
        const bool uncH = hlo != hhi;
        f |= (active && tlo != thi) ? CPL_TAIL : 0;
        f |= (active && uncH && (hhi > end || (beg >= hlo && beg < hhi && h10init != 0))) ? CPL_HEAD : 0;
        const int lo = imax(0, i - w);
        const bool left = beg > lo && (fzMax >= lo || (lo == 0 && hlo <= 0 && hv_next != 0));  // H_v[i + 1] at column 0
        f |= (active && left) ? CPL_LEFT : 0;
        const int Emax = imin(i + w + 1, cmax);
        const int c0 = imax(imax(end, tlo), maxEnd) + 1;
        f |= (active && end < Emax && end < thi) ? CPL_RIGHT : 0;
        f |= (active && end < Emax && c0 <= imin(Emax, len2 - 1) && c0 < K0) ? CPL_STALE : 0;
        flag |= f;
    }
    // the range [beg, trim_hi) whose old entries must be zero when the lane
    // does not trim the row or its head is uncertain (empty: beg >= trim_hi)
    __device__ int trim_hi(bool changed, int end, int head) const {
        if (changed && hlo == hhi) return -1;
        return imin(end, imax(head, hhi));
    }
    // F' of a column from its old entries h, f and score s
    __device__ static int fnext(int h, int f, int s, int e_del, int oe_del) {
        const int M = h ? h + s : 0;
        return imax(f - e_del, imax(M - oe_del, 0));
    }
    // the tail column's and the band end's F (old entries, before the row)
    __device__ void f_checks(bool active, int i, int w, int beg, int end, int head,
                                      int tail, int len2, int cmax, bool tail_in_band,
                                      int f_tail, int f_end) {
        if (!active) return;
        const int Emax = imin(i + w + 1, cmax);
        if (tail_in_band && f_tail != 0 && tail < Emax) flag |= CPL_TAILF;
        if (end < Emax && end == tail && head <= end && end < len2 && f_end != 0) flag |= CPL_ENDF;
    }
    // after the row's last-column store at column jl: Hjl = its H, s_dummy =
    // the row's score against the padding code past the query
    __device__ void stored_last(int jl, int len2, int Hjl, int s_dummy, int head, int tail,
                                         int e_del, int oe_del) {
        maxEnd = imax(maxEnd, jl);
        if (jl == len2) {
            reached = true;
            const int nf = fnext(Hjl, Fv, s_dummy, e_del, oe_del);
            Fv = (len2 > tail || head > len2) ? 0 : nf;
        }
    }
    // first column in (a, b] that may be non-zero in a group's view, right of
    // everything this lane wrote; -1 if none
    __device__ int first_right_nz(int a, int b, int len2, int cmax) const {
        const int c0 = imax(a, maxEnd) + 1;
        const int c1 = imax(a, len2) + 1;
        const bool own = c0 <= b && c0 < len2 && c0 < K0;
        const bool atq = len2 > a && len2 <= b && (Fv > 0 || (!reached && len2 < K0));
        const bool past = c1 <= b && c1 < cmax && c1 < K0;
        return own ? c0 : atq ? len2 : past ? c1 : -1;
    }
    // the head / tail scans' results (bandedSWA.cpp:3265-3316): sb / se their
    // ranges, nz_sb / nz_se whether the lane is non-zero there, newhead /
    // index the lane's own results, run_end / run_bot whether its runs
    // reached the range's end; last_row: no row of this lane follows.
    // Straight-line selects, as row_checks.
    __device__ void scans(bool ex, bool last_row, bool is8, int i, int w, int beg, int end,
                          int sb, int se, bool nz_sb, bool nz_se, bool run_end, bool hse_nz,
                          bool run_bot, int newhead, int index, int qlenE, int len2, int cmax) {
        const bool go = ex && !last_row;
        int f = (run_end && !(se <= end && hse_nz)) ? CPL_RUNEND : 0;
        f |= run_bot ? CPL_RUNBOT : 0;
        flag |= go ? f : 0;
        const int lo = imax(0, i - w);
        const int los = is8 ? lo : 0;
        int nhlo = nz_sb ? hlo : newhead, nhhi = nz_sb ? hhi : newhead;
        const int Pl16 = fzMin < sb ? imin(fzMax, sb - 1) : -1;
        const int Pl8 = fzMax >= lo ? fzMax : -1;
        const int Pl = sb > los ? (is8 ? Pl8 : Pl16) : -1;
        const bool c1 = sb > los && nz_sb && Pl < sb - 1;
        nhlo = c1 ? imin(nhlo, sb) : nhlo;
        nhhi = c1 ? imax(nhhi, sb) : nhhi;
        const bool c2 = Pl >= 0;
        nhlo = c2 ? imin(imin(nhlo, hlo), los) : nhlo;
        nhhi = c2 ? imax(imax(nhhi, hhi), Pl) : nhhi;
        const int Emax = imin(i + w + 1, cmax);
        const int Smax = is8 ? Emax : imin(Emax + 2, cmax);
        int rlo = nz_se ? tlo : index, rhi = nz_se ? thi : index;
        const bool c3 = Smax > se;
        const int Qr = c3 ? first_right_nz(imax(se, end), Smax, len2, cmax) : -1;
        const bool c4 = c3 && nz_se;
        rlo = c4 ? imin(rlo, se) : rlo;
        rhi = c4 ? imax(rhi, se) : rhi;
        const bool c5 = Qr >= 0;
        rlo = c5 ? imin(imin(rlo, tlo), Qr) : rlo;
        rhi = c5 ? imax(imax(rhi, thi), Smax - 1) : rhi;
        tlo = go ? imin(rlo + 2, qlenE) : tlo;
        thi = go ? imin(rhi + 2, qlenE) : thi;
        hlo = go ? nhlo : hlo;
        hhi = go ? nhhi : hhi;
    }
    // keeps the lane's own head / tail inside the intervals (after a row)
    __device__ void settle(bool ex, bool last_row, int head, int tail) {
        if (!(ex && !last_row)) { hlo = hhi = head; tlo = thi = tail; }
        if (hlo > head) hlo = head;
        if (hhi < head) hhi = head;
        if (tlo > tail) tlo = tail;
        if (thi < tail) thi = tail;
    }
};

}  // namespace talbsw
