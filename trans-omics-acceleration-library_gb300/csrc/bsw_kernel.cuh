// Banded Smith-Waterman seed extension on sm_103a: G lanes per pair (32/G
// pairs per warp), row-synchronous, each lane owning K consecutive columns of
// a G*K-column strip of the current row.
//
// Semantics: the reference's getScores16 / getScores8 kernels
// (src/alignment/BSW/bandedSWA.cpp:2962-3356 / :2263-2661) for a pair scored on
// its own, as if alone in its SIMD group.  The reference's outputs almost
// never depend on which other pairs share the group (equal on every workload
// shape checked; the rare exceptions, narrow bands next to the group's, are
// scored exactly by the grouped kernel in bsw_group.cuh), so a pair is the
// unit of work here and the per-lane head/tail bookkeeping of the vector code
// collapses to per-pair scalars held uniformly by the pair's G lanes.
// Several pairs share a warp so that this per-row bookkeeping (band edges,
// narrowing, z-drop) is paid once per warp-instruction for 32/G pairs; each
// group takes its next pair from the work counter as soon as it finishes.
//
// Per row i the reference computes, over its band [beg, end):
//   M(j)   = H(i-1,j-1) ? H(i-1,j-1) + S(i,j) : 0
//   H(j)   = max(M(j), E(j), F(j))
//   E(j+1) = max(E(j) - e_ins, max(M(j) - oe_ins, 0))      (horizontal, E(beg)=0)
//   F'(j)  = max(F(j) - e_del, max(M(j) - oe_del, 0))      (vertical, next row)
// E does not depend on H, so it is a max-plus prefix scan of
// T(k) = max(M(k) - oe_ins, 0):  E(j) = max_{beg<=k<j} T(k) - e_ins*(j-1-k),
// computed as a plain prefix max of P(k) = T(k) + e_ins*(k-beg): first within
// a lane's K columns, then across the warp with shuffles, then carried from
// strip to strip.  Everything else in a row is elementwise or a warp
// reduction, so a whole strip is one pass with no serial dependency.
//
// The row buffers live in shared memory, one per warp, exactly as the
// reference's scratch rows H_h[j] and F[j] (int32 each); columns outside the
// computed band keep their old ("stale") values, which the reference's
// narrowing reads.
//
// A row is cut into strips of G*K columns, each lane owning K consecutive
// columns.  All collectives (shuffles, ballots) run with the full warp mask in
// warp-uniform loops; a group with nothing to do in an iteration is masked by
// predicates, never by divergence around a collective.
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

// The per-block dynamic shared memory; a host build of this file for the
// CPU emulator in the tests defines the macro to a plain pointer first.
#ifndef TALBSW_DYNAMIC_SMEM
#define TALBSW_DYNAMIC_SMEM(name) extern __shared__ __align__(16) unsigned char name[]
#endif

namespace talbsw {

struct KernelParams {
    int o_del, e_del, o_ins, e_ins, zdrop, end_bonus, a, b;
};

struct DevPair {  // SeqPair, bandedSWA.h:90-99
    int32_t idr, idq, id, len1, len2, h0, seqid, regid;
    int32_t score, tle, gtle, qle, gscore, max_off;
};

// error word layout: bit 0 = domain error seen; the first offending pair
// index is recorded separately with atomicMin.
enum : int { ERR_DOMAIN = 1, ERR_CAPACITY = 2, ERR_BASE = 4, ERR_FLAGCAP = 8 };

// One request of a serving tick: the tick's pairs are the concatenation of
// its requests' pair arrays, each request with its own sequence buffers,
// band and precision.  Pair `first + k` of the tick is pair k of the request.
// The kernels record errors per request here (err, bad), so that one
// request's bad pair does not fail the others.
struct ReqDesc {
    DevPair *pairs;
    const uint8_t *ref;
    const uint8_t *qer;
    const int32_t *wpair;     // optional per-pair band
    long long ref_lo, ref_hi, qer_lo, qer_hi;
    long long bad;            // first offending pair, request-local (LLONG_MAX if none)
    int first, n, w, bits;
    int err;                  // ERR_* flags
    int pad_;
};

struct LaunchArgs {
    DevPair *pairs;
    // ref / qer point at a device copy of the caller's buffer window
    // [*_lo, *_hi): byte `off` of the caller's buffer is ref[off - ref_lo].
    const uint8_t *ref;
    const uint8_t *qer;
    long long ref_lo, ref_hi, qer_lo, qer_hi;
    const int32_t *order;    // optional permutation (batched form)
    const int32_t *seg;      // optional {offset, count} pairs into order (overrides n):
    int nseg;                // the launch takes the nseg (>= 1) consecutive segments there
    const int32_t *wpair;    // optional per-pair band
    int32_t n;
    int32_t w;
    int bits;                // 8, 16 or 0 = per-pair routing
    int cols_cap, rows_cap;  // shared-memory row capacity per pair
    int win;                 // lane kernel: ring of win columns per pair (0: whole rows)
    int *work_counter;       // next work item (dynamic scheduling)
    unsigned long long *cells;  // optional: total DP cells computed
    int *err_flags;
    long long *err_index;
    KernelParams P;
    // serving tick: when reqs is set, order[] holds request-local pair
    // indices and order_req[] (parallel to order) the request of each;
    // pairs / ref / qer / wpair / w / bits above are unused
    ReqDesc *reqs;
    const int32_t *order_req;
    // group-coupling detector (bsw_couple.cuh): when `flagged` is set, the
    // kernels flag every pair whose outputs may depend on its SIMD group (or
    // that lies outside their exact range but inside the grouped kernel's),
    // append it as ((request + 1) << 32) | pair to flagged[0, flag_cap) and
    // leave its outputs to the grouped re-scoring; when it is not set, such
    // pairs are scored alone (or refused, outside the range)
    long long *flagged = nullptr;
    int *nflagged = nullptr;
    int flag_cap = 0;
    int flag_base = 0;  // added to a flagged pair's index (a chunk of a larger call)
};

// Appends a flagged pair to the launch's list.
__device__ __forceinline__ void flag_pair(const LaunchArgs &A, int req, int pidx) {
    const int k = atomicAdd(A.nflagged, 1);
    if (k < A.flag_cap) A.flagged[k] = ((long long)(req + 1) << 32) | (unsigned)(pidx + A.flag_base);
    else atomicOr(A.err_flags, ERR_FLAGCAP);
}

// Is the pair inside the grouped kernel's range (the reference's own limits:
// lengths up to the element type's, h0 >= 0; any gap weights)?
__device__ __forceinline__ bool pair_in_group_range(int len1, int len2, int h0, int w, bool is8) {
    const int lim = is8 ? 127 : 32767;
    return len1 >= 0 && len2 >= 0 && len1 <= lim && len2 <= lim && h0 >= 0 && w >= 0;
}

// Where one pair's record, sequences, band and precision live.
struct PairSrc {
    DevPair *pp;
    const uint8_t *ref, *qer;
    long long ref_lo, ref_hi, qer_lo, qer_hi;
    int w, bits;
};

// item: position in the (optionally sorted) work list; pidx: the pair's
// index (request-local for a serving tick); req: its request or -1.
__device__ __forceinline__ PairSrc pair_src(const LaunchArgs &A, int pidx, int req) {
    PairSrc s;
    if (req >= 0) {
        const ReqDesc &d = A.reqs[req];
        s.pp = d.pairs + pidx;
        s.ref = d.ref; s.qer = d.qer;
        s.ref_lo = d.ref_lo; s.ref_hi = d.ref_hi; s.qer_lo = d.qer_lo; s.qer_hi = d.qer_hi;
        s.w = d.wpair ? d.wpair[pidx] : d.w;
        s.bits = d.bits;
    } else {
        s.pp = A.pairs + pidx;
        s.ref = A.ref; s.qer = A.qer;
        s.ref_lo = A.ref_lo; s.ref_hi = A.ref_hi; s.qer_lo = A.qer_lo; s.qer_hi = A.qer_hi;
        s.w = A.wpair ? A.wpair[pidx] : A.w;
        s.bits = A.bits;
    }
    return s;
}

// Work items of a launch: the consecutive segments seg[0 .. nseg) of the
// sorted order, or items 0..n of the launch's pairs.
__device__ __forceinline__ int work_count(const LaunchArgs &A) {
    if (!A.seg) return A.n;
    const int last = A.nseg > 1 ? A.nseg - 1 : 0;
    return A.seg[2 * last] + A.seg[2 * last + 1] - A.seg[0];
}

// Records an error for pair pidx (of request req, or of the launch).
__device__ __forceinline__ void report_error(const LaunchArgs &A, int req, int flag, int pidx) {
    atomicOr(A.err_flags, flag);
    if (req >= 0) {
        atomicOr(&A.reqs[req].err, flag);
        atomicMin(&A.reqs[req].bad, (long long)pidx);
    } else {
        atomicMin(A.err_index, (long long)pidx);
    }
}

// Element-width wrap of the reference's per-row int16 / int8 arithmetic,
// emulated exactly: sh = 16 (int16) or 24 (int8), msk = 0xffff or 0xff.
__device__ __forceinline__ int wrapS(int x, int sh) { return (int)((unsigned)x << sh) >> sh; }
__device__ __forceinline__ int wrapU(int x, int msk) { return x & msk; }

__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }
__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }

// Can this pair be scored exactly with the 8-bit (is8) or 16-bit rules?
// The per-cell arithmetic runs in int32, which equals the reference's
// wrapping int8/int16 arithmetic as long as no DP value leaves the element
// range; these are the conditions for that.
__device__ __forceinline__ bool pair_in_range(const KernelParams &P, int len1, int len2,
                                              int h0, int w, bool is8) {
    const int lim = is8 ? 127 : 32767;
    if (len1 < 0 || len2 < 0 || len1 > lim || len2 > lim || h0 < 0) return false;
    long long top = (long long)h0 + (long long)P.a * (long long)imin(len1, len2);
    if (top > lim) return false;
    const int lo = is8 ? -128 : -32768;
    // gap scores: M - oe >= element minimum, M >= 1 - max(b, 1)
    const int oe = imax(P.o_del + P.e_del, P.o_ins + P.e_ins);
    if (is8 && oe > 127) return false;
    if (1 - imax(P.b, 1) - oe < lo) return false;
    // first column H_v[k] = max(h0 - o_del - k*e_del, 0) must not wrap where
    // it is read (k <= w + 1, k < len1)
    long long kmax = (long long)imin(len1 - 1, (w < 0 ? 0 : w) + 1);
    if (kmax >= 1) {
        long long v = (long long)h0 - P.o_del - kmax * (long long)P.e_del;
        if (v < lo) return false;
    }
    return true;
}

template <int K>
struct VecIO;
template <>
struct VecIO<1> {
    __device__ static void ld(const int *p, int (&v)[1]) { v[0] = p[0]; }
    __device__ static void st(int *p, const int (&v)[1]) { p[0] = v[0]; }
    __device__ static void ldq(const uint16_t *q, uint32_t (&v)[1]) { v[0] = q[0]; }
};
template <>
struct VecIO<2> {
    __device__ static void ld(const int *p, int (&v)[2]) {
        int2 t = *reinterpret_cast<const int2 *>(p);
        v[0] = t.x; v[1] = t.y;
    }
    __device__ static void st(int *p, const int (&v)[2]) {
        *reinterpret_cast<int2 *>(p) = make_int2(v[0], v[1]);
    }
    __device__ static void ldq(const uint16_t *q, uint32_t (&v)[2]) {
        uint32_t w = *reinterpret_cast<const uint32_t *>(q);
        v[0] = w; v[1] = w >> 16;   // PRMT reads only the low 16 bits of a selector
    }
};
template <>
struct VecIO<4> {
    __device__ static void ld(const int *p, int (&v)[4]) {
        int4 t = *reinterpret_cast<const int4 *>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    __device__ static void st(int *p, const int (&v)[4]) {
        *reinterpret_cast<int4 *>(p) = make_int4(v[0], v[1], v[2], v[3]);
    }
    __device__ static void ldq(const uint16_t *q, uint32_t (&v)[4]) {
        uint2 w = *reinterpret_cast<const uint2 *>(q);
        v[0] = w.x; v[1] = w.x >> 16; v[2] = w.y; v[3] = w.y >> 16;
    }
};

constexpr int KPAD = 4;  // widest strip's columns per lane: row padding

// Shared-memory footprint of one pair's rows, in bytes (16-byte aligned parts):
// H_h and F (int32 each) and the query as 16-bit byte-permute selectors, for
// whole rows of cols_cap columns or -- win > 0 -- rings of win columns (a
// power of two; column j in slot j & (win - 1)).  The target is read from
// global memory, one base per row.
__host__ __device__ __forceinline__ size_t smem_hh_bytes(int cols_cap, int win = 0) {
    if (win > 0) return (size_t)win * 4;
    return ((size_t)(cols_cap + 2 + KPAD) * 4 + 15) & ~(size_t)15;
}
__host__ __device__ __forceinline__ size_t smem_q_bytes(int cols_cap, int win = 0) {
    if (win > 0) return (size_t)win * 2;
    return ((size_t)(cols_cap + KPAD + 8) * 2 + 15) & ~(size_t)15;
}
__host__ __device__ __forceinline__ size_t pair_smem_bytes(int cols_cap, int rows_cap, int win = 0) {
    (void)rows_cap;
    return 2 * smem_hh_bytes(cols_cap, win) + smem_q_bytes(cols_cap, win);
}
// one warp = 32/G pairs
__host__ __device__ __forceinline__ size_t warp_smem_bytes(int cols_cap, int rows_cap, int G,
                                                           int win = 0) {
    return (size_t)(32 / G) * pair_smem_bytes(cols_cap, rows_cap, win);
}

constexpr int NEG = -(1 << 29);  // "minus infinity" for the E scan, no overflow

// Byte permute with the PTX sign-replicate bit honoured: selector nibble
// 8|q copies the sign of source byte q.  A query code q is stored as the
// selector q*0x1111 + 0x8880, so the result is the score byte q of the row's
// table, sign-extended to 32 bits.
__device__ __forceinline__ int prmt_sext(uint32_t lo, uint32_t hi, uint32_t sel) {
#if defined(__CUDA_ARCH__)
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(lo), "r"(hi), "r"(sel));
    return (int)r;
#else
    const uint64_t v = ((uint64_t)hi << 32) | lo;
    uint32_t r = 0;
    for (int n = 0; n < 4; n++) {
        const uint32_t c = (sel >> (4 * n)) & 0xfu;
        uint32_t b = (uint32_t)(v >> (8 * (c & 7u))) & 0xffu;
        if (c & 8u) b = (b & 0x80u) ? 0xffu : 0u;
        r |= b << (8 * n);
    }
    return (int)r;
#endif
}

// (hi16 of the result) = h, (lo16) = k: h << 16 | k for 0 <= h, k < 65536.
__device__ __forceinline__ uint32_t pack_key(int h, uint32_t k) {
    return __byte_perm(k, (uint32_t)h, 0x5410u);
}

// Constants of the cell recurrence.  The gap parameters are at most 127 and
// o + e fits every pair routed to the 8-bit rules, so they need no wrap.
struct CellConsts {
    int e_ins, e_del, oe_del;
    int ke[4];    // k * e_ins
    int keoe[4];  // k * e_ins - oe_ins
    int ce[4];    // -(k - 1) * e_ins
    uint32_t kp1[4];  // k + 1
};

// Per-row state of one pair, shared by the strips of the row.
struct RowState {
    int beg, end, head, tail;
    uint32_t tlo, thi;  // score table of the row's target base (signed bytes)
    int carryP;         // max over columns left of the strip of P (units of (j - beg))
    int hprev;          // H of the column left of the strip
    int h10init;        // H(i, beg - 1): first-column value or 0
    uint32_t key;       // lane's max of (H << 16) | (j + 1) over valid columns
    int hlast;          // H(i, end - 1), held by the lane that owns the column
};

// Strip kinds, chosen warp-uniformly (the most general any pair needs):
// interior strips lie inside [beg, end) and the head/tail window, edge strips
// cross beg or end, masked strips also cross the head/tail window.
enum { STRIP_INTERIOR = 0, STRIP_EDGE = 1, STRIP_MASKED = 2 };

// One strip of a pair's row: columns [base, base + G*K), lane gl owning
// [base + gl*K, +K).  `act` false: the pair has no strip here (no effects).
template <int G, int K, int MODE>
__device__ __forceinline__ void do_strip(const int base, const bool act, const int gl,
                                         RowState &r, const CellConsts &c, int *Hh, int *Fv,
                                         const uint16_t *Qs, const int wm) {
    const unsigned full = 0xffffffffu;
    const int j0 = base + gl * K;
    const int s0 = j0 & wm;  // K-aligned, so the lane's K columns are contiguous slots
    int hv[K], fv[K];
    uint32_t qs[K];
    const bool ld = act && (MODE == STRIP_INTERIOR || j0 < r.end);
    if (ld) {
        VecIO<K>::ld(Hh + s0, hv);
        VecIO<K>::ld(Fv + s0, fv);
        VecIO<K>::ldq(Qs + s0, qs);
    } else {
#pragma unroll
        for (int k = 0; k < K; k++) { hv[k] = 0; fv[k] = 0; qs[k] = 0x8880u; }
    }
    const int lo = r.beg - j0;  // columns k < lo lie left of the band
    const int hi = r.end - j0;  // columns k >= hi lie right of it
    // pass 1: M and the lane-local prefix of P'(k) = max(M - oe_ins, 0) + k*e_ins
    int mm[K], lp[K];
    int run = NEG;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int sb = prmt_sext(r.tlo, r.thi, qs[k]);               // S(t, q)
        mm[k] = __viaddmin_s32(hv[k], sb, hv[k] << 12);              // h00 ? h00 + S : <= 0
        int p = __viaddmax_s32(mm[k], c.keoe[k], c.ke[k]);
        if (MODE != STRIP_INTERIOR && k < lo) p = NEG;
        run = imax(run, p);
        lp[k] = run;
    }
    // scan of the lane summaries across the pair's G lanes (units of (j - beg))
    const int off = c.e_ins * (j0 - r.beg);
    int incl = lp[K - 1] + off;
#pragma unroll
    for (int d = 1; d < G; d <<= 1) incl = imax(incl, __shfl_up_sync(full, incl, d, G));
    int excl = __shfl_up_sync(full, incl, 1, G);
    excl = (gl == 0) ? r.carryP : imax(excl, r.carryP);
    const int ctot = __shfl_sync(full, incl, G - 1, G);
    if (act) r.carryP = imax(r.carryP, ctot);
    const int X = excl - off;
    // pass 2: E and H
    int H[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int R = (k == 0) ? X : imax(X, lp[k - 1]);
        H[k] = __vimax3_s32(mm[k], R + c.ce[k], fv[k]);
    }
    int hl = __shfl_up_sync(full, H[K - 1], 1, G);
    if (gl == 0) hl = r.hprev;
    const int hnext = __shfl_sync(full, H[K - 1], G - 1, G);
    if (act) r.hprev = hnext;   // a pair with no strip here keeps its last H
    // pass 3: stores and the row maximum
    int ho[K], fo[K];
    uint32_t lkey = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
        int hst = (k == 0) ? hl : H[k - 1];
        int f2 = __viaddmax_s32_relu(fv[k], -c.e_del, mm[k] - c.oe_del);
        uint32_t kk = pack_key(H[k], c.kp1[k]);
        if (MODE != STRIP_INTERIOR) {
            const bool in = k >= lo && k < hi;
            if (k == lo) hst = r.h10init;
            bool valid = in;
            if (MODE == STRIP_MASKED) {
                const int j = j0 + k;
                if (j < r.head || j > r.tail) { hst = 0; f2 = 0; }
                valid = in && j >= r.head && j < r.tail;
            }
            if (!valid) kk = 0;
            if (k == hi - 1) r.hlast = H[k];
        }
        ho[k] = hst;
        fo[k] = f2;
        lkey = kk > lkey ? kk : lkey;
    }
    if (act) {
        if (lkey) lkey += (uint32_t)j0;
        r.key = lkey > r.key ? lkey : r.key;
    }
    if (ld) {
        if (MODE == STRIP_INTERIOR || (lo <= 0 && hi >= K)) {
            VecIO<K>::st(Hh + s0, ho);
            VecIO<K>::st(Fv + s0, fo);
        } else {
#pragma unroll
            for (int k = 0; k < K; k++) {
                if (k >= lo && k < hi) {
                    Hh[s0 + k] = ho[k];
                    Fv[s0 + k] = fo[k];
                }
            }
        }
    }
}

// Max over a pair's G lanes.
template <int G>
__device__ __forceinline__ unsigned group_max(unsigned v) {
    if constexpr (G == 32) {
        return __reduce_max_sync(0xffffffffu, v);
    } else {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            unsigned t = __shfl_xor_sync(0xffffffffu, v, o, G);
            v = t > v ? t : v;
        }
        return v;
    }
}

// First column of [lo, hi) with H_h | F non-zero, scanning up; hi if none.
// Warp-uniform loop; each pair searches with its own G lanes.
template <int G>
__device__ __forceinline__ int scan_first_nz(const int *Hh, const int *Fv, int lo, int hi,
                                             bool act, int gl, int gshift, unsigned gbits, int wm) {
    int found = hi;
    bool srch = act && lo < hi;
    int b = lo;
    while (__any_sync(0xffffffffu, srch)) {
        const int j = b + gl;
        const bool nz = srch && j < hi && ((Hh[j & wm] | Fv[j & wm]) != 0);
        const unsigned m = (__ballot_sync(0xffffffffu, nz) & gbits) >> gshift;
        if (srch) {
            if (m) { found = b + __ffs(m) - 1; srch = false; }
            else { b += G; if (b >= hi) srch = false; }
        }
    }
    return found;
}
// Last column of [lo, hi] with H_h | F non-zero, scanning down; lo-1 if none.
template <int G>
__device__ __forceinline__ int scan_last_nz(const int *Hh, const int *Fv, int lo, int hi,
                                            bool act, int gl, int gshift, unsigned gbits, int wm) {
    int found = lo - 1;
    bool srch = act && hi >= lo;
    int t = hi;
    while (__any_sync(0xffffffffu, srch)) {
        const int j = t - gl;
        const bool nz = srch && j >= lo && ((Hh[j & wm] | Fv[j & wm]) != 0);
        const unsigned m = (__ballot_sync(0xffffffffu, nz) & gbits) >> gshift;
        if (srch) {
            if (m) { found = t - (__ffs(m) - 1); srch = false; }
            else { t -= G; if (t < lo) srch = false; }
        }
    }
    return found;
}

}  // namespace talbsw

#include "bsw_couple.cuh"

namespace talbsw {

// One pass over [a, c) for the coupling detector: the lowest and highest
// non-zero column of [a, b) (columns freezing this row) and whether [b, c)
// (old entries a group may trim) holds a non-zero.  Warp-uniform loop; each
// pair searches with its own G lanes, G columns per ballot.
template <int G>
__device__ __forceinline__ void scan_frozen_trim(const int *Hh, const int *Fv, int a, int b, int c,
                                                 bool act, int gl, int gshift, unsigned gbits, int wm,
                                                 int &fmin, int &fmax, bool &tnz) {
    fmin = 1 << 30;
    fmax = -1;
    tnz = false;
    bool srch = act && a < c;
    int base = a;
    while (__any_sync(0xffffffffu, srch)) {
        const int j = base + gl;
        const bool nz = srch && j < c && ((Hh[j & wm] | Fv[j & wm]) != 0);
        const unsigned m = (__ballot_sync(0xffffffffu, nz) & gbits) >> gshift;  // bit k: column base + k
        if (srch) {
            const int nf = imin(imax(b - base, 0), G);  // frozen columns in this window
            const unsigned lowm = nf >= 32 ? 0xffffffffu : ((1u << nf) - 1u);
            const unsigned fm = m & lowm;
            if (fm) {
                fmin = imin(fmin, base + __ffs(fm) - 1);
                fmax = imax(fmax, base + 31 - __clz(fm));
            }
            if (m & ~lowm) tnz = true;
            base += G;
            if (base >= c) srch = false;
        }
    }
}

// Per-pair state, uniform across the pair's G lanes.
struct PairState {
    DevPair *pp;
    const uint8_t *Qg;   // the query in global memory (staged lazily)
    int pidx, req, nrow, ncol, i;
    int initc, v1;       // next column to initialise; its row-0 value base
    int fend, p;         // frozen columns [nbeg, fend) seen; p: first nonzero of them, or -1
    int beg, end, nbeg, nend, head, tail;
    int maxScore, x, y, gscore, max_ie, max_off;
    int h0e, o_delE, e_delE, bandE, wk, qlenE, mlen, zdropE;
    int sh, msk;  // element width: wrap shift and unsigned mask
    bool is8;
    unsigned long long ncells;
    Couple cp;  // group-coupling detector state (uniform over the pair's lanes)
};

template <int G, int K>
__global__ void __launch_bounds__(128, 5) bsw_kernel(LaunchArgs A) {
    TALBSW_DYNAMIC_SMEM(smem_raw);
    constexpr int NG = 32 / G;
    constexpr int SPAN = G * K;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int g = lane / G, gl = lane % G, gshift = g * G;
    const unsigned gbits = (G == 32) ? full : (((1u << G) - 1u) << gshift);
    const size_t pbytes = pair_smem_bytes(A.cols_cap, A.rows_cap, A.win);
    unsigned char *pbase = smem_raw + ((size_t)wib * NG + g) * pbytes;
    int *Hh = reinterpret_cast<int *>(pbase);
    int *Fv = reinterpret_cast<int *>(pbase + smem_hh_bytes(A.cols_cap, A.win));
    uint16_t *Qs = reinterpret_cast<uint16_t *>(pbase + 2 * smem_hh_bytes(A.cols_cap, A.win));
    const bool ring = A.win > 0;
    const int wm = ring ? A.win - 1 : -1;  // column -> slot mask (-1: whole rows)
    const uint8_t *Tg = nullptr;  // this pair's target in global memory
    int tnext = 0;                // its next row's base, loaded one row ahead
    const KernelParams P = A.P;

    CellConsts cc;
    cc.e_ins = P.e_ins;
    cc.e_del = P.e_del;
    cc.oe_del = P.o_del + P.e_del;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        cc.ke[k] = k * P.e_ins;
        cc.keoe[k] = k * P.e_ins - (P.o_ins + P.e_ins);
        cc.ce[k] = -(k - 1) * P.e_ins;
        cc.kp1[k] = (uint32_t)(k + 1);
    }
    const int oe_ins = P.o_ins + P.e_ins;

    PairState ps;
    ps.pidx = 0; ps.req = -1; ps.pp = nullptr; ps.nrow = 0; ps.ncol = 0; ps.i = 0; ps.ncells = 0;
    bool active = false, done = false;
    const bool det = A.flagged != nullptr;  // run the group-coupling detector
    // drops a flagged pair: its group is re-scored by the grouped kernel
    auto drop = [&]() {
        if (gl == 0) flag_pair(A, ps.req, ps.pidx);
        active = false;
    };
    const int nwork = work_count(A);
    const int32_t *order = A.seg ? A.order + A.seg[0] : A.order;
    const int32_t *order_req = A.reqs ? (A.seg ? A.order_req + A.seg[0] : A.order_req) : nullptr;

    auto finish = [&]() {
        if (gl == 0) {
            DevPair *pp = ps.pp;
            if (A.cells) atomicAdd(A.cells, ps.ncells);
            pp->score = ps.maxScore;
            pp->tle = ps.x;
            pp->qle = ps.y;
            pp->max_off = ps.max_off;
            pp->gscore = ps.gscore;
            pp->gtle = ps.max_ie;
        }
        active = false;
    };

    for (;;) {
        // ---- groups without a pair take the next one
        const bool need = !active && !done;
        if (__any_sync(full, need)) {
            int item = 0;
            if (need && gl == 0) item = atomicAdd(A.work_counter, 1);
            item = __shfl_sync(full, item, gshift);
            const bool take = need && item < nwork;
            if (need && !take) done = true;
            int len1 = 0, len2 = 0, h0in = 0, idr = 0, idq = 0, wcall = 0, pidx = 0, req = -1;
            bool is8 = false, ok = false;
            PairSrc src = {};
            if (take) {
                pidx = order ? order[item] : item;
                req = order_req ? order_req[item] : -1;
                src = pair_src(A, pidx, req);
                const DevPair *pp = src.pp;
                len1 = pp->len1; len2 = pp->len2; h0in = pp->h0;
                idr = pp->idr; idq = pp->idq;
                wcall = src.w;
                if (src.bits == 8) is8 = true;
                else if (src.bits == 16) is8 = false;
                else is8 = pair_in_range(P, len1, len2, h0in, wcall, true);
                const bool inwin = (long long)idr >= src.ref_lo && (long long)idq >= src.qer_lo &&
                                   (long long)idr + len1 <= src.ref_hi && (long long)idq + len2 <= src.qer_hi;
                ok = pair_in_range(P, len1, len2, h0in, wcall, is8) && wcall >= 0 && inwin;
                if (!ok) {
                    // outside the exact range of int32 cells: the grouped
                    // kernel computes in the element type and takes it
                    if (gl == 0) {
                        if (det && inwin && pair_in_group_range(len1, len2, h0in, wcall, is8)) flag_pair(A, req, pidx);
                        else report_error(A, req, ERR_DOMAIN, pidx);
                    }
                } else if (ring ? (2LL * wcall + 12 > A.win && len2 + 4 > A.win)
                                : (len2 > A.cols_cap)) {
                    ok = false;
                    if (gl == 0) {
                        if (det) flag_pair(A, req, pidx);
                        else report_error(A, req, ERR_CAPACITY, pidx);
                    }
                }
            }
            const bool st = take && ok;
            if (st) {
                // per-pair constants (smithWatermanBatchWrapper16/8 set-up)
                const int sh = is8 ? 24 : 16, msk = is8 ? 0xff : 0xffff;
                ps.is8 = is8; ps.sh = sh; ps.msk = msk;
                ps.pidx = pidx; ps.req = req; ps.pp = src.pp;
                ps.nrow = len1; ps.ncol = len2; ps.i = 0; ps.ncells = 0;
                Tg = src.ref + (idr - src.ref_lo);
                tnext = len1 > 0 ? Tg[0] : 0;
                ps.Qg = src.qer + (idq - src.qer_lo);
                ps.h0e = wrapS(wrapU(h0in, msk), sh);
                ps.o_delE = P.o_del;
                ps.e_delE = P.e_del;
                int maxsc = 0;  // max(0, a, -b, -1) in the element type (:2779-2782)
                {
                    int av = wrapS((int8_t)P.a, sh), bv = wrapS((int8_t)(-P.b), sh);
                    if (maxsc < av) maxsc = av;
                    if (maxsc < bv) maxsc = bv;
                    if (maxsc < -1) maxsc = -1;
                }
                // band clamp (:2882-2904): integer division, then +1
                int myband;
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
                    ps.wk = wcall < myband ? myband : wcall;
                }
                ps.qlenE = wrapS(len2, sh);
                const int tlenE = wrapS(len1, sh);
                ps.mlen = wrapS(imin(wrapU(ps.qlenE + myband, msk), wrapU(tlenE, msk)), sh);
                ps.zdropE = wrapS(P.zdrop, sh);
                ps.bandE = wrapS(myband, sh);
                ps.head = 0; ps.tail = ps.qlenE;
                ps.maxScore = ps.h0e; ps.x = 0; ps.y = 0; ps.gscore = -1; ps.max_off = 0;
                ps.max_ie = 0;
                ps.beg = 0; ps.end = len2; ps.nbeg = 0; ps.nend = len2;
                // row 0 values H_h[k] and F[k] = 0 (:2839-2879), set lazily
                // as columns come within reach
                ps.v1 = (ps.h0e > oe_ins) ? wrapS(ps.h0e - oe_ins, sh) : 0;
                ps.initc = 0;
                ps.fend = 0; ps.p = -1;
                ps.cp.init(ps.qlenE, ps.v1, P.e_ins);
                active = true;
            }
            __syncwarp();
        }
        if (__all_sync(full, done)) break;

        // ---- one row of every active pair (smithWaterman512_16 :3053-3321)
        bool rowact = active;
        if (rowact && ps.i >= ps.nrow) { finish(); rowact = false; }
        const int sh = ps.sh, msk = ps.msk;
        const int i = ps.i;
        const int i1 = wrapS(i + 1, sh);
        // columns up to i + wk + 3 can be touched by this row (band end + 2):
        // their row-0 values and query selectors, by the pair's G lanes
        {
            bool badq = false;
            if (rowact) {
                const int lim = imin(imax(ps.ncol, 1), i + ps.wk + 3);
                for (int k = ps.initc + gl; k <= lim; k += G) {
                    int hv;
                    if (k == 0) hv = ps.h0e;
                    else if (k == 1) hv = ps.v1;
                    else if (k < ps.ncol) hv = imax(ps.v1 - (k - 1) * P.e_ins, 0);
                    else hv = 0;
                    Hh[k & wm] = hv;
                    Fv[k & wm] = 0;
                    if (k < ps.ncol) {
                        const uint32_t qc = ps.Qg[k];
                        badq |= qc > 4u;
                        Qs[k & wm] = (uint16_t)(qc * 0x1111u + 0x8880u);
                    }
                }
                ps.initc = imax(ps.initc, lim + 1);
            }
            if ((__ballot_sync(full, badq) & gbits) && rowact) {  // a query base code above 4
                if (gl == 0) report_error(A, ps.req, ERR_BASE, ps.pidx);
                active = false;
                rowact = false;
            }
            __syncwarp();
        }
        int beg = 0, end = 0, h10init = 0, hv_next = 0;
        bool changed = false;
        if (rowact) {
            beg = ps.nbeg; end = ps.nend;
            if (beg < i - ps.wk) beg = i - ps.wk;
            if (end > i + ps.wk + 1) end = i + ps.wk + 1;
            if (end > ps.ncol) end = ps.ncol;
            // column -1 value: H_v[i+1] (:3065-3067); DUMMY1 past the last row (:2821-2825)
            {
                const int k = i + 1;
                hv_next = (k == ps.nrow) ? 99 : imax(wrapS(ps.h0e - ps.o_delE - k * ps.e_delE, sh), 0);
                if (beg == 0) h10init = hv_next;
            }
            // per-pair band (:3080-3089)
            const int phead = ps.head, ptail = ps.tail;
            ps.head = imax(ps.head, wrapS(i - ps.bandE, sh));
            int t = imin(wrapU(ps.tail, msk), wrapU(i1 + ps.bandE, msk));
            t = imin(t, wrapU(ps.qlenE, msk));
            ps.tail = wrapS(t, sh);
            changed = ps.head != phead || ps.tail != ptail;
            if (det) ps.cp.clamp(wrapS(i - ps.bandE, sh), wrapU(i1 + ps.bandE, msk), wrapU(ps.qlenE, msk), sh, msk);
        }
        // group-coupling detector: frozen columns, the row's scalar checks and
        // the old entries a group may trim
        if (det) {
            const bool stay = rowact && !(i1 > ps.mlen || ps.tail == ps.head || ps.head > ps.tail);
            // one pass: columns freezing this row [frozenTo, beg), and the old
            // entries a group may trim [beg, th) when the lane does not
            const int th = stay ? imax(ps.cp.trim_hi(changed, end, ps.head), beg) : beg;
            const int a = rowact ? imin(ps.cp.frozenTo, beg) : 0;
            // the usual row: one column froze and no old entry is in question --
            // read it directly; otherwise the ballot pass over [a, th)
            const bool one = rowact && th <= beg && beg - a <= 1;
            int fmin = 1 << 30, fmax = -1, smin, smax;
            bool tnz = false, stnz;
            if (one && beg - a == 1 && (Hh[(beg - 1) & wm] | Fv[(beg - 1) & wm]) != 0) fmin = fmax = beg - 1;
            scan_frozen_trim<G>(Hh, Fv, a, beg, th, rowact && !one, gl, gshift, gbits, wm, smin, smax, stnz);
            if (!one) { fmin = smin; fmax = smax; tnz = stnz; }
            if (rowact) {
                if (fmax >= 0) { ps.cp.frozen_nz(fmin); ps.cp.frozen_nz(fmax); }
                ps.cp.frozenTo = imax(ps.cp.frozenTo, beg);
                ps.cp.row_checks(true, i1 > ps.mlen, stay, i, ps.wk, beg, end, ps.ncol, h10init, hv_next,
                                 ps.is8 ? 127 : 32767);
                if (stay && tnz) ps.cp.flag |= CPL_TRIM;
                if (ps.cp.flag) { drop(); rowact = false; }
            }
            __syncwarp();
        }
        // columns that left the band since the last row are frozen: note the
        // first nonzero one at or after nbeg (16-bit head re-derivation)
        {
            const int lo = imax(ps.fend, ps.nbeg);
            const bool fr = rowact && !ps.is8 && ps.p < 0 && lo < beg;
            const int f = scan_first_nz<G>(Hh, Fv, lo, beg, fr, gl, gshift, gbits, wm);
            if (fr && f < beg) ps.p = f;
            if (rowact) ps.fend = imax(ps.fend, beg);
        }
        // trimming (:3091-3112): zero [beg, min(end, head))
        if (rowact && changed) {
            const int hi = imin(end, ps.head);
            for (int l = beg + gl; l < hi; l += G) { Hh[l & wm] = 0; Fv[l & wm] = 0; }
        }
        __syncwarp();
        // row exit status (:3119-3129); outputs freeze once a pair exits
        if (rowact && (i1 > ps.mlen || ps.tail == ps.head || ps.head > ps.tail)) {
            finish();
            rowact = false;
        }

        // score table of this row's target base: byte q of {thi:tlo} is
        // S(t, q) as a signed byte for query code q (0..3 bases, 4 = N)
        RowState r;
        int tbrow = 0;
        {
            const int tb = rowact ? tnext : 0;
            tbrow = tb;
            if (rowact && i + 1 < ps.nrow) tnext = Tg[i + 1];
            if (rowact && tb > 4) {  // a target base code above 4
                if (gl == 0) report_error(A, ps.req, ERR_BASE, ps.pidx);
                active = false;
                rowact = false;
            }
            const uint32_t mis = (uint32_t)(-P.b) & 0xffu;
            const uint32_t mat = (uint32_t)P.a & 0xffu;
            if (tb >= 4) {
                r.tlo = 0xffffffffu;  // N in the target: -1 against anything
            } else {
                r.tlo = mis * 0x01010101u;
                r.tlo = (r.tlo & ~(0xffu << (8 * tb))) | (mat << (8 * tb));
            }
            r.thi = 0x000000ffu;      // N in the query: -1
        }
        if (det && rowact) {  // F the group could store differently at the tail column and band end
            const int tl = ps.tail;
            const bool tin = tl >= beg && tl < end;
            int ftl = 0, fen = 0;
            if (tin) ftl = Couple::fnext(Hh[tl & wm], Fv[tl & wm], prmt_sext(r.tlo, r.thi, Qs[tl & wm]), P.e_del, cc.oe_del);
            if (end < ps.ncol && end == tl)
                fen = Couple::fnext(Hh[end & wm], Fv[end & wm], prmt_sext(r.tlo, r.thi, Qs[end & wm]), P.e_del, cc.oe_del);
            ps.cp.f_checks(true, i, ps.wk, beg, end, ps.head, tl, ps.ncol, ps.is8 ? 127 : 32767, tin, ftl, fen);
            if (ps.cp.flag) { drop(); rowact = false; }
        }
        r.beg = beg; r.end = end; r.head = ps.head; r.tail = ps.tail;
        r.carryP = -P.e_ins;          // makes E(beg) = 0
        r.hprev = h10init;
        r.h10init = h10init;
        r.key = 0;
        r.hlast = 0;
        const bool ran = rowact && end > beg;
        if (ran) ps.ncells += (unsigned long long)(end - beg);

        // ---- the row, strip by strip (warp-uniform count and kind)
        const int sbase = beg & ~(K - 1);
        const int nstr = ran ? (end - sbase + SPAN - 1) / SPAN : 0;
        const int smax = (int)__reduce_max_sync(full, (unsigned)nstr);
        const bool needmask = ran && (ps.head > beg || ps.tail < end);
        bool lastint = false;
        for (int s = 0; s < smax; s++) {
            const int base = sbase + s * SPAN;
            const bool act = s < nstr;
            const bool inner = base >= beg && base >= ps.head && base + SPAN <= end &&
                               base + SPAN <= ps.tail;
            const int want = (!act || inner) ? STRIP_INTERIOR : (needmask ? STRIP_MASKED : STRIP_EDGE);
            if (act && s == nstr - 1) lastint = inner;
            const int mode = (int)__reduce_max_sync(full, (unsigned)want);
            if (mode == STRIP_INTERIOR) do_strip<G, K, STRIP_INTERIOR>(base, act, gl, r, cc, Hh, Fv, Qs, wm);
            else if (mode == STRIP_EDGE) do_strip<G, K, STRIP_EDGE>(base, act, gl, r, cc, Hh, Fv, Qs, wm);
            else do_strip<G, K, STRIP_MASKED>(base, act, gl, r, cc, Hh, Fv, Qs, wm);
        }
        __syncwarp();
        const uint32_t key = group_max<G>(r.key);
        const int hlast_g = (int)group_max<G>((uint32_t)r.hlast);
        const int hlast = lastint ? r.hprev : hlast_g;
        if (rowact) {
            // last column of the row (:3197-3203)
            const int jl = ran ? end : beg;
            const int h10 = ran ? hlast : h10init;
            const bool m = (ps.head > jl) || (jl > ps.tail);
            if (gl == 0 && jl <= ps.ncol + 1) {
                Hh[jl & wm] = m ? 0 : h10;
                Fv[jl & wm] = 0;
            }
            if (det) ps.cp.stored_last(jl, ps.ncol, m ? 0 : h10, tbrow >= 4 ? -1 : -P.b, ps.head, ps.tail,
                                       P.e_del, cc.oe_del);
            // gscore at the query's last column (:3177-3195); it is in the
            // band exactly when end == ncol, and then it is column end-1
            if (ran && end == ps.ncol && !(ps.qlenE > ps.tail)) {
                ps.max_ie = (ps.gscore > hlast) ? ps.max_ie : i1;
                ps.gscore = imax(ps.gscore, hlast);
            }
        }
        __syncwarp();
        if (rowact) {
            const int maxRS1 = (int)(key >> 16);
            const int y1 = (int)(key & 0xffffu);
            if (maxRS1 == 0) {  // a zero row ends the pair (:3206-3211)
                finish();
                rowact = false;
            } else {
                // maximum, its position and max_off (:3213-3226)
                const int bmax = ps.maxScore;
                ps.maxScore = imax(ps.maxScore, maxRS1);
                if (ps.maxScore > bmax) {
                    ps.y = y1;
                    ps.x = i1;
                    int ind = wrapS(y1 - i1, sh);
                    if (ind < 0) ind = wrapS(-ind, sh);
                    ps.max_off = imax(ps.max_off, ind);
                }
                // z-drop (:3229 -> ZSCORE16 :1868-1881, ZSCORE8 :1826-1839)
                const int tmpi = wrapS(i1 - ps.x, sh);
                const int tmpj = wrapS(y1 - ps.y, sh);
                const int d = (tmpi > tmpj) ? wrapS(tmpi - tmpj, sh) : wrapS(tmpj - tmpi, sh);
                const int t1 = wrapS(wrapS(ps.maxScore - maxRS1, sh) - d, sh);
                if (t1 > ps.zdropE) {
                    finish();
                    rowact = false;
                }
            }
        }
        // band narrowing (:3235-3260)
        {
            const int f = scan_first_nz<G>(Hh, Fv, beg, end, rowact, gl, gshift, gbits, wm);
            const int L = scan_last_nz<G>(Hh, Fv, beg, end, rowact, gl, gshift, gbits, wm);
            if (rowact) {
                if (f > beg) {  // nbeg >= beg: no frozen columns at or after it yet
                    ps.nbeg = f - 1;
                    ps.fend = ps.nbeg;
                    ps.p = -1;
                }
                ps.nend = (L + 2 < ps.ncol) ? L + 2 : ps.ncol;
            }
        }
        // per-pair head / tail (:3265-3316; the 8-bit kernel scans the row's
        // own range, :2571-2621)
        {
            const int B = ps.is8 ? beg : ps.nbeg;
            const int E = ps.is8 ? end : ps.nend;
            // the frozen columns [B, beg) answer from p; the rest is live
            const bool use_p = B < beg && ps.p >= 0 && ps.p < E;
            const int Bl = B < beg ? imin(beg, E) : B;
            int f2 = scan_first_nz<G>(Hh, Fv, Bl, E, rowact && E > B && !use_p, gl, gshift, gbits, wm);
            if (use_p) f2 = ps.p;
            // a cell with H > 0 left a nonzero in [beg + 1, end]: this scan
            // stops inside the band
            const int L2 = scan_last_nz<G>(Hh, Fv, imax(B, beg), E, rowact && E >= B, gl, gshift, gbits, wm);
            if (rowact && ring && E >= B && L2 < beg) {  // would have read a reused ring slot
                if (det) drop();
                else {
                    if (gl == 0) report_error(A, ps.req, ERR_CAPACITY, ps.pidx);
                    active = false;
                }
                rowact = false;
            }
            if (rowact) {
                if (E > B && f2 > B) ps.head = wrapS(f2, sh);
                int index = ps.tail;
                if (E >= B && L2 != E) index = L2;
                const int index0 = index;
                index = wrapS(index + 2, sh);
                ps.tail = index < ps.qlenE ? index : ps.qlenE;
                ps.i = i + 1;
                if (det) {
                    const bool last_row = i + 1 >= ps.nrow;
                    const bool nz_sb = B < beg ? ps.p == B : (Hh[B & wm] | Fv[B & wm]) != 0;
                    const int hse = Hh[E & wm], fse = Fv[E & wm];
                    ps.cp.scans(true, last_row, ps.is8, i, ps.wk, beg, end, B, E, nz_sb, (hse | fse) != 0,
                                E > B && f2 >= E, hse != 0, E >= B && L2 < imax(B, beg), ps.head, index0,
                                ps.qlenE, ps.ncol, ps.is8 ? 127 : 32767);
                    ps.cp.settle(true, last_row, ps.head, ps.tail);
                    if (ps.cp.flag) drop();
                }
            }
        }
    }
}

}  // namespace talbsw
