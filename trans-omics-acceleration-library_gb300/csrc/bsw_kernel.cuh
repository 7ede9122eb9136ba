// Banded Smith-Waterman seed extension on sm_103a: one warp per pair,
// row-synchronous, each lane owning K consecutive columns of a 32*K-column
// strip of the current row.
//
// Semantics: the reference's getScores16 / getScores8 kernels
// (src/alignment/BSW/bandedSWA.cpp:2962-3356 / :2263-2661) for a pair scored on
// its own.  Their outputs do not depend on which other pairs share the SIMD
// group (checked against the reference on every workload shape), so a pair is
// the unit of work here and the per-lane head/tail bookkeeping of the vector
// code collapses to per-pair scalars held uniformly by the warp.
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
// reference's scratch rows: HF[j] packs H_h[j] (low 16 bits) and F[j] (high 16
// bits); columns outside the computed band keep their old ("stale") values,
// which the reference's narrowing reads.
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
enum : int { ERR_DOMAIN = 1, ERR_CAPACITY = 2, ERR_BASE = 4 };

struct LaunchArgs {
    DevPair *pairs;
    // ref / qer point at a device copy of the caller's buffer window
    // [*_lo, *_hi): byte `off` of the caller's buffer is ref[off - ref_lo].
    const uint8_t *ref;
    const uint8_t *qer;
    long long ref_lo, ref_hi, qer_lo, qer_hi;
    const int32_t *order;    // optional permutation (batched form)
    const int32_t *wpair;    // optional per-pair band
    int32_t n;
    int32_t w;
    int bits;                // 8, 16 or 0 = per-pair routing
    int cols_cap, rows_cap;  // shared-memory row capacity per warp
    int *work_counter;       // next work item (dynamic scheduling)
    unsigned long long *cells;  // optional: total DP cells computed
    int *err_flags;
    long long *err_index;
    KernelParams P;
};

// Element-width wrap helpers: the reference's per-row bookkeeping is int16
// (or int8) arithmetic that wraps; it is emulated exactly.
__device__ __forceinline__ int wrapS(int x, bool is8) {
    return is8 ? (int)(int8_t)x : (int)(int16_t)x;
}
__device__ __forceinline__ int wrapU(int x, bool is8) {
    return is8 ? (int)(uint8_t)x : (int)(uint16_t)x;
}

__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }
__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }

// first non-zero word of HF in [lo, hi) scanning up; hi if none
__device__ __forceinline__ int scan_first_nz(const uint32_t *HF, int lo, int hi, int lane) {
    for (int b = lo; b < hi; b += 32) {
        int j = b + lane;
        bool nz = (j < hi) && HF[j] != 0u;
        unsigned m = __ballot_sync(0xffffffffu, nz);
        if (m) return b + __ffs(m) - 1;
    }
    return hi;
}
// last non-zero word of HF in [lo, hi] scanning down from hi; lo-1 if none
__device__ __forceinline__ int scan_last_nz(const uint32_t *HF, int lo, int hi, int lane) {
    for (int t = hi; t >= lo; t -= 32) {
        int j = t - lane;
        bool nz = (j >= lo) && HF[j] != 0u;
        unsigned m = __ballot_sync(0xffffffffu, nz);
        if (m) return t - (__ffs(m) - 1);
    }
    return lo - 1;
}

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
    __device__ static void ld(const uint32_t *p, uint32_t (&v)[1]) { v[0] = p[0]; }
    __device__ static void st(uint32_t *p, const uint32_t (&v)[1]) { p[0] = v[0]; }
    __device__ static uint32_t ldq(const uint8_t *q) { return q[0]; }
};
template <>
struct VecIO<2> {
    __device__ static void ld(const uint32_t *p, uint32_t (&v)[2]) {
        uint2 t = *reinterpret_cast<const uint2 *>(p);
        v[0] = t.x; v[1] = t.y;
    }
    __device__ static void st(uint32_t *p, const uint32_t (&v)[2]) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(v[0], v[1]);
    }
    __device__ static uint32_t ldq(const uint8_t *q) {
        return *reinterpret_cast<const uint16_t *>(q);
    }
};
template <>
struct VecIO<4> {
    __device__ static void ld(const uint32_t *p, uint32_t (&v)[4]) {
        uint4 t = *reinterpret_cast<const uint4 *>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    __device__ static void st(uint32_t *p, const uint32_t (&v)[4]) {
        *reinterpret_cast<uint4 *>(p) = make_uint4(v[0], v[1], v[2], v[3]);
    }
    __device__ static uint32_t ldq(const uint8_t *q) {
        return *reinterpret_cast<const uint32_t *>(q);
    }
};

// Shared-memory footprint of one warp's rows, in bytes (16-byte aligned parts).
__host__ __device__ __forceinline__ size_t warp_smem_bytes(int cols_cap, int rows_cap, int K) {
    size_t hf = ((size_t)(cols_cap + 2 + K) * 4 + 15) & ~(size_t)15;
    size_t q = ((size_t)(cols_cap + K + 16) + 15) & ~(size_t)15;
    size_t t = ((size_t)(rows_cap + 16) + 15) & ~(size_t)15;
    return hf + q + t;
}

// Stage len bytes at window offset `off` of the device window src (window
// length buf_bytes, 16-byte aligned start) into shared dst as base codes,
// with 16-byte vector loads; returns false (warp-uniform) if any byte is
// above 4.
__device__ __forceinline__ bool stage_bases(uint8_t *dst, const uint8_t *src, int len,
                                            size_t buf_bytes, size_t off, int lane) {
    // aligned 16-byte chunks covering [off, off+len), never past the window
    size_t a0 = off & ~(size_t)15;
    size_t a1 = (off + (size_t)len + 15) & ~(size_t)15;
    if (a1 > (buf_bytes & ~(size_t)15)) a1 = buf_bytes & ~(size_t)15;
    bool bad = false;
    for (size_t c = a0 + (size_t)lane * 16; c < a1; c += 32 * 16) {
        uint4 v = *reinterpret_cast<const uint4 *>(src + c);
        uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int b = 0; b < 16; b++) {
            size_t pos = c + b;
            if (pos >= off && pos < off + (size_t)len) {
                uint32_t byte = (wv[b >> 2] >> ((b & 3) * 8)) & 0xffu;
                if (byte > 4u) bad = true;
                dst[pos - off] = (uint8_t)byte;
            }
        }
    }
    // tail bytes past the last whole 16-byte unit of the buffer
    size_t done = a1 > off ? a1 - off : 0;
    for (size_t p = done + lane; p < (size_t)len; p += 32) {
        uint32_t byte = src[off + p];
        if (byte > 4u) bad = true;
        dst[p] = (uint8_t)byte;
    }
    return __any_sync(0xffffffffu, bad) == 0;
}

template <int K>
__global__ void __launch_bounds__(128) bsw_warp_kernel(LaunchArgs A) {
    TALBSW_DYNAMIC_SMEM(smem_raw);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const size_t wbytes = warp_smem_bytes(A.cols_cap, A.rows_cap, K);
    unsigned char *wbase = smem_raw + (size_t)wib * wbytes;
    uint32_t *HF = reinterpret_cast<uint32_t *>(wbase);
    uint8_t *Q = wbase + (((size_t)(A.cols_cap + 2 + K) * 4 + 15) & ~(size_t)15);
    uint8_t *Tt = Q + (((size_t)(A.cols_cap + K + 16) + 15) & ~(size_t)15);
    const KernelParams P = A.P;
    const int span = 32 * K;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.work_counter, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= A.n) break;
        const int pidx = A.order ? A.order[item] : item;
        DevPair *pp = A.pairs + pidx;
        const int len1 = pp->len1, len2 = pp->len2, h0in = pp->h0;
        const int idr = pp->idr, idq = pp->idq;
        const int wcall = A.wpair ? A.wpair[pidx] : A.w;

        // ---- precision routing and range checks (warp-uniform)
        bool is8;
        if (A.bits == 8) is8 = true;
        else if (A.bits == 16) is8 = false;
        else is8 = pair_in_range(P, len1, len2, h0in, wcall, true);
        bool ok = pair_in_range(P, len1, len2, h0in, wcall, is8) && wcall >= 0;
        ok = ok && (long long)idr >= A.ref_lo && (long long)idq >= A.qer_lo &&
             (long long)idr + len1 <= A.ref_hi && (long long)idq + len2 <= A.qer_hi;
        if (!ok) {
            if (lane == 0) {
                atomicOr(A.err_flags, ERR_DOMAIN);
                atomicMin(A.err_index, (long long)pidx);
            }
            continue;
        }
        if (len2 > A.cols_cap || len1 > A.rows_cap) {
            if (lane == 0) {
                atomicOr(A.err_flags, ERR_CAPACITY);
                atomicMin(A.err_index, (long long)pidx);
            }
            continue;
        }
        const int ncol = len2, nrow = len1;

        // ---- stage bases (codes 0..4) into shared memory
        bool gq = stage_bases(Q, A.qer, len2, (size_t)(A.qer_hi - A.qer_lo),
                              (size_t)(idq - A.qer_lo), lane);
        bool gt = stage_bases(Tt, A.ref, len1, (size_t)(A.ref_hi - A.ref_lo),
                              (size_t)(idr - A.ref_lo), lane);
        if (!(gq && gt)) {
            if (lane == 0) {
                atomicOr(A.err_flags, ERR_BASE);
                atomicMin(A.err_index, (long long)pidx);
            }
            __syncwarp();
            continue;
        }

        // ---- per-pair constants (smithWatermanBatchWrapper16/8 set-up)
        const int h0e = wrapS(wrapU(h0in, is8), is8);
        const int oe_insE = wrapS(P.o_ins + P.e_ins, is8);
        const int e_insE = wrapS(P.e_ins, is8), e_delE = wrapS(P.e_del, is8);
        const int o_delE = wrapS(P.o_del, is8);
        int maxsc = 0;  // max(0, a, -b, -1) in the element type (:2779-2782)
        {
            int av = wrapS((int8_t)P.a, is8), bv = wrapS((int8_t)(-P.b), is8);
            if (maxsc < av) maxsc = av;
            if (maxsc < bv) maxsc = bv;
            if (maxsc < -1) maxsc = -1;
        }
        // band clamp (:2882-2904): integer division, then +1
        int myband, wk;
        {
            const int qlen_b = wrapU(len2 * maxsc, is8);
            const int tmp1 = wrapU(qlen_b + wrapS(P.end_bonus - P.o_ins, is8), is8);
            int mi = tmp1 / P.e_ins + 1;
            if (mi < 1) mi = 1;
            myband = wrapU(wcall > mi ? mi : wcall, is8);
            const int tmp2 = wrapU(qlen_b + wrapS(P.end_bonus - P.o_del, is8), is8);
            int md = tmp2 / P.e_del + 1;
            if (md < 1) md = 1;
            myband = wrapU(myband > md ? md : myband, is8);
            wk = wcall < myband ? myband : wcall;
        }
        const int qlenE = wrapS(len2, is8);
        const int tlenE = wrapS(len1, is8);
        const int mlen = wrapS(imin(wrapU(qlenE + myband, is8), wrapU(tlenE, is8)), is8);
        const int zdropE = wrapS(P.zdrop, is8);
        const int bandE = wrapS(myband, is8);

        // ---- row 0 values H_h[k] and F[k] = 0 (:2839-2879)
        {
            const int v1 = (h0e > oe_insE) ? wrapS(h0e - oe_insE, is8) : 0;
            const int top = ncol > 1 ? ncol : 1;
            for (int k = lane; k <= top; k += 32) {
                int hv;
                if (k == 0) hv = h0e;
                else if (k == 1) hv = v1;
                else if (k < ncol) hv = imax(v1 - (k - 1) * e_insE, 0);
                else hv = 0;
                HF[k] = (uint32_t)hv & 0xffffu;
            }
        }
        __syncwarp();

        // ---- per-pair state (smithWaterman512_16 :3000-3047)
        int head = 0, tail = qlenE;
        int maxScore = h0e, x = 0, y = 0, gscore = -1, max_off = 0, max_ie = 0;
        int beg = 0, end = ncol, nbeg = 0, nend = ncol;
        const uint32_t full = 0xffffffffu;
        unsigned long long ncells = 0;

        for (int i = 0; i < nrow; i++) {
            const int i1 = wrapS(i + 1, is8);
            beg = nbeg; end = nend;
            if (beg < i - wk) beg = i - wk;
            if (end > i + wk + 1) end = i + wk + 1;
            if (end > ncol) end = ncol;
            // column -1 value: H_v[i+1] (:3065-3067)
            int h10init = 0;
            if (beg == 0) {
                const int k = i + 1;
                if (k == nrow) h10init = 99;  // DUMMY1 past the last row (:2821-2825)
                else h10init = imax(wrapS(h0e - o_delE - k * e_delE, is8), 0);
            }
            // per-pair band (:3080-3089)
            const int phead = head, ptail = tail;
            head = imax(head, wrapS(i - bandE, is8));
            {
                int t = imin(wrapU(tail, is8), wrapU(i1 + bandE, is8));
                t = imin(t, wrapU(qlenE, is8));
                tail = wrapS(t, is8);
            }
            // trimming (:3091-3112): zero [beg, min(end, head))
            if (head != phead || tail != ptail) {
                const int hi = imin(end, head);
                for (int l = beg + lane; l < hi; l += 32) HF[l] = 0u;
                __syncwarp();
            }
            // row exit status (:3119-3129); outputs freeze once a pair exits
            if (i1 > mlen || tail == head || head > tail) break;

            // score lookup for this row's target base: byte q of {thi:tlo} is
            // S(t, q) + 128 for query code q (0..3 bases, 4 = N); bytes 5..7 are
            // zero so a selector q | 0x7770 yields the byte zero-extended
            const int tb = Tt[i];
            uint32_t tlo, thi;
            {
                const uint32_t mis = (uint32_t)(128 - P.b) & 0xffu;
                const uint32_t mat = (uint32_t)(128 + P.a) & 0xffu;
                if (tb >= 4) {
                    tlo = 0x7f7f7f7fu;  // N in the target: -1 against anything
                } else {
                    tlo = mis * 0x01010101u;
                    tlo = (tlo & ~(0xffu << (8 * tb))) | (mat << (8 * tb));
                }
                thi = 0x0000007fu;      // N in the query: -1
            }

            // ---- the row, strip by strip
            if (end > beg) ncells += (unsigned long long)(end - beg);
            int carryP = INT_MIN;      // max of P over earlier strips
            int hprev = h10init;       // H of the column left of the strip
            uint32_t key = 0;          // (H << 16) | (j + 1), row max, last j wins ties
            int hq = 0;                // H at column qlen-1
            int hlast = 0;             // H at column end-1
            const int sbase = (beg / K) * K;
            for (int base = sbase; base < end; base += span) {
                const int j0 = base + lane * K;
                uint32_t hf[K];
                int mm[K], ff[K], hh[K];
                uint32_t qv = 0;
                const bool anyin = (j0 < end) && (j0 + K - 1 >= beg);
                if (anyin) {
                    VecIO<K>::ld(HF + j0, hf);
                    qv = VecIO<K>::ldq(Q + j0);
                } else {
#pragma unroll
                    for (int k = 0; k < K; k++) hf[k] = 0u;
                }
                int summ = INT_MIN;
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const int j = j0 + k;
                    const int h00 = (int)(hf[k] & 0xffffu);
                    const int f11 = (int)(hf[k] >> 16);
                    const uint32_t q = (qv >> (8 * k)) & 0xffu;
                    const int sbt = (int)__byte_perm(tlo, thi, q | 0x7770u);  // S + 128
                    const int m = h00 ? h00 + sbt - 128 : 0;
                    mm[k] = m;
                    ff[k] = f11;
                    const int Pk = imax(m - oe_insE, 0) + e_insE * (j - beg);
                    if (j >= beg && j < end) summ = imax(summ, Pk);
                }
                // inclusive max-scan of lane summaries across the warp
                int incl = summ;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    int v = __shfl_up_sync(full, incl, d);
                    if (lane >= d) incl = imax(incl, v);
                }
                int excl = __shfl_up_sync(full, incl, 1);
                excl = (lane == 0) ? carryP : imax(excl, carryP);
                carryP = imax(carryP, __shfl_sync(full, incl, 31));
                int run = excl;
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const int j = j0 + k;
                    const int E = (j <= beg) ? 0 : run - e_insE * (j - 1 - beg);
                    const int Pk = imax(mm[k] - oe_insE, 0) + e_insE * (j - beg);
                    if (j >= beg) run = imax(run, Pk);
                    hh[k] = imax(imax(mm[k], E), ff[k]);
                }
                int hl = __shfl_up_sync(full, hh[K - 1], 1);
                if (lane == 0) hl = hprev;
                hprev = __shfl_sync(full, hh[K - 1], 31);
                uint32_t outv[K];
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const int j = j0 + k;
                    const bool in = (j >= beg) && (j < end);
                    const int hleft = (j == beg) ? h10init : ((k == 0) ? hl : hh[k - 1]);
                    const bool mask = (j < head) || (j > tail);
                    const int f21 = imax(imax(mm[k] - wrapS(P.o_del + P.e_del, is8), 0),
                                         ff[k] - e_delE);
                    const int hst = mask ? 0 : hleft;
                    const int fst = mask ? 0 : f21;
                    outv[k] = in ? (((uint32_t)fst << 16) | ((uint32_t)hst & 0xffffu)) : hf[k];
                    const bool valid = in && !((j + 1) > tail) && !(j < head);
                    if (valid) {
                        const uint32_t kk = ((uint32_t)hh[k] << 16) | (uint32_t)(j + 1);
                        key = kk > key ? kk : key;
                    }
                    if (in && j == ncol - 1) hq = hh[k];
                    if (in && j == end - 1) hlast = hh[k];
                }
                if (anyin) VecIO<K>::st(HF + j0, outv);
            }
            __syncwarp();
            key = __reduce_max_sync(full, key);
            const bool ran = end > beg;
            hq = __reduce_max_sync(full, (uint32_t)hq);
            hlast = (int)__reduce_max_sync(full, (uint32_t)hlast);
            // last column of the row (:3197-3203)
            {
                const int jl = ran ? end : beg;
                const int h10 = ran ? hlast : h10init;
                const bool m = (head > jl) || (jl > tail);
                if (lane == 0 && jl <= ncol + 1) HF[jl] = m ? 0u : ((uint32_t)h10 & 0xffffu);
            }
            // gscore at the query's last column (:3177-3195)
            if (ran && (ncol - 1) >= beg && (ncol - 1) < end && !(qlenE > tail)) {
                max_ie = (gscore > hq) ? max_ie : i1;
                gscore = imax(gscore, hq);
            }
            __syncwarp();
            const int maxRS1 = (int)(key >> 16);
            const int y1 = (int)(key & 0xffffu);
            // a zero row ends the pair (:3206-3211)
            if (maxRS1 == 0) break;
            // maximum, its position and max_off (:3213-3226)
            {
                const int bmax = maxScore;
                maxScore = imax(maxScore, maxRS1);
                if (maxScore > bmax) {
                    y = y1;
                    x = i1;
                    int ind = wrapS(y1 - i1, is8);
                    if (ind < 0) ind = wrapS(-ind, is8);
                    max_off = imax(max_off, ind);
                }
            }
            // z-drop (:3229 -> ZSCORE16 :1868-1881, ZSCORE8 :1826-1839)
            {
                const int tmpi = wrapS(i1 - x, is8);
                const int tmpj = wrapS(y1 - y, is8);
                const int d = (tmpi > tmpj) ? wrapS(tmpi - tmpj, is8) : wrapS(tmpj - tmpi, is8);
                const int t1 = wrapS(wrapS(maxScore - maxRS1, is8) - d, is8);
                if (t1 > zdropE) break;
            }
            // band narrowing (:3235-3260)
            {
                const int f = scan_first_nz(HF, beg, end, lane);
                if (f > beg) nbeg = f - 1;
                const int L = scan_last_nz(HF, beg, end, lane);
                nend = (L + 2 < ncol) ? L + 2 : ncol;
            }
            // per-pair head / tail (:3265-3316; the 8-bit kernel scans the
            // row's own range, :2571-2621)
            {
                const int B = is8 ? beg : nbeg;
                const int E = is8 ? end : nend;
                if (E > B) {
                    const int f2 = scan_first_nz(HF, B, E, lane);
                    if (f2 > B) head = wrapS(f2, is8);
                }
                int index = tail;
                if (E >= B) {
                    const int L2 = scan_last_nz(HF, B, E, lane);
                    if (L2 != E) index = L2;
                }
                index = wrapS(index + 2, is8);
                tail = index < qlenE ? index : qlenE;
            }
        }
        if (lane == 0) {
            if (A.cells) atomicAdd(A.cells, ncells);
            pp->score = maxScore;
            pp->tle = x;
            pp->qle = y;
            pp->max_off = max_off;
            pp->gscore = gscore;
            pp->gtle = max_ie;
        }
        __syncwarp();
    }
}

}  // namespace talbsw
