// Dynamic-programming anchor chaining on sm_103a: the reference's
// dp_chain::mm_dp_vectorized (src/chaining/parallel_chaining_32_bit.h:216-436),
// the minimap2 chaining step that precedes extension, one warp per read.
//
// For each anchor i of a read in order (the recurrence is sequential in i):
//   st: first predecessor with r_i - r_st <= dr (64-bit), at least i - max_iter
//   each j in [st, i) passing, in 32-bit arithmetic on the low words of r,
//       ddr = r_i - r_j, ddq = q_i - q_j, dd = |ddr - ddq|:
//       dd <= bw, ddr != 0, 0 < ddq <= dq, ddq <= dr
//   scores f_j + min(ddr, ddq, l_i) - gap(dd)
//   f_i = max(l_i, best score); p_i = the largest j with that score when it
//   exceeds l_i, else -1; v_i = max(v_{p_i}, f_i)
// gap(dd) = floor(dd * 0.01 * avg_l) + (floor(log2 dd) >> 1) with the rounding
// of the reference's path: more than six predecessors -> its 16-lane vector
// loop, float product (float)dd * (float)(0.01 * avg_l) rounded down (:129-150);
// at most six -> its scalar loop, double product (dd * 0.01) * avg_l truncated
// (:414-415).  Out-of-range conversions give INT_MIN as the x86 ones do.
//
// The warp's 32 lanes split the predecessors of anchor i (lane t takes
// j = i-1-t, i-1-t-32, ...; descending, so a strict '>' keeps the larger j of
// a tie), then two warp reductions (__reduce_max_sync) give f_i and p_i, and
// lane 0 stores them before the next anchor.  The warp first writes its read's
// (low word of r, q) pairs to an 8-byte scratch array, so a predecessor costs
// two coalesced loads (that pair and f), served from L1 as long as the
// windows of the resident warps fit it (consecutive anchors' windows overlap
// almost entirely; the launch keeps few warps per SM for that).  Integer work
// only, except one float product per predecessor (one double product in the
// scalar path, at most six predecessors).
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

#include <climits>

#include "bucket_scan.cuh"

#ifndef TALBSW_DYNAMIC_SMEM
#define TALBSW_DYNAMIC_SMEM(name) extern __shared__ __align__(16) unsigned char name[]
#endif

namespace talchain {

struct Anchor {  // anchor_t (parallel_chaining_32_bit.h:58-67)
    uint64_t r;
    int32_t q;
    int32_t l;
};

enum : int { CHERR_DOMAIN = 1 };

struct ChainArgs {
    const Anchor *anchors;
    const int64_t *offsets;  // read k: anchors [offsets[k], offsets[k+1])
    const int32_t *order;    // optional read order
    int n_reads;
    int bw, max_iter, dr, dq;
    int2 *rq;                // scratch, one per anchor: (low word of r, q)
    uint32_t *f;
    int32_t *p, *v;
    int *work_counter;
    unsigned long long *evals;  // optional: predecessors scored
    int *err_flags;
    long long *err_index;
};

__device__ __forceinline__ int32_t ch_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t ch_sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

// floor(log2 dd) >> 1, 0 for dd == 0 (dd read as unsigned)
__device__ __forceinline__ int32_t ch_log_term(int32_t dd) {
    return dd != 0 ? (31 - __clz((unsigned)dd)) >> 1 : 0;
}

__device__ __forceinline__ int32_t ch_gap_float(int32_t dd, float aq) {
    const float prod = __fmul_rn(__int2float_rn(dd), aq);
    const int32_t c = prod >= 2147483648.0f ? INT_MIN : __float2int_rd(prod);
    return ch_add(c, ch_log_term(dd));
}

__device__ __forceinline__ int32_t ch_gap_double(int32_t dd, double avg) {
    const double prod = __dmul_rn(__dmul_rn((double)dd, 0.01), avg);
    const int32_t c = prod >= 2147483648.0 ? INT_MIN : __double2int_rz(prod);
    return ch_add(c, ch_log_term(dd));
}

// Read order for device-resident batches: by anchor count, longest first, in
// buckets of 16 anchors (a counting sort), so no long read starts last.
constexpr int kChainBuckets = talbsw::kScanBuckets;  // scanned by talbsw::bucket_scan_4096

__device__ __forceinline__ int ch_bucket(const int64_t *offsets, int k) {
    int64_t n = offsets[k + 1] - offsets[k];
    n = n < 0 ? 0 : n >> 4;
    return (kChainBuckets - 1) - (int)(n > kChainBuckets - 1 ? kChainBuckets - 1 : n);
}

__global__ void ch_bucket_count(const int64_t *offsets, int n_reads, int *hist) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_reads; k += gridDim.x * blockDim.x)
        atomicAdd(&hist[ch_bucket(offsets, k)], 1);
}

__global__ void ch_bucket_scatter(const int64_t *offsets, int n_reads, int *offs, int32_t *order) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_reads; k += gridDim.x * blockDim.x)
        order[atomicAdd(&offs[ch_bucket(offsets, k)], 1)] = k;
}

constexpr int kChainBatch = 4;       // anchors scored per pass over a window
constexpr int kGapTableMax = 2048;   // bw up to this: vector-path gap costs from a table
constexpr int kRing = 1024;          // newest predecessors kept in shared memory (power of 2)

// Per warp: the ring of the newest kRing anchors' (low r, q) and f, then the
// gap table (bw + 1 entries when bw <= kGapTableMax).
__host__ __device__ __forceinline__ size_t chain_table_bytes(int bw) {
    return (bw >= 0 && bw <= kGapTableMax) ? (((size_t)(bw + 1) * 4 + 15) & ~(size_t)15) : 0;
}
__host__ __device__ __forceinline__ size_t chain_warp_smem_bytes(int bw) {
    return (size_t)kRing * 12 + chain_table_bytes(bw);
}

// The predecessor test in one unsigned compare for the query gap:
// 0 < ddq <= min(dq, dr)  <=>  (unsigned)(ddq - 1) < max(min(dq, dr), 0).
__device__ __forceinline__ bool ch_valid(int32_t dd, int32_t ddr, int32_t ddq, int bw, uint32_t limq) {
    return dd <= bw && ddr != 0 && (uint32_t)ch_sub(ddq, 1) < limq;
}

// Vector-path gap cost: from the warp's table (dd in [0, bw]) or computed
// (dd = INT_MIN, the wrapped |INT_MIN| the reference's SIMD abs leaves).
__device__ __forceinline__ int32_t ch_gap_vec(const int32_t *tbl, int32_t dd, int bw, float aq) {
    if (tbl == nullptr || dd < 0) return ch_gap_float(dd, aq);
    return tbl[(uint32_t)dd <= (uint32_t)bw ? dd : 0];
}

// Where predecessor j's (low r, q) and f are read: the warp's ring when
// j >= i - kRing (i: the first anchor being scored), else global memory.
struct ChSrc {
    const int2 *rq;
    const uint32_t *f;
    const int2 *ring_rq;
    const int32_t *ring_f;
    __device__ __forceinline__ void load_global(int j, int2 &c, int32_t &fj) const {
        c = rq[j];
        fj = (int32_t)f[j];
    }
    __device__ __forceinline__ void load_ring(int j, int2 &c, int32_t &fj) const {
        c = ring_rq[j & (kRing - 1)];
        fj = ring_f[j & (kRing - 1)];
    }
};

// Score of predecessor (c, fj) for an anchor (ri, qi, li); false if the
// reference skips it.
template <typename GAP>
__device__ __forceinline__ bool ch_score(int2 c, int32_t fj, uint32_t ri, int32_t qi, int32_t li, int bw,
                                         uint32_t limq, GAP gap, int32_t &sc) {
    const int32_t ddr = (int32_t)(ri - (uint32_t)c.x);
    const int32_t ddq = ch_sub(qi, c.y);
    const int32_t x = ch_sub(ddr, ddq);
    const int32_t dd = x < 0 ? ch_sub(0, x) : x;
    int32_t oc = ddr < ddq ? ddr : ddq;
    oc = oc < li ? oc : li;
    sc = ch_sub(ch_add(fj, oc), gap(dd));
    return ch_valid(dd, ddr, ddq, bw, limq);
}

// Lane `lane`'s predecessors j = i-1-lane, i-1-lane-32, ... split at lo: the
// first one below lo (the first read from global memory).
__device__ __forceinline__ int ch_first_below(int i, int lane, int lo) {
    const int j0 = i - 1 - lane;
    return j0 < lo ? j0 : j0 - 32 * ((j0 - lo) / 32 + 1);
}

// One anchor: best (score, largest j) over lane `lane`'s share of [st, i).
template <typename GAP>
__device__ __forceinline__ void ch_scan1(const ChSrc &S, int i, int st, int lane, uint32_t ri, int32_t qi,
                                         int32_t li, int bw, uint32_t limq, GAP gap, int32_t &best,
                                         int &bj) {
    const int lo = i - kRing > st ? i - kRing : st;
#pragma unroll 4
    for (int j = i - 1 - lane; j >= lo; j -= 32) {
        int2 c;
        int32_t fj, sc;
        S.load_ring(j, c, fj);
        if (ch_score(c, fj, ri, qi, li, bw, limq, gap, sc) && sc > best) {
            best = sc;
            bj = j;
        }
    }
    for (int j = ch_first_below(i, lane, lo); j >= st; j -= 32) {  // older than the ring
        int2 c;
        int32_t fj, sc;
        S.load_global(j, c, fj);
        if (ch_score(c, fj, ri, qi, li, bw, limq, gap, sc) && sc > best) {
            best = sc;
            bj = j;
        }
    }
}

// kChainBatch anchors i..i+K-1 (vector-loop rounding) over one pass of
// [stk[0], i): predecessors j >= stk[K-1] are in every window; below it each
// anchor checks its own start.
template <bool CHECK, bool RING>
__device__ __forceinline__ void ch_scanK(const ChSrc &S, int jfrom, int jto, const int *stk,
                                         const uint32_t *rk, const int32_t *qk, const int32_t *lk,
                                         const int32_t *tbl, int bw, uint32_t limq, float aq,
                                         int32_t *best, int *bj) {
#pragma unroll 2
    for (int j = jfrom; j >= jto; j -= 32) {
        int2 c;
        int32_t fj;
        if (RING) S.load_ring(j, c, fj);
        else S.load_global(j, c, fj);
#pragma unroll
        for (int k = 0; k < kChainBatch; k++) {
            int32_t sc;
            const bool ok = ch_score(c, fj, rk[k], qk[k], lk[k], bw, limq,
                                     [tbl, bw, aq](int32_t dd) { return ch_gap_vec(tbl, dd, bw, aq); }, sc);
            if ((!CHECK || j >= stk[k]) && ok && sc > best[k]) {
                best[k] = sc;
                bj[k] = j;
            }
        }
    }
}

__global__ void __launch_bounds__(128) chain_kernel(ChainArgs A) {
    TALBSW_DYNAMIC_SMEM(ch_smem);
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint64_t drw = (uint64_t)(uint32_t)A.dr;
    const int bw = A.bw;
    const int lq = A.dq < A.dr ? A.dq : A.dr;
    const uint32_t limq = lq > 0 ? (uint32_t)lq : 0u;
    unsigned char *wsm = ch_smem + (threadIdx.x >> 5) * chain_warp_smem_bytes(bw);
    int2 *ring_rq = reinterpret_cast<int2 *>(wsm);
    int32_t *ring_f = reinterpret_cast<int32_t *>(wsm + (size_t)kRing * 8);
    int32_t *tbl = chain_table_bytes(bw) ? reinterpret_cast<int32_t *>(wsm + (size_t)kRing * 12) : nullptr;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.work_counter, 1);
        item = __shfl_sync(full, item, 0);
        if (item >= A.n_reads) break;
        const int rd = A.order ? A.order[item] : item;
        const int64_t o = A.offsets[rd];
        const int64_t n64 = A.offsets[rd + 1] - o;
        if (n64 < 0 || n64 > INT_MAX) {
            if (lane == 0) {
                atomicOr(A.err_flags, CHERR_DOMAIN);
                atomicMin(A.err_index, (long long)rd);
            }
            continue;
        }
        if (n64 == 0) continue;
        const Anchor *a = A.anchors + o;
        int2 *rq = A.rq + o;
        uint32_t *f = A.f + o;
        int32_t *p = A.p + o;
        int32_t *v = A.v + o;
        const int n = (int)n64;
        // mean anchor length, float(sum) / float(n) as the reference, and the
        // (r, q) words the predecessor scan reads (ring: the first kRing)
        unsigned long long sum = 0;
        int neg = 0;
        for (int i = lane; i < n; i += 32) {
            const Anchor ai = a[i];
            neg |= ai.l < 0;
            sum += (uint32_t)ai.l;
            const int2 c = make_int2((int)(uint32_t)ai.r, ai.q);
            rq[i] = c;
            if (i < kRing) ring_rq[i] = c;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(full, sum, d);
        if (__any_sync(full, neg)) {  // lengths are non-negative int32
            if (lane == 0) {
                atomicOr(A.err_flags, CHERR_DOMAIN);
                atomicMin(A.err_index, (long long)rd);
            }
            continue;
        }
        const float avg = __fdiv_rn(__ull2float_rn(sum), __ll2float_rn(n64));
        const float aq = __double2float_rn(__dmul_rn(0.01, (double)avg));
        const double davg = (double)avg;
        if (tbl)
            for (int d = lane; d <= bw; d += 32) tbl[d] = ch_gap_float(d, aq);
        __syncwarp();
        const ChSrc S = {rq, f, ring_rq, ring_f};
        auto gapv = [tbl, bw, aq](int32_t dd) { return ch_gap_vec(tbl, dd, bw, aq); };
        auto gaps = [davg](int32_t dd) { return ch_gap_double(dd, davg); };
        // anchor k's outputs: global f, p, v; its f and (r, q) also into the ring
        auto put = [&](int k, int32_t fk, int32_t pk, int32_t vk, uint32_t rk, int32_t qk) {
            if (lane == 0) {
                f[k] = (uint32_t)fk;
                p[k] = pk;
                v[k] = vk;
                ring_f[k & (kRing - 1)] = fk;
                ring_rq[k & (kRing - 1)] = make_int2((int)rk, qk);
            }
        };
        unsigned long long evals = 0;
        int st = 0;
        int i = 0;
        while (i < n) {
            // the next kChainBatch anchors and their windows
            int stk[kChainBatch];
            bool batch = n - i >= kChainBatch;
#pragma unroll
            for (int k = 0; k < kChainBatch; k++) {
                if (i + k < n) {
                    const uint64_t rk = a[i + k].r;
                    while (st < i + k && rk - a[st].r > drw) ++st;
                    if (i + k - st > A.max_iter) st = i + k - A.max_iter;
                    stk[k] = st;
                    batch = batch && (i + k - 1 - st > 5);
                }
            }
            if (!batch) {
                // one anchor, either loop of the reference
                const Anchor ai = a[i];
                const int s0 = stk[0];
                st = s0;
                int32_t best = ai.l;
                int bj = -1;
                if (i - 1 - s0 > 5)
                    ch_scan1(S, i, s0, lane, (uint32_t)ai.r, ai.q, ai.l, bw, limq, gapv, best, bj);
                else
                    ch_scan1(S, i, s0, lane, (uint32_t)ai.r, ai.q, ai.l, bw, limq, gaps, best, bj);
                evals += (uint64_t)(i - s0);
                const int32_t fi = __reduce_max_sync(full, best);
                const int32_t pj = __reduce_max_sync(full, best == fi ? bj : -1);
                const int32_t pi = fi > ai.l ? pj : -1;
                const int32_t vi = lane == 0 && pi >= 0 && v[pi] > fi ? v[pi] : fi;
                put(i, fi, pi, vi, (uint32_t)ai.r, ai.q);
                __syncwarp();
                i += 1;
                continue;
            }
            // kChainBatch anchors (all in the vector loop's rounding) over one
            // pass of the shared window: each predecessor's (r, q) and f are
            // loaded once for all of them
            uint32_t rk[kChainBatch];
            int32_t qk[kChainBatch], lk[kChainBatch], best[kChainBatch];
            int bj[kChainBatch];
#pragma unroll
            for (int k = 0; k < kChainBatch; k++) {
                const Anchor ak = a[i + k];
                rk[k] = (uint32_t)ak.r;
                qk[k] = ak.q;
                lk[k] = ak.l;
                best[k] = ak.l;
                bj[k] = -1;
                evals += (uint64_t)(i + k - stk[k]);
            }
            const int lo = i - kRing > stk[0] ? i - kRing : stk[0];  // ring part: [lo, i)
            const int sall = stk[kChainBatch - 1];                    // in every window
            if (sall >= lo) {
                // ring, all windows; ring, own starts; global (windows over kRing)
                const int j0 = i - 1 - lane;
                const int j1 = j0 < sall ? j0 : j0 - 32 * ((j0 - sall) / 32 + 1);
                ch_scanK<false, true>(S, j0, sall, stk, rk, qk, lk, tbl, bw, limq, aq, best, bj);
                ch_scanK<true, true>(S, j1, lo, stk, rk, qk, lk, tbl, bw, limq, aq, best, bj);
                ch_scanK<true, false>(S, ch_first_below(i, lane, lo), stk[0], stk, rk, qk, lk, tbl, bw,
                                      limq, aq, best, bj);
            } else {
                const int j0 = i - 1 - lane;
                const int j1 = j0 < lo ? j0 : j0 - 32 * ((j0 - lo) / 32 + 1);
                ch_scanK<false, true>(S, j0, lo, stk, rk, qk, lk, tbl, bw, limq, aq, best, bj);
                const int j2 = j1 < sall ? j1 : j1 - 32 * ((j1 - sall) / 32 + 1);
                ch_scanK<false, false>(S, j1, sall, stk, rk, qk, lk, tbl, bw, limq, aq, best, bj);
                ch_scanK<true, false>(S, j2, stk[0], stk, rk, qk, lk, tbl, bw, limq, aq, best, bj);
            }
            // merge the lanes, then the predecessors inside the batch (j = i..i+k-1,
            // larger than every window index: '>=' keeps the larger j of a tie)
            int32_t fk[kChainBatch], vk[kChainBatch] = {};
#pragma unroll
            for (int k = 0; k < kChainBatch; k++) {
                int32_t fbest = __reduce_max_sync(full, best[k]);
                int pbest = __reduce_max_sync(full, best[k] == fbest ? bj[k] : -1);
#pragma unroll
                for (int m = 0; m < k; m++) {
                    int32_t sc;
                    const bool ok = ch_score(make_int2((int)rk[m], qk[m]), fk[m], rk[k], qk[k], lk[k], bw,
                                             limq, gapv, sc);
                    if (i + m >= stk[k] && ok && sc >= fbest) {
                        fbest = sc;
                        pbest = i + m;
                    }
                }
                const int32_t pi = fbest > lk[k] ? pbest : -1;
                fk[k] = fbest;
                int32_t vp = 0;
                if (lane == 0) {
                    if (pi >= i) {
#pragma unroll
                        for (int m = 0; m < k; m++)
                            if (pi == i + m) vp = vk[m];
                    } else if (pi >= 0) {
                        vp = v[pi];
                    }
                }
                vk[k] = (pi >= 0 && vp > fbest) ? vp : fbest;
                put(i + k, fbest, pi, vk[k], rk[k], qk[k]);
            }
            __syncwarp();
            i += kChainBatch;
        }
        if (lane == 0 && A.evals) atomicAdd(A.evals, evals);
    }
}

}  // namespace talchain
