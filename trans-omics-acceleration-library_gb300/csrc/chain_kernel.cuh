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
constexpr int kChainBuckets = 4096;  // = 4 x the 1024 threads of ch_bucket_offsets

__device__ __forceinline__ int ch_bucket(const int64_t *offsets, int k) {
    int64_t n = offsets[k + 1] - offsets[k];
    n = n < 0 ? 0 : n >> 4;
    return (kChainBuckets - 1) - (int)(n > kChainBuckets - 1 ? kChainBuckets - 1 : n);
}

__global__ void ch_bucket_count(const int64_t *offsets, int n_reads, int *hist) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_reads; k += gridDim.x * blockDim.x)
        atomicAdd(&hist[ch_bucket(offsets, k)], 1);
}

// Counts -> first positions (exclusive scan), one block of 1024 threads, four
// buckets per thread.
__global__ void __launch_bounds__(1024) ch_bucket_offsets(int *hist) {
    __shared__ int wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int c[4], run = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        c[k] = hist[4 * t + k];
        run += c[k];
    }
    int incl = run;  // inclusive scan of the per-thread sums over the warp
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        int x = wsum[lane];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        wsum[lane] = x;  // inclusive over warps
    }
    __syncthreads();
    int pos = incl - run + (w > 0 ? wsum[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        hist[4 * t + k] = pos;
        pos += c[k];
    }
}

__global__ void ch_bucket_scatter(const int64_t *offsets, int n_reads, int *offs, int32_t *order) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_reads; k += gridDim.x * blockDim.x)
        order[atomicAdd(&offs[ch_bucket(offsets, k)], 1)] = k;
}

// Best (score, largest j) of lane `lane`'s share of the predecessors of
// anchor i: j = i-1-lane, i-1-lane-32, ... >= st.  GAP: the path's gap cost.
template <typename GAP>
__device__ __forceinline__ void ch_scan(const int2 *rq, const uint32_t *f, int i, int st, int lane,
                                        uint32_t ri, int32_t qi, int32_t li, const ChainArgs &A,
                                        GAP gap, int32_t &best, int &bj) {
#pragma unroll 4
    for (int j = i - 1 - lane; j >= st; j -= 32) {
        const int2 c = rq[j];
        const int32_t ddr = (int32_t)(ri - (uint32_t)c.x);
        const int32_t ddq = ch_sub(qi, c.y);
        const int32_t x = ch_sub(ddr, ddq);
        const int32_t dd = x < 0 ? ch_sub(0, x) : x;
        const bool ok = !(dd > A.bw || ddr == 0 || ddq <= 0 || ddq > A.dq || ddq > A.dr);
        int32_t oc = ddr < ddq ? ddr : ddq;
        oc = oc < li ? oc : li;
        const int32_t sc = ch_sub(ch_add((int32_t)f[j], oc), gap(dd));
        if (ok && sc > best) {
            best = sc;
            bj = j;
        }
    }
}

__global__ void __launch_bounds__(128) chain_kernel(ChainArgs A) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint64_t drw = (uint64_t)(uint32_t)A.dr;
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
        // (r, q) words the predecessor scan reads
        unsigned long long sum = 0;
        int neg = 0;
        for (int i = lane; i < n; i += 32) {
            const Anchor ai = a[i];
            neg |= ai.l < 0;
            sum += (uint32_t)ai.l;
            rq[i] = make_int2((int)(uint32_t)ai.r, ai.q);
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
        __syncwarp();
        const float avg = __fdiv_rn(__ull2float_rn(sum), __ll2float_rn(n64));
        const float aq = __double2float_rn(__dmul_rn(0.01, (double)avg));
        const double davg = (double)avg;
        unsigned long long evals = 0;
        int st = 0;
        for (int i = 0; i < n; i++) {
            const Anchor ai = a[i];
            while (st < i && ai.r - a[st].r > drw) ++st;
            if (i - st > A.max_iter) st = i - A.max_iter;
            const uint32_t ri = (uint32_t)ai.r;
            int32_t best = ai.l;
            int bj = -1;
            // warp-uniform: the reference's vector loop (> 6 predecessors,
            // float gap cost) or its scalar loop (double gap cost)
            if (i - 1 - st > 5)
                ch_scan(rq, f, i, st, lane, ri, ai.q, ai.l, A,
                        [aq](int32_t dd) { return ch_gap_float(dd, aq); }, best, bj);
            else
                ch_scan(rq, f, i, st, lane, ri, ai.q, ai.l, A,
                        [davg](int32_t dd) { return ch_gap_double(dd, davg); }, best, bj);
            evals += (uint64_t)(i - st);
            const int32_t fi = __reduce_max_sync(full, best);
            const int32_t pj = __reduce_max_sync(full, best == fi ? bj : -1);
            if (lane == 0) {
                const int32_t pi = fi > ai.l ? pj : -1;
                f[i] = (uint32_t)fi;
                p[i] = pi;
                v[i] = (pi >= 0 && v[pi] > fi) ? v[pi] : fi;
            }
            __syncwarp();
        }
        if (lane == 0 && A.evals) atomicAdd(A.evals, evals);
    }
}

}  // namespace talchain
