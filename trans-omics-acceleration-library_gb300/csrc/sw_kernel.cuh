// Unbanded Smith-Waterman scores on sm_103a: the reference's PairWiseSW_8 /
// _16 / _32::getScores (src/alignment/Smith-Waterman/PairWiseSW_16.cpp:151-229,
// cell MAIN_CODE :62-76), one warp per pair, rows in bands of 32.
//
// Per cell (row i of seq1, column j of seq2):
//   M = H(i-1, j-1) + (seq1[i] == seq2[j] ? match : mismatch)
//   H = max(M, E, F, 0)
//   E' = max(H + open, E + extend)   -> the next column
//   F' = max(F + extend, H + open)   -> the next row
// E = open at the start of a row; the row above the first holds H = 0, F = open.
// The answer is the largest H.
//
// Lane t of the warp owns rows [R*t, R*t + R) of a band of 32*R rows and walks
// the columns one step behind lane t - 1 (an anti-diagonal wavefront): at
// step s it computes column s - t of its R rows, top to bottom, taking H and
// F' of the row above its block from lane t - 1 through a shuffle (lane t - 1
// computed that column at step s - 1); each row keeps its diagonal H and its
// E in registers.  Lane 31 writes its bottom row's H and F' to shared memory,
// where lane 0 of the next band reads them.  R rows per lane share one
// shuffle pair, one query load and the loop control.  E and F' are kept less
// the open weight: V = max(E + open, M, 0), H = max(F + open, V), and
// E - open <- max(E - open + extend, H), the same for F' (four DPX add-max
// instructions a cell).  Every cell is computed once, in int32 (exact inside
// the range the host checks), or two pairs per warp in int16x2 below.
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

#ifndef TALBSW_DYNAMIC_SMEM
#define TALBSW_DYNAMIC_SMEM(name) extern __shared__ __align__(16) unsigned char name[]
#endif

namespace talsw {

struct SwPair {  // PairWiseSW.h:44-49
    int32_t id;
    int16_t len1, len2;
    int32_t score;
};

enum : int { SWERR_DOMAIN = 1, SWERR_CAPACITY = 2 };

struct SwArgs {
    SwPair *pairs;
    // seq holds bytes [seq_lo, seq_hi) of the caller's sequence buffer; pair
    // k's seq1 starts at 2*id*stride, its seq2 at (2*id + 1)*stride
    const uint8_t *seq;
    long long seq_lo, seq_hi, stride;
    int n;
    int cols_cap;     // shared-memory row length (longest seq2 of the launch)
    int maxlen;       // longest sequence of the precision
    int score_lim;    // largest score the precision holds
    int match, mismatch, open, ext;
    const int32_t *order;  // optional work order (pair indices), else 0..n-1
    int *work_counter;
    unsigned long long *cells;  // optional: len1 * len2 summed
    int *err_flags;
    long long *err_index;
};

__host__ __device__ __forceinline__ size_t sw_warp_smem_bytes(int cols_cap) {
    // H and F' rows (int32) and seq2 (bytes)
    return ((size_t)cols_cap * 9 + 16 + 15) & ~(size_t)15;
}

constexpr int kSwRows = 8;  // rows per lane

// 0 if pair p is inside the exact range and fits the launch's rows, else the
// error flag it raises.
__device__ __forceinline__ int sw_pair_check(const SwArgs &A, const SwPair &p) {
    const long long o1 = 2LL * p.id * A.stride, o2 = o1 + A.stride;
    bool ok = p.id >= 0 && p.len1 >= 0 && p.len2 >= 0 && p.len1 <= A.maxlen && p.len2 <= A.maxlen &&
              o1 >= A.seq_lo && o1 + p.len1 <= A.seq_hi && o2 >= A.seq_lo && o2 + p.len2 <= A.seq_hi;
    // every value stays inside the reference's element type
    const int mn = p.len1 < p.len2 ? p.len1 : p.len2;
    ok = ok && ((long long)mn + 1) * (A.match > 0 ? A.match : 0) <= A.score_lim;
    if (!ok) return SWERR_DOMAIN;
    return p.len2 > A.cols_cap ? SWERR_CAPACITY : 0;
}

// Work order: pairs by their longer sequence, longest first, in buckets of 8
// bases (a counting sort).  The longest pairs start first, so none is left
// to run alone at the end, and neighbours in the order have about the same
// lengths, which the two-pairs-per-warp kernel walks together.
constexpr int kSwBuckets = 128;

__device__ __forceinline__ int sw_bucket(const SwPair &p) {
    int l = p.len1 > p.len2 ? p.len1 : p.len2;
    l = l < 0 ? 0 : l > 8 * kSwBuckets - 1 ? 8 * kSwBuckets - 1 : l;
    return (kSwBuckets - 1) - (l >> 3);
}

__global__ void sw_bucket_count(const SwPair *pairs, int n, int *hist) {
    __shared__ int sh[kSwBuckets];
    for (int t = threadIdx.x; t < kSwBuckets; t += blockDim.x) sh[t] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&sh[sw_bucket(pairs[i])], 1);
    __syncthreads();
    for (int t = threadIdx.x; t < kSwBuckets; t += blockDim.x)
        if (sh[t]) atomicAdd(&hist[t], sh[t]);
}

__global__ void sw_bucket_offsets(int *hist) {  // one thread: counts -> first positions
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int run = 0;
        for (int b = 0; b < kSwBuckets; b++) {
            const int c = hist[b];
            hist[b] = run;
            run += c;
        }
    }
}

__global__ void sw_bucket_scatter(const SwPair *pairs, int n, int *offs, int32_t *order) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        order[atomicAdd(&offs[sw_bucket(pairs[i])], 1)] = i;
}

template <int R>
__global__ void __launch_bounds__(128) sw_wave_kernel(SwArgs A) {
    TALBSW_DYNAMIC_SMEM(smem_raw);
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    unsigned char *wsm = smem_raw + (size_t)wib * sw_warp_smem_bytes(A.cols_cap);
    int *Hrow = reinterpret_cast<int *>(wsm);
    int *Frow = Hrow + A.cols_cap;
    uint8_t *Q = reinterpret_cast<uint8_t *>(Frow + A.cols_cap);
    const int match = A.match, mismatch = A.mismatch, open = A.open, ext = A.ext;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.work_counter, 1);
        item = __shfl_sync(full, item, 0);
        if (item >= A.n) break;
        const int idx = A.order ? A.order[item] : item;
        SwPair *pp = A.pairs + idx;
        const SwPair pv = *pp;
        const int bad = sw_pair_check(A, pv);
        if (bad) {
            if (lane == 0) {
                atomicOr(A.err_flags, bad);
                atomicMin(A.err_index, (long long)idx);
            }
            continue;
        }
        const int nrow = pv.len1, ncol = pv.len2;
        const long long o1 = 2LL * pv.id * A.stride, o2 = o1 + A.stride;
        const uint8_t *s1 = A.seq + (o1 - A.seq_lo);
        const uint8_t *s2 = A.seq + (o2 - A.seq_lo);
        for (int j = lane; j < ncol; j += 32) {
            Q[j] = s2[j];
            Hrow[j] = 0;
            Frow[j] = 0;  // F' - open of the row above the first
        }
        __syncwarp();
        int best = 0;
        for (int rb = 0; rb < nrow; rb += 32 * R) {
            // rows past seq1 hold a code equal to no byte: their cells take
            // gaps and mismatches from the real cells above, stay below the
            // best real cell and feed nothing that is read
            int c1[R], e[R], hdiag[R];
#pragma unroll
            for (int k = 0; k < R; k++) {
                const int r = rb + lane * R + k;
                c1[k] = r < nrow ? (int)s1[r] : -1;
                e[k] = 0;  // E - open at the start of a row
                hdiag[k] = 0;
            }
            int hout = 0, fout = 0;
            const int steps = ncol + 31;
            for (int s = 0; s < steps; s++) {
                int hu = __shfl_up_sync(full, hout, 1);
                int fu = __shfl_up_sync(full, fout, 1);
                const int j = s - lane;
                if (lane == 0 && j < ncol) {
                    hu = Hrow[j];
                    fu = Frow[j];
                }
                if (j >= 0 && j < ncol) {
                    const int q = Q[j];
                    int hp = 0;
#pragma unroll
                    for (int k = 0; k < R; k++) {
                        // hu: H of the row above, this column; e, fu hold E
                        // and F' less the open weight:
                        //   H = max(M, E + open, F + open, 0)
                        //   E - open <- max(E - open + extend, H), F the same
                        const int m = hdiag[k] + ((c1[k] == q) ? match : mismatch);
                        const int v = __viaddmax_s32_relu(e[k], open, m);
                        const int h = __viaddmax_s32(fu, open, v);
                        if (k & 1) best = __vimax3_s32(best, hp, h);
                        else if (k == R - 1) best = best > h ? best : h;
                        hp = h;
                        e[k] = __viaddmax_s32(e[k], ext, h);
                        fu = __viaddmax_s32(fu, ext, h);
                        hdiag[k] = hu;
                        hu = h;
                    }
                    hout = hu;
                    fout = fu;
                    if (lane == 31) {
                        Hrow[j] = hout;
                        Frow[j] = fout;
                    }
                }
            }
            __syncwarp();  // the band's last row, in shared memory, for the next band
        }
        best = (int)__reduce_max_sync(full, (unsigned)best);
        if (lane == 0) {
            pp->score = best;
            if (A.cells) atomicAdd(A.cells, (unsigned long long)nrow * (unsigned long long)ncol);
        }
        __syncwarp();
    }
}

// Two pairs per warp in int16x2: the low halves of every register score pair
// A, the high halves pair B (DPX 16x2 instructions: one instruction, two
// cells), for precisions whose values fit int16 (8- and 16-bit kernels).  The
// warp walks the larger of the two pairs' rows and columns; a pair's rows
// past its seq1 read the code 0x100 and its columns past its seq2 the code
// 0x200, which equal nothing, so those cells only mismatch or open gaps from
// its real cells and never exceed its best real cell (the weights are not
// positive) -- the reference pads its SIMD groups the same way
// (PairWiseSW_16.cpp:295-320, DUMMY1 / DUMMY2).
__host__ __device__ __forceinline__ size_t sw2_warp_smem_bytes(int cols_cap) {
    // packed H and F' rows and packed seq2 codes, 4 B each per column
    return ((size_t)cols_cap * 12 + 16 + 15) & ~(size_t)15;
}

template <int R>
__global__ void __launch_bounds__(128) sw_wave2_kernel(SwArgs A) {
    TALBSW_DYNAMIC_SMEM(smem_raw);
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    unsigned char *wsm = smem_raw + (size_t)wib * sw2_warp_smem_bytes(A.cols_cap);
    uint32_t *Hrow = reinterpret_cast<uint32_t *>(wsm);
    uint32_t *Frow = Hrow + A.cols_cap;
    uint32_t *Q = Frow + A.cols_cap;
    auto pk = [](int lo, int hi) -> uint32_t { return ((uint32_t)lo & 0xffffu) | ((uint32_t)hi << 16); };
    const uint32_t open2 = pk(A.open, A.open), ext2 = pk(A.ext, A.ext);
    const uint32_t match2 = pk(A.match, A.match);
    const uint32_t ones2 = 0x00010001u, neg2 = 0x80008000u;
    // -(match - mismatch) in 16 bits: the host keeps match - mismatch <= 2^15
    const uint32_t negdiff = (uint32_t)(-(A.match - A.mismatch)) & 0xffffu;

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.work_counter, 2);
        item = __shfl_sync(full, item, 0);
        if (item >= A.n) break;
        // pair A = item, pair B = item + 1 (absent past the end); a pair that
        // fails its checks is reported and scored as empty
        int idx[2] = {-1, -1};
        int len1[2] = {0, 0}, len2[2] = {0, 0};
        const uint8_t *s1[2] = {nullptr, nullptr}, *s2[2] = {nullptr, nullptr};
        bool real[2] = {false, false};
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (item + h >= A.n) continue;
            const int it = A.order ? A.order[item + h] : item + h;
            idx[h] = it;
            const SwPair p = A.pairs[it];
            const int bad = sw_pair_check(A, p);
            if (bad) {
                if (lane == 0) {
                    atomicOr(A.err_flags, bad);
                    atomicMin(A.err_index, (long long)it);
                }
                continue;
            }
            real[h] = true;
            len1[h] = p.len1;
            len2[h] = p.len2;
            s1[h] = A.seq + (2LL * p.id * A.stride - A.seq_lo);
            s2[h] = s1[h] + A.stride;
        }
        const int nrow = len1[0] > len1[1] ? len1[0] : len1[1];
        const int ncol = len2[0] > len2[1] ? len2[0] : len2[1];
        for (int j = lane; j < ncol; j += 32) {
            const int qa = j < len2[0] ? (int)s2[0][j] : 0x200;
            const int qb = j < len2[1] ? (int)s2[1][j] : 0x200;
            Q[j] = pk(qa, qb);
            Hrow[j] = 0u;
            Frow[j] = 0u;  // F' - open of the row above the first
        }
        __syncwarp();
        uint32_t best = 0u;
        for (int rb = 0; rb < nrow; rb += 32 * R) {
            uint32_t c1[R], e[R], hdm[R];
#pragma unroll
            for (int k = 0; k < R; k++) {
                const int r = rb + lane * R + k;
                const int ca = r < len1[0] ? (int)s1[0][r] : 0x100;
                const int cb = r < len1[1] ? (int)s1[1][r] : 0x100;
                c1[k] = pk(ca, cb);
                e[k] = 0u;        // E - open at the start of a row
                hdm[k] = match2;  // diagonal H (0) + match
            }
            uint32_t hout = 0u, fout = 0u;
            const int steps = ncol + 31;
            for (int s = 0; s < steps; s++) {
                uint32_t hu = __shfl_up_sync(full, hout, 1);
                uint32_t fu = __shfl_up_sync(full, fout, 1);
                const int j = s - lane;
                if (lane == 0 && j < ncol) {
                    hu = Hrow[j];
                    fu = Frow[j];
                }
                if (j >= 0 && j < ncol) {
                    const uint32_t q = Q[j];
                    uint32_t hp = 0u;
#pragma unroll
                    for (int k = 0; k < R; k++) {
                        // per half: codes differ -> 1, else 0; M = diagonal
                        // H + match - that * (match - mismatch)
                        const uint32_t d = __vimin3_u16x2(c1[k] ^ q, ones2, ones2);
                        const uint32_t m = __viaddmax_s16x2(hdm[k], d * negdiff, neg2);
                        const uint32_t v = __viaddmax_s16x2_relu(e[k], open2, m);
                        const uint32_t h = __viaddmax_s16x2(fu, open2, v);
                        if (k & 1) best = __vimax3_s16x2_relu(best, hp, h);
                        else if (k == R - 1) best = __vimax3_s16x2_relu(best, h, h);
                        hp = h;
                        e[k] = __viaddmax_s16x2(e[k], ext2, h);
                        fu = __viaddmax_s16x2(fu, ext2, h);
                        // both halves stay in [0, 2^15): a 32-bit add is exact
                        hdm[k] = hu + match2;
                        hu = h;
                    }
                    hout = hu;
                    fout = fu;
                    if (lane == 31) {
                        Hrow[j] = hout;
                        Frow[j] = fout;
                    }
                }
            }
            __syncwarp();
        }
        const unsigned ba = __reduce_max_sync(full, best & 0xffffu);
        const unsigned bb = __reduce_max_sync(full, best >> 16);
        if (lane == 0) {
            if (real[0]) {
                A.pairs[idx[0]].score = (int)ba;
                if (A.cells) atomicAdd(A.cells, (unsigned long long)len1[0] * (unsigned long long)len2[0]);
            }
            if (real[1]) {
                A.pairs[idx[1]].score = (int)bb;
                if (A.cells) atomicAdd(A.cells, (unsigned long long)len1[1] * (unsigned long long)len2[1]);
            }
        }
        __syncwarp();
    }
}

}  // namespace talsw
