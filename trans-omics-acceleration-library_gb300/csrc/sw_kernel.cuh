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
// shuffle pair, one query load and the loop control.  Every cell is computed
// once, in int32 (exact inside the range the host checks).
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
        SwPair *pp = A.pairs + item;
        const int id = pp->id, nrow = pp->len1, ncol = pp->len2;
        const long long o1 = 2LL * id * A.stride, o2 = o1 + A.stride;
        bool ok = id >= 0 && nrow >= 0 && ncol >= 0 && nrow <= A.maxlen && ncol <= A.maxlen &&
                  o1 >= A.seq_lo && o1 + nrow <= A.seq_hi && o2 >= A.seq_lo && o2 + ncol <= A.seq_hi;
        // every value stays inside the reference's element type
        ok = ok && ((long long)(nrow < ncol ? nrow : ncol) + 1) * (match > 0 ? match : 0) <= A.score_lim;
        if (ok && ncol > A.cols_cap) {
            if (lane == 0) {
                atomicOr(A.err_flags, SWERR_CAPACITY);
                atomicMin(A.err_index, (long long)item);
            }
            continue;
        }
        if (!ok) {
            if (lane == 0) {
                atomicOr(A.err_flags, SWERR_DOMAIN);
                atomicMin(A.err_index, (long long)item);
            }
            continue;
        }
        const uint8_t *s1 = A.seq + (o1 - A.seq_lo);
        const uint8_t *s2 = A.seq + (o2 - A.seq_lo);
        for (int j = lane; j < ncol; j += 32) {
            Q[j] = s2[j];
            Hrow[j] = 0;
            Frow[j] = open;
        }
        __syncwarp();
        int best = 0;
        for (int rb = 0; rb < nrow; rb += 32 * R) {
            int c1[R], e[R], hdiag[R];
            bool rv[R];
#pragma unroll
            for (int k = 0; k < R; k++) {
                const int r = rb + lane * R + k;
                rv[k] = r < nrow;
                c1[k] = rv[k] ? (int)s1[r] : -1;  // never equal to a byte
                e[k] = open;
                hdiag[k] = 0;
            }
            int hout = 0, fout = open;
            const int steps = ncol + 31;
            for (int s = 0; s < steps; s++) {
                int hu = __shfl_up_sync(full, hout, 1);
                int fu = __shfl_up_sync(full, fout, 1);
                const int j = s - lane;
                if (lane == 0 && j < ncol) {
                    hu = Hrow[j];
                    fu = Frow[j];
                }
                if (rv[0] && j >= 0 && j < ncol) {
                    const int q = Q[j];
#pragma unroll
                    for (int k = 0; k < R; k++) {
                        if (rv[k]) {  // hu, fu: H and F' of the row above, this column
                            const int m = hdiag[k] + ((c1[k] == q) ? match : mismatch);
                            const int h = __vimax3_s32_relu(m, e[k], fu);
                            best = best > h ? best : h;
                            const int t = h + open;
                            e[k] = __viaddmax_s32(e[k], ext, t);
                            fu = __viaddmax_s32(fu, ext, t);
                            hdiag[k] = hu;
                            hu = h;
                        }
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

}  // namespace talsw
