// Exclusive scan of 4,096 bucket counts in place, one block of 1,024 threads
// (four buckets per thread): the middle step of the counting sorts that order
// work by length (plain BSW launches, chaining reads).
#pragma once

#include <cuda_runtime.h>

namespace talbsw {

constexpr int kScanBuckets = 4096;  // = 4 x the 1,024 threads of bucket_scan_4096

// static: each translation unit that launches it keeps its own copy
static __global__ void __launch_bounds__(1024) bucket_scan_4096(int *hist) {
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

}  // namespace talbsw
