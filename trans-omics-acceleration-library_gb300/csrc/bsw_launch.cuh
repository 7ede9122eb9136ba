// Launch configuration of the scoring kernel: lanes per pair (G), columns per
// lane (K), warps per block, grid size.  Shared by the C ABI entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdlib.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "bsw_kernel.cuh"
#include "bsw_lane.cuh"

namespace talbsw {

struct KConfig {
    int G, K;
};

// Short queries: one lane per pair (G = 1, bsw_lane_kernel), the rows of 32
// pairs interleaved in a warp's shared memory.  Longer queries: G lanes per
// pair (bsw_kernel), narrow bands with few lanes (more pairs share each
// warp-instruction of per-row bookkeeping), wide bands with more lanes so a
// row is not a long serial walk.  TAL_BSW_G / TAL_BSW_K override (tuning).
constexpr int kLaneMaxCols = 384;

// Ring size for a launch whose pairs all have band <= w and query length
// <= cols_cap: 0 (whole rows) unless a ring is smaller.
inline int lane_window(long long w, int cols_cap) {
    if (w < 0) return 0;
    // sized exactly (a multiple of 32) when the lane kernel takes it, a power
    // of two when the G kernel does (TAL_BSW_POW2_RING: always, for tuning)
    int W = lane_ring_exact(w);
    if (W - 4 > kLaneMaxCols || getenv("TAL_BSW_POW2_RING")) W = lane_window_for(w);
    return W < cols_cap + 4 ? W : 0;
}

inline KConfig choose_config(int w, int cols_cap, int win = 0) {
    long long bw = std::min<long long>(2LL * std::max(w, 0) + 1, (long long)cols_cap);
    KConfig c;
    c.K = 4;
    if ((win > 0 ? win - 4 : cols_cap) <= kLaneMaxCols) c.G = 1;
    else if (bw <= 64) c.G = 4;
    else if (bw <= 256) c.G = 8;
    else if (bw <= 640) c.G = 16;
    else c.G = 32;
    if (const char *e = getenv("TAL_BSW_G")) {
        int g = atoi(e);
        if (g == 1 || g == 4 || g == 8 || g == 16 || g == 32) c.G = g;
    }
    if (const char *e = getenv("TAL_BSW_K")) {
        int k = atoi(e);
        if (k == 2 || k == 4) c.K = k;
    }
    return c;
}

// Resident blocks per SM of kernel kern at (threads, smem) on the current
// device.  The shared-memory opt-in is raised to the device limit once per
// kernel and device, and the occupancy is cached: both queries cost
// microseconds, and a serving tick issues dozens of launches.
inline cudaError_t resident_blocks(const void *kern, int threads, size_t smem, size_t smem_optin,
                                   int *bps) {
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, int, size_t>, int> occ;
    static std::map<std::pair<const void *, int>, bool> raised;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_tuple(kern, dev, threads, smem);
    auto it = occ.find(key);
    if (it != occ.end()) {
        *bps = it->second;
        return cudaSuccess;
    }
    if (!raised[std::make_pair(kern, dev)]) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_optin);
        if (e != cudaSuccess) return e;
        raised[std::make_pair(kern, dev)] = true;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, kern, threads, smem);
    if (e == cudaSuccess) occ[key] = *bps;
    return e;
}

template <int G, int K>
inline cudaError_t launch_gk(const LaunchArgs &A, int num_sms, size_t smem_optin, cudaStream_t s) {
    auto kern = bsw_kernel<G, K>;
    const size_t wbytes = warp_smem_bytes(A.cols_cap, A.rows_cap, G, A.win);
    int wpb = 4;
    while (wpb > 1 && (size_t)wpb * wbytes * 2 > smem_optin) wpb >>= 1;
    const size_t smem = (size_t)wpb * wbytes;
    if (smem > smem_optin) return cudaErrorInvalidValue;
    int bps = 0;
    cudaError_t e = resident_blocks((const void *)kern, 32 * wpb, smem, smem_optin, &bps);
    if (e != cudaSuccess) return e;
    if (bps < 1) return cudaErrorInvalidConfiguration;
    long long blocks = (long long)bps * num_sms;
    const long long pairs_per_block = (long long)wpb * (32 / G);
    const long long need = ((long long)A.n + pairs_per_block - 1) / pairs_per_block;
    if (blocks > need) blocks = std::max<long long>(need, 1);
    kern<<<(unsigned)blocks, 32 * wpb, smem, s>>>(A);
    return cudaGetLastError();
}

inline cudaError_t launch_lane(const LaunchArgs &A, int num_sms, size_t smem_optin, cudaStream_t s) {
    const bool sym = A.P.o_del == A.P.o_ins && A.P.e_del == A.P.e_ins;
    int v = sym ? 3 : 1;
    if (const char *ev = getenv("TAL_BSW_LV")) v = atoi(ev) & 3;
    if (!sym) v &= 1;
    if (A.win > 0 && (A.win & (A.win - 1)) != 0) v |= 4;  // a ring that is not a power of two
    void (*kern)(LaunchArgs);
    switch (v) {
        case 0: kern = bsw_lane_kernel<0>; break;
        case 1: kern = bsw_lane_kernel<1>; break;
        case 2: kern = bsw_lane_kernel<2>; break;
        case 3: kern = bsw_lane_kernel<3>; break;
        case 4: kern = bsw_lane_kernel<4>; break;
        case 5: kern = bsw_lane_kernel<5>; break;
        case 6: kern = bsw_lane_kernel<6>; break;
        default: kern = bsw_lane_kernel<7>; break;
    }
    const size_t wbytes = lane_warp_smem_bytes(A.cols_cap, A.win);
    int wpb = 4;
    while (wpb > 1 && (size_t)wpb * wbytes > 48 * 1024) wpb >>= 1;
    const size_t smem = (size_t)wpb * wbytes;
    if (smem > smem_optin) return cudaErrorInvalidValue;
    int bps = 0;
    cudaError_t e = resident_blocks((const void *)kern, 32 * wpb, smem, smem_optin, &bps);
    if (e != cudaSuccess) return e;
    if (bps < 1) return cudaErrorInvalidConfiguration;
    long long blocks = (long long)bps * num_sms;
    const long long need = ((long long)A.n + 32LL * wpb - 1) / (32LL * wpb);
    if (blocks > need) blocks = std::max<long long>(need, 1);
    kern<<<(unsigned)blocks, 32 * wpb, smem, s>>>(A);
    return cudaGetLastError();
}

// Lowest-latency configuration for queries up to cols_cap columns: one lane
// walks a whole pair in the lane kernel, so a pair of many hundred columns
// holds its warp for milliseconds; G lanes per pair split each row.  Used
// when a launch is too small to fill the GPU, where the slowest pair, not the
// cells per second, sets the time.
constexpr int kLongQuery = 768;  // queries above this always run with G lanes per pair in ticks

inline KConfig latency_config(int cols_cap, int win) {
    if (cols_cap <= 256) return choose_config(0, cols_cap, win);
    KConfig c;
    c.K = 4;
    c.G = cols_cap <= 512 ? 8 : cols_cap <= 1024 ? 16 : 32;
    return c;
}

// Shared memory one warp of the chosen configuration needs.
inline size_t config_smem(const KConfig &c, int cols_cap, int rows_cap, int win = 0) {
    if (c.G == 1) return lane_warp_smem_bytes(cols_cap, win);
    return warp_smem_bytes(cols_cap, rows_cap, c.G, win);
}

// Widens the lanes per pair (fewer pairs per warp, less shared memory per
// warp) until one warp's rows fit a block.
inline KConfig fit_config(KConfig c, int cols_cap, size_t smem_optin, int win = 0) {
    while (c.G < 32 && config_smem(c, cols_cap, 1, win) > smem_optin) c.G = c.G == 1 ? 4 : c.G * 2;
    return c;
}

inline cudaError_t launch_config(const LaunchArgs &A, const KConfig &c, int num_sms,
                                 size_t smem_optin, cudaStream_t s) {
    if (c.G == 1) return launch_lane(A, num_sms, smem_optin, s);
    switch (c.G * 10 + c.K) {
        case 44: return launch_gk<4, 4>(A, num_sms, smem_optin, s);
        case 42: return launch_gk<4, 2>(A, num_sms, smem_optin, s);
        case 84: return launch_gk<8, 4>(A, num_sms, smem_optin, s);
        case 82: return launch_gk<8, 2>(A, num_sms, smem_optin, s);
        case 164: return launch_gk<16, 4>(A, num_sms, smem_optin, s);
        case 162: return launch_gk<16, 2>(A, num_sms, smem_optin, s);
        case 324: return launch_gk<32, 4>(A, num_sms, smem_optin, s);
        case 322: return launch_gk<32, 2>(A, num_sms, smem_optin, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace talbsw
