// Handle state of the C ABI (include/tal_bsw.h), shared by the translation
// units that implement its entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/tal_bsw.h"
#include "bsw_launch.cuh"

namespace talbsw {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        size_t want = std::max(bytes, cap + cap / 2);
        want = (want + 255) & ~(size_t)255;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// Length bins of the batched form: bin b holds pairs with query length in
// (kBinUpper[b-1], kBinUpper[b]]; within a bin pairs are ordered by target
// length (rows), longest first, in buckets of 8 rows.
constexpr int kNumBins = 21;
__host__ __device__ constexpr int bin_upper(int b) {
    switch (b) {
        case 0: return 32;     case 1: return 64;     case 2: return 96;     case 3: return 128;
        case 4: return 160;    case 5: return 192;    case 6: return 224;    case 7: return 256;
        case 8: return 320;    case 9: return 384;    case 10: return 512;   case 11: return 768;
        case 12: return 1024;  case 13: return 1536;  case 14: return 2048;  case 15: return 3072;
        case 16: return 4096;  case 17: return 6144;  case 18: return 8192;  case 19: return 16384;
        default: return 32767;
    }
}
constexpr int kRowBuckets = 4096;  // len1 / 8, capped
constexpr int kNumBuckets = kNumBins * kRowBuckets;

// Control block on the device for one call: work counters (one per bin),
// error flags, first bad pair, cell count.
struct BatchCtrl {
    int counter[kNumBins + 1];
    int flags;
    long long bad_index;
    unsigned long long cells;
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
};

// One stream per length bin, forked from and joined back into a caller
// stream with events, so the bins' launches run side by side: a bin whose
// last pairs are long no longer holds back the bins after it.
struct BinFork {
    cudaStream_t st[kNumBins] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kNumBins] = {};
    bool ready = false;
    cudaError_t create() {
        if (ready) return cudaSuccess;
        cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
        for (int b = 0; b < kNumBins && e == cudaSuccess; b++) {
            e = cudaStreamCreateWithFlags(&st[b], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join[b], cudaEventDisableTiming);
        }
        ready = e == cudaSuccess;
        return e;
    }
    void release() {
        for (int b = 0; b < kNumBins; b++) {
            if (st[b]) cudaStreamDestroy(st[b]);
            if (join[b]) cudaEventDestroy(join[b]);
            st[b] = nullptr;
            join[b] = nullptr;
        }
        if (fork) cudaEventDestroy(fork);
        fork = nullptr;
        ready = false;
    }
};

// Device buffers of one sort: bucket counts (kNumBuckets), sorted order and
// -- for a serving tick -- the request of each sorted item, bin segments
// {offset, count} x kNumBins, control block.
struct SortBufs {
    int *counts;
    int32_t *order;
    int32_t *order_req;
    int32_t *seg;
    BatchCtrl *ctrl;
};

}  // namespace talbsw

struct tal_bsw_ctx;

namespace talbsw {
// Implemented in bsw_batched.cu; used by the serving loop (bsw_serve.cu).
int bin_cols(const tal_bsw_ctx *h, int b);
// Kernel and tile of length bin b: the autotuner's choice, else the default
// for band w.
KConfig bin_kconfig(const tal_bsw_ctx *h, int b, int w);
LaunchArgs bin_launch_args(const tal_bsw_ctx *h, const SortBufs &sb, LaunchArgs A, int b, int n,
                           const int32_t *seg);
cudaError_t enqueue_sort(tal_bsw_ctx *h, const SortBufs &sb, const DevPair *pairs,
                         const ReqDesc *reqs, int nreqs, int n, cudaStream_t s);
// One launch per bin with count[b] > 0 (all bins when count is NULL), each on
// its own stream of f, longest queries first, forked from and joined into s.
// base: the launch's pair source (pairs / windows / bands, or a request table).
cudaError_t enqueue_bins_forked(tal_bsw_ctx *h, const SortBufs &sb, const LaunchArgs &base,
                                const int *count, int n, int w, BinFork &f, cudaStream_t s);
}  // namespace talbsw

struct tal_bsw_ctx {
    tal_bsw_params prm;
    talbsw::KernelParams kp;
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    talbsw::DevBuf pairs, ref, qer, ctrl, wpair, caps;
    // batched form
    talbsw::DevBuf bcounts, border, bseg, bctrl, btune_seg;
    talbsw::BinFork bfork;
    bool tuned = false;
    talbsw::KConfig bin_cfg[talbsw::kNumBins];
    std::map<std::tuple<const void *, const void *, size_t, const void *, size_t, int, int,
                        const void *, int>, talbsw::GraphEntry> graphs;
    std::mutex mu;
    std::string last_error;
    int64_t last_bad = -1;
    uint64_t launches = 0;
    uint64_t last_cells = 0;
    int pending_status = TAL_OK;
};
