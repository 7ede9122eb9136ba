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
// Band classes within a length bin: class c < kRingCls holds pairs whose
// band fits a ring of 64 << c columns (2w + 12 <= 64 << c; rings of 64 ..
// 2,048 columns), class kRingCls holds whole rows.  A class whose ring would
// be no smaller than the bin's whole rows folds into the whole-row class.
// A segment is a (length bin, band class).
constexpr int kRingCls = 6;
constexpr int kNumCls = kRingCls + 1;
__host__ __device__ inline int seg_cls(int b, long long w) {
    for (int c = 0; c < kRingCls; c++) {
        const long long W = 64LL << c;
        if (W >= bin_upper(b) + 4) return kRingCls;
        if (2 * w + 12 <= W) return c;
    }
    return kRingCls;
}

// Segment order of the sort (positions 0..kNumSegs-1): first the whole-row
// segments of queries above 384 columns (too wide for the lane kernel),
// bins longest first; then every other segment, bins longest first, classes
// in order.  Each bin's segments are consecutive there, and so is any run of
// bins from bin 0 up, so a launch can take one bin, or all bins up to a
// length, as one range.
constexpr int kRowSegs = 11;  // positions 0..10: bins 20..10, whole rows
constexpr int kNumSegs = kRowSegs + 11 * kRingCls + 10 * kNumCls;
__host__ __device__ inline int seg_index(int b, int c) {
    if (c == kRingCls && b >= 10) return 20 - b;
    return kRowSegs + (b >= 10 ? (20 - b) * kRingCls : 11 * kRingCls + (9 - b) * kNumCls) + c;
}
__host__ __device__ inline int seg_bin(int s) {
    if (s < kRowSegs) return 20 - s;
    const int r = s - kRowSegs;
    return r < 11 * kRingCls ? 20 - r / kRingCls : 9 - (r - 11 * kRingCls) / kNumCls;
}
__host__ __device__ inline int seg_class(int s) {
    if (s < kRowSegs) return kRingCls;
    const int r = s - kRowSegs;
    return r < 11 * kRingCls ? r % kRingCls : (r - 11 * kRingCls) % kNumCls;
}
// First and last position of bin b's ring / lane segments (not its
// whole-row segment when b >= 10).
__host__ __device__ inline int seg_first(int b) { return seg_index(b, 0); }
__host__ __device__ inline int seg_last(int b) { return seg_index(b, b >= 10 ? kRingCls - 1 : kRingCls); }
// The ring of segment s: 64 << c columns for class c < kRingCls, 0 (whole
// rows) otherwise.  The lane kernel's query ring is win / 8 words.
__host__ __device__ inline int seg_window(int s) {
    const int c = seg_class(s);
    return c < kRingCls ? (64 << c) : 0;
}

constexpr int kRowBuckets = 512;  // len1 / 8, capped
constexpr int kNumBuckets = kNumSegs * kRowBuckets;

// Control block on the device for one call: work counters (one per
// segment), error flags, first bad pair, cell count.
struct BatchCtrl {
    int counter[kNumSegs + 1];
    int flags;
    long long bad_index;
    unsigned long long cells;
};

// Arena of the regroup pass (bsw_regroup.cu), which re-scores the SIMD
// groups of the pairs the per-pair kernels flag: the flagged list (the
// kernels' LaunchArgs::flagged), the flagged pairs' classes (band,
// precision, request) in a hash table of kRegroupClasses slots, per-chunk
// class counts and their scan, the marked groups in a hash table, their
// members and the grouped kernel's scratch.  ctr: [0] flagged pairs,
// [1] / [2] marked 16- / 8-bit groups, [3] / [4] grouped-kernel work
// counters, [5] overflow bits; [6] / [7] the last pass's flagged pairs and
// re-scored groups.
constexpr int kRegroupClasses = 1024;  // distinct classes among one call's flagged pairs
constexpr int kRegroupChunk = 2048;
// Shared memory of the regroup pass's first scoring launch: room (after the
// 25 KB of cross-warp exchange of a 16-warp block) for a 16-bit group's
// 256-column ring (bands up to 124) with the lane masks of up to ~2,600
// columns, or an 8-bit group's whole rows.
constexpr int kRegroupSmem1 = 75 * 1024;    // pairs per counting chunk
struct RegroupView {
    int *ctr = nullptr;
    long long *flagged = nullptr;
    int *cls_of = nullptr;
    long long *gidx = nullptr;
    unsigned long long *ckeys = nullptr;
    int4 *cinfo = nullptr;
    int *counts = nullptr, *offsets = nullptr, *totals = nullptr;
    unsigned long long *mhash = nullptr;
    unsigned long long *needh = nullptr;  // per hash slot: the flagged lanes of its group
    unsigned long long *gneed = nullptr;  // per marked group: the same, in list order
    int2 *mlist = nullptr;
    int *mslot = nullptr;
    long long *members = nullptr;
    int4 *ginfo = nullptr;
    int16_t *scratch = nullptr;
    int nchunks = 0, fcap = 0, mcap = 0, hcap = 0, col_cap = 0, slots = 0;
    int smem = 0;          // the second scoring launch's shared memory (the opt-in limit)
    int smem1 = 0, grid1[2] = {0, 0};  // the first launch's (16-, 8-bit): several blocks per SM
};
struct RegroupBufs {
    DevBuf arena;
    RegroupView V;
    // Sizes the arena for ntotal pairs with queries up to cols_cap (grow-only;
    // *grown: the pointers changed, so captured graphs are stale).  Not
    // while a capture is open: it may allocate and synchronises.
    cudaError_t ensure(long long ntotal, int cols_cap, int num_sms, bool *grown);
    void release() { arena.release(); V = RegroupView(); }
};
// Enqueues the regroup pass after a scoring launch of A's pairs (ntotal in
// the launch's pair space; nreq requests when A.reqs is set).  Flags it
// cannot handle (the tables overflowed) end as ERR_FLAGCAP in A.err_flags.
cudaError_t enqueue_regroup(const RegroupView &V, LaunchArgs A, int nreq, long long ntotal,
                            int num_sms, cudaStream_t s, uint64_t *launches);
// The flagged-list fields of a scoring launch that feeds the pass.
inline void attach_regroup(LaunchArgs &A, const RegroupView &V) {
    A.flagged = V.flagged;
    A.nflagged = V.ctr;
    A.flag_cap = V.fcap;
}

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
};

// Streams forked from and joined back into a caller stream with events, so
// the segments' launches run side by side: a segment whose last pairs are
// long no longer holds back the ones after it.  Captured in a graph, segment
// s runs on stream s % kForkStreams (one branch per segment measured 1 %
// slower on the mixed batch); launched directly (a serving tick, whose
// segment counts the host knows), the non-empty segments take the streams
// one each while they last, and the shortest-query segments after that queue
// behind the shortest ones before them, not behind the longest -- launches on
// one stream run in order (and a process has CUDA_DEVICE_MAX_CONNECTIONS, at
// most 32, hardware queues).
constexpr int kForkStreams = 32;
struct BinFork {
    cudaStream_t st[kForkStreams] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kForkStreams] = {};
    bool ready = false;
    cudaError_t create() {
        if (ready) return cudaSuccess;
        cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
        for (int b = 0; b < kForkStreams && e == cudaSuccess; b++) {
            e = cudaStreamCreateWithFlags(&st[b], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join[b], cudaEventDisableTiming);
        }
        ready = e == cudaSuccess;
        return e;
    }
    void release() {
        for (int b = 0; b < kForkStreams; b++) {
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
// -- for a serving tick -- the request of each sorted item, segments
// {offset, count} x kNumSegs, control block.
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
// Kernel and tile of segment seg: the autotuner's choice, else the default
// for band w.
KConfig seg_kconfig(const tal_bsw_ctx *h, int seg, int w);
LaunchArgs seg_launch_args(const tal_bsw_ctx *h, const SortBufs &sb, LaunchArgs A, int seg, int n);
// Sorts the pairs into (segment, target-length bucket) order.  The pairs are
// base's (pairs, bands wpair / w) or, when base.reqs is set, the
// concatenation of the nreqs requests of that table.
cudaError_t enqueue_sort(tal_bsw_ctx *h, const SortBufs &sb, const LaunchArgs &base, int nreqs,
                         int n, cudaStream_t s);
// A serving tick's launches (count: pairs per segment, known on the host):
// bins above lane_bin with G lanes per pair, bins 0..lane_bin in one
// lane-kernel launch.
cudaError_t enqueue_tick(tal_bsw_ctx *h, const SortBufs &sb, const LaunchArgs &base,
                         const int *count, int lane_bin, BinFork &f, cudaStream_t s);
// One launch per segment with count[seg] > 0 (all when count is NULL),
// longest queries first, on streams of f forked from and joined into s;
// latency: per-pair latency configurations instead of the tuned ones.
cudaError_t enqueue_segs_forked(tal_bsw_ctx *h, const SortBufs &sb, const LaunchArgs &base,
                                const int *count, int n, int w, BinFork &f, cudaStream_t s,
                                bool latency);
}  // namespace talbsw

struct tal_bsw_ctx {
    tal_bsw_params prm;
    talbsw::KernelParams kp;
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    talbsw::DevBuf pairs, ref, qer, ctrl, wpair, caps;
    talbsw::DevBuf gscratch;  // grouped scoring: one row slot per warp
    talbsw::RegroupBufs regroup;  // exact scoring of flagged pairs' SIMD groups
    talbsw::DevBuf porder;  // plain launch: work order by target length, and its buckets
    // seed extension: reference, reads, copy jobs + seeds, pairs, arenas, regions
    talbsw::DevBuf xref, xreads, xjobs, xpairs, xtarena, xqarena, xout, xretry;
    // host-buffer calls in chunks: copies on cstream, chunk k's scoring waits on cev[k]
    cudaStream_t cstream = nullptr;
    cudaEvent_t cev[4] = {};
    // around the last scoring launch (plain calls): its device time
    cudaEvent_t kev0 = nullptr, kev1 = nullptr;
    float last_kernel_ms = 0.f;
    // batched form
    talbsw::DevBuf bcounts, border, bseg, bctrl, btune_seg;
    talbsw::BinFork bfork;
    bool tuned = false;
    talbsw::KConfig bin_cfg[talbsw::kNumSegs];
    std::map<std::tuple<const void *, const void *, size_t, const void *, size_t, int, int,
                        const void *, int>, talbsw::GraphEntry> graphs;
    std::mutex mu;
    std::string last_error;
    int64_t last_bad = -1;
    uint64_t launches = 0;
    uint64_t last_cells = 0;
    int pending_status = TAL_OK;
};
