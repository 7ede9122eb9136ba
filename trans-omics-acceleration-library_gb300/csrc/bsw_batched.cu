// Batched form of the scorer (tal_bsw_scores_batched*): one call scores a
// large, mixed batch -- uneven lengths, bands and 8/16-bit pairs -- as a CUDA
// graph of
//   1. a counting sort of the pairs into (segment, 8-row target bucket)
//      order on the device, a segment being a query-length bin and a band
//      class (bsw_ctx.h);
//   2. one persistent launch per segment, side by side on forked streams,
//      each taking its pairs from the sorted order through a work counter,
//      with the kernel and tile chosen for that segment by an autotuner on
//      the first call, and -- for the lane-per-pair kernel -- row rings sized
//      to the segment's band class.
// Sorting makes the pairs that share a warp alike in shape (same row count,
// similar band widths), which is what the lane-per-pair kernel needs to keep
// its lanes busy, and lets each segment size its shared memory to its pairs.
// Outputs do not depend on the order pairs are scored in.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <climits>
#include <string>
#include <vector>

#include "bsw_ctx.h"

namespace talbsw {

__device__ __forceinline__ int bin_of(int len2) {
    int b = 0;
#pragma unroll
    for (int k = 0; k < kNumBins - 1; k++) b += (len2 > bin_upper(k)) ? 1 : 0;
    return b;
}

__device__ __forceinline__ int bucket_of(const DevPair &p, int w) {
    const int b = bin_of(p.len2);
    const int r = imin(imax(p.len1, 0) >> 3, kRowBuckets - 1);
    return seg_index(b, seg_cls(b, w)) * kRowBuckets + r;
}

// Sort key of work item k: of the launch's pairs (band wpair[k] or w), or --
// for a serving tick -- of the request whose range [first, first + n) holds
// k (binary search over the tick's request table).
__device__ __forceinline__ int item_key(const LaunchArgs &A, int nreqs, int k, int &req, int &local) {
    if (!A.reqs) {
        req = -1;
        local = k;
        return bucket_of(A.pairs[k], A.wpair ? A.wpair[k] : A.w);
    }
    int lo = 0, hi = nreqs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.reqs[mid].first <= k) lo = mid;
        else hi = mid - 1;
    }
    const ReqDesc &d = A.reqs[lo];
    req = lo;
    local = k - d.first;
    return bucket_of(d.pairs[local], d.wpair ? d.wpair[local] : d.w);
}

__global__ void batch_init_kernel(BatchCtrl *c) {
    for (int k = threadIdx.x; k <= kNumSegs; k += blockDim.x) c->counter[k] = 0;
    if (threadIdx.x == 0) {
        c->flags = 0;
        c->bad_index = LLONG_MAX;
        c->cells = 0ull;
    }
}

// bucket histogram, one atomic per distinct bucket per warp
__global__ void batch_hist_kernel(const LaunchArgs A, int nreqs, int n, int *counts) {
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int k = base + threadIdx.x;
        const bool valid = k < n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        int req, local;
        const int key = item_key(A, nreqs, k, req, local);
        const unsigned m = __match_any_sync(act, key);
        if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(counts + key, __popc(m));
    }
}

// exclusive scan of the bucket counts in place (one block of 1024 threads),
// and each segment's {offset, count} into seg
__global__ void __launch_bounds__(1024) batch_scan_kernel(int *counts, int *seg) {
    __shared__ int warp_tot[32];
    __shared__ int total;
    constexpr int per = (kNumBuckets + 1023) / 1024;
    const int t = threadIdx.x;
    const int lo = t * per, hi = imin(lo + per, kNumBuckets);
    int sum = 0;
    for (int k = lo; k < hi; k++) sum += counts[k];
    // block exclusive scan of the per-thread sums
    const int lane = t & 31, wid = t >> 5;
    int incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int v = warp_tot[lane];
        int wi = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += u;
        }
        warp_tot[lane] = wi - v;
        if (lane == 31) total = wi;
    }
    __syncthreads();
    int run = warp_tot[wid] + incl - sum;
    for (int k = lo; k < hi; k++) {
        const int c = counts[k];
        counts[k] = run;
        run += c;
    }
    __syncthreads();
    if (t < kNumSegs) {
        const int s0 = counts[t * kRowBuckets];
        const int s1 = (t + 1 < kNumSegs) ? counts[(t + 1) * kRowBuckets] : total;
        seg[2 * t] = s0;
        seg[2 * t + 1] = s1 - s0;
    }
}

// scatter work items into bucket order; within a segment the order is
// reversed so the longest targets come first
__global__ void batch_scatter_kernel(const LaunchArgs A, int nreqs, int n, int *cursor,
                                     const int *seg, int32_t *order, int32_t *order_req) {
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int k = base + threadIdx.x;
        const bool valid = k < n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        int req, local;
        const int key = item_key(A, nreqs, k, req, local);
        const unsigned m = __match_any_sync(act, key);
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(m) - 1;
        int b0 = 0;
        if (lane == leader) b0 = atomicAdd(cursor + key, __popc(m));
        b0 = __shfl_sync(m, b0, leader);
        const int pos = b0 + __popc(m & ((1u << lane) - 1u));
        const int sg = key / kRowBuckets;
        const int s0 = seg[2 * sg], s1 = s0 + seg[2 * sg + 1];
        order[s0 + s1 - 1 - pos] = local;
        if (order_req) order_req[s0 + s1 - 1 - pos] = req;
    }
}

// A serving tick holds few pairs per segment, and only eight kernels run side
// by side (the device's hardware queues), so a tick is a handful of
// launches: bins above lane_bin with G lanes per pair (latency
// configuration), one launch per bin over all its segments, and ONE
// lane-kernel launch over bins 0..lane_bin, its ring the largest any
// non-empty segment of them needs.  A lane walks a whole pair, so a pair of
// several hundred columns holds its warp for milliseconds; G lanes per pair
// split each row.  The lane launch takes its longest queries first.
cudaError_t enqueue_tick(tal_bsw_ctx *h, const SortBufs &sb, const LaunchArgs &base,
                         const int *count, int lane_bin, BinFork &f, cudaStream_t s) {
    cudaError_t e = cudaEventRecord(f.fork, s);
    int k = 0;
    // one G launch over the consecutive segments [s0, s1] of bin b, with the
    // largest ring its non-empty segments need (whole rows if any needs them)
    auto g_launch = [&](int s0, int s1, int b) {
        int n = 0, win = 0;
        bool rows = false;
        for (int sg = s0; sg <= s1; sg++) {
            if (count[sg] <= 0) continue;
            n += count[sg];
            if (seg_window(sg) == 0) rows = true;
            win = std::max(win, seg_window(sg));
        }
        if (n <= 0 || e != cudaSuccess) return;
        e = cudaStreamWaitEvent(f.st[k], f.fork, 0);
        LaunchArgs A = seg_launch_args(h, sb, base, s0, n);
        A.nseg = s1 - s0 + 1;
        A.cols_cap = bin_cols(h, b);
        A.win = rows ? 0 : win;
        const KConfig cfg = fit_config(latency_config(A.cols_cap, A.win), A.cols_cap, h->smem_optin, A.win);
        if (e == cudaSuccess) e = launch_config(A, cfg, h->num_sms, h->smem_optin, f.st[k]);
        h->launches++;
        if (e == cudaSuccess) e = cudaEventRecord(f.join[k], f.st[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, f.join[k], 0);
        k = (k + 1) % kForkStreams;
    };
    for (int sg = 0; sg < kRowSegs; sg++) g_launch(sg, sg, seg_bin(sg));
    for (int b = kNumBins - 1; b > lane_bin; b--) g_launch(seg_first(b), seg_last(b), b);
    const int first = seg_first(lane_bin);
    int lane_pairs = 0, win = 0;
    for (int sg = first; sg < kNumSegs; sg++) {
        if (count[sg] <= 0) continue;
        lane_pairs += count[sg];
        int W = seg_window(sg);
        if (W == 0) W = lane_ring_at_least(bin_upper(seg_bin(sg)) + 4);  // whole rows
        win = std::max(win, W);
    }
    if (lane_pairs > 0 && e == cudaSuccess) {
        LaunchArgs A = seg_launch_args(h, sb, base, first, lane_pairs);
        A.nseg = kNumSegs - first;
        A.win = win;
        A.cols_cap = bin_upper(lane_bin);
        e = launch_config(A, KConfig{1, 4}, h->num_sms, h->smem_optin, s);
        h->launches++;
    }
    return e;
}

int bin_cols(const tal_bsw_ctx *h, int b) {
    int c = bin_upper(b);
    // the widest one-pair-per-warp configuration must fit the block limit
    while (c > 32 && warp_smem_bytes(c, 1, 32) > h->smem_optin) c -= 512;
    return c;
}

KConfig seg_default(const tal_bsw_ctx *h, int seg, int w) {
    const int cols = bin_cols(h, seg_bin(seg)), win = seg_window(seg);
    return fit_config(choose_config(w, cols, win), cols, h->smem_optin, win);
}

KConfig seg_kconfig(const tal_bsw_ctx *h, int seg, int w) {
    return h->tuned ? h->bin_cfg[seg] : seg_default(h, seg, w);
}

// The per-segment fields of a launch over a sorted work list: row capacity
// and ring, the segment's {offset, count}, its work counter, the control block.
LaunchArgs seg_launch_args(const tal_bsw_ctx *h, const SortBufs &sb, LaunchArgs A, int seg, int n) {
    A.order = sb.order;
    A.order_req = sb.order_req;
    A.seg = sb.seg + 2 * seg;
    A.nseg = 1;
    A.n = n;  // upper bound, sizes the persistent grid
    A.cols_cap = bin_cols(h, seg_bin(seg));
    A.rows_cap = 1;
    A.win = seg_window(seg);
    A.work_counter = &sb.ctrl->counter[seg];
    A.err_flags = &sb.ctrl->flags;
    A.err_index = &sb.ctrl->bad_index;
    A.cells = &sb.ctrl->cells;
    A.P = h->kp;
    return A;
}

// Memset + sort kernels: bucket histogram, scan into segments, scatter into
// the sorted order.
cudaError_t enqueue_sort(tal_bsw_ctx *h, const SortBufs &sb, const LaunchArgs &base, int nreqs,
                         int n, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(sb.counts, 0, sizeof(int) * kNumBuckets, s);
    if (e != cudaSuccess) return e;
    batch_init_kernel<<<1, 128, 0, s>>>(sb.ctrl);
    const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, (long long)h->num_sms * 8);
    batch_hist_kernel<<<blocks, 256, 0, s>>>(base, nreqs, n, sb.counts);
    batch_scan_kernel<<<1, 1024, 0, s>>>(sb.counts, sb.seg);
    batch_scatter_kernel<<<blocks, 256, 0, s>>>(base, nreqs, n, sb.counts, sb.seg, sb.order,
                                                sb.order_req);
    h->launches += 4;
    return cudaGetLastError();
}

// Batches at least this large hide the long pairs' lane-kernel walk behind
// the other segments; smaller ones give those pairs several lanes each.
constexpr int kHideLongPairs = 2 << 20;

// TAL_BSW_TRACE=1: each segment launch outside graph capture is bracketed by
// timing events and, after the join, its start / end (ms after the fork),
// pairs and configuration go to stderr.  Synchronises: for profiling only.
bool trace_on() {
    static const bool on = getenv("TAL_BSW_TRACE") && atoi(getenv("TAL_BSW_TRACE")) > 0;
    return on;
}

cudaError_t enqueue_segs_forked(tal_bsw_ctx *h, const SortBufs &sb, const LaunchArgs &base,
                                const int *count, int n, int w, BinFork &f, cudaStream_t s,
                                bool latency) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    const bool trace = trace_on() && cap == cudaStreamCaptureStatusNone;
    struct Span { int sg, ns, G, win; cudaEvent_t a, b; };
    std::vector<Span> spans;
    cudaEvent_t t0 = nullptr;
    if (trace) {
        cudaEventCreate(&t0);
        cudaEventRecord(t0, s);
    }
    cudaError_t e = cudaEventRecord(f.fork, s);
    bool used[kForkStreams] = {};
    int nz = 0;  // non-empty segments so far
    for (int sg = 0; sg < kNumSegs && e == cudaSuccess; sg++) {  // longest queries first
        const int ns = count ? count[sg] : n;
        if (ns <= 0) continue;
        const int k = cap != cudaStreamCaptureStatusNone ? sg % kForkStreams
                      : nz < kForkStreams ? nz : kForkStreams - 1 - (nz - kForkStreams) % kForkStreams;
        nz++;
        if (!used[k]) {
            e = cudaStreamWaitEvent(f.st[k], f.fork, 0);
            used[k] = true;
        }
        if (e != cudaSuccess) break;
        const LaunchArgs A = seg_launch_args(h, sb, base, sg, ns);
        // long queries: the slowest pair sets the end of the launch unless the
        // batch is large enough to hide it behind other segments
        const bool lat = latency || (n < kHideLongPairs && A.cols_cap > kLongQuery);
        const KConfig cfg = lat ? fit_config(latency_config(A.cols_cap, A.win), A.cols_cap,
                                             h->smem_optin, A.win)
                                : seg_kconfig(h, sg, w);
        Span sp = {sg, ns, cfg.G, A.win, nullptr, nullptr};
        if (trace) {
            cudaEventCreate(&sp.a);
            cudaEventCreate(&sp.b);
            cudaEventRecord(sp.a, f.st[k]);
        }
        e = launch_config(A, cfg, h->num_sms, h->smem_optin, f.st[k]);
        h->launches++;
        if (trace) {
            cudaEventRecord(sp.b, f.st[k]);
            spans.push_back(sp);
        }
    }
    for (int k = 0; k < kForkStreams; k++) {
        if (!used[k]) continue;
        cudaError_t e2 = cudaEventRecord(f.join[k], f.st[k]);
        if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(s, f.join[k], 0);
        if (e == cudaSuccess) e = e2;
    }
    if (trace) {
        cudaStreamSynchronize(s);
        for (const Span &sp : spans) {
            float ta = 0, tb = 0;
            cudaEventElapsedTime(&ta, t0, sp.a);
            cudaEventElapsedTime(&tb, t0, sp.b);
            fprintf(stderr, "[tal_bsw trace] seg %3d (len2<=%5d ring %4d) pairs %7d G%-2d  %8.3f -> %8.3f ms\n",
                    sp.sg, bin_upper(seg_bin(sp.sg)), sp.win, sp.ns, sp.G, ta, tb);
            cudaEventDestroy(sp.a);
            cudaEventDestroy(sp.b);
        }
        cudaEventDestroy(t0);
    }
    return e;
}

}  // namespace talbsw

using namespace talbsw;

namespace {

// Byte extents of the sequence buffers a device SeqPair array references
// (out[0]: max idr + len1, out[1]: max idq + len2) and its first pair with a
// negative length or offset (out[2]: n - its index; 0 if none), all by
// atomicMax into a zeroed out[3].
__global__ void extent_kernel(const talbsw::DevPair *p, int n, unsigned long long *out) {
    unsigned long long r = 0, q = 0, bad = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const talbsw::DevPair x = p[k];
        if (x.len1 < 0 || x.len2 < 0 || x.idr < 0 || x.idq < 0) {
            bad = bad > (unsigned long long)(n - k) ? bad : (unsigned long long)(n - k);
        } else {
            const unsigned long long re = (unsigned long long)x.idr + (unsigned long long)x.len1;
            const unsigned long long qe = (unsigned long long)x.idq + (unsigned long long)x.len2;
            r = r > re ? r : re;
            q = q > qe ? q : qe;
        }
    }
    for (int o = 16; o; o >>= 1) {
        const unsigned long long r2 = __shfl_xor_sync(0xffffffffu, r, o);
        const unsigned long long q2 = __shfl_xor_sync(0xffffffffu, q, o);
        const unsigned long long b2 = __shfl_xor_sync(0xffffffffu, bad, o);
        r = r > r2 ? r : r2;
        q = q > q2 ? q : q2;
        bad = bad > b2 ? bad : b2;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out + 0, r);
        atomicMax(out + 1, q);
        if (bad) atomicMax(out + 2, bad);
    }
}

int bfail(tal_bsw_ctx *h, int code, const std::string &msg) {
    h->last_error = msg;
    return code;
}

SortBufs handle_sort_bufs(tal_bsw_ctx *h) {
    SortBufs sb;
    sb.counts = reinterpret_cast<int *>(h->bcounts.p);
    sb.order = reinterpret_cast<int32_t *>(h->border.p);
    sb.order_req = nullptr;
    sb.seg = reinterpret_cast<int32_t *>(h->bseg.p);
    sb.ctrl = reinterpret_cast<BatchCtrl *>(h->bctrl.p);
    return sb;
}

LaunchArgs base_args(DevPair *pairs, const uint8_t *ref, size_t ref_bytes, const uint8_t *qer,
                     size_t qer_bytes, int w, const int32_t *d_w, int bits) {
    LaunchArgs A;
    memset(&A, 0, sizeof(A));
    A.pairs = pairs;
    A.ref = ref;
    A.qer = qer;
    A.ref_lo = 0; A.ref_hi = (long long)ref_bytes;
    A.qer_lo = 0; A.qer_hi = (long long)qer_bytes;
    A.wpair = d_w;
    A.w = w;
    A.bits = bits;
    return A;
}

// Per segment, times each candidate configuration on up to kSample of the
// segment's pairs (scoring them, so the work is not wasted) and keeps the
// fastest.
int autotune(tal_bsw_ctx *h, const LaunchArgs &base, int n, int w) {
    constexpr int kSample = 16384;
    cudaError_t e = enqueue_sort(h, handle_sort_bufs(h), base, 0, n, h->stream);
    int seg[2 * kNumSegs];
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(seg, h->bseg.p, sizeof(seg), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("autotune sort: ") + cudaGetErrorString(e));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    BatchCtrl *c = reinterpret_cast<BatchCtrl *>(h->bctrl.p);
    SortBufs tsb = handle_sort_bufs(h);  // tuning launches read {offset, count} from btune_seg
    tsb.seg = reinterpret_cast<int32_t *>(h->btune_seg.p);
    for (int sg = 0; sg < kNumSegs; sg++) {
        h->bin_cfg[sg] = seg_default(h, sg, w);
        const int cnt = seg[2 * sg + 1];
        if (cnt < 1024) continue;
        const int cols = bin_cols(h, seg_bin(sg)), win = seg_window(sg);
        const int slots = win > 0 ? win : cols + 4;
        std::vector<KConfig> cands;
        if (slots <= kLaneMaxCols + 4) cands = {{1, 4}, {8, 4}, {4, 4}};
        else if (slots <= 1028) cands = {{1, 4}, {8, 4}, {16, 4}, {32, 4}};
        else cands = {{8, 4}, {16, 4}, {32, 4}, {16, 2}};
        int ts[2] = {seg[2 * sg], std::min(cnt, kSample)};
        int32_t *tseg = reinterpret_cast<int32_t *>(h->btune_seg.p) + 2 * sg;
        e = cudaMemcpyAsync(tseg, ts, sizeof(ts), cudaMemcpyHostToDevice, h->stream);
        float best = 1e30f;
        for (const KConfig &k : cands) {
            if (config_smem(k, cols, 1, win) > h->smem_optin) continue;
            LaunchArgs A = seg_launch_args(h, tsb, base, sg, ts[1]);
            // timed with the coupling detector on, as the captured launches run
            // (its flags are dropped: the sample's outputs are scored again)
            attach_regroup(A, h->regroup.V);
            float ms = 1e30f;
            for (int rep = 0; rep < 2 && e == cudaSuccess; rep++) {
                e = cudaMemsetAsync(&c->counter[sg], 0, sizeof(int), h->stream);
                if (e == cudaSuccess) e = cudaMemsetAsync(h->regroup.V.ctr, 0, sizeof(int), h->stream);
                if (e != cudaSuccess) break;
                cudaEventRecord(e0, h->stream);
                e = launch_config(A, k, h->num_sms, h->smem_optin, h->stream);
                cudaEventRecord(e1, h->stream);
                h->launches++;
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float t = 0;
                cudaEventElapsedTime(&t, e0, e1);
                if (rep) ms = std::min(ms, t);
            }
            if (e != cudaSuccess) break;
            if (ms < best) {
                best = ms;
                h->bin_cfg[sg] = k;
            }
        }
        if (e != cudaSuccess) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->regroup.V.ctr, 0, sizeof(int), h->stream);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("autotune: ") + cudaGetErrorString(e));
    h->tuned = true;
    return TAL_OK;
}

int collect_batch(tal_bsw_ctx *h) {
    BatchCtrl c;
    cudaError_t e = cudaMemcpyAsync(&c, h->bctrl.p, sizeof(c), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("batched scoring: ") + cudaGetErrorString(e));
    h->last_cells = c.cells;
    if (c.flags) {
        h->last_bad = c.bad_index;
        std::string why;
        if (c.flags & ERR_DOMAIN) why += "pair outside the exact 8/16-bit range; ";
        if (c.flags & ERR_CAPACITY) why += "pair longer than the row capacity; ";
        if (c.flags & ERR_BASE) why += "base code above 4; ";
        if (c.flags & ERR_FLAGCAP)
            why += "more than 1024 band / precision classes among pairs that need group scoring; ";
        return bfail(h, TAL_EDOMAIN, why + "first bad pair " + std::to_string(c.bad_index));
    }
    return TAL_OK;
}

int batched_device_locked(tal_bsw_ctx *h, tal_seq_pair *d_pairs, const uint8_t *d_ref,
                          size_t ref_bytes, const uint8_t *d_qer, size_t qer_bytes,
                          int32_t numPairs, int32_t w, const int32_t *d_w, int bits) {
    if (numPairs < 0 || (bits != 0 && bits != 8 && bits != 16))
        return bfail(h, TAL_EINVAL, "bad numPairs or bits");
    if (numPairs == 0) return TAL_OK;
    if (!d_pairs || !d_ref || !d_qer) return bfail(h, TAL_EINVAL, "NULL buffer");
    if (((uintptr_t)d_ref & 15) || ((uintptr_t)d_qer & 15))
        return bfail(h, TAL_EINVAL, "device sequence buffers must be 16-byte aligned");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, "cudaSetDevice");
    const bool grow = (size_t)numPairs * sizeof(int32_t) > h->border.cap;
    if ((e = h->bcounts.ensure(sizeof(int) * kNumBuckets)) != cudaSuccess ||
        (e = h->border.ensure(sizeof(int32_t) * (size_t)numPairs)) != cudaSuccess ||
        (e = h->bseg.ensure(sizeof(int) * 2 * kNumSegs)) != cudaSuccess ||
        (e = h->bctrl.ensure(sizeof(BatchCtrl))) != cudaSuccess ||
        (e = h->btune_seg.ensure(sizeof(int) * 2 * kNumSegs)) != cudaSuccess ||
        (e = h->bfork.create()) != cudaSuccess)
        return bfail(h, TAL_ENOMEM, std::string("batched buffers: ") + cudaGetErrorString(e));
    // the regroup pass's arena: queries up to the 16-bit limit (a captured
    // graph is replayed on new contents of the same buffers)
    bool rgrow = false;
    if ((e = h->regroup.ensure(numPairs, 32767, h->num_sms, &rgrow)) != cudaSuccess)
        return bfail(h, TAL_ENOMEM, std::string("regroup buffers: ") + cudaGetErrorString(e));
    if (grow || rgrow) {  // captured graphs hold the old order / regroup buffers
        for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
        h->graphs.clear();
    }
    DevPair *pairs = reinterpret_cast<DevPair *>(d_pairs);
    LaunchArgs base = base_args(pairs, d_ref, ref_bytes, d_qer, qer_bytes, w, d_w, bits);
    if (!h->tuned) {
        int rc = autotune(h, base, numPairs, w);
        if (rc != TAL_OK) return rc;
        for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
        h->graphs.clear();
    }
    auto key = std::make_tuple((const void *)d_pairs, (const void *)d_ref, ref_bytes,
                               (const void *)d_qer, qer_bytes, (int)numPairs, (int)w,
                               (const void *)d_w, bits);
    auto it = h->graphs.find(key);
    if (it == h->graphs.end()) {
        cudaGraph_t g = nullptr;
        // the scoring launches flag pairs whose outputs may depend on their
        // SIMD group; the regroup pass re-scores those groups exactly
        attach_regroup(base, h->regroup.V);
        LaunchArgs rg = base;
        rg.n = numPairs;
        rg.err_flags = &handle_sort_bufs(h).ctrl->flags;
        rg.err_index = &handle_sort_bufs(h).ctrl->bad_index;
        rg.cells = &handle_sort_bufs(h).ctrl->cells;
        rg.P = h->kp;
        e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e1 = enqueue_sort(h, handle_sort_bufs(h), base, 0, numPairs, h->stream);
            cudaError_t e2 = e1 == cudaSuccess
                                 ? enqueue_segs_forked(h, handle_sort_bufs(h), base, nullptr,
                                                       numPairs, w, h->bfork, h->stream, false)
                                 : e1;
            if (e2 == cudaSuccess)
                e2 = enqueue_regroup(h->regroup.V, rg, 0, numPairs, h->num_sms, h->stream, &h->launches);
            e = cudaStreamEndCapture(h->stream, &g);
            if (e == cudaSuccess) e = e2;
        }
        cudaGraphExec_t exec = nullptr;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        GraphEntry ge;
        ge.exec = exec;
        it = h->graphs.emplace(key, ge).first;
    } else {
        h->launches += 4 + kNumSegs + 11;
    }
    e = cudaGraphLaunch(it->second.exec, h->stream);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    return collect_batch(h);
}

}  // namespace

extern "C" {

int tal_bsw_scores_batched_device(tal_bsw_handle h, tal_seq_pair *d_pairs, const uint8_t *d_ref,
                                  size_t ref_bytes, const uint8_t *d_qer, size_t qer_bytes,
                                  int32_t numPairs, int32_t w, const int32_t *d_w, int bits) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->last_error.clear();
    h->last_bad = -1;
    return batched_device_locked(h, d_pairs, d_ref, ref_bytes, d_qer, qer_bytes, numPairs, w,
                                 d_w, bits);
}

int tal_bsw_scores_batched(tal_bsw_handle h, tal_seq_pair *pairs, const uint8_t *seqBufRef,
                           const uint8_t *seqBufQer, int32_t numPairs, int32_t w,
                           const int32_t *wpair, int bits) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->last_error.clear();
    h->last_bad = -1;
    if (numPairs < 0) return bfail(h, TAL_EINVAL, "bad numPairs");
    if (numPairs == 0) return TAL_OK;
    if (!pairs || !seqBufRef || !seqBufQer) return bfail(h, TAL_EINVAL, "NULL buffer");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, "cudaSetDevice");
    // the pairs first; the extents of the sequence buffers they reference
    // (and the first pair with a negative length or offset) are reduced on
    // the device, not by a pass of the host over the array
    const size_t pbytes = (size_t)numPairs * sizeof(tal_seq_pair);
    if ((e = h->pairs.ensure(pbytes)) != cudaSuccess || (e = h->caps.ensure(4 * sizeof(unsigned long long))) != cudaSuccess)
        return bfail(h, TAL_ENOMEM, std::string("device buffers: ") + cudaGetErrorString(e));
    unsigned long long *ext = reinterpret_cast<unsigned long long *>(h->caps.p);
    e = cudaMemcpyAsync(h->pairs.p, pairs, pbytes, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ext, 0, 3 * sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess) {
        const int blocks = (int)std::min<long long>(((long long)numPairs + 255) / 256, (long long)h->num_sms * 8);
        extent_kernel<<<blocks, 256, 0, h->stream>>>(reinterpret_cast<const talbsw::DevPair *>(h->pairs.p),
                                                     numPairs, ext);
        h->launches++;
        e = cudaGetLastError();
    }
    unsigned long long hext[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hext, ext, sizeof(hext), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("H2D: ") + cudaGetErrorString(e));
    if (hext[2]) {
        const long long k = (long long)numPairs - (long long)hext[2];
        h->last_bad = k;
        return bfail(h, TAL_EDOMAIN, "negative length or offset at pair " + std::to_string(k));
    }
    const long long rhi = std::max<long long>(16, (long long)hext[0]);
    const long long qhi = std::max<long long>(16, (long long)hext[1]);
    if ((e = h->ref.ensure((size_t)rhi + 16)) != cudaSuccess ||
        (e = h->qer.ensure((size_t)qhi + 16)) != cudaSuccess ||
        (wpair && (e = h->wpair.ensure(sizeof(int32_t) * (size_t)numPairs)) != cudaSuccess))
        return bfail(h, TAL_ENOMEM, std::string("device buffers: ") + cudaGetErrorString(e));
    e = cudaMemcpyAsync(h->ref.p, seqBufRef, (size_t)rhi, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->qer.p, seqBufQer, (size_t)qhi, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && wpair)
        e = cudaMemcpyAsync(h->wpair.p, wpair, sizeof(int32_t) * (size_t)numPairs,
                            cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("H2D: ") + cudaGetErrorString(e));
    int rc = batched_device_locked(h, reinterpret_cast<tal_seq_pair *>(h->pairs.p),
                                   reinterpret_cast<const uint8_t *>(h->ref.p), (size_t)rhi,
                                   reinterpret_cast<const uint8_t *>(h->qer.p), (size_t)qhi,
                                   numPairs, w, wpair ? reinterpret_cast<const int32_t *>(h->wpair.p) : nullptr,
                                   bits);
    if (rc != TAL_OK) return rc;
    e = cudaMemcpyAsync(pairs, h->pairs.p, pbytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("D2H: ") + cudaGetErrorString(e));
    return TAL_OK;
}

int tal_bsw_autotune_reset(tal_bsw_handle h) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->tuned = false;
    for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
    h->graphs.clear();
    return TAL_OK;
}

int tal_bsw_segment_config(tal_bsw_handle h, int seg, int *lanes_per_pair, int *cols_per_lane,
                           int *max_len2, int *window) {
    if (!h || seg < 0 || seg >= kNumSegs) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    const KConfig c = seg_kconfig(h, seg, 100);
    if (lanes_per_pair) *lanes_per_pair = c.G;
    if (cols_per_lane) *cols_per_lane = c.K;
    if (max_len2) *max_len2 = bin_cols(h, seg_bin(seg));
    if (window) *window = seg_window(seg);
    return TAL_OK;
}

int tal_bsw_bin_config(tal_bsw_handle h, int bin, int *lanes_per_pair, int *cols_per_lane,
                       int *max_len2) {
    if (bin < 0 || bin >= kNumBins) return TAL_EINVAL;
    return tal_bsw_segment_config(h, seg_index(bin, kRingCls), lanes_per_pair, cols_per_lane,
                                  max_len2, nullptr);
}

}  // extern "C"
