// Batched form of the scorer (tal_bsw_scores_batched*): one call scores a
// large, mixed batch -- uneven lengths, bands and 8/16-bit pairs -- as a CUDA
// graph of
//   1. a counting sort of the pairs into (query-length bin, 8-row target
//      bucket) order, on the device;
//   2. one persistent launch per length bin, each taking its pairs from the
//      sorted order through a work counter, with the kernel and tile chosen
//      for that bin by an autotuner on the first call.
// Sorting makes the pairs that share a warp alike in shape (same row count,
// similar band widths), which is what the lane-per-pair kernel needs to keep
// its lanes busy, and lets each bin size its shared-memory rows to the bin.
// Outputs do not depend on the order pairs are scored in.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <string>

#include "bsw_ctx.h"

namespace talbsw {

__device__ __forceinline__ int bin_of(int len2) {
    int b = 0;
#pragma unroll
    for (int k = 0; k < kNumBins - 1; k++) b += (len2 > bin_upper(k)) ? 1 : 0;
    return b;
}

__device__ __forceinline__ int bucket_of(const DevPair &p) {
    const int r = imin(imax(p.len1, 0) >> 3, kRowBuckets - 1);
    return bin_of(p.len2) * kRowBuckets + r;
}

// Pair k of the work list: of the launch's pair array, or -- for a serving
// tick -- of the request whose range [first, first + n) holds k (binary
// search over the tick's request table).
__device__ __forceinline__ const DevPair &pair_of(const DevPair *p, const ReqDesc *reqs, int nreqs,
                                                  int k, int &req, int &local) {
    if (!reqs) {
        req = -1;
        local = k;
        return p[k];
    }
    int lo = 0, hi = nreqs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (reqs[mid].first <= k) lo = mid;
        else hi = mid - 1;
    }
    req = lo;
    local = k - reqs[lo].first;
    return reqs[lo].pairs[local];
}

__global__ void batch_init_kernel(BatchCtrl *c) {
    for (int k = threadIdx.x; k <= kNumBins; k += blockDim.x) c->counter[k] = 0;
    if (threadIdx.x == 0) {
        c->flags = 0;
        c->bad_index = LLONG_MAX;
        c->cells = 0ull;
    }
}

// bucket histogram, one atomic per distinct bucket per warp
__global__ void batch_hist_kernel(const DevPair *p, const ReqDesc *reqs, int nreqs, int n,
                                  int *counts) {
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int k = base + threadIdx.x;
        const bool valid = k < n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        int req, local;
        const int key = bucket_of(pair_of(p, reqs, nreqs, k, req, local));
        const unsigned m = __match_any_sync(act, key);
        if ((int)(threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(counts + key, __popc(m));
    }
}

// exclusive scan of the bucket counts in place (one block of 1024 threads),
// and each bin's {offset, count} into seg
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
    if (t < kNumBins) {
        const int s0 = counts[t * kRowBuckets];
        const int s1 = (t + 1 < kNumBins) ? counts[(t + 1) * kRowBuckets] : total;
        seg[2 * t] = s0;
        seg[2 * t + 1] = s1 - s0;
    }
}

// scatter pair indices into bucket order; within a bin the order is reversed
// so the longest targets come first
__global__ void batch_scatter_kernel(const DevPair *p, const ReqDesc *reqs, int nreqs, int n,
                                     int *cursor, const int *seg, int32_t *order,
                                     int32_t *order_req) {
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int k = base + threadIdx.x;
        const bool valid = k < n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        int req, local;
        const int key = bucket_of(pair_of(p, reqs, nreqs, k, req, local));
        const unsigned m = __match_any_sync(act, key);
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(m) - 1;
        int b0 = 0;
        if (lane == leader) b0 = atomicAdd(cursor + key, __popc(m));
        b0 = __shfl_sync(m, b0, leader);
        const int pos = b0 + __popc(m & ((1u << lane) - 1u));
        const int bin = key / kRowBuckets;
        const int s0 = seg[2 * bin], s1 = s0 + seg[2 * bin + 1];
        order[s0 + s1 - 1 - pos] = local;
        if (order_req) order_req[s0 + s1 - 1 - pos] = req;
    }
}

}  // namespace talbsw

using namespace talbsw;

namespace {

int bfail(tal_bsw_ctx *h, int code, const std::string &msg) {
    h->last_error = msg;
    return code;
}

KConfig default_cfg(const tal_bsw_ctx *h, int b, int w) {
    return fit_config(choose_config(w, bin_cols(h, b)), bin_cols(h, b), h->smem_optin);
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

LaunchArgs bin_args(tal_bsw_ctx *h, int b, DevPair *pairs, const uint8_t *ref, size_t ref_bytes,
                    const uint8_t *qer, size_t qer_bytes, int n, int w, const int32_t *d_w, int bits,
                    const int32_t *seg) {
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
    return bin_launch_args(h, handle_sort_bufs(h), A, b, n, seg);
}

}  // namespace

namespace talbsw {

// The per-bin fields of a launch over a sorted work list: row capacity, the
// bin's {offset, count}, its work counter, the control block.
LaunchArgs bin_launch_args(const tal_bsw_ctx *h, const SortBufs &sb, LaunchArgs A, int b, int n,
                           const int32_t *seg) {
    A.order = sb.order;
    A.order_req = sb.order_req;
    A.seg = seg;
    A.n = n;  // upper bound, sizes the persistent grid
    A.cols_cap = bin_cols(h, b);
    A.rows_cap = 1;
    A.work_counter = &sb.ctrl->counter[b];
    A.err_flags = &sb.ctrl->flags;
    A.err_index = &sb.ctrl->bad_index;
    A.cells = &sb.ctrl->cells;
    A.P = h->kp;
    return A;
}

// Memset + sort kernels: bucket histogram, scan into bin segments, scatter
// into the sorted order.  reqs (device table of nreqs requests) replaces
// pairs for a serving tick.
cudaError_t enqueue_sort(tal_bsw_ctx *h, const SortBufs &sb, const DevPair *pairs,
                         const ReqDesc *reqs, int nreqs, int n, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(sb.counts, 0, sizeof(int) * kNumBuckets, s);
    if (e != cudaSuccess) return e;
    batch_init_kernel<<<1, 64, 0, s>>>(sb.ctrl);
    const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, (long long)h->num_sms * 8);
    batch_hist_kernel<<<blocks, 256, 0, s>>>(pairs, reqs, nreqs, n, sb.counts);
    batch_scan_kernel<<<1, 1024, 0, s>>>(sb.counts, sb.seg);
    batch_scatter_kernel<<<blocks, 256, 0, s>>>(pairs, reqs, nreqs, n, sb.counts, sb.seg, sb.order,
                                                sb.order_req);
    h->launches += 4;
    return cudaGetLastError();
}

KConfig bin_kconfig(const tal_bsw_ctx *h, int b, int w) {
    if (h->tuned) return h->bin_cfg[b];
    return fit_config(choose_config(w, bin_cols(h, b)), bin_cols(h, b), h->smem_optin);
}

cudaError_t enqueue_bins_forked(tal_bsw_ctx *h, const SortBufs &sb, const LaunchArgs &base,
                                const int *count, int n, int w, BinFork &f, cudaStream_t s) {
    cudaError_t e = cudaEventRecord(f.fork, s);
    for (int b = kNumBins - 1; b >= 0 && e == cudaSuccess; b--) {
        const int nb = count ? count[b] : n;
        if (nb <= 0) continue;
        e = cudaStreamWaitEvent(f.st[b], f.fork, 0);
        if (e != cudaSuccess) break;
        const LaunchArgs A = bin_launch_args(h, sb, base, b, nb, sb.seg + 2 * b);
        e = launch_config(A, bin_kconfig(h, b, w), h->num_sms, h->smem_optin, f.st[b]);
        h->launches++;
        if (e == cudaSuccess) e = cudaEventRecord(f.join[b], f.st[b]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, f.join[b], 0);
    }
    return e;
}

int bin_cols(const tal_bsw_ctx *h, int b) {
    int c = bin_upper(b);
    // the widest one-pair-per-warp configuration must fit the block limit
    while (c > 32 && warp_smem_bytes(c, 1, 32) > h->smem_optin) c -= 512;
    return c;
}

}  // namespace talbsw

namespace {

cudaError_t enqueue_bins(tal_bsw_ctx *h, DevPair *pairs, const uint8_t *ref, size_t ref_bytes,
                         const uint8_t *qer, size_t qer_bytes, int n, int w, const int32_t *d_w,
                         int bits) {
    cudaError_t e = h->bfork.create();
    if (e != cudaSuccess) return e;
    LaunchArgs base;
    memset(&base, 0, sizeof(base));
    base.pairs = pairs;
    base.ref = ref;
    base.qer = qer;
    base.ref_lo = 0; base.ref_hi = (long long)ref_bytes;
    base.qer_lo = 0; base.qer_hi = (long long)qer_bytes;
    base.wpair = d_w;
    base.w = w;
    base.bits = bits;
    return enqueue_bins_forked(h, handle_sort_bufs(h), base, nullptr, n, w, h->bfork, h->stream);
}

// Per bin, times each candidate configuration on up to kSample of the bin's
// pairs (scoring them, so the work is not wasted) and keeps the fastest.
int autotune(tal_bsw_ctx *h, DevPair *pairs, const uint8_t *ref, size_t ref_bytes,
             const uint8_t *qer, size_t qer_bytes, int n, int w, const int32_t *d_w, int bits) {
    constexpr int kSample = 16384;
    cudaError_t e = enqueue_sort(h, handle_sort_bufs(h), pairs, nullptr, 0, n, h->stream);
    int seg[2 * kNumBins];
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(seg, h->bseg.p, sizeof(seg), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return bfail(h, TAL_ECUDA, std::string("autotune sort: ") + cudaGetErrorString(e));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    BatchCtrl *c = reinterpret_cast<BatchCtrl *>(h->bctrl.p);
    for (int b = 0; b < kNumBins; b++) {
        h->bin_cfg[b] = default_cfg(h, b, w);
        const int cnt = seg[2 * b + 1];
        if (cnt < 1024) continue;
        const int cols = bin_cols(h, b);
        std::vector<KConfig> cands;
        if (cols <= kLaneMaxCols) cands = {{1, 4}, {8, 4}, {4, 4}};
        else cands = {{8, 4}, {16, 4}, {32, 4}, {16, 2}};
        int ts[2] = {seg[2 * b], std::min(cnt, kSample)};
        int32_t *tseg = reinterpret_cast<int32_t *>(h->btune_seg.p);
        e = cudaMemcpyAsync(tseg, ts, sizeof(ts), cudaMemcpyHostToDevice, h->stream);
        float best = 1e30f;
        for (const KConfig &k : cands) {
            if (config_smem(k, cols, 1) > h->smem_optin) continue;
            LaunchArgs A = bin_args(h, b, pairs, ref, ref_bytes, qer, qer_bytes, n, w, d_w, bits, tseg);
            float ms = 1e30f;
            for (int rep = 0; rep < 2 && e == cudaSuccess; rep++) {
                e = cudaMemsetAsync(&c->counter[b], 0, sizeof(int), h->stream);
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
                h->bin_cfg[b] = k;
            }
        }
        if (e != cudaSuccess) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
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
        (e = h->bseg.ensure(sizeof(int) * 2 * kNumBins)) != cudaSuccess ||
        (e = h->bctrl.ensure(sizeof(BatchCtrl))) != cudaSuccess ||
        (e = h->btune_seg.ensure(sizeof(int) * 2)) != cudaSuccess)
        return bfail(h, TAL_ENOMEM, std::string("batched buffers: ") + cudaGetErrorString(e));
    if (grow) {  // captured graphs hold the old order buffer
        for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
        h->graphs.clear();
    }
    DevPair *pairs = reinterpret_cast<DevPair *>(d_pairs);
    if (!h->tuned) {
        int rc = autotune(h, pairs, d_ref, ref_bytes, d_qer, qer_bytes, numPairs, w, d_w, bits);
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
        e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e1 = enqueue_sort(h, handle_sort_bufs(h), pairs, nullptr, 0, numPairs,
                                          h->stream);
            cudaError_t e2 = e1 == cudaSuccess
                                 ? enqueue_bins(h, pairs, d_ref, ref_bytes, d_qer, qer_bytes,
                                                numPairs, w, d_w, bits)
                                 : e1;
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
        h->launches += 4 + kNumBins;
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
    long long rhi = 16, qhi = 16;
    for (int32_t k = 0; k < numPairs; k++) {
        const tal_seq_pair &p = pairs[k];
        if (p.len1 < 0 || p.len2 < 0 || p.idr < 0 || p.idq < 0) {
            h->last_bad = k;
            return bfail(h, TAL_EDOMAIN, "negative length or offset at pair " + std::to_string(k));
        }
        rhi = std::max<long long>(rhi, (long long)p.idr + p.len1);
        qhi = std::max<long long>(qhi, (long long)p.idq + p.len2);
    }
    const size_t pbytes = (size_t)numPairs * sizeof(tal_seq_pair);
    if ((e = h->pairs.ensure(pbytes)) != cudaSuccess ||
        (e = h->ref.ensure((size_t)rhi + 16)) != cudaSuccess ||
        (e = h->qer.ensure((size_t)qhi + 16)) != cudaSuccess ||
        (wpair && (e = h->wpair.ensure(sizeof(int32_t) * (size_t)numPairs)) != cudaSuccess))
        return bfail(h, TAL_ENOMEM, std::string("device buffers: ") + cudaGetErrorString(e));
    e = cudaMemcpyAsync(h->pairs.p, pairs, pbytes, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
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

int tal_bsw_bin_config(tal_bsw_handle h, int bin, int *lanes_per_pair, int *cols_per_lane,
                       int *max_len2) {
    if (!h || bin < 0 || bin >= kNumBins) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    const KConfig c = h->tuned ? h->bin_cfg[bin] : default_cfg(h, bin, 100);
    if (lanes_per_pair) *lanes_per_pair = c.G;
    if (cols_per_lane) *cols_per_lane = c.K;
    if (max_len2) *max_len2 = bin_cols(h, bin);
    return TAL_OK;
}

}  // extern "C"
