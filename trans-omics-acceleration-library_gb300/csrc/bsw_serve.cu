// Serving loop of the scorer (tal_bsw_server_*, tal_bsw_submit, tal_bsw_poll).
//
// Continuous batching over a device-resident pool:
//   submit (caller's thread)  checks the request, measures the byte windows
//                             its pairs reference and its pairs per length
//                             bin, stages pageable buffers into pinned
//                             memory, and queues it;
//   admission (worker)        in arrival order, while the head request's
//                             pairs + sequence windows fit the device pool,
//                             reserves its region and issues its host->device
//                             copies on the copy stream (they overlap the
//                             ticks running on the device);
//   tick (worker)             when a slot is free, every admitted request not
//                             yet running becomes one tick on the slot's own
//                             stream: wait for their copies, upload the tick's
//                             request table, sort all their pairs into
//                             segments (length bin x band class) on the
//                             device, one persistent launch per non-empty
//                             segment side by side on forked streams, copy
//                             the results back, record the slot's event;
//   completion (worker)       a finished slot's requests get their status
//                             (per request: the kernels record errors per
//                             request in the table), their pool regions are
//                             released, and pollers are woken.
// Several slots run ticks at once, so work admitted while a tick runs starts
// on the SMs that tick leaves idle.  A pair's outputs do not depend on the
// pairs it is scored with, so a request's results are the same alone or in
// any tick.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bsw_ctx.h"

using namespace talbsw;

namespace {

constexpr size_t kAlign = 256;
constexpr int kMaxTickRequests = 4096;

size_t round_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

int64_t steady_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

int host_seg(int len2, int w) {
    int b = 0;
    while (b < kNumBins - 1 && len2 > bin_upper(b)) b++;
    return seg_index(b, seg_cls(b, w));
}

// First-fit allocator of byte ranges in [0, cap), 256-byte granules, with
// coalescing of neighbouring free ranges.
class Arena {
public:
    void init(size_t cap) {
        cap_ = cap;
        used_ = peak_ = 0;
        free_.clear();
        if (cap) free_[0] = cap;
    }
    bool alloc(size_t bytes, size_t *off) {
        bytes = round_up(std::max<size_t>(bytes, 1));
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off = it->first;
            const size_t rest = it->second - bytes, noff = it->first + bytes;
            free_.erase(it);
            if (rest) free_[noff] = rest;
            used_ += bytes;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = round_up(std::max<size_t>(bytes, 1));
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }
    size_t peak() const { return peak_; }

private:
    size_t cap_ = 0, used_ = 0, peak_ = 0;
    std::map<size_t, size_t> free_;
};

enum ReqState { QUEUED, ADMITTED, RUNNING, DONE };

struct Request {
    uint64_t ticket = 0;
    tal_seq_pair *pairs = nullptr;  // caller's array (outputs land here)
    const uint8_t *ref = nullptr, *qer = nullptr;
    const int32_t *wpair = nullptr;
    int n = 0, w = 0, bits = 0;
    long long rlo = 0, rhi = 0, qlo = 0, qhi = 0;  // byte windows of the caller's buffers
    int segs[kNumSegs] = {};  // pairs per segment
    // one region, in the device pool and (pageable callers) in the staging:
    // pairs | ref window | qer window | bands
    size_t off_pairs = 0, off_ref = 0, off_qer = 0, off_w = 0, bytes = 0;
    size_t dev_off = 0;
    bool pinned = true;
    bool staged = false;
    size_t st_off = 0;
    cudaEvent_t h2d = nullptr;
    ReqState state = QUEUED;
    int status = TAL_OK;
    long long bad = -1;
    int tick_requests = 0;
    long long tick_pairs = 0;
    int64_t t_submit = 0, t_admit = 0, t_launch = 0, t_done = 0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    DevBuf counts, order, order_req, seg, ctrl, dreqs;
    RegroupBufs rg;  // exact scoring of the tick's flagged pairs' SIMD groups
    BinFork fork;
    ReqDesc *hreqs = nullptr;  // pinned copy of the tick's request table
    std::vector<Request *> reqs;
    bool busy = false;
};

}  // namespace

struct tal_bsw_server {
    tal_bsw_ctx *h = nullptr;  // private handle: parameters, device, bin configurations
    tal_bsw_server_config cfg = {};
    uint8_t *pool = nullptr;
    Arena pool_arena;          // worker only (stats read under mu)
    uint8_t *staging = nullptr;
    Arena staging_arena;       // under mu
    cudaStream_t copy_stream = nullptr;
    std::vector<Slot> slots;
    std::thread worker;

    std::mutex mu;  // queue, tickets, staging, request states, stats
    std::condition_variable cv_done;
    std::deque<Request *> queue;
    std::unordered_map<uint64_t, Request *> tickets;
    uint64_t next_ticket = 1;
    bool stop = false;
    int fatal = TAL_OK;  // a CUDA error that poisons the context

    std::mutex wake_mu;
    std::condition_variable cv_wake;
    bool wake_flag = false;

    std::vector<Request *> ready;  // worker only: admitted, not yet in a tick

    tal_bsw_server_stats st = {};

    void wake() {
        {
            std::lock_guard<std::mutex> lk(wake_mu);
            wake_flag = true;
        }
        cv_wake.notify_one();
    }
    void run();
    bool admit();
    bool launch_ticks();
    bool finish_ticks();
    int launch_tick(Slot &sl);
    void complete(Request *r, int status, long long bad);
};

namespace {

void CUDART_CB wake_cb(void *p) { static_cast<tal_bsw_server *>(p)->wake(); }

}  // namespace

// Marks r complete (worker thread; takes mu).
void tal_bsw_server::complete(Request *r, int status, long long bad) {
    {
        std::lock_guard<std::mutex> lk(mu);
        if (r->staged) staging_arena.release(r->st_off, r->bytes);
        r->staged = false;
        r->status = status;
        r->bad = bad;
        r->t_done = steady_ns();
        r->state = DONE;
        st.completed++;
        if (status != TAL_OK) st.failed++;
    }
    cv_done.notify_all();
}

// Admission in arrival order while the head request fits the pool.
bool tal_bsw_server::admit() {
    std::vector<Request *> got;
    {
        std::lock_guard<std::mutex> lk(mu);
        while (!queue.empty()) {
            Request *r = queue.front();
            size_t off = 0;
            if (fatal != TAL_OK) {
                queue.pop_front();
                got.push_back(r);
                continue;
            }
            if (!pool_arena.alloc(r->bytes, &off)) break;
            r->dev_off = off;
            r->state = ADMITTED;
            queue.pop_front();
            got.push_back(r);
        }
    }
    for (Request *r : got) {
        if (fatal != TAL_OK) {
            complete(r, fatal, -1);
            continue;
        }
        uint8_t *d = pool + r->dev_off;
        cudaError_t e = cudaSuccess;
        if (r->pinned) {
            e = cudaMemcpyAsync(d + r->off_pairs, r->pairs, (size_t)r->n * sizeof(tal_seq_pair),
                                cudaMemcpyHostToDevice, copy_stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d + r->off_ref, r->ref + r->rlo, (size_t)(r->rhi - r->rlo),
                                    cudaMemcpyHostToDevice, copy_stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d + r->off_qer, r->qer + r->qlo, (size_t)(r->qhi - r->qlo),
                                    cudaMemcpyHostToDevice, copy_stream);
            if (e == cudaSuccess && r->wpair)
                e = cudaMemcpyAsync(d + r->off_w, r->wpair, (size_t)r->n * sizeof(int32_t),
                                    cudaMemcpyHostToDevice, copy_stream);
        } else {  // the staged region has the pool region's layout: one copy
            e = cudaMemcpyAsync(d, staging + r->st_off, r->bytes, cudaMemcpyHostToDevice, copy_stream);
        }
        if (e == cudaSuccess && !r->h2d) e = cudaEventCreateWithFlags(&r->h2d, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(r->h2d, copy_stream);
        r->t_admit = steady_ns();
        if (e != cudaSuccess) {
            fatal = TAL_ECUDA;
            {
                std::lock_guard<std::mutex> lk(mu);
                pool_arena.release(r->dev_off, r->bytes);
            }
            complete(r, TAL_ECUDA, -1);
            continue;
        }
        ready.push_back(r);
    }
    return !got.empty();
}

// One tick on slot sl from the front of `ready`.
int tal_bsw_server::launch_tick(Slot &sl) {
    const int max_pairs = cfg.max_tick_pairs;
    int nreq = 0;
    long long total = 0;
    int segs[kNumSegs] = {};
    while (nreq < (int)ready.size() && nreq < kMaxTickRequests) {
        Request *r = ready[nreq];
        if (nreq > 0 && total + r->n > max_pairs) break;
        ReqDesc &d = sl.hreqs[nreq];
        uint8_t *base = pool + r->dev_off;
        d.pairs = reinterpret_cast<DevPair *>(base + r->off_pairs);
        d.ref = base + r->off_ref;
        d.qer = base + r->off_qer;
        d.wpair = r->wpair ? reinterpret_cast<const int32_t *>(base + r->off_w) : nullptr;
        d.ref_lo = r->rlo; d.ref_hi = r->rhi;
        d.qer_lo = r->qlo; d.qer_hi = r->qhi;
        d.bad = LLONG_MAX;
        d.first = (int)total;
        d.n = r->n;
        d.w = r->w;
        d.bits = r->bits;
        d.err = 0;
        d.pad_ = 0;
        for (int g = 0; g < kNumSegs; g++) segs[g] += r->segs[g];
        total += r->n;
        nreq++;
    }
    sl.reqs.assign(ready.begin(), ready.begin() + nreq);
    ready.erase(ready.begin(), ready.begin() + nreq);

    cudaError_t e = cudaSuccess;
    for (Request *r : sl.reqs)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sl.stream, r->h2d, 0);
    ReqDesc *dreqs = reinterpret_cast<ReqDesc *>(sl.dreqs.p);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dreqs, sl.hreqs, sizeof(ReqDesc) * nreq, cudaMemcpyHostToDevice, sl.stream);
    SortBufs sb;
    sb.counts = reinterpret_cast<int *>(sl.counts.p);
    sb.order = reinterpret_cast<int32_t *>(sl.order.p);
    sb.order_req = reinterpret_cast<int32_t *>(sl.order_req.p);
    sb.seg = reinterpret_cast<int32_t *>(sl.seg.p);
    sb.ctrl = reinterpret_cast<BatchCtrl *>(sl.ctrl.p);
    LaunchArgs base;
    memset(&base, 0, sizeof(base));
    base.reqs = dreqs;
    attach_regroup(base, sl.rg.V);  // the scoring launches flag pairs for the regroup pass
    if (e == cudaSuccess && total > 0) e = enqueue_sort(h, sb, base, nreq, (int)total, sl.stream);
    // a small tick cannot hide a lane walking a long pair behind other work:
    // a handful of launches, pairs above 256 columns with G lanes each; a
    // large tick runs like the batched form, one tuned launch per segment
    if (e == cudaSuccess && total > 0) {
        if (total < cfg.latency_pairs)
            e = enqueue_tick(h, sb, base, segs, 7, sl.fork, sl.stream);
        else
            e = enqueue_segs_forked(h, sb, base, segs, (int)total, 100, sl.fork, sl.stream, false);
    }
    // the SIMD groups of flagged pairs, per request (errors into its table entry)
    if (e == cudaSuccess && total > 0) {
        LaunchArgs rg = base;
        rg.err_flags = &sb.ctrl->flags;
        rg.err_index = &sb.ctrl->bad_index;
        rg.cells = &sb.ctrl->cells;
        rg.P = h->kp;
        e = enqueue_regroup(sl.rg.V, rg, nreq, total, h->num_sms, sl.stream, nullptr);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.hreqs, dreqs, sizeof(ReqDesc) * nreq, cudaMemcpyDeviceToHost, sl.stream);
    for (Request *r : sl.reqs) {
        if (e != cudaSuccess) break;
        const uint8_t *src = pool + r->dev_off + r->off_pairs;
        void *dst = r->pinned ? (void *)r->pairs : (void *)(staging + r->st_off + r->off_pairs);
        e = cudaMemcpyAsync(dst, src, (size_t)r->n * sizeof(tal_seq_pair), cudaMemcpyDeviceToHost,
                            sl.stream);
    }
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, sl.stream);
    if (e == cudaSuccess) e = cudaLaunchHostFunc(sl.stream, wake_cb, this);
    const int64_t now = steady_ns();
    {
        std::lock_guard<std::mutex> lk(mu);
        for (Request *r : sl.reqs) {
            r->state = RUNNING;
            r->t_launch = now;
            r->tick_requests = nreq;
            r->tick_pairs = total;
        }
        st.ticks++;
        st.pairs += (uint64_t)total;
        st.max_tick_requests = std::max(st.max_tick_requests, nreq);
        st.launches = h->launches;
    }
    sl.busy = true;
    if (e != cudaSuccess) fatal = TAL_ECUDA;
    return e == cudaSuccess ? TAL_OK : TAL_ECUDA;
}

bool tal_bsw_server::launch_ticks() {
    bool any = false;
    for (Slot &sl : slots) {
        if (ready.empty()) break;
        if (sl.busy) continue;
        launch_tick(sl);
        any = true;
    }
    int running = 0;
    for (Slot &sl : slots) running += sl.busy ? 1 : 0;
    if (running > st.max_ticks_in_flight) {
        std::lock_guard<std::mutex> lk(mu);
        st.max_ticks_in_flight = std::max(st.max_ticks_in_flight, running);
    }
    return any;
}

bool tal_bsw_server::finish_ticks() {
    bool any = false;
    for (Slot &sl : slots) {
        if (!sl.busy) continue;
        const cudaError_t q = fatal != TAL_OK ? cudaErrorUnknown : cudaEventQuery(sl.done);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) {
            fatal = TAL_ECUDA;
            cudaStreamSynchronize(sl.stream);  // the work of a broken context ends at once
        }
        for (size_t k = 0; k < sl.reqs.size(); k++) {
            Request *r = sl.reqs[k];
            int status = TAL_OK;
            long long bad = -1;
            if (q != cudaSuccess) {
                status = TAL_ECUDA;
            } else if (sl.hreqs[k].err) {
                status = TAL_EDOMAIN;
                bad = sl.hreqs[k].bad;
            }
            if (q == cudaSuccess && !r->pinned)
                memcpy(r->pairs, staging + r->st_off + r->off_pairs, (size_t)r->n * sizeof(tal_seq_pair));
            {
                std::lock_guard<std::mutex> lk(mu);
                pool_arena.release(r->dev_off, r->bytes);
            }
            complete(r, status, bad);
        }
        sl.reqs.clear();
        sl.busy = false;
        any = true;
    }
    return any;
}

void tal_bsw_server::run() {
    cudaSetDevice(h->device);
    for (;;) {
        bool progress = finish_ticks();
        progress |= admit();
        progress |= launch_ticks();
        if (progress) continue;
        bool idle;
        {
            std::lock_guard<std::mutex> lk(mu);
            bool busy = false;
            for (Slot &sl : slots) busy |= sl.busy;
            idle = queue.empty() && ready.empty() && !busy;
            if (stop && idle) break;
        }
        std::unique_lock<std::mutex> lk(wake_mu);
        cv_wake.wait_for(lk, std::chrono::milliseconds(2), [&] { return wake_flag; });
        wake_flag = false;
    }
}

namespace {

bool is_pinned(const void *p, size_t bytes) {
    if (!p || bytes == 0) return true;
    for (const uint8_t *q : {(const uint8_t *)p, (const uint8_t *)p + bytes - 1}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost) return false;
    }
    return true;
}

void free_server(tal_bsw_server *s) {
    for (Slot &sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        sl.counts.release(); sl.order.release(); sl.order_req.release();
        sl.seg.release(); sl.ctrl.release(); sl.dreqs.release();
        sl.rg.release();
        if (sl.hreqs) cudaFreeHost(sl.hreqs);
        sl.fork.release();
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    if (s->copy_stream) {
        cudaStreamSynchronize(s->copy_stream);
        cudaStreamDestroy(s->copy_stream);
    }
    for (auto &kv : s->tickets) {
        if (kv.second->h2d) cudaEventDestroy(kv.second->h2d);
        delete kv.second;
    }
    if (s->pool) cudaFree(s->pool);
    if (s->staging) cudaFreeHost(s->staging);
    if (s->h) tal_bsw_destroy(s->h);
    delete s;
}

}  // namespace

extern "C" {

int64_t tal_bsw_now_ns(void) { return steady_ns(); }

int tal_bsw_server_create(tal_bsw_handle src, const tal_bsw_server_config *cfg,
                          tal_bsw_server_handle *out) {
    if (!src || !out) return TAL_EINVAL;
    *out = nullptr;
    tal_bsw_server_config c = cfg ? *cfg : tal_bsw_server_config{};
    // two ticks in flight: the next tick overlaps the current one's tail,
    // while more would split the GPU between ticks and stretch each one
    // (measured at 70 % of the batched peak: p99 31 ms with two, 47 with four)
    if (c.slots == 0) c.slots = 2;
    if (c.latency_pairs == 0) c.latency_pairs = 131072;
    if (c.max_tick_pairs == 0) c.max_tick_pairs = 8 << 20;
    if (c.staging_bytes == 0) c.staging_bytes = (size_t)1 << 30;
    if (c.slots < 1 || c.slots > 4 || c.max_tick_pairs < 1) return TAL_EINVAL;
    tal_bsw_server *s = new (std::nothrow) tal_bsw_server();
    if (!s) return TAL_ENOMEM;
    int rc = tal_bsw_create(&src->prm, src->device, &s->h);
    if (rc != TAL_OK) {
        delete s;
        return rc;
    }
    {
        std::lock_guard<std::mutex> lk(src->mu);
        s->h->tuned = src->tuned;
        for (int g = 0; g < kNumSegs; g++) s->h->bin_cfg[g] = src->bin_cfg[g];
    }
    cudaError_t e = cudaSetDevice(s->h->device);
    size_t free_b = 0, total_b = 0;
    if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) {
        free_server(s);
        return TAL_ECUDA;
    }
    if (c.pool_bytes == 0) c.pool_bytes = std::min<size_t>((size_t)64 << 30, free_b / 100 * 85);
    c.pool_bytes = round_up(c.pool_bytes);
    s->cfg = c;
    // device pool first: admission is by its free space
    e = cudaMalloc(&s->pool, c.pool_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        s->pool = nullptr;
        free_server(s);
        return TAL_ENOMEM;
    }
    s->pool_arena.init(c.pool_bytes);
    e = cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking);
    s->slots.resize(c.slots);
    for (Slot &sl : s->slots) {
        if (e != cudaSuccess) break;
        e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = sl.counts.ensure(sizeof(int) * kNumBuckets);
        if (e == cudaSuccess) e = sl.order.ensure(sizeof(int32_t) * (size_t)c.max_tick_pairs);
        if (e == cudaSuccess) e = sl.order_req.ensure(sizeof(int32_t) * (size_t)c.max_tick_pairs);
        if (e == cudaSuccess) e = sl.seg.ensure(sizeof(int32_t) * 2 * kNumSegs);
        if (e == cudaSuccess) e = sl.ctrl.ensure(sizeof(BatchCtrl));
        if (e == cudaSuccess) e = sl.dreqs.ensure(sizeof(ReqDesc) * kMaxTickRequests);
        bool grown = false;
        if (e == cudaSuccess) e = sl.rg.ensure(c.max_tick_pairs, 32767, s->h->num_sms, &grown);
        if (e == cudaSuccess) e = sl.fork.create();
        if (e == cudaSuccess)
            e = cudaHostAlloc(reinterpret_cast<void **>(&sl.hreqs), sizeof(ReqDesc) * kMaxTickRequests,
                              cudaHostAllocDefault);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        free_server(s);
        return e == cudaErrorMemoryAllocation ? TAL_ENOMEM : TAL_ECUDA;
    }
    s->st.pool_bytes = c.pool_bytes;
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return TAL_OK;
}

int tal_bsw_server_destroy(tal_bsw_server_handle s) {
    if (!s) return TAL_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->wake();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->h->device);
    free_server(s);
    return TAL_OK;
}

int tal_bsw_submit(tal_bsw_server_handle s, tal_seq_pair *pairs, const uint8_t *seqBufRef,
                   const uint8_t *seqBufQer, int32_t numPairs, int32_t w, const int32_t *wpair,
                   int bits, uint64_t *ticket) {
    if (!s || !ticket) return TAL_EINVAL;
    const int64_t t0 = steady_ns();
    if (numPairs < 0 || numPairs > s->cfg.max_tick_pairs || (bits != 0 && bits != 8 && bits != 16))
        return TAL_EINVAL;
    if (numPairs > 0 && (!pairs || !seqBufRef || !seqBufQer)) return TAL_EINVAL;
    Request *r = new (std::nothrow) Request();
    if (!r) return TAL_ENOMEM;
    r->pairs = pairs; r->ref = seqBufRef; r->qer = seqBufQer; r->wpair = wpair;
    r->n = numPairs; r->w = w; r->bits = bits;
    r->t_submit = t0;
    // windows of the sequence buffers and pairs per length bin
    long long rlo = LLONG_MAX, rhi = 0, qlo = LLONG_MAX, qhi = 0;
    long long bad = -1;
    for (int32_t k = 0; k < numPairs; k++) {
        const tal_seq_pair &p = pairs[k];
        if (p.len1 < 0 || p.len2 < 0 || p.idr < 0 || p.idq < 0) {
            bad = k;
            break;
        }
        rlo = std::min<long long>(rlo, p.idr);
        qlo = std::min<long long>(qlo, p.idq);
        rhi = std::max<long long>(rhi, (long long)p.idr + p.len1);
        qhi = std::max<long long>(qhi, (long long)p.idq + p.len2);
        r->segs[host_seg(p.len2, wpair ? wpair[k] : w)]++;
    }
    bool done_now = numPairs == 0 || bad >= 0;
    if (!done_now) {
        rlo &= ~15LL;
        // the padding lanes of a request's last partial 8-bit group, when its
        // SIMD groups are re-scored exactly, read the query at offset 0
        if (bits != 16 && qlo <= (1 << 20)) qlo = 0;
        qlo &= ~15LL;
        if (rhi <= rlo) rhi = rlo + 16;
        if (qhi <= qlo) qhi = qlo + 16;
        r->rlo = rlo; r->rhi = rhi; r->qlo = qlo; r->qhi = qhi;
        r->off_pairs = 0;
        r->off_ref = round_up((size_t)numPairs * sizeof(tal_seq_pair));
        r->off_qer = r->off_ref + round_up((size_t)(rhi - rlo) + 16);
        r->off_w = r->off_qer + round_up((size_t)(qhi - qlo) + 16);
        r->bytes = r->off_w + (wpair ? round_up((size_t)numPairs * sizeof(int32_t)) : 0);
        if (r->bytes > s->cfg.pool_bytes) {
            delete r;
            return TAL_ENOMEM;
        }
        r->pinned = is_pinned(pairs, (size_t)numPairs * sizeof(tal_seq_pair)) &&
                    is_pinned(seqBufRef + rlo, (size_t)(rhi - rlo)) &&
                    is_pinned(seqBufQer + qlo, (size_t)(qhi - qlo)) &&
                    (!wpair || is_pinned(wpair, (size_t)numPairs * sizeof(int32_t)));
        if (!r->pinned) {
            if (r->bytes > s->cfg.staging_bytes) {
                delete r;
                return TAL_ENOMEM;
            }
            std::lock_guard<std::mutex> lk(s->mu);
            if (!s->staging) {
                if (cudaSetDevice(s->h->device) != cudaSuccess ||
                    cudaHostAlloc(reinterpret_cast<void **>(&s->staging), s->cfg.staging_bytes,
                                  cudaHostAllocDefault) != cudaSuccess) {
                    cudaGetLastError();
                    s->staging = nullptr;
                    delete r;
                    return TAL_ENOMEM;
                }
                s->staging_arena.init(s->cfg.staging_bytes);
            }
            if (!s->staging_arena.alloc(r->bytes, &r->st_off)) {
                delete r;
                return TAL_EBUSY;
            }
            r->staged = true;
        }
        if (r->staged) {  // the caller's buffers into the pinned region, pool layout
            uint8_t *d = s->staging + r->st_off;
            memcpy(d + r->off_pairs, pairs, (size_t)numPairs * sizeof(tal_seq_pair));
            memcpy(d + r->off_ref, seqBufRef + rlo, (size_t)(rhi - rlo));
            memcpy(d + r->off_qer, seqBufQer + qlo, (size_t)(qhi - qlo));
            if (wpair) memcpy(d + r->off_w, wpair, (size_t)numPairs * sizeof(int32_t));
        }
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->ticket = s->next_ticket++;
        s->tickets[r->ticket] = r;
        s->st.submitted++;
        if (done_now) {
            r->status = bad >= 0 ? TAL_EDOMAIN : TAL_OK;
            r->bad = bad;
            r->state = DONE;
            r->t_admit = r->t_launch = r->t_done = steady_ns();
            s->st.completed++;
            if (bad >= 0) s->st.failed++;
        } else {
            s->queue.push_back(r);
        }
        *ticket = r->ticket;
    }
    if (!done_now) s->wake();
    return TAL_OK;
}

int tal_bsw_poll(tal_bsw_server_handle s, uint64_t ticket, int64_t timeout_us,
                 tal_bsw_request_info *info) {
    if (!s) return TAL_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return TAL_EINVAL;
    Request *r = it->second;
    auto done = [&] { return r->state == DONE; };
    if (!done()) {
        if (timeout_us == 0) return TAL_ETIMEOUT;
        if (timeout_us < 0) s->cv_done.wait(lk, done);
        else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), done))
            return TAL_ETIMEOUT;
    }
    if (info) {
        info->status = r->status;
        info->tick_requests = r->tick_requests;
        info->bad_pair = r->bad;
        info->tick_pairs = r->tick_pairs;
        info->submit_ns = r->t_submit;
        info->admit_ns = r->t_admit;
        info->launch_ns = r->t_launch;
        info->done_ns = r->t_done;
    }
    s->tickets.erase(it);
    lk.unlock();
    if (r->h2d) cudaEventDestroy(r->h2d);
    delete r;
    return TAL_OK;
}

int tal_bsw_server_get_stats(tal_bsw_server_handle s, tal_bsw_server_stats *out) {
    if (!s || !out) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->pool_used_bytes = s->pool_arena.used();
    out->pool_peak_bytes = s->pool_arena.peak();
    int q = 0, a = 0, ru = 0;
    for (auto &kv : s->tickets) {
        q += kv.second->state == QUEUED;
        a += kv.second->state == ADMITTED;
        ru += kv.second->state == RUNNING;
    }
    out->queued = q;
    out->admitted = a;
    out->running = ru;
    return TAL_OK;
}

}  // extern "C"
