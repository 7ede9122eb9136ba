// C ABI of the anchor chaining DP (include/tal_chain.h): handle, host<->device
// staging, read ordering, launch of chain_kernel.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/tal_chain.h"
#include "bsw_ctx.h"
#include "chain_kernel.cuh"

static_assert(sizeof(tal_anchor) == 16, "anchor_t is 16 bytes");
static_assert(sizeof(talchain::Anchor) == 16, "device view");

namespace {

constexpr int kBlocksPerSm = 8;

struct ChainCtrl {
    int counter;
    int flags;
    long long bad;
    unsigned long long evals;
};

}  // namespace

struct tal_chain_ctx {
    tal_chain_params prm;
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    talbsw::DevBuf anchors, offsets, order, out_f, out_p, out_v, ctrl, rq;
    std::mutex mu;
    std::string last_error;
    int64_t last_bad = -1;
    uint64_t last_evals = 0;
};

namespace {

int cfail(tal_chain_ctx *h, int code, const std::string &msg) {
    h->last_error = msg;
    return code;
}

// Blocks (of four warps) resident per SM: few, so that the predecessor
// windows of the resident warps stay in L1.  TAL_CHAIN_BPS overrides (tuning).
int blocks_per_sm() {
    if (const char *e = getenv("TAL_CHAIN_BPS")) {
        const int b = atoi(e);
        if (b >= 1 && b <= 16) return b;
    }
    return kBlocksPerSm;
}

// Launches the kernel over device-resident reads and collects the status.
int run_locked(tal_chain_ctx *h, const tal_anchor *d_anchors, const int64_t *d_offsets,
               const int32_t *d_order, int32_t n_reads, int64_t n_anchors, int32_t dr, int32_t dq,
               uint32_t *d_f, int32_t *d_p, int32_t *d_v) {
    cudaError_t e;
    if ((e = h->ctrl.ensure(sizeof(ChainCtrl))) != cudaSuccess)
        return cfail(h, TAL_ENOMEM, "control block");
    if ((e = h->rq.ensure(8 * (size_t)std::max<int64_t>(n_anchors, 1))) != cudaSuccess)
        return cfail(h, TAL_ENOMEM, "scan scratch");
    ChainCtrl init = {0, 0, LLONG_MAX, 0ull};
    e = cudaMemcpyAsync(h->ctrl.p, &init, sizeof(init), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cfail(h, TAL_ECUDA, cudaGetErrorString(e));
    ChainCtrl *c = reinterpret_cast<ChainCtrl *>(h->ctrl.p);
    talchain::ChainArgs A;
    memset(&A, 0, sizeof(A));
    A.anchors = reinterpret_cast<const talchain::Anchor *>(d_anchors);
    A.offsets = d_offsets;
    A.order = d_order;
    A.n_reads = n_reads;
    A.bw = h->prm.bw;
    A.max_iter = h->prm.max_iter;
    A.dr = dr;
    A.dq = dq;
    A.rq = reinterpret_cast<int2 *>(h->rq.p);
    A.f = d_f;
    A.p = d_p;
    A.v = d_v;
    A.work_counter = &c->counter;
    A.evals = &c->evals;
    A.err_flags = &c->flags;
    A.err_index = &c->bad;
    const int wpb = 4;
    const size_t smem = wpb * talchain::chain_warp_smem_bytes(A.bw);  // rings and gap tables
    e = cudaFuncSetAttribute(talchain::chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cfail(h, TAL_ECUDA, "shared memory opt-in");
    int bps = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, talchain::chain_kernel, 32 * wpb, smem);
    if (e != cudaSuccess || bps < 1) return cfail(h, TAL_ECUDA, "occupancy query");
    long long blocks = (long long)std::min(bps, blocks_per_sm()) * h->num_sms;
    blocks = std::min<long long>(blocks, ((long long)n_reads + wpb - 1) / wpb);
    talchain::chain_kernel<<<(unsigned)std::max<long long>(blocks, 1), 32 * wpb, smem, h->stream>>>(A);
    if ((e = cudaGetLastError()) != cudaSuccess) return cfail(h, TAL_ECUDA, cudaGetErrorString(e));
    ChainCtrl out;
    e = cudaMemcpyAsync(&out, c, sizeof(out), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cfail(h, TAL_ECUDA, cudaGetErrorString(e));
    h->last_evals = out.evals;
    if (out.flags) {
        h->last_bad = out.bad;
        return cfail(h, TAL_EDOMAIN, "read outside the domain (negative anchor length or "
                                     "2^31+ anchors), first bad read " + std::to_string(out.bad));
    }
    return TAL_OK;
}

}  // namespace

extern "C" {

int tal_chain_create(const tal_chain_params *params, int device, tal_chain_handle *out) {
    if (!params || !out) return TAL_EINVAL;
    *out = nullptr;
    if (params->max_iter < 0 || params->bw < 0) return TAL_EINVAL;
    int dev = device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return TAL_ENODEV;
    if (cudaSetDevice(dev) != cudaSuccess) return TAL_ENODEV;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major != 10) return TAL_ENODEV;
    tal_chain_ctx *h = new (std::nothrow) tal_chain_ctx();
    if (!h) return TAL_ENOMEM;
    h->prm = *params;
    h->device = dev;
    h->num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return TAL_ECUDA;
    }
    *out = h;
    return TAL_OK;
}

int tal_chain_destroy(tal_chain_handle h) {
    if (!h) return TAL_EINVAL;
    {
        std::lock_guard<std::mutex> lk(h->mu);
        cudaSetDevice(h->device);
        cudaStreamSynchronize(h->stream);
        for (talbsw::DevBuf *b : {&h->anchors, &h->offsets, &h->order, &h->out_f, &h->out_p,
                                  &h->out_v, &h->ctrl, &h->rq})
            b->release();
        cudaStreamDestroy(h->stream);
    }
    delete h;
    return TAL_OK;
}

int tal_chain_dp(tal_chain_handle h, const tal_anchor *anchors, const int64_t *offsets,
                 int32_t n_reads, int32_t dr, int32_t dq, uint32_t *f, int32_t *p, int32_t *v) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->last_error.clear();
    h->last_bad = -1;
    h->last_evals = 0;
    if (n_reads < 0 || !offsets) return cfail(h, TAL_EINVAL, "bad n_reads or NULL offsets");
    if (n_reads == 0) return TAL_OK;
    const int64_t base = offsets[0];
    if (base < 0) return cfail(h, TAL_EINVAL, "negative offset");
    for (int32_t k = 0; k < n_reads; k++) {
        const int64_t n = offsets[k + 1] - offsets[k];
        if (n < 0) return cfail(h, TAL_EINVAL, "offsets decrease at read " + std::to_string(k));
        if (n > INT_MAX) {
            h->last_bad = k;
            return cfail(h, TAL_EDOMAIN, "read " + std::to_string(k) + " has 2^31 anchors or more");
        }
    }
    const int64_t total = offsets[n_reads] - base;
    if (total == 0) return TAL_OK;
    if (!anchors || !f || !p || !v) return cfail(h, TAL_EINVAL, "NULL buffer");
    if (cudaSetDevice(h->device) != cudaSuccess) return cfail(h, TAL_ECUDA, "cudaSetDevice");
    // rebased offsets, and the reads longest first so no long read starts last
    std::vector<int64_t> offs((size_t)n_reads + 1);
    for (int32_t k = 0; k <= n_reads; k++) offs[k] = offsets[k] - base;
    std::vector<int32_t> order((size_t)n_reads);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return offs[x + 1] - offs[x] > offs[y + 1] - offs[y];
    });
    const size_t ab = sizeof(tal_anchor) * (size_t)total, ob = 4 * (size_t)total;
    cudaError_t e;
    if ((e = h->anchors.ensure(ab)) != cudaSuccess || (e = h->offsets.ensure(8 * offs.size())) != cudaSuccess ||
        (e = h->order.ensure(4 * order.size())) != cudaSuccess || (e = h->out_f.ensure(ob)) != cudaSuccess ||
        (e = h->out_p.ensure(ob)) != cudaSuccess || (e = h->out_v.ensure(ob)) != cudaSuccess)
        return cfail(h, TAL_ENOMEM, cudaGetErrorString(e));
    e = cudaMemcpyAsync(h->anchors.p, anchors + base, ab, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->offsets.p, offs.data(), 8 * offs.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->order.p, order.data(), 4 * order.size(), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cfail(h, TAL_ECUDA, cudaGetErrorString(e));
    int rc = run_locked(h, reinterpret_cast<const tal_anchor *>(h->anchors.p),
                        reinterpret_cast<const int64_t *>(h->offsets.p),
                        reinterpret_cast<const int32_t *>(h->order.p), n_reads, total, dr, dq,
                        reinterpret_cast<uint32_t *>(h->out_f.p), reinterpret_cast<int32_t *>(h->out_p.p),
                        reinterpret_cast<int32_t *>(h->out_v.p));
    if (rc != TAL_OK) return rc;
    e = cudaMemcpyAsync(f + base, h->out_f.p, ob, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p + base, h->out_p.p, ob, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v + base, h->out_v.p, ob, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cfail(h, TAL_ECUDA, cudaGetErrorString(e));
    return TAL_OK;
}

int tal_chain_dp_device(tal_chain_handle h, const tal_anchor *d_anchors, const int64_t *d_offsets,
                        int32_t n_reads, int32_t dr, int32_t dq, uint32_t *d_f, int32_t *d_p,
                        int32_t *d_v) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->last_error.clear();
    h->last_bad = -1;
    h->last_evals = 0;
    if (n_reads < 0) return cfail(h, TAL_EINVAL, "bad n_reads");
    if (n_reads == 0) return TAL_OK;
    if (!d_anchors || !d_offsets || !d_f || !d_p || !d_v) return cfail(h, TAL_EINVAL, "NULL buffer");
    if (cudaSetDevice(h->device) != cudaSuccess) return cfail(h, TAL_ECUDA, "cudaSetDevice");
    // the scan scratch is indexed like the anchors: their count is the last offset
    int64_t n_anchors = 0;
    cudaError_t e = cudaMemcpyAsync(&n_anchors, d_offsets + n_reads, sizeof(n_anchors),
                                    cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cfail(h, TAL_ECUDA, cudaGetErrorString(e));
    if (n_anchors < 0) return cfail(h, TAL_EINVAL, "negative last offset");
    // longest reads first (a device counting sort of the reads by anchor count)
    const size_t hb = sizeof(int) * talchain::kChainBuckets;
    if ((e = h->order.ensure(4 * (size_t)n_reads + hb)) != cudaSuccess)
        return cfail(h, TAL_ENOMEM, "read order");
    int32_t *order = reinterpret_cast<int32_t *>(h->order.p);
    int *hist = reinterpret_cast<int *>(order + n_reads);
    e = cudaMemsetAsync(hist, 0, hb, h->stream);
    if (e != cudaSuccess) return cfail(h, TAL_ECUDA, cudaGetErrorString(e));
    const int gb = (int)std::min<long long>(((long long)n_reads + 255) / 256, 4LL * h->num_sms);
    talchain::ch_bucket_count<<<gb, 256, 0, h->stream>>>(d_offsets, n_reads, hist);
    talbsw::bucket_scan_4096<<<1, 1024, 0, h->stream>>>(hist);
    talchain::ch_bucket_scatter<<<gb, 256, 0, h->stream>>>(d_offsets, n_reads, hist, order);
    if ((e = cudaGetLastError()) != cudaSuccess) return cfail(h, TAL_ECUDA, cudaGetErrorString(e));
    return run_locked(h, d_anchors, d_offsets, order, n_reads, n_anchors, dr, dq, d_f, d_p, d_v);
}

void *tal_chain_stream(tal_chain_handle h) { return h ? (void *)h->stream : nullptr; }
const char *tal_chain_last_error(tal_chain_handle h) { return h ? h->last_error.c_str() : "null handle"; }
int64_t tal_chain_last_bad_read(tal_chain_handle h) { return h ? h->last_bad : -1; }
uint64_t tal_chain_last_evals(tal_chain_handle h) { return h ? h->last_evals : 0; }

}  // extern "C"
