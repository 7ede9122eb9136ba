// C ABI of the GB300 banded Smith-Waterman (include/tal_bsw.h): handle
// management, host<->device staging and kernel launches.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "bsw_ctx.h"
#include "bsw_group.cuh"
#include "bucket_scan.cuh"

static_assert(sizeof(tal_seq_pair) == 56, "SeqPair is 14 x int32 (bandedSWA.h:90-99)");
static_assert(sizeof(talbsw::DevPair) == 56, "device SeqPair view");

using talbsw::DevBuf;

namespace {

int fail(tal_bsw_ctx *h, int code, const std::string &msg) {
    if (h) h->last_error = msg;
    return code;
}

int cuda_fail(tal_bsw_ctx *h, cudaError_t e, const char *what) {
    return fail(h, TAL_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// control block on the device: work counter, error flags, first bad index
struct Ctrl {
    int counter;
    int flags;
    long long bad_index;
    unsigned long long cells;
};

// Work order of a plain launch: the reference sorts each thread's pairs by
// target length before scoring them (sortPairsLen, bandedSWA.cpp:1909-1950,
// called at :2742 and :2046) so that a SIMD group's pairs end together; here
// the order groups pairs of about the same target length (buckets of four
// bases, longest first) into the same warp.  Outputs do not depend on it.
constexpr int kOrderMin = 2048;  // smaller batches keep their order

__device__ __forceinline__ int plain_bucket(const talbsw::DevPair &p) {
    int b = p.len1 < 0 ? 0 : p.len1 >> 2;
    b = b > talbsw::kScanBuckets - 1 ? talbsw::kScanBuckets - 1 : b;
    return (talbsw::kScanBuckets - 1) - b;
}

__global__ void plain_count(const talbsw::DevPair *pairs, int n, int *hist) {
    __shared__ int sh[talbsw::kScanBuckets];
    for (int t = threadIdx.x; t < talbsw::kScanBuckets; t += blockDim.x) sh[t] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&sh[plain_bucket(pairs[i])], 1);
    __syncthreads();
    for (int t = threadIdx.x; t < talbsw::kScanBuckets; t += blockDim.x)
        if (sh[t]) atomicAdd(&hist[t], sh[t]);
}

// Each block places a contiguous chunk of pairs: it counts the chunk per
// bucket, reserves the chunk's range of every bucket with one global atomic,
// then hands out positions inside those ranges with shared-memory atomics.
__global__ void plain_scatter(const talbsw::DevPair *pairs, int n, int *offs, int32_t *order) {
    __shared__ int sh[talbsw::kScanBuckets];
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    for (int t = threadIdx.x; t < talbsw::kScanBuckets; t += blockDim.x) sh[t] = 0;
    __syncthreads();
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) atomicAdd(&sh[plain_bucket(pairs[i])], 1);
    __syncthreads();
    for (int t = threadIdx.x; t < talbsw::kScanBuckets; t += blockDim.x)
        if (sh[t]) sh[t] = atomicAdd(&offs[t], sh[t]);
    __syncthreads();
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x)
        order[atomicAdd(&sh[plain_bucket(pairs[i])], 1)] = i;
}

cudaError_t enqueue_plain_order(tal_bsw_ctx *h, talbsw::LaunchArgs &A) {
    const size_t hb = sizeof(int) * talbsw::kScanBuckets;
    cudaError_t e = h->porder.ensure(4 * (size_t)A.n + hb);
    if (e != cudaSuccess) return e;
    int32_t *order = reinterpret_cast<int32_t *>(h->porder.p);
    int *hist = reinterpret_cast<int *>(order + A.n);
    if ((e = cudaMemsetAsync(hist, 0, hb, h->stream)) != cudaSuccess) return e;
    const int gb = (int)std::min<long long>(((long long)A.n + 255) / 256, 2LL * h->num_sms);
    plain_count<<<gb, 256, 0, h->stream>>>(A.pairs, A.n, hist);
    talbsw::bucket_scan_4096<<<1, 1024, 0, h->stream>>>(hist);
    plain_scatter<<<gb, 256, 0, h->stream>>>(A.pairs, A.n, hist, order);
    h->launches += 3;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    A.order = order;
    return cudaSuccess;
}

// Host-buffer calls from this many pairs copy and score in kChunks chunks
// (chunk k + 1's copies overlap chunk k's scoring); each chunk has its own
// control block.
constexpr int kChunks = 4;
constexpr int kChunkMin = 262144;

int collect_chunks(tal_bsw_ctx *h, int nslots, int32_t per);
int collect(tal_bsw_ctx *h) { return collect_chunks(h, 1, 0); }

// Issues the scoring launch for pairs already on the device (control block
// `slot`).
int launch_scoring(tal_bsw_ctx *h, talbsw::LaunchArgs A, int w_for_k, int slot = 0) {
    Ctrl *c = reinterpret_cast<Ctrl *>(h->ctrl.p) + slot;
    A.work_counter = &c->counter;
    A.err_flags = &c->flags;
    A.err_index = &c->bad_index;
    A.cells = &c->cells;
    A.P = h->kp;
    // one band for every pair: the lane kernel keeps a ring of columns
    A.win = A.wpair ? 0 : talbsw::lane_window(A.w, A.cols_cap);
    talbsw::KConfig cfg = talbsw::fit_config(talbsw::choose_config(w_for_k, A.cols_cap, A.win),
                                             A.cols_cap, h->smem_optin, A.win);
    if (talbsw::config_smem(cfg, A.cols_cap, A.rows_cap, A.win) > h->smem_optin) {
        if (!A.flagged) return fail(h, TAL_EDOMAIN, "pair too long for the shared-memory row buffers");
        // exact mode: the per-pair kernels take the pairs whose rows fit and
        // flag the longer ones, whose groups the regroup pass scores (rows in
        // global scratch)
        int cc = A.cols_cap;
        do {
            cc = cc > 1056 ? cc - 512 : cc / 2;
            A.win = A.wpair ? 0 : talbsw::lane_window(A.w, cc);
            cfg = talbsw::fit_config(talbsw::choose_config(w_for_k, cc, A.win), cc, h->smem_optin, A.win);
        } while (cc > 32 && talbsw::config_smem(cfg, cc, A.rows_cap, A.win) > h->smem_optin);
        A.cols_cap = cc;
    }
    Ctrl init = {0, 0, (long long)INT64_MAX, 0ull};
    cudaError_t e = cudaMemcpyAsync(c, &init, sizeof(Ctrl), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemcpyAsync(ctrl)");
    if (A.order == nullptr && A.n >= kOrderMin && !getenv("TAL_BSW_NO_ORDER")) {
        if ((e = enqueue_plain_order(h, A)) != cudaSuccess) return cuda_fail(h, e, "work order");
    }
    if (h->kev0) cudaEventRecord(h->kev0, h->stream);
    e = talbsw::launch_config(A, cfg, h->num_sms, h->smem_optin, h->stream);
    if (h->kev1) cudaEventRecord(h->kev1, h->stream);
    h->launches++;
    if (e != cudaSuccess) return cuda_fail(h, e, "kernel launch");
    return TAL_OK;
}

// Grouped scoring (TAL_BSW_GROUPED) of pairs already on the device: one warp
// per SIMD group of the reference, each with a scratch slot of the group's
// rows (cols_cap = the longest query), up to 48 warps per SM (as many as
// fit) and 1 GiB of scratch.
int launch_grouped(tal_bsw_ctx *h, const talbsw::LaunchArgs &A, int slot = 0) {
    Ctrl *c = reinterpret_cast<Ctrl *>(h->ctrl.p) + slot;
    talbsw::GroupArgs G;
    memset(&G, 0, sizeof(G));
    G.pairs = A.pairs;
    G.ref = A.ref; G.qer = A.qer;
    G.ref_lo = A.ref_lo; G.ref_hi = A.ref_hi; G.qer_lo = A.qer_lo; G.qer_hi = A.qer_hi;
    G.n = A.n;
    G.w = A.w;
    G.bits = A.bits;
    G.col_cap = std::max(A.cols_cap, 1) + 3;
    G.slot_elems = talbsw::group_slot_elems(G.col_cap, A.bits);
    G.work_counter = &c->counter;
    G.err_flags = &c->flags;
    G.err_index = &c->bad_index;
    G.cells = &c->cells;
    G.P = h->kp;
    const long long ngroups = ((long long)A.n + talbsw::group_lanes(A.bits) - 1) / talbsw::group_lanes(A.bits);
    const long long slot_bytes = (long long)G.slot_elems * 2;
    int wps = 48;  // warps per SM, as many as fit (tuning: TAL_BSW_GROUP_WARPS; 32 / 48 measured 142 / 150 GCUPS on C2)
    if (const char *ev = getenv("TAL_BSW_GROUP_WARPS")) wps = std::min(std::max(atoi(ev), 4), 64);
    long long warps = std::min<long long>((long long)h->num_sms * wps, ngroups);
    warps = std::min<long long>(warps, std::max<long long>(4, (1LL << 30) / slot_bytes));
    const int blocks = (int)((warps + 3) / 4);
    cudaError_t e = h->gscratch.ensure((size_t)blocks * 4 * (size_t)slot_bytes);
    if (e != cudaSuccess) return fail(h, TAL_ENOMEM, "grouped scoring scratch");
    G.scratch = reinterpret_cast<int16_t *>(h->gscratch.p);
    Ctrl init = {0, 0, (long long)INT64_MAX, 0ull};
    e = cudaMemcpyAsync(c, &init, sizeof(Ctrl), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemcpyAsync(ctrl)");
    if (h->kev0) cudaEventRecord(h->kev0, h->stream);
    if (A.bits == 8)
        talbsw::bsw_group_kernel<8><<<blocks, 128, 0, h->stream>>>(G);
    else
        talbsw::bsw_group_kernel<16><<<blocks, 128, 0, h->stream>>>(G);
    e = cudaGetLastError();
    if (h->kev1) cudaEventRecord(h->kev1, h->stream);
    h->launches++;
    if (e != cudaSuccess) return cuda_fail(h, e, "grouped kernel launch");
    return TAL_OK;
}

// Sizes the regroup arena for a call of n pairs with queries up to max2;
// captured batched graphs hold its old pointers when it grows.
int ensure_regroup(tal_bsw_ctx *h, long long n, int max2) {
    bool grown = false;
    cudaError_t e = h->regroup.ensure(n, max2, h->num_sms, &grown);
    if (e != cudaSuccess) return fail(h, TAL_ENOMEM, std::string("regroup buffers: ") + cudaGetErrorString(e));
    if (grown) {
        for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
        h->graphs.clear();
    }
    return TAL_OK;
}

// Re-scores the SIMD groups of the pairs a plain launch flagged (A: the
// call's pairs, windows, band and precision); status into control block 0.
int launch_regroup(tal_bsw_ctx *h, talbsw::LaunchArgs A) {
    Ctrl *c = reinterpret_cast<Ctrl *>(h->ctrl.p);
    A.err_flags = &c->flags;
    A.err_index = &c->bad_index;
    A.cells = &c->cells;
    A.P = h->kp;
    cudaError_t e = talbsw::enqueue_regroup(h->regroup.V, A, 0, A.n, h->num_sms, h->stream, &h->launches);
    if (e != cudaSuccess) return cuda_fail(h, e, "regroup launch");
    return TAL_OK;
}

// Waits for the launches of control blocks [0, nslots) and merges their
// status: flags or-ed, the first bad pair (block k's pair indices start at
// k * per), cells summed.
int collect_chunks(tal_bsw_ctx *h, int nslots, int32_t per) {
    Ctrl cs[kChunks];
    cudaError_t e = cudaMemcpyAsync(cs, h->ctrl.p, sizeof(Ctrl) * nslots, cudaMemcpyDeviceToHost,
                                    h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "scoring");
    if (h->kev0 && h->kev1 && cudaEventElapsedTime(&h->last_kernel_ms, h->kev0, h->kev1) != cudaSuccess)
        h->last_kernel_ms = 0.f;
    Ctrl c = {0, 0, (long long)INT64_MAX, 0ull};
    for (int k = 0; k < nslots; k++) {
        c.flags |= cs[k].flags;
        if (cs[k].flags) c.bad_index = std::min(c.bad_index, (long long)k * per + cs[k].bad_index);
        c.cells += cs[k].cells;
    }
    h->last_cells = c.cells;
    if (c.flags) {
        h->last_bad = c.bad_index;
        std::string why;
        if (c.flags & talbsw::ERR_DOMAIN) why += "pair outside the exact 8/16-bit range; ";
        if (c.flags & talbsw::ERR_CAPACITY) why += "pair longer than the row capacity; ";
        if (c.flags & talbsw::ERR_BASE) why += "base code above 4; ";
        if (c.flags & talbsw::ERR_FLAGCAP)
            why += "more than 1024 band / precision classes among pairs that need group scoring; ";
        return fail(h, TAL_EDOMAIN, why + "first bad pair " + std::to_string(c.bad_index));
    }
    return TAL_OK;
}

}  // namespace

extern "C" {

int tal_bsw_create(const tal_bsw_params *params, int device, tal_bsw_handle *out) {
    if (!params || !out) return TAL_EINVAL;
    *out = nullptr;
    const tal_bsw_params &p = *params;
    auto in = [](int v, int lo, int hi) { return v >= lo && v <= hi; };
    if (!in(p.o_del, 0, 127) || !in(p.o_ins, 0, 127) || !in(p.e_del, 1, 127) ||
        !in(p.e_ins, 1, 127) || !in(p.w_match, 0, 127) || !in(p.w_mismatch, 0, 127))
        return TAL_EINVAL;
    int dev = device;
    cudaError_t e;
    if (dev < 0) {
        e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return TAL_ENODEV;
    }
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) return TAL_ENODEV;
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return TAL_ENODEV;
    if (prop.major != 10) return TAL_ENODEV;
    tal_bsw_ctx *h = new (std::nothrow) tal_bsw_ctx();
    if (!h) return TAL_ENOMEM;
    h->prm = p;
    h->kp = {p.o_del, p.e_del, p.o_ins, p.e_ins, p.zdrop, p.end_bonus, p.w_match, p.w_mismatch};
    h->device = dev;
    h->num_sms = prop.multiProcessorCount;
    h->smem_optin = prop.sharedMemPerBlockOptin;
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = h->ctrl.ensure(sizeof(Ctrl) * kChunks);
    if (e == cudaSuccess) e = cudaEventCreate(&h->kev0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->kev1);
    if (e != cudaSuccess) {
        if (h->kev0) cudaEventDestroy(h->kev0);
        if (h->kev1) cudaEventDestroy(h->kev1);
        if (h->stream) cudaStreamDestroy(h->stream);
        h->ctrl.release();
        delete h;
        return e == cudaErrorMemoryAllocation ? TAL_ENOMEM : TAL_ECUDA;
    }
    *out = h;
    return TAL_OK;
}

int tal_bsw_destroy(tal_bsw_handle h) {
    if (!h) return TAL_EINVAL;
    {
        std::lock_guard<std::mutex> lk(h->mu);
        cudaSetDevice(h->device);
        cudaStreamSynchronize(h->stream);
        h->pairs.release();
        h->ref.release();
        h->qer.release();
        h->ctrl.release();
        h->wpair.release();
        h->caps.release();
        h->bcounts.release();
        h->border.release();
        h->porder.release();
        for (DevBuf *b : {&h->xref, &h->xreads, &h->xjobs, &h->xpairs, &h->xtarena, &h->xqarena,
                          &h->xout, &h->xretry, &h->gscratch})
            b->release();
        h->regroup.release();
        h->bseg.release();
        h->bctrl.release();
        h->btune_seg.release();
        h->bfork.release();
        for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second.exec);
        h->graphs.clear();
        for (cudaEvent_t &ev : h->cev)
            if (ev) cudaEventDestroy(ev);
        if (h->kev0) cudaEventDestroy(h->kev0);
        if (h->kev1) cudaEventDestroy(h->kev1);
        if (h->cstream) cudaStreamDestroy(h->cstream);
        cudaStreamDestroy(h->stream);
    }
    delete h;
    return TAL_OK;
}

int tal_bsw_scores(tal_bsw_handle h, tal_seq_pair *pairs, const uint8_t *seqBufRef,
                   const uint8_t *seqBufQer, int32_t numPairs, int32_t w, int bits) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->last_error.clear();
    h->last_bad = -1;
    const bool grouped = (bits & TAL_BSW_GROUPED) != 0;
    const bool perpair = (bits & TAL_BSW_PER_PAIR) != 0;  // each pair alone: no regrouping
    bits &= ~(TAL_BSW_GROUPED | TAL_BSW_PER_PAIR);
    if (numPairs < 0 || (bits != 0 && bits != 8 && bits != 16) || (grouped && bits == 0) ||
        (grouped && perpair))
        return fail(h, TAL_EINVAL, "bad numPairs or bits");
    const bool exact = !grouped && !perpair;  // per-pair kernels + regroup pass
    if (numPairs == 0) return TAL_OK;
    if (!pairs || !seqBufRef || !seqBufQer) return fail(h, TAL_EINVAL, "NULL buffer");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    // Per chunk of pairs: the byte windows they reference and their row
    // capacities (one host thread per chunk)
    struct Ext {
        long long rlo = LLONG_MAX, rhi = 0, qlo = LLONG_MAX, qhi = 0;
        int max1 = 0, max2 = 0;
        int32_t bad = -1;
    };
    int nch = numPairs >= kChunkMin ? kChunks : 1;
    if (const char *ev = getenv("TAL_BSW_CHUNKS")) {  // tuning: 1 .. kChunks
        const int c = atoi(ev);
        if (c >= 1 && c <= kChunks) nch = numPairs >= kChunkMin ? c : 1;
    }
    int32_t per = (numPairs + nch - 1) / nch;
    if (grouped) per = (per + 63) & ~63;  // chunks end on SIMD-group boundaries
    Ext ext[kChunks];
    auto scan = [&](int c) {
        Ext &x = ext[c];
        const int32_t k1 = std::min<int32_t>(numPairs, (c + 1) * per);
        for (int32_t k = c * per; k < k1; k++) {
            const tal_seq_pair &p = pairs[k];
            if (p.len1 < 0 || p.len2 < 0 || p.idr < 0 || p.idq < 0) {
                x.bad = k;
                return;
            }
            x.rlo = std::min<long long>(x.rlo, p.idr);
            x.qlo = std::min<long long>(x.qlo, p.idq);
            x.rhi = std::max<long long>(x.rhi, (long long)p.idr + p.len1);
            x.qhi = std::max<long long>(x.qhi, (long long)p.idq + p.len2);
            x.max1 = std::max(x.max1, p.len1);
            x.max2 = std::max(x.max2, p.len2);
        }
    };
    if (nch > 1) {
        std::vector<std::thread> th;
        for (int c = 0; c < nch; c++) th.emplace_back(scan, c);
        for (auto &t : th) t.join();
    } else {
        scan(0);
    }
    Ext all;
    for (int c = 0; c < nch; c++) {
        if (ext[c].bad >= 0) {
            h->last_bad = ext[c].bad;
            return fail(h, TAL_EDOMAIN, "negative length or offset at pair " + std::to_string(ext[c].bad));
        }
        if ((int64_t)c * per >= numPairs) continue;
        all.rlo = std::min(all.rlo, ext[c].rlo);
        all.qlo = std::min(all.qlo, ext[c].qlo);
        all.rhi = std::max(all.rhi, ext[c].rhi);
        all.qhi = std::max(all.qhi, ext[c].qhi);
        all.max1 = std::max(all.max1, ext[c].max1);
        all.max2 = std::max(all.max2, ext[c].max2);
    }
    auto align = [](Ext &x) {
        x.rlo &= ~15LL;
        x.qlo &= ~15LL;
        if (x.rhi <= x.rlo) x.rhi = x.rlo + 16;
        if (x.qhi <= x.qlo) x.qhi = x.qlo + 16;
    };
    // grouped 8-bit: the padding lanes of a last partial group read the
    // query bytes at offset 0 (the reference pads with zeroed SeqPairs)
    if (grouped && bits == 8 && numPairs % 64) {
        const long long need = pairs[numPairs - 1].len2;
        all.qlo = 0;
        all.qhi = std::max(all.qhi, need);
        for (int c = 0; c < nch; c++) {
            const int32_t k1 = std::min<int32_t>(numPairs, (c + 1) * per);
            if (k1 == numPairs && (int64_t)c * per < numPairs) {
                ext[c].qlo = 0;
                ext[c].qhi = std::max(ext[c].qhi, need);
            }
        }
    }
    // exact scoring: a last partial 8-bit group re-scored in the reference's
    // grouping has padding lanes that read the query bytes at the caller's
    // offset 0 (the reference pads with zeroed SeqPairs); copy them too
    // when the windows start within 1 MiB of it
    if (exact && bits != 16 && all.qlo <= (1 << 20)) {
        all.qlo = 0;
        for (int c = 0; c < nch; c++)
            if (ext[c].qlo <= (1 << 20)) ext[c].qlo = 0;
    }
    align(all);
    for (int c = 0; c < nch; c++) align(ext[c]);
    // chunk windows that overlap much (pairs sharing sequences) copy once, whole
    long long sum = 0;
    for (int c = 0; c < nch; c++) sum += (ext[c].rhi - ext[c].rlo) + (ext[c].qhi - ext[c].qlo);
    if (nch > 1 && sum * 4 > ((all.rhi - all.rlo) + (all.qhi - all.qlo)) * 5) nch = 1;
    if (nch == 1) {
        ext[0] = all;
        per = numPairs;
    }
    // device layout: the call's whole window, each chunk's window copied to its
    // place in it (so any pair -- and the SIMD groups re-scored across chunk
    // boundaries -- resolves through one window); sparse windows copy as one chunk
    if (nch > 1 && ((all.rhi - all.rlo) + (all.qhi - all.qlo)) > 2 * sum) {
        nch = 1;
        ext[0] = all;
        per = numPairs;
    }
    long long roff[kChunks], qoff[kChunks];
    const long long rtot = all.rhi - all.rlo, qtot = all.qhi - all.qlo;
    for (int c = 0; c < nch; c++) {
        roff[c] = ext[c].rlo - all.rlo;
        qoff[c] = ext[c].qlo - all.qlo;
    }
    const size_t pbytes = (size_t)numPairs * sizeof(tal_seq_pair);
    if ((e = h->pairs.ensure(pbytes)) != cudaSuccess ||
        (e = h->ref.ensure((size_t)rtot + 16)) != cudaSuccess ||
        (e = h->qer.ensure((size_t)qtot + 16)) != cudaSuccess)
        return fail(h, TAL_ENOMEM, std::string("device buffers: ") + cudaGetErrorString(e));
    if (exact) {
        int rc = ensure_regroup(h, numPairs, all.max2);
        if (rc != TAL_OK) return rc;
    }
    if (nch > 1 && !h->cstream) {
        e = cudaStreamCreateWithFlags(&h->cstream, cudaStreamNonBlocking);
        for (int c = 0; c < kChunks && e == cudaSuccess; c++)
            e = cudaEventCreateWithFlags(&h->cev[c], cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(h, e, "copy stream");
    }
    // the copy stream starts after the previous call's work on the scoring stream
    if (nch > 1) {
        if ((e = cudaEventRecord(h->cev[0], h->stream)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(h->cstream, h->cev[0], 0)) != cudaSuccess)
            return cuda_fail(h, e, "stream order");
    }
    for (int c = 0; c < nch; c++) {
        const int32_t k0 = c * per, k1 = std::min<int32_t>(numPairs, (c + 1) * per);
        if (k1 <= k0) {
            nch = c;
            break;
        }
        cudaStream_t cs = nch > 1 ? h->cstream : h->stream;
        uint8_t *dp = reinterpret_cast<uint8_t *>(h->pairs.p) + (size_t)k0 * sizeof(tal_seq_pair);
        uint8_t *dr = reinterpret_cast<uint8_t *>(h->ref.p) + roff[c];
        uint8_t *dq = reinterpret_cast<uint8_t *>(h->qer.p) + qoff[c];
        e = cudaMemcpyAsync(dp, pairs + k0, (size_t)(k1 - k0) * sizeof(tal_seq_pair),
                            cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dr, seqBufRef + ext[c].rlo, (size_t)(ext[c].rhi - ext[c].rlo),
                                cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dq, seqBufQer + ext[c].qlo, (size_t)(ext[c].qhi - ext[c].qlo),
                                cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess && nch > 1) {
            e = cudaEventRecord(h->cev[c], cs);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, h->cev[c], 0);
        }
        if (e != cudaSuccess) {
            cudaStreamSynchronize(h->stream);
            if (h->cstream) cudaStreamSynchronize(h->cstream);
            return cuda_fail(h, e, "cudaMemcpyAsync(H2D)");
        }
        talbsw::LaunchArgs A;
        memset(&A, 0, sizeof(A));
        A.pairs = reinterpret_cast<talbsw::DevPair *>(dp);
        A.ref = reinterpret_cast<uint8_t *>(h->ref.p);
        A.qer = reinterpret_cast<uint8_t *>(h->qer.p);
        A.ref_lo = all.rlo; A.ref_hi = all.rhi; A.qer_lo = all.qlo; A.qer_hi = all.qhi;
        if (exact) {
            talbsw::attach_regroup(A, h->regroup.V);
            A.flag_base = k0;
        }
        A.order = nullptr;
        A.wpair = nullptr;
        A.n = k1 - k0;
        A.w = w;
        A.bits = bits;
        // one row capacity for all chunks: the kernel configuration stays the same
        A.cols_cap = std::max(all.max2, 1);
        A.rows_cap = std::max(all.max1, 1);
        int rc = grouped ? launch_grouped(h, A, c) : launch_scoring(h, A, w, c);
        if (rc != TAL_OK) {
            cudaStreamSynchronize(h->stream);
            if (h->cstream) cudaStreamSynchronize(h->cstream);
            return rc;
        }
    }
    // the SIMD groups of flagged pairs, over the whole call (errors into
    // chunk 0's control block, whose pair indices are the call's)
    if (exact) {
        talbsw::LaunchArgs A;
        memset(&A, 0, sizeof(A));
        A.pairs = reinterpret_cast<talbsw::DevPair *>(h->pairs.p);
        A.ref = reinterpret_cast<uint8_t *>(h->ref.p);
        A.qer = reinterpret_cast<uint8_t *>(h->qer.p);
        A.ref_lo = all.rlo; A.ref_hi = all.rhi; A.qer_lo = all.qlo; A.qer_hi = all.qhi;
        A.n = numPairs;
        A.w = w;
        A.bits = bits;
        int rc = launch_regroup(h, A);
        if (rc != TAL_OK) {
            cudaStreamSynchronize(h->stream);
            if (h->cstream) cudaStreamSynchronize(h->cstream);
            return rc;
        }
    }
    // a bad pair index is local to its chunk: chunks are launched in order, so
    // map it back through the chunk bounds after the merge
    int rc = collect_chunks(h, nch, per);
    if (rc != TAL_OK) return rc;
    e = cudaMemcpyAsync(pairs, h->pairs.p, pbytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemcpyAsync(D2H)");
    return TAL_OK;
}

}  // extern "C"

namespace {

// max len1 / len2 over a device SeqPair array (or a per-pair band), for
// sizing the shared-memory rows of a device-resident call
__global__ void caps_kernel(const talbsw::DevPair *p, int n, int *out) {
    int m1 = 0, m2 = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        m1 = max(m1, p[k].len1);
        m2 = max(m2, p[k].len2);
    }
    m1 = __reduce_max_sync(0xffffffffu, (unsigned)max(m1, 0));
    m2 = __reduce_max_sync(0xffffffffu, (unsigned)max(m2, 0));
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out + 0, m1);
        atomicMax(out + 1, m2);
    }
}

// Integer-pipe throughput probes: 8 independent dependency chains per thread.
__global__ void probe_dpx_kernel(int iters, unsigned *out) {
    unsigned a[8];
    const unsigned b = 0xffff0001u;
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = threadIdx.x * 0x00010003u + k;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = __viaddmax_s16x2(a[k], b, 0x00020002u + k);
    }
    unsigned r = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) r ^= a[k];
    if (r == 0x12345678u) out[0] = r;
}

__global__ void probe_i32_kernel(int iters, int *out) {
    int a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = (int)threadIdx.x * 3 + k;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = max(a[k] + 1, k - (int)i);
    }
    int r = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) r ^= a[k];
    if (r == 0x12345678) out[0] = r;
}

}  // namespace

extern "C" {

int tal_bsw_probe_int_peak(int device, double *dpx_per_s, double *i32_per_s) {
    if (!dpx_per_s || !i32_per_s) return TAL_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return TAL_ENODEV;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return TAL_ENODEV;
    unsigned *d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) return TAL_ENOMEM;
    const int threads = 256, blocks = prop.multiProcessorCount * 8, iters = 8192;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_dpx = 1e30f, best_i32 = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        float ms;
        cudaEventRecord(e0);
        probe_dpx_kernel<<<blocks, threads>>>(iters, d);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep) best_dpx = std::min(best_dpx, ms);
        cudaEventRecord(e0);
        probe_i32_kernel<<<blocks, threads>>>(iters, reinterpret_cast<int *>(d));
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep) best_i32 = std::min(best_i32, ms);
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) return TAL_ECUDA;
    const double ops = (double)blocks * threads * iters * 8.0;
    *dpx_per_s = ops / (best_dpx * 1e-3);
    // the i32 chain step is an add and a max: two instructions
    *i32_per_s = 2.0 * ops / (best_i32 * 1e-3);
    return TAL_OK;
}

int tal_bsw_last_regroup(tal_bsw_handle h, int64_t *flagged_pairs, int64_t *groups) {
    if (!h || !flagged_pairs || !groups) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    *flagged_pairs = 0;
    *groups = 0;
    if (!h->regroup.V.ctr) return TAL_OK;
    int c[8];
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c, h->regroup.V.ctr, sizeof(c), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "regroup counters");
    *flagged_pairs = c[6];
    *groups = c[7];
    return TAL_OK;
}

int tal_bsw_scores_device(tal_bsw_handle h, tal_seq_pair *d_pairs, const uint8_t *d_ref,
                          size_t ref_bytes, const uint8_t *d_qer, size_t qer_bytes,
                          int32_t numPairs, int32_t w, const int32_t *d_w, int bits) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->last_error.clear();
    h->last_bad = -1;
    const bool grouped = (bits & TAL_BSW_GROUPED) != 0;
    const bool perpair = (bits & TAL_BSW_PER_PAIR) != 0;
    bits &= ~(TAL_BSW_GROUPED | TAL_BSW_PER_PAIR);
    if (numPairs < 0 || (bits != 0 && bits != 8 && bits != 16) || (grouped && (bits == 0 || d_w)) ||
        (grouped && perpair))
        return fail(h, TAL_EINVAL, "bad numPairs or bits");
    const bool exact = !grouped && !perpair;
    if (numPairs == 0) return TAL_OK;
    if (!d_pairs || !d_ref || !d_qer) return fail(h, TAL_EINVAL, "NULL buffer");
    if (((uintptr_t)d_ref & 15) || ((uintptr_t)d_qer & 15))
        return fail(h, TAL_EINVAL, "device sequence buffers must be 16-byte aligned");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    if ((e = h->caps.ensure(2 * sizeof(int))) != cudaSuccess)
        return fail(h, TAL_ENOMEM, "caps buffer");
    int *caps = reinterpret_cast<int *>(h->caps.p);
    e = cudaMemsetAsync(caps, 0, 2 * sizeof(int), h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemsetAsync");
    int blocks = std::min<long long>(((long long)numPairs + 255) / 256, (long long)h->num_sms * 8);
    caps_kernel<<<blocks, 256, 0, h->stream>>>(reinterpret_cast<talbsw::DevPair *>(d_pairs),
                                                numPairs, caps);
    h->launches++;
    int hc[2] = {0, 0};
    e = cudaMemcpyAsync(hc, caps, sizeof(hc), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "caps");
    talbsw::LaunchArgs A;
    memset(&A, 0, sizeof(A));
    A.pairs = reinterpret_cast<talbsw::DevPair *>(d_pairs);
    A.ref = d_ref;
    A.qer = d_qer;
    A.ref_lo = 0; A.ref_hi = (long long)ref_bytes;
    A.qer_lo = 0; A.qer_hi = (long long)qer_bytes;
    A.wpair = d_w;
    A.n = numPairs;
    A.w = w;
    A.bits = bits;
    A.cols_cap = std::max(hc[1], 1);
    A.rows_cap = std::max(hc[0], 1);
    if (exact) {
        int rc = ensure_regroup(h, numPairs, hc[1]);
        if (rc != TAL_OK) return rc;
        talbsw::attach_regroup(A, h->regroup.V);
    }
    int rc = grouped ? launch_grouped(h, A) : launch_scoring(h, A, w);
    if (rc == TAL_OK && exact) rc = launch_regroup(h, A);
    if (rc != TAL_OK) return rc;
    h->pending_status = TAL_OK;
    return TAL_OK;
}

int tal_bsw_sync(tal_bsw_handle h) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return collect(h);
}

void *tal_bsw_stream(tal_bsw_handle h) { return h ? (void *)h->stream : nullptr; }

const char *tal_bsw_last_error(tal_bsw_handle h) { return h ? h->last_error.c_str() : "null handle"; }

int64_t tal_bsw_last_bad_pair(tal_bsw_handle h) { return h ? h->last_bad : -1; }

uint64_t tal_bsw_launch_count(tal_bsw_handle h) { return h ? h->launches : 0; }

float tal_bsw_last_kernel_ms(tal_bsw_handle h) { return h ? h->last_kernel_ms : 0.f; }

uint64_t tal_bsw_last_cells(tal_bsw_handle h) { return h ? h->last_cells : 0; }

}  // extern "C"
