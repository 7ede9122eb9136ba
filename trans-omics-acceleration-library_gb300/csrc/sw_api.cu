// C ABI of the unbanded Smith-Waterman scorer (include/tal_sw.h): handle,
// host<->device staging, launch of sw_wave_kernel.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <string>

#include "../../include/tal_sw.h"
#include "bsw_ctx.h"
#include "sw_kernel.cuh"

static_assert(sizeof(tal_sw_pair) == 12, "SeqPair of the unbanded kernels is 12 bytes");
static_assert(sizeof(talsw::SwPair) == 12, "device view");

namespace {

struct SwCtrl {
    int counter;
    int flags;
    long long bad;
    unsigned long long cells;
    int hist[talsw::kSwBuckets];  // work-order buckets
};

int max_seq_len(int bits) { return bits == 8 ? 128 : 1024; }  // PairWiseSW_{8,16,32}.h

constexpr int kSortMin = 256;  // batches from this size are scored in length order

}  // namespace

struct tal_sw_ctx {
    tal_sw_params prm;
    int device = 0, num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    talbsw::DevBuf pairs, seq, ctrl, order;
    std::mutex mu;
    std::string last_error;
    int64_t last_bad = -1;
    uint64_t last_cells = 0;
};

namespace {

int sfail(tal_sw_ctx *h, int code, const std::string &msg) {
    h->last_error = msg;
    return code;
}

// Launches the kernel over device-resident pairs and sequences and collects
// the status.
int run_locked(tal_sw_ctx *h, tal_sw_pair *d_pairs, const uint8_t *d_seq, long long lo, long long hi,
               int32_t n, int bits, int cols_cap) {
    const int lim = bits == 8 ? 127 : bits == 16 ? 32767 : INT_MAX;
    const tal_sw_params &p = h->prm;
    const int lo_el = bits == 8 ? -128 : bits == 16 ? -32768 : INT_MIN / 2;
    if (p.w_match > lim || p.w_mismatch < lo_el || (long long)p.w_open + p.w_extend < lo_el)
        return sfail(h, TAL_EDOMAIN, "weights outside the precision's element type");
    cudaError_t e;
    if ((e = h->ctrl.ensure(sizeof(SwCtrl))) != cudaSuccess)
        return sfail(h, TAL_ENOMEM, "control block");
    SwCtrl init;
    memset(&init, 0, sizeof(init));
    init.bad = LLONG_MAX;
    e = cudaMemcpyAsync(h->ctrl.p, &init, sizeof(init), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return sfail(h, TAL_ECUDA, cudaGetErrorString(e));
    SwCtrl *c = reinterpret_cast<SwCtrl *>(h->ctrl.p);
    talsw::SwArgs A;
    memset(&A, 0, sizeof(A));
    A.pairs = reinterpret_cast<talsw::SwPair *>(d_pairs);
    A.seq = d_seq;
    A.seq_lo = lo;
    A.seq_hi = hi;
    A.stride = max_seq_len(bits);
    A.n = n;
    A.cols_cap = std::max(cols_cap, 1);
    A.maxlen = max_seq_len(bits) - 4;
    A.score_lim = lim;
    A.match = p.w_match; A.mismatch = p.w_mismatch; A.open = p.w_open; A.ext = p.w_extend;
    // work order by length, longest first (small batches keep theirs)
    if (n >= kSortMin) {
        if ((e = h->order.ensure(sizeof(int32_t) * (size_t)n)) != cudaSuccess)
            return sfail(h, TAL_ENOMEM, "work order");
        int32_t *order = reinterpret_cast<int32_t *>(h->order.p);
        const int gb = (int)std::min<long long>(((long long)n + 255) / 256, 4LL * h->num_sms);
        talsw::sw_bucket_count<<<gb, 256, 0, h->stream>>>(A.pairs, n, c->hist);
        talsw::sw_bucket_offsets<<<1, 32, 0, h->stream>>>(c->hist);
        talsw::sw_bucket_scatter<<<gb, 256, 0, h->stream>>>(A.pairs, n, c->hist, order);
        if ((e = cudaGetLastError()) != cudaSuccess) return sfail(h, TAL_ECUDA, cudaGetErrorString(e));
        A.order = order;
    }
    A.work_counter = &c->counter;
    A.cells = &c->cells;
    A.err_flags = &c->flags;
    A.err_index = &c->bad;
    // 8- and 16-bit values fit int16: two pairs per warp in 16x2 lanes (the
    // mismatch step, match - mismatch, must fit too)
    const bool packed = bits != 32 && (long long)p.w_match - p.w_mismatch <= 32768;
    const size_t wbytes = packed ? talsw::sw2_warp_smem_bytes(A.cols_cap)
                                 : talsw::sw_warp_smem_bytes(A.cols_cap);
    const int wpb = 4;
    const size_t smem = wbytes * wpb;
    if (smem > h->smem_optin) return sfail(h, TAL_EDOMAIN, "sequences too long for shared memory");
    int bps = 0;
    auto kern = packed ? talsw::sw_wave2_kernel<talsw::kSwRows> : talsw::sw_wave_kernel<talsw::kSwRows>;
    e = talbsw::resident_blocks((const void *)kern, 32 * wpb, smem, h->smem_optin, &bps);
    if (e != cudaSuccess || bps < 1) return sfail(h, TAL_ECUDA, "occupancy query");
    long long blocks = (long long)bps * h->num_sms;
    const long long pairs_per_block = (long long)wpb * (packed ? 2 : 1);
    blocks = std::min<long long>(blocks, ((long long)n + pairs_per_block - 1) / pairs_per_block);
    kern<<<(unsigned)std::max<long long>(blocks, 1), 32 * wpb, smem, h->stream>>>(A);
    if ((e = cudaGetLastError()) != cudaSuccess) return sfail(h, TAL_ECUDA, cudaGetErrorString(e));
    SwCtrl out;
    e = cudaMemcpyAsync(&out, c, sizeof(out), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return sfail(h, TAL_ECUDA, cudaGetErrorString(e));
    h->last_cells = out.cells;
    if (out.flags) {
        h->last_bad = out.bad;
        return sfail(h, TAL_EDOMAIN, "pair outside the exact range, first bad pair " + std::to_string(out.bad));
    }
    return TAL_OK;
}

}  // namespace

extern "C" {

int tal_sw_create(const tal_sw_params *params, int device, tal_sw_handle *out) {
    if (!params || !out) return TAL_EINVAL;
    *out = nullptr;
    const tal_sw_params &p = *params;
    if (p.w_mismatch > 0 || p.w_open > 0 || p.w_extend > 0 || p.w_match < 0) return TAL_EINVAL;
    int dev = device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return TAL_ENODEV;
    if (cudaSetDevice(dev) != cudaSuccess) return TAL_ENODEV;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major != 10) return TAL_ENODEV;
    tal_sw_ctx *h = new (std::nothrow) tal_sw_ctx();
    if (!h) return TAL_ENOMEM;
    h->prm = p;
    h->device = dev;
    h->num_sms = prop.multiProcessorCount;
    h->smem_optin = prop.sharedMemPerBlockOptin;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return TAL_ECUDA;
    }
    *out = h;
    return TAL_OK;
}

int tal_sw_destroy(tal_sw_handle h) {
    if (!h) return TAL_EINVAL;
    {
        std::lock_guard<std::mutex> lk(h->mu);
        cudaSetDevice(h->device);
        cudaStreamSynchronize(h->stream);
        h->pairs.release();
        h->seq.release();
        h->ctrl.release();
        h->order.release();
        cudaStreamDestroy(h->stream);
    }
    delete h;
    return TAL_OK;
}

int tal_sw_scores(tal_sw_handle h, tal_sw_pair *pairs, const uint8_t *seqBuf, int32_t numPairs,
                  int bits) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->last_error.clear();
    h->last_bad = -1;
    h->last_cells = 0;
    if (numPairs < 0 || (bits != 8 && bits != 16 && bits != 32)) return sfail(h, TAL_EINVAL, "bad numPairs or bits");
    if (numPairs == 0) return TAL_OK;
    if (!pairs || !seqBuf) return sfail(h, TAL_EINVAL, "NULL buffer");
    if (cudaSetDevice(h->device) != cudaSuccess) return sfail(h, TAL_ECUDA, "cudaSetDevice");
    const long long L = max_seq_len(bits);
    long long lo = LLONG_MAX, hi = 0;
    int cols = 1;
    for (int32_t k = 0; k < numPairs; k++) {
        const tal_sw_pair &p = pairs[k];
        if (p.id < 0 || p.len1 < 0 || p.len2 < 0 || p.len1 > L - 4 || p.len2 > L - 4) {
            h->last_bad = k;
            return sfail(h, TAL_EDOMAIN, "bad id or length at pair " + std::to_string(k));
        }
        lo = std::min(lo, 2LL * p.id * L);
        hi = std::max(hi, (2LL * p.id + 1) * L + p.len2);
        cols = std::max<int>(cols, p.len2);
    }
    lo &= ~15LL;
    const size_t pbytes = sizeof(tal_sw_pair) * (size_t)numPairs;
    cudaError_t e;
    if ((e = h->pairs.ensure(pbytes)) != cudaSuccess || (e = h->seq.ensure((size_t)(hi - lo) + 16)) != cudaSuccess)
        return sfail(h, TAL_ENOMEM, cudaGetErrorString(e));
    e = cudaMemcpyAsync(h->pairs.p, pairs, pbytes, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->seq.p, seqBuf + lo, (size_t)(hi - lo), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return sfail(h, TAL_ECUDA, cudaGetErrorString(e));
    int rc = run_locked(h, reinterpret_cast<tal_sw_pair *>(h->pairs.p),
                        reinterpret_cast<const uint8_t *>(h->seq.p), lo, hi, numPairs, bits, cols);
    if (rc != TAL_OK) return rc;
    e = cudaMemcpyAsync(pairs, h->pairs.p, pbytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return sfail(h, TAL_ECUDA, cudaGetErrorString(e));
    return TAL_OK;
}

int tal_sw_scores_device(tal_sw_handle h, tal_sw_pair *d_pairs, const uint8_t *d_seqbuf,
                         size_t seq_bytes, int32_t numPairs, int bits) {
    if (!h) return TAL_EINVAL;
    std::lock_guard<std::mutex> lk(h->mu);
    h->last_error.clear();
    h->last_bad = -1;
    h->last_cells = 0;
    if (numPairs < 0 || (bits != 8 && bits != 16 && bits != 32)) return sfail(h, TAL_EINVAL, "bad numPairs or bits");
    if (numPairs == 0) return TAL_OK;
    if (!d_pairs || !d_seqbuf) return sfail(h, TAL_EINVAL, "NULL buffer");
    if (cudaSetDevice(h->device) != cudaSuccess) return sfail(h, TAL_ECUDA, "cudaSetDevice");
    // row capacity: the precision's longest sequence (the pairs stay on the device)
    return run_locked(h, d_pairs, d_seqbuf, 0, (long long)seq_bytes, numPairs, bits,
                      max_seq_len(bits) - 4);
}

void *tal_sw_stream(tal_sw_handle h) { return h ? (void *)h->stream : nullptr; }
const char *tal_sw_last_error(tal_sw_handle h) { return h ? h->last_error.c_str() : "null handle"; }
int64_t tal_sw_last_bad_pair(tal_sw_handle h) { return h ? h->last_bad : -1; }
uint64_t tal_sw_last_cells(tal_sw_handle h) { return h ? h->last_cells : 0; }

}  // extern "C"
