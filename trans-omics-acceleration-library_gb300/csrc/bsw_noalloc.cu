// Allocation-free scoring entry point (tal_bsw_scores_device_noalloc).
//
// Who needs it: callers that must not allocate device memory during the
// call -- for example a process whose device memory is fully owned by its own
// caching pool (a cudaMalloc behind the pool's back can fail or fragment it),
// or a real-time pipeline that forbids allocation on its hot path because
// cudaMalloc/cudaFree can synchronise the whole device.  They already hold
// the pairs and the sequences in device memory; this entry point scores them
// without a handle and without allocating anything.
//
// The only memory the scoring kernel needs beyond its inputs and outputs is a
// small control block (work counter, error flags, first offending pair, cell
// count) and two words for the row-capacity reduction.  Here that scratch is
// the file-scope device array below, of a fixed size.  Host code cannot use
// the array's name as a device address (it names a host-side shadow), so the
// device address is fetched once per device with cudaGetSymbolAddress.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <mutex>

#include "../../include/tal_bsw.h"
#include "bsw_launch.cuh"

namespace {

// Control block layout inside the scratch array.
struct NoAllocCtrl {
    int counter;
    int flags;
    long long bad_index;
    unsigned long long cells;
    int caps[2];  // max len1, max len2
};

static_assert(sizeof(NoAllocCtrl) <= TAL_BSW_NOALLOC_SCRATCH_BYTES,
              "control block must fit the static scratch array");

// The scratch: one per device that loads this library, alive until exit.
// Every call uses the same bytes, so calls that overlap on the GPU race.
static __device__ __align__(256) unsigned char g_noalloc_scratch[TAL_BSW_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_dev[kMaxDevices];
int g_num_sms[kMaxDevices];
size_t g_smem_optin[kMaxDevices];
bool g_ready[kMaxDevices];
long long g_last_bad1[kMaxDevices];  // the last call's first offending pair + 1 (0: none)

// Zeroes the control block (the first offending index starts at INT64_MAX).
__global__ void noalloc_reset_kernel(NoAllocCtrl *c) {
    c->counter = 0;
    c->flags = 0;
    c->bad_index = LLONG_MAX;
    c->cells = 0ull;
    c->caps[0] = 0;
    c->caps[1] = 0;
}

__global__ void noalloc_caps_kernel(const talbsw::DevPair *p, int n, NoAllocCtrl *c) {
    int m1 = 0, m2 = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        m1 = max(m1, p[k].len1);
        m2 = max(m2, p[k].len2);
    }
    m1 = (int)__reduce_max_sync(0xffffffffu, (unsigned)max(m1, 0));
    m2 = (int)__reduce_max_sync(0xffffffffu, (unsigned)max(m2, 0));
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&c->caps[0], m1);
        atomicMax(&c->caps[1], m2);
    }
}

// Per-device set-up, done by the first call on each device with that device
// current: resolve the scratch array's device address and cache the device's
// SM count and shared-memory limit.
int setup_device(int dev) {
    if (dev < 0 || dev >= kMaxDevices) return TAL_ENODEV;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (g_ready[dev]) return TAL_OK;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major != 10) return TAL_ENODEV;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr)
        return TAL_ECUDA;
    g_scratch_dev[dev] = p;
    g_num_sms[dev] = prop.multiProcessorCount;
    g_smem_optin[dev] = prop.sharedMemPerBlockOptin;
    g_ready[dev] = true;
    return TAL_OK;
}

}  // namespace

extern "C" int tal_bsw_scores_device_noalloc(const tal_bsw_params *params, tal_seq_pair *d_pairs,
                                             const uint8_t *d_ref, size_t ref_bytes,
                                             const uint8_t *d_qer, size_t qer_bytes,
                                             int32_t numPairs, int32_t w, const int32_t *d_w,
                                             int bits, void *stream) {
    if (!params) return TAL_EINVAL;
    const tal_bsw_params &p = *params;
    auto in = [](int v, int lo, int hi) { return v >= lo && v <= hi; };
    if (!in(p.o_del, 0, 127) || !in(p.o_ins, 0, 127) || !in(p.e_del, 1, 127) ||
        !in(p.e_ins, 1, 127) || !in(p.w_match, 0, 127) || !in(p.w_mismatch, 0, 127))
        return TAL_EINVAL;
    if (numPairs < 0 || (bits != 0 && bits != 8 && bits != 16)) return TAL_EINVAL;
    {
        int d = 0;
        if (cudaGetDevice(&d) == cudaSuccess && d >= 0 && d < kMaxDevices) g_last_bad1[d] = 0;
    }
    if (numPairs == 0) return TAL_OK;
    if (!d_pairs || !d_ref || !d_qer) return TAL_EINVAL;
    if (((uintptr_t)d_ref & 15) || ((uintptr_t)d_qer & 15)) return TAL_EINVAL;
    // The scratch this call needs must fit the static array: one control block.
    if (sizeof(NoAllocCtrl) > (size_t)TAL_BSW_NOALLOC_SCRATCH_BYTES) return TAL_EDOMAIN;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TAL_ENODEV;
    int rc = setup_device(dev);
    if (rc != TAL_OK) return rc;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    NoAllocCtrl *c = reinterpret_cast<NoAllocCtrl *>(g_scratch_dev[dev]);

    noalloc_reset_kernel<<<1, 1, 0, s>>>(c);
    int blocks = (int)std::min<long long>(((long long)numPairs + 255) / 256, (long long)g_num_sms[dev] * 8);
    noalloc_caps_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<talbsw::DevPair *>(d_pairs), numPairs, c);
    int caps[2] = {0, 0};
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(caps, c->caps, sizeof(caps), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return TAL_ECUDA;

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
    A.cols_cap = std::max(caps[1], 1);
    A.rows_cap = std::max(caps[0], 1);
    A.work_counter = &c->counter;
    A.err_flags = &c->flags;
    A.err_index = &c->bad_index;
    A.cells = &c->cells;
    A.P = {p.o_del, p.e_del, p.o_ins, p.e_ins, p.zdrop, p.end_bonus, p.w_match, p.w_mismatch};
    A.win = d_w ? 0 : talbsw::lane_window(w, A.cols_cap);
    const talbsw::KConfig cfg = talbsw::fit_config(talbsw::choose_config(w, A.cols_cap, A.win),
                                                   A.cols_cap, g_smem_optin[dev], A.win);
    if (talbsw::config_smem(cfg, A.cols_cap, A.rows_cap, A.win) > g_smem_optin[dev])
        return TAL_ENOMEM;  // a pair too long for the shared-memory rows
    e = talbsw::launch_config(A, cfg, g_num_sms[dev], g_smem_optin[dev], s);
    if (e != cudaSuccess) return TAL_ECUDA;
    NoAllocCtrl st;
    e = cudaMemcpyAsync(&st, c, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return TAL_ECUDA;
    const int flags = st.flags;
    if (flags && st.bad_index != LLONG_MAX) g_last_bad1[dev] = st.bad_index + 1;
    // a pair whose rows do not fit shared memory: a capacity refusal; a pair
    // outside the exact range or with a base code above 4: a domain error
    if (flags & (talbsw::ERR_DOMAIN | talbsw::ERR_BASE)) return TAL_EDOMAIN;
    if (flags) return TAL_ENOMEM;
    return TAL_OK;
}

extern "C" int64_t tal_bsw_noalloc_last_bad_pair(void) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -1;
    return g_last_bad1[dev] - 1;
}
