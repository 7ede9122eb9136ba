// Exact scoring of the pairs the per-pair kernels flag (bsw_couple.cuh): the
// reference scores a caller's array in SIMD groups of 32 (16-bit) / 64
// (8-bit) consecutive pairs (bandedSWA.cpp:2722-2955 / :2030-2258); a flagged
// pair's outputs may depend on the other pairs of its group, so its group is
// scored again by the block-wide grouped kernel (bsw_group_wide.cuh), which
// stops once the group's flagged lanes have exited and writes their outputs
// (the other members keep their per-pair outputs, equal to the grouped ones).
//
// A group is defined by the caller's array: the reference takes one band and
// one precision per call, so a batch with per-pair bands and 8/16-bit routing
// is scored as the caller would issue it -- one call per (band, precision)
// with that class's pairs in array order -- and, for a serving tick, per
// request.  The pass finds, for each flagged pair, its rank within its class
// (per-chunk class counts and a scan), marks its group, gathers the group's
// members in order and re-scores the marked groups.  Everything runs on the
// device on the scoring stream, so it can be captured into the batched
// form's graph; each stage returns at once when no pair was flagged.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "bsw_ctx.h"
#include "bsw_group_wide.cuh"

namespace talbsw {

namespace {

constexpr unsigned long long kEmpty = ~0ull;

__device__ __forceinline__ unsigned long long mix64(unsigned long long k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
    return k;
}

// The class of pair `pidx` of request `req` (-1: the launch's pairs): the
// precision the reference call would use and the band.
struct PairClass {
    unsigned long long key;
    int w, bits;
};
__device__ __forceinline__ PairClass class_of(const LaunchArgs &A, int req, int pidx) {
    const PairSrc src = pair_src(A, pidx, req);
    int bits = src.bits;
    if (bits != 8 && bits != 16) {
        const DevPair &p = *src.pp;
        bits = pair_in_range(A.P, p.len1, p.len2, p.h0, src.w, true) ? 8 : 16;
    }
    PairClass c;
    c.w = src.w;
    c.bits = bits;
    c.key = ((unsigned long long)(req + 1) << 40) | ((unsigned long long)(unsigned)(src.w & 0x7fffffff) << 1) |
            (bits == 16 ? 1ull : 0ull);
    return c;
}

// Global index (the tick's pair space, or the launch's pairs) -> request.
__device__ __forceinline__ int req_at(const LaunchArgs &A, int nreq, long long gi) {
    return A.reqs ? group_req_of(A.reqs, nreq, gi) : -1;
}
__device__ __forceinline__ int local_of(const LaunchArgs &A, int req, long long gi) {
    return (int)(req >= 0 ? gi - A.reqs[req].first : gi);
}

__device__ __forceinline__ int class_slot(const RegroupView &V, unsigned long long key) {
    unsigned s = (unsigned)mix64(key) & (kRegroupClasses - 1);
    for (int probe = 0; probe < kRegroupClasses; probe++) {
        const unsigned long long k = V.ckeys[s];
        if (k == key) return (int)s;
        if (k == kEmpty) return -1;
        s = (s + 1) & (kRegroupClasses - 1);
    }
    return -1;
}

// 1. the classes of the flagged pairs
__global__ void rg_classes(LaunchArgs A, int nreq, RegroupView V) {
    const int nf = min(V.ctr[0], V.fcap);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nf; e += gridDim.x * blockDim.x) {
        const long long f = V.flagged[e];
        const int req = (int)(f >> 32) - 1, pidx = (int)(f & 0xffffffffll);
        const PairClass c = class_of(A, req, pidx);
        unsigned s = (unsigned)mix64(c.key) & (kRegroupClasses - 1);
        int slot = -1;
        for (int probe = 0; probe < kRegroupClasses; probe++) {
            const unsigned long long old = atomicCAS(&V.ckeys[s], kEmpty, c.key);
            if (old == kEmpty) { V.cinfo[s] = make_int4(c.w, req, c.bits, 0); slot = (int)s; break; }
            if (old == c.key) { slot = (int)s; break; }
            s = (s + 1) & (kRegroupClasses - 1);
        }
        if (slot < 0) atomicOr(&V.ctr[5], 1);  // more classes than the table holds
        V.cls_of[e] = slot;
        V.gidx[e] = (req >= 0 ? A.reqs[req].first : 0) + pidx;
    }
}

// 2. members of each flagged class per chunk of kRegroupChunk pairs
__global__ void __launch_bounds__(256) rg_count(LaunchArgs A, int nreq, long long ntotal, RegroupView V) {
    if (V.ctr[0] == 0) return;
    __shared__ int cnt[kRegroupClasses];
    for (int c = threadIdx.x; c < kRegroupClasses; c += blockDim.x) cnt[c] = 0;
    __syncthreads();
    const long long c0 = (long long)blockIdx.x * kRegroupChunk;
    const long long c1 = min(c0 + kRegroupChunk, ntotal);
    for (long long gi = c0 + threadIdx.x; gi < c1; gi += blockDim.x) {
        const int req = req_at(A, nreq, gi);
        const int s = class_slot(V, class_of(A, req, local_of(A, req, gi)).key);
        if (s >= 0) atomicAdd(&cnt[s], 1);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < kRegroupClasses; c += blockDim.x)
        V.counts[(size_t)c * V.nchunks + blockIdx.x] = cnt[c];
}

// 3. exclusive scan of each class's chunk counts
__global__ void __launch_bounds__(256) rg_scan(RegroupView V, int nck) {
    if (V.ctr[0] == 0 || V.ckeys[blockIdx.x] == kEmpty) return;
    __shared__ int part[256];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int *cn = V.counts + (size_t)blockIdx.x * V.nchunks;
    int *off = V.offsets + (size_t)blockIdx.x * V.nchunks;
    for (int b = 0; b < nck; b += 256) {
        const int k = b + threadIdx.x;
        const int v = k < nck ? cn[k] : 0;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int d = 1; d < 256; d <<= 1) {
            const int t = threadIdx.x >= d ? part[threadIdx.x - d] : 0;
            __syncthreads();
            part[threadIdx.x] += t;
            __syncthreads();
        }
        if (k < nck) off[k] = carry + part[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 255) carry += part[255];
        __syncthreads();
    }
    if (threadIdx.x == 0) V.totals[blockIdx.x] = carry;
}

// 4. each flagged pair's rank in its class -> its group, marked once
__global__ void __launch_bounds__(256) rg_mark(LaunchArgs A, int nreq, long long ntotal, RegroupView V) {
    const int nf = min(V.ctr[0], V.fcap);
    const int lane = threadIdx.x & 31;
    for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < nf; e += (gridDim.x * blockDim.x) >> 5) {
        const int c = V.cls_of[e];
        if (c < 0) continue;
        const unsigned long long key = V.ckeys[c];
        const long long gi = V.gidx[e];
        const int k = (int)(gi / kRegroupChunk);
        int intra = 0;
        for (long long b = (long long)k * kRegroupChunk; b < gi; b += 32) {
            const long long x = b + lane;
            bool m = false;
            if (x < gi) {
                const int req = req_at(A, nreq, x);
                m = class_of(A, req, local_of(A, req, x)).key == key;
            }
            intra += __popc(__ballot_sync(0xffffffffu, m));
        }
        if (lane != 0) continue;
        const long long rank = (long long)V.offsets[(size_t)c * V.nchunks + k] + intra;
        const int bits = V.cinfo[c].z;
        const long long grp = rank / group_lanes(bits);
        const unsigned long long lbit = 1ull << (int)(rank % group_lanes(bits));
        const unsigned long long gkey = ((unsigned long long)c << 40) | (unsigned long long)grp;
        unsigned s = (unsigned)mix64(gkey) & (unsigned)(V.hcap - 1);
        for (int probe = 0; probe < V.hcap; probe++) {
            const unsigned long long old = atomicCAS(&V.mhash[s], kEmpty, gkey);
            if (old == kEmpty || old == gkey) atomicOr(&V.needh[s], lbit);  // this pair's lane is wanted
            if (old == kEmpty) {
                const int b = bits == 8 ? 1 : 0;
                const int m = atomicAdd(&V.ctr[1 + b], 1);
                if (m < V.mcap) {
                    V.mlist[(size_t)b * V.mcap + m] = make_int2(c, (int)grp);
                    V.mslot[(size_t)b * V.mcap + m] = (int)s;
                } else {
                    atomicOr(&V.ctr[5], 2);
                }
                break;
            }
            if (old == gkey) break;
            s = (s + 1) & (unsigned)(V.hcap - 1);
            if (probe == V.hcap - 1) atomicOr(&V.ctr[5], 2);
        }
    }
}

// 5. the members of each marked group, in array order (-1: padding lanes)
__global__ void __launch_bounds__(256) rg_gather(LaunchArgs A, int nreq, long long ntotal, RegroupView V) {
    const int nck = (int)((ntotal + kRegroupChunk - 1) / kRegroupChunk);
    const int n16 = min(V.ctr[1], V.mcap), n8 = min(V.ctr[2], V.mcap);
    const int lane = threadIdx.x & 31;
    for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n16 + n8; e += (gridDim.x * blockDim.x) >> 5) {
        const int b = e < n16 ? 0 : 1;
        const size_t slot = (size_t)b * V.mcap + (e < n16 ? e : e - n16);
        const int2 cg = V.mlist[slot];
        const int c = cg.x;
        const int4 ci = V.cinfo[c];
        const int W = group_lanes(ci.z);
        const unsigned long long key = V.ckeys[c];
        const long long r0 = (long long)cg.y * W;
        const long long r1 = min(r0 + W, (long long)V.totals[c]);
        long long *mem = V.members + slot * 64;
        for (int l = lane; l < 64; l += 32) mem[l] = -1;
        __syncwarp();
        // the first chunk holding rank r0
        const int *off = V.offsets + (size_t)c * V.nchunks;
        const int *cn = V.counts + (size_t)c * V.nchunks;
        int lo = 0, hi = nck - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= r0) lo = mid; else hi = mid - 1;
        }
        int k = lo;
        while (k < nck && (long long)off[k] + cn[k] <= r0) k++;
        long long run = k < nck ? off[k] : r1;
        int padq = 0;
        while (run < r1 && k < nck) {
            if (cn[k] == 0) { k++; if (k < nck) run = off[k]; continue; }
            const long long c0 = (long long)k * kRegroupChunk, c1 = min(c0 + kRegroupChunk, ntotal);
            for (long long x0 = c0; x0 < c1 && run < r1; x0 += 32) {
                const long long x = x0 + lane;
                bool m = false;
                int len2 = 0;
                if (x < c1) {
                    const int req = req_at(A, nreq, x);
                    const int li = local_of(A, req, x);
                    m = class_of(A, req, li).key == key;
                    if (m) len2 = pair_src(A, li, req).pp->len2;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, m);
                const long long r = run + __popc(bal & ((1u << lane) - 1u));
                if (m && r >= r0 && r < r1) mem[r - r0] = x;
                if (m && r == r1 - 1) padq = len2;
                run += __popc(bal);
            }
            k++;
            if (k < nck) run = max(run, (long long)off[k]);
        }
        padq = __reduce_max_sync(0xffffffffu, padq);
        if (lane == 0) {
            V.ginfo[slot] = make_int4(ci.x, ci.y, padq, 0);
            V.gneed[slot] = V.needh[V.mslot[slot]];
        }
    }
}

// 7. leaves the tables empty for the next call
__global__ void rg_cleanup(RegroupView V) {
    const int n16 = min(V.ctr[1], V.mcap), n8 = min(V.ctr[2], V.mcap);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nth = gridDim.x * blockDim.x;
    for (int e = tid; e < n16 + n8; e += nth) {
        const size_t slot = e < n16 ? (size_t)e : (size_t)V.mcap + (e - n16);
        V.mhash[V.mslot[slot]] = kEmpty;
        V.needh[V.mslot[slot]] = 0ull;
    }
    for (int c = tid; c < kRegroupClasses; c += nth) V.ckeys[c] = kEmpty;
}
__global__ void rg_reset(RegroupView V, int *err_flags, ReqDesc *reqs, int nreq) {
    if (V.ctr[5]) {  // tables overflowed: the call (every request of a tick) fails
        if (threadIdx.x == 0) atomicOr(err_flags, ERR_FLAGCAP);
        for (int r = threadIdx.x; reqs && r < nreq; r += blockDim.x) atomicOr(&reqs[r].err, ERR_FLAGCAP);
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // kept for the caller: the call's flagged pairs and re-scored groups
        V.ctr[6] = V.ctr[0];
        V.ctr[7] = V.ctr[1] + V.ctr[2];
    }
    __syncthreads();
    if (threadIdx.x < 6 || (threadIdx.x >= 8 && threadIdx.x < 10)) V.ctr[threadIdx.x] = 0;
}

}  // namespace

cudaError_t RegroupBufs::ensure(long long ntotal, int cols_cap, int num_sms, bool *grown) {
    *grown = false;
    const long long nchunks = std::max<long long>(1, (ntotal + kRegroupChunk - 1) / kRegroupChunk);
    const long long fcap = std::max<long long>(1, ntotal);
    const long long mcap = std::min<long long>(fcap, ntotal / 32 + kRegroupClasses + 1);
    long long hcap = 64;
    while (hcap < 2 * mcap) hcap <<= 1;
    // group-kernel scratch: slots for the longer of the 16- and 8-bit rows
    const int col_cap = std::max(cols_cap, 1) + 3;
    const long long slot_bytes = (long long)std::max(wide_slot_elems(col_cap, 16), wide_slot_elems(col_cap, 8)) * 2;
    // one global slot per block, for the groups whose rows do not fit shared memory
    const long long slots = std::min<long long>((long long)num_sms, std::max<long long>(4, (1LL << 30) / slot_bytes));
    if (nchunks <= V.nchunks && fcap <= V.fcap && col_cap <= V.col_cap && V.ctr) {
        return cudaSuccess;
    }
    // the block-wide kernel, one block per group: a first launch with several
    // blocks per SM takes the groups whose rows (a ring of the band for long
    // queries) fit its shared memory, a second with the opt-in limit per block
    // and a global slot per block the rest
    int dev = 0, optin = 0;
    cudaError_t e0 = cudaGetDevice(&dev);
    if (e0 == cudaSuccess) e0 = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e0 == cudaSuccess) e0 = cudaFuncSetAttribute(bsw_group_wide_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e0 == cudaSuccess) e0 = cudaFuncSetAttribute(bsw_group_wide_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    const int smem1 = std::min(optin, kRegroupSmem1);
    int bps16 = 1, bps8 = 1;
    if (e0 == cudaSuccess)
        e0 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps16, bsw_group_wide_kernel<16>, 32 * wide_warps<16>(), smem1);
    if (e0 == cudaSuccess)
        e0 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps8, bsw_group_wide_kernel<8>, 32 * wide_warps<8>(), smem1);
    if (e0 != cudaSuccess) return e0;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~(size_t)255; return o; };
    const size_t o_ctr = take(sizeof(int) * 16);
    const size_t o_flag = take(sizeof(long long) * fcap);
    const size_t o_cls = take(sizeof(int) * fcap);
    const size_t o_gidx = take(sizeof(long long) * fcap);
    const size_t o_ck = take(sizeof(unsigned long long) * kRegroupClasses);
    const size_t o_ci = take(sizeof(int4) * kRegroupClasses);
    const size_t o_cnt = take(sizeof(int) * kRegroupClasses * nchunks);
    const size_t o_off = take(sizeof(int) * kRegroupClasses * nchunks);
    const size_t o_tot = take(sizeof(int) * kRegroupClasses);
    const size_t o_mh = take(sizeof(unsigned long long) * hcap);
    const size_t o_nh = take(sizeof(unsigned long long) * hcap);
    const size_t o_gn = take(sizeof(unsigned long long) * 2 * mcap);
    const size_t o_ml = take(sizeof(int2) * 2 * mcap);
    const size_t o_ms = take(sizeof(int) * 2 * mcap);
    const size_t o_mem = take(sizeof(long long) * 64 * 2 * mcap);
    const size_t o_gi = take(sizeof(int4) * 2 * mcap);
    const size_t o_scr = take((size_t)slots * (size_t)slot_bytes);
    arena.release();
    cudaError_t e = arena.ensure(off);
    if (e != cudaSuccess) { V = RegroupView(); return e; }
    unsigned char *b = reinterpret_cast<unsigned char *>(arena.p);
    V.ctr = reinterpret_cast<int *>(b + o_ctr);
    V.flagged = reinterpret_cast<long long *>(b + o_flag);
    V.cls_of = reinterpret_cast<int *>(b + o_cls);
    V.gidx = reinterpret_cast<long long *>(b + o_gidx);
    V.ckeys = reinterpret_cast<unsigned long long *>(b + o_ck);
    V.cinfo = reinterpret_cast<int4 *>(b + o_ci);
    V.counts = reinterpret_cast<int *>(b + o_cnt);
    V.offsets = reinterpret_cast<int *>(b + o_off);
    V.totals = reinterpret_cast<int *>(b + o_tot);
    V.mhash = reinterpret_cast<unsigned long long *>(b + o_mh);
    V.needh = reinterpret_cast<unsigned long long *>(b + o_nh);
    V.gneed = reinterpret_cast<unsigned long long *>(b + o_gn);
    V.mlist = reinterpret_cast<int2 *>(b + o_ml);
    V.mslot = reinterpret_cast<int *>(b + o_ms);
    V.members = reinterpret_cast<long long *>(b + o_mem);
    V.ginfo = reinterpret_cast<int4 *>(b + o_gi);
    V.scratch = reinterpret_cast<int16_t *>(b + o_scr);
    V.nchunks = (int)nchunks;
    V.fcap = (int)fcap;
    V.mcap = (int)mcap;
    V.hcap = (int)hcap;
    V.col_cap = col_cap;
    V.slots = (int)slots;
    V.smem1 = smem1;
    V.grid1[0] = num_sms * std::max(1, bps16);
    V.grid1[1] = num_sms * std::max(1, bps8);
    V.smem = optin;
    // empty tables, zero counters (the passes leave them so)
    if ((e = cudaMemset(V.ctr, 0, sizeof(int) * 16)) != cudaSuccess) return e;
    if ((e = cudaMemset(V.ckeys, 0xff, sizeof(unsigned long long) * kRegroupClasses)) != cudaSuccess) return e;
    if ((e = cudaMemset(V.mhash, 0xff, sizeof(unsigned long long) * hcap)) != cudaSuccess) return e;
    if ((e = cudaMemset(V.needh, 0, sizeof(unsigned long long) * hcap)) != cudaSuccess) return e;
    *grown = true;
    return cudaDeviceSynchronize();
}

cudaError_t enqueue_regroup(const RegroupView &V, LaunchArgs A, int nreq, long long ntotal,
                            int num_sms, cudaStream_t s, uint64_t *launches) {
    if (ntotal <= 0) return cudaSuccess;
    const int nck = (int)((ntotal + kRegroupChunk - 1) / kRegroupChunk);
    const int g1 = std::max(1, std::min(num_sms * 4, (int)((ntotal + 255) / 256)));
    rg_classes<<<g1, 256, 0, s>>>(A, nreq, V);
    rg_count<<<nck, 256, 0, s>>>(A, nreq, ntotal, V);
    rg_scan<<<kRegroupClasses, 256, 0, s>>>(V, nck);
    rg_mark<<<num_sms * 4, 256, 0, s>>>(A, nreq, ntotal, V);
    rg_gather<<<num_sms * 2, 256, 0, s>>>(A, nreq, ntotal, V);
    // 6. the marked groups, scored in the reference's grouping
    for (int b = 0; b < 2; b++) {
        GroupArgs G;
        G.pairs = A.pairs;
        G.ref = A.ref; G.qer = A.qer;
        G.ref_lo = A.ref_lo; G.ref_hi = A.ref_hi; G.qer_lo = A.qer_lo; G.qer_hi = A.qer_hi;
        G.n = 0;
        G.w = A.w;
        G.bits = b == 0 ? 16 : 8;
        G.col_cap = V.col_cap;
        G.slot_elems = wide_slot_elems(V.col_cap, G.bits);
        G.scratch = V.scratch;
        G.work_counter = &V.ctr[3 + b];
        G.cells = A.cells;
        G.err_flags = A.err_flags;
        G.err_index = A.err_index;
        G.P = A.P;
        G.members = V.members + (size_t)b * V.mcap * 64;
        G.ginfo = V.ginfo + (size_t)b * V.mcap;
        G.need = V.gneed + (size_t)b * V.mcap;
        G.ngroups_dev = &V.ctr[1 + b];
        G.ngroups_cap = V.mcap;
        G.reqs = A.reqs;
        G.nreq = nreq;
        // first launch: the groups that fit smem1, several blocks per SM
        G.smem_bytes = (size_t)V.smem1;
        G.defer = true;
        G.skip_upto = 0;
        if (b == 0) bsw_group_wide_kernel<16><<<V.grid1[0], 32 * wide_warps<16>(), V.smem1, s>>>(G);
        else bsw_group_wide_kernel<8><<<V.grid1[1], 32 * wide_warps<8>(), V.smem1, s>>>(G);
        // second: the rest, one block per SM, global slot = block index
        G.work_counter = &V.ctr[8 + b];
        G.defer = false;
        const size_t xb = b == 0 ? wide_x_bytes<wide_warps<16>()>() : wide_x_bytes<wide_warps<8>()>();
        G.skip_upto = (size_t)V.smem1 > xb ? (size_t)V.smem1 - xb : 0;
        G.smem_bytes = (size_t)V.smem;
        const int blocks = std::min(V.slots, num_sms);
        if (b == 0) bsw_group_wide_kernel<16><<<blocks, 32 * wide_warps<16>(), V.smem, s>>>(G);
        else bsw_group_wide_kernel<8><<<blocks, 32 * wide_warps<8>(), V.smem, s>>>(G);
    }
    rg_cleanup<<<std::max(1, num_sms), 256, 0, s>>>(V);
    rg_reset<<<1, 32, 0, s>>>(V, A.err_flags, A.reqs, nreq);
    if (launches) *launches += 11;
    return cudaGetLastError();
}

}  // namespace talbsw
