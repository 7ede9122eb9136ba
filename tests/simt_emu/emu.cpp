// Runs the CUDA kernel source (csrc/bsw_kernel.cuh), compiled for the host,
// one std::thread per lane, so its logic can be checked against the oracle on
// a machine without a GPU.  Test infrastructure only; the product path never
// uses it.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cuda_runtime.h"

namespace simt {
thread_local Dim tl_threadIdx, tl_blockIdx, tl_blockDim, tl_gridDim;
thread_local Warp *tl_warp;
thread_local unsigned char *tl_smem;
std::mutex atomic_mu;
}  // namespace simt

// The kernel's dynamic shared memory resolves to the per-block buffer.
#define TALBSW_DYNAMIC_SMEM(name) unsigned char *name = simt::tl_smem
#include "bsw_kernel.cuh"
#include "bsw_lane.cuh"
#include "sw_kernel.cuh"
#include "chain_kernel.cuh"
#include "bsw_group.cuh"
#include "bsw_group_wide.cuh"
#include <functional>

// Runs one launch of A (one block of `warps` warps); -1 if a warp's lanes
// did not finish together (a divergent exit).
// sw != nullptr: the unbanded Smith-Waterman kernel with those arguments
// instead (G, K unused).
static int sw_packed = 0;  // the unbanded kernel: 1 = two pairs per warp (16x2)
static const talbsw::GroupArgs *g_group = nullptr;  // set: the grouped kernel instead

static int run_launch(talbsw::LaunchArgs &A, int G, int K, int warps,
                      const talsw::SwArgs *sw = nullptr, const talchain::ChainArgs *ch = nullptr) {
    size_t wbytes = g_group ? 64
                  : ch ? talchain::chain_warp_smem_bytes(ch->bw) + 16
                  : sw ? (sw_packed ? talsw::sw2_warp_smem_bytes(sw->cols_cap) : talsw::sw_warp_smem_bytes(sw->cols_cap))
                  : G == 1 ? talbsw::lane_warp_smem_bytes(A.cols_cap, A.win)
                           : talbsw::warp_smem_bytes(A.cols_cap, A.rows_cap, G, A.win);
    std::vector<unsigned char> smem(wbytes * warps + 64, 0xA5);  // poisoned, like fresh smem
    // warps run one after another; the 32 lanes of a warp are fibers
    int divergent = 0;
    for (int wi = 0; wi < warps; wi++) {
        simt::Warp *W = new simt::Warp();
        std::vector<std::vector<char>> stacks(32, std::vector<char>(1 << 18));
        struct Arg { int t; simt::Warp *W; const talbsw::LaunchArgs *A; int G, K; unsigned char *sm; int warps; const talsw::SwArgs *sw; const talchain::ChainArgs *ch; };
        static thread_local Arg args[32];
        for (int l = 0; l < 32; l++) {
            args[l] = Arg{wi * 32 + l, W, &A, G, K, smem.data(), warps, sw, ch};
            getcontext(&W->lane_ctx[l]);
            W->lane_ctx[l].uc_stack.ss_sp = stacks[l].data();
            W->lane_ctx[l].uc_stack.ss_size = stacks[l].size();
            W->lane_ctx[l].uc_link = &W->sched;
            makecontext(&W->lane_ctx[l], (void (*)())+[](int l2) {
                Arg &a = args[l2];
                simt::tl_threadIdx.x = a.t;
                simt::tl_blockIdx.x = 0;
                simt::tl_blockDim.x = 32 * a.warps;
                simt::tl_gridDim.x = 1;
                simt::tl_warp = a.W;
                simt::tl_smem = a.sm;
                if (g_group) { if (g_group->bits == 8) talbsw::bsw_group_kernel<8>(*g_group); else talbsw::bsw_group_kernel<16>(*g_group); a.W->done[a.t & 31] = true; return; }
                if (a.ch) { talchain::chain_kernel(*a.ch); a.W->done[a.t & 31] = true; return; }
                if (a.sw) { if (sw_packed) talsw::sw_wave2_kernel<talsw::kSwRows>(*a.sw); else talsw::sw_wave_kernel<talsw::kSwRows>(*a.sw); a.W->done[a.t & 31] = true; return; }
                if (a.G == 1) { const bool sym = a.A->P.o_del == a.A->P.o_ins && a.A->P.e_del == a.A->P.e_ins; int v = a.K == 4 ? 3 : a.K == 2 ? 2 : 1; if (!sym) v &= 1; if (a.A->win > 0 && (a.A->win & (a.A->win - 1))) v |= 4;
                    switch (v) { case 7: talbsw::bsw_lane_kernel<7>(*a.A); break; case 6: talbsw::bsw_lane_kernel<6>(*a.A); break; case 5: talbsw::bsw_lane_kernel<5>(*a.A); break; case 4: talbsw::bsw_lane_kernel<4>(*a.A); break; case 3: talbsw::bsw_lane_kernel<3>(*a.A); break; case 2: talbsw::bsw_lane_kernel<2>(*a.A); break; case 1: talbsw::bsw_lane_kernel<1>(*a.A); break; default: talbsw::bsw_lane_kernel<0>(*a.A); }
                    a.W->done[a.t & 31] = true; return; }
                switch (a.G * 10 + a.K) {
                    case 44: talbsw::bsw_kernel<4, 4>(*a.A); break;
                    case 42: talbsw::bsw_kernel<4, 2>(*a.A); break;
                    case 84: talbsw::bsw_kernel<8, 4>(*a.A); break;
                    case 82: talbsw::bsw_kernel<8, 2>(*a.A); break;
                    case 164: talbsw::bsw_kernel<16, 4>(*a.A); break;
                    case 162: talbsw::bsw_kernel<16, 2>(*a.A); break;
                    case 322: talbsw::bsw_kernel<32, 2>(*a.A); break;
                    default: talbsw::bsw_kernel<32, 4>(*a.A); break;
                }
                a.W->done[a.t & 31] = true;
            }, 1, l);
        }
        for (;;) {
            int ndone = 0;
            for (int l = 0; l < 32; l++) {
                if (W->done[l]) { ndone++; continue; }
                simt::tl_warp = W;
                simt::tl_threadIdx.x = wi * 32 + l;
                swapcontext(&W->sched, &W->lane_ctx[l]);
                if (W->done[l]) ndone++;
            }
            if (ndone == 32) break;
            if (ndone > 0) { divergent = 1; break; }
        }
        delete W;
    }
    if (divergent) return -1;
    return 0;
}

extern "C" int emu_bsw_run(talbsw::DevPair *pairs, const uint8_t *ref, long long ref_lo,
                           long long ref_hi, const uint8_t *qer, long long qer_lo,
                           long long qer_hi, int n, int w, const int32_t *wpair, int bits,
                           const int32_t *kp, int G, int K, int warps, int win, int *err_flags,
                           long long *err_index) {
    talbsw::LaunchArgs A;
    std::memset(&A, 0, sizeof(A));
    A.pairs = pairs;
    A.ref = ref; A.ref_lo = ref_lo; A.ref_hi = ref_hi;
    A.qer = qer; A.qer_lo = qer_lo; A.qer_hi = qer_hi;
    A.wpair = wpair;
    A.n = n; A.w = w; A.bits = bits; A.win = win;
    int m1 = 1, m2 = 1;
    for (int i = 0; i < n; i++) { m1 = std::max(m1, pairs[i].len1); m2 = std::max(m2, pairs[i].len2); }
    A.cols_cap = m2; A.rows_cap = m1;
    int counter = 0;
    *err_flags = 0; *err_index = (long long)INT64_MAX;
    A.work_counter = &counter; A.err_flags = err_flags; A.err_index = err_index;
    A.P = {kp[0], kp[1], kp[2], kp[3], kp[4], kp[5], kp[6], kp[7]};
    return run_launch(A, G, K, warps);
}

// The same with the group-coupling detector on: flagged pairs are appended
// to flagged[0, cap) ((request + 1) << 32 | pair), their count to *nflagged.
extern "C" int emu_bsw_run_det(talbsw::DevPair *pairs, const uint8_t *ref, long long ref_lo,
                               long long ref_hi, const uint8_t *qer, long long qer_lo,
                               long long qer_hi, int n, int w, const int32_t *wpair, int bits,
                               const int32_t *kp, int G, int K, int warps, int win, int *err_flags,
                               long long *err_index, long long *flagged, int *nflagged, int cap) {
    talbsw::LaunchArgs A;
    std::memset(&A, 0, sizeof(A));
    A.pairs = pairs;
    A.ref = ref; A.ref_lo = ref_lo; A.ref_hi = ref_hi;
    A.qer = qer; A.qer_lo = qer_lo; A.qer_hi = qer_hi;
    A.wpair = wpair;
    A.n = n; A.w = w; A.bits = bits; A.win = win;
    int m1 = 1, m2 = 1;
    for (int i = 0; i < n; i++) { m1 = std::max(m1, pairs[i].len1); m2 = std::max(m2, pairs[i].len2); }
    A.cols_cap = m2; A.rows_cap = m1;
    int counter = 0;
    *err_flags = 0; *err_index = (long long)INT64_MAX; *nflagged = 0;
    A.work_counter = &counter; A.err_flags = err_flags; A.err_index = err_index;
    A.flagged = flagged; A.nflagged = nflagged; A.flag_cap = cap;
    A.P = {kp[0], kp[1], kp[2], kp[3], kp[4], kp[5], kp[6], kp[7]};
    return run_launch(A, G, K, warps);
}

// The grouped kernel (the reference's SIMD groups, one warp each) over n
// pairs with one band; `warps` warps share the groups.
extern "C" int emu_bsw_group_run(talbsw::DevPair *pairs, const uint8_t *ref, long long ref_lo,
                                 long long ref_hi, const uint8_t *qer, long long qer_lo,
                                 long long qer_hi, int n, int w, int bits, const int32_t *kp,
                                 int warps, int *err_flags, long long *err_index) {
    talbsw::GroupArgs G;
    std::memset(&G, 0, sizeof(G));
    G.pairs = pairs;
    G.ref = ref; G.ref_lo = ref_lo; G.ref_hi = ref_hi;
    G.qer = qer; G.qer_lo = qer_lo; G.qer_hi = qer_hi;
    G.n = n; G.w = w; G.bits = bits;
    int m2 = 1;
    for (int i = 0; i < n; i++) m2 = std::max(m2, pairs[i].len2);
    G.col_cap = m2 + 3;
    G.slot_elems = talbsw::group_slot_elems(G.col_cap, bits);
    std::vector<int16_t> scratch(G.slot_elems * warps, (int16_t)0x5a5a);  // poisoned
    G.scratch = scratch.data();
    int counter = 0;
    unsigned long long cells = 0;
    *err_flags = 0; *err_index = (long long)INT64_MAX;
    G.work_counter = &counter; G.cells = &cells; G.err_flags = err_flags; G.err_index = err_index;
    G.P = {kp[0], kp[1], kp[2], kp[3], kp[4], kp[5], kp[6], kp[7]};
    talbsw::LaunchArgs A;
    std::memset(&A, 0, sizeof(A));
    g_group = &G;
    const int rc = run_launch(A, 1, 4, warps);
    g_group = nullptr;
    return rc;
}

// One block of `warps` warps running body() in every lane, the warps
// interleaved so that __syncthreads() holds: a warp whose lanes all wait at
// the block barrier is skipped until every warp still running waits there.
// -1 on a divergent warp (its lanes at different barriers or exits).
static int run_block(void (*body)(const void *), const void *arg, int warps, unsigned char *smem) {
    std::vector<simt::Warp *> Ws(warps);
    std::vector<std::vector<char>> stacks((size_t)32 * warps, std::vector<char>(1 << 18));
    struct BArg { int t; simt::Warp *W; unsigned char *sm; int warps; void (*body)(const void *); const void *arg; };
    static thread_local std::vector<BArg> bargs;
    bargs.assign((size_t)32 * warps, BArg{});
    for (int wi = 0; wi < warps; wi++) {
        Ws[wi] = new simt::Warp();
        for (int l = 0; l < 32; l++) {
            const int t = wi * 32 + l;
            bargs[t] = BArg{t, Ws[wi], smem, warps, body, arg};
            getcontext(&Ws[wi]->lane_ctx[l]);
            Ws[wi]->lane_ctx[l].uc_stack.ss_sp = stacks[t].data();
            Ws[wi]->lane_ctx[l].uc_stack.ss_size = stacks[t].size();
            Ws[wi]->lane_ctx[l].uc_link = &Ws[wi]->sched;
            makecontext(&Ws[wi]->lane_ctx[l], (void (*)())+[](int t2) {
                BArg &a = bargs[t2];
                simt::tl_threadIdx.x = a.t;
                simt::tl_blockIdx.x = 0;
                simt::tl_blockDim.x = 32 * a.warps;
                simt::tl_gridDim.x = 1;
                simt::tl_warp = a.W;
                simt::tl_smem = a.sm;
                a.body(a.arg);
                a.W->done[a.t & 31] = true;
            }, 1, t);
        }
    }
    int divergent = 0;
    for (;;) {
        bool ran = false, live = false;
        for (int wi = 0; wi < warps && !divergent; wi++) {
            simt::Warp *W = Ws[wi];
            int nlive = 0, nbar = 0;
            for (int l = 0; l < 32; l++) {
                if (W->done[l]) continue;
                nlive++;
                nbar += W->at_bar[l];
            }
            if (nlive == 0) continue;
            live = true;
            if (nbar == nlive) continue;  // waiting at the block barrier
            if (nbar != 0 || nlive != 32) { divergent = 1; break; }
            for (int l = 0; l < 32; l++) {
                simt::tl_warp = W;
                simt::tl_threadIdx.x = wi * 32 + l;
                simt::tl_smem = smem;
                swapcontext(&W->sched, &W->lane_ctx[l]);
            }
            ran = true;
        }
        if (divergent || !live) break;
        if (!ran)  // every running warp waits at the barrier: release it
            for (int wi = 0; wi < warps; wi++)
                for (int l = 0; l < 32; l++) Ws[wi]->at_bar[l] = false;
    }
    for (int wi = 0; wi < warps; wi++) delete Ws[wi];
    return divergent ? -1 : 0;
}

// The block-wide grouped kernel (bsw_group_wide.cuh) over n pairs with one
// band, one block taking every group; smem_rows: shared-memory bytes for the
// group's rows (0: every group uses the global slot).  members / ginfo /
// need / ngroups: member mode (null members: consecutive groups of n).
extern "C" int emu_bsw_group_wide_run(talbsw::DevPair *pairs, const uint8_t *ref, long long ref_lo,
                                      long long ref_hi, const uint8_t *qer, long long qer_lo,
                                      long long qer_hi, int n, int w, int bits, const int32_t *kp,
                                      const long long *members, const int *ginfo,
                                      const unsigned long long *need, int ngroups,
                                      long long smem_rows, int *err_flags, long long *err_index,
                                      unsigned long long *cells) {
    talbsw::GroupArgs G;
    std::memset(&G, 0, sizeof(G));
    G.pairs = pairs;
    G.ref = ref; G.ref_lo = ref_lo; G.ref_hi = ref_hi;
    G.qer = qer; G.qer_lo = qer_lo; G.qer_hi = qer_hi;
    G.n = n; G.w = w; G.bits = bits;
    int m2 = 1;
    for (int i = 0; i < n; i++) m2 = std::max(m2, pairs[i].len2);
    G.col_cap = m2 + 3;
    G.slot_elems = talbsw::wide_slot_elems(G.col_cap, bits);
    std::vector<int16_t> scratch(G.slot_elems, (int16_t)0x5a5a);  // poisoned
    G.scratch = scratch.data();
    int counter = 0, ng = ngroups;
    *cells = 0;
    *err_flags = 0; *err_index = (long long)INT64_MAX;
    G.work_counter = &counter; G.cells = cells; G.err_flags = err_flags; G.err_index = err_index;
    G.P = {kp[0], kp[1], kp[2], kp[3], kp[4], kp[5], kp[6], kp[7]};
    G.ngroups_cap = 1 << 30;
    if (members) {
        G.members = members;
        G.ginfo = reinterpret_cast<const int4 *>(ginfo);
        G.need = need;
        G.ngroups_dev = &ng;
    }
    const int nw = bits == 8 ? talbsw::wide_warps<8>() : talbsw::wide_warps<16>();
    const size_t xb = bits == 8 ? talbsw::wide_x_bytes<talbsw::wide_warps<8>()>()
                                : talbsw::wide_x_bytes<talbsw::wide_warps<16>()>();
    G.smem_bytes = xb + (size_t)smem_rows;
    std::vector<unsigned char> smem(G.smem_bytes + 64, 0xA5);  // poisoned, like fresh smem
    auto body = [](const void *a) {
        const talbsw::GroupArgs &g = *static_cast<const talbsw::GroupArgs *>(a);
        if (g.bits == 8) talbsw::group_wide_body<8, talbsw::wide_warps<8>()>(g, simt::tl_smem);
        else talbsw::group_wide_body<16, talbsw::wide_warps<16>()>(g, simt::tl_smem);
    };
    return run_block(body, &G, nw, smem.data());
}

// A serving tick: nreq requests, each with its own pair array, sequence
// windows, band and precision, scored in the work order given by
// order (request-local index) / order_req (request).  Per request errors go
// to req_err / req_bad.
extern "C" int emu_bsw_run_reqs(int nreq, talbsw::DevPair **pairs, const uint8_t **ref,
                                const long long *ref_lo, const long long *ref_hi,
                                const uint8_t **qer, const long long *qer_lo,
                                const long long *qer_hi, const int32_t **wpair, const int *n,
                                const int *w, const int *bits, int nwork, const int32_t *order,
                                const int32_t *order_req, const int32_t *kp, int G, int K,
                                int warps, int win, int *req_err, long long *req_bad) {
    std::vector<talbsw::ReqDesc> R(nreq);
    int first = 0, m1 = 1, m2 = 1;
    for (int r = 0; r < nreq; r++) {
        talbsw::ReqDesc &d = R[r];
        std::memset(&d, 0, sizeof(d));
        d.pairs = pairs[r]; d.ref = ref[r]; d.qer = qer[r]; d.wpair = wpair[r];
        d.ref_lo = ref_lo[r]; d.ref_hi = ref_hi[r]; d.qer_lo = qer_lo[r]; d.qer_hi = qer_hi[r];
        d.bad = (long long)INT64_MAX;
        d.first = first; d.n = n[r]; d.w = w[r]; d.bits = bits[r];
        first += n[r];
        for (int k = 0; k < n[r]; k++) {
            m1 = std::max(m1, pairs[r][k].len1);
            m2 = std::max(m2, pairs[r][k].len2);
        }
    }
    talbsw::LaunchArgs A;
    std::memset(&A, 0, sizeof(A));
    A.reqs = R.data();
    A.order = order;
    A.order_req = order_req;
    A.n = nwork;
    A.cols_cap = m2; A.rows_cap = m1; A.win = win;
    int counter = 0, flags = 0;
    long long bad = (long long)INT64_MAX;
    A.work_counter = &counter; A.err_flags = &flags; A.err_index = &bad;
    A.P = {kp[0], kp[1], kp[2], kp[3], kp[4], kp[5], kp[6], kp[7]};
    const int rc = run_launch(A, G, K, warps);
    for (int r = 0; r < nreq; r++) {
        req_err[r] = R[r].err;
        req_bad[r] = R[r].bad;
    }
    return rc;
}


// The unbanded Smith-Waterman kernel over n 12-byte pairs; seqbuf holds the
// whole caller buffer (window [0, seq_bytes)).  params: match, mismatch,
// open, extend.  Returns the kernel's error flags (bad index in *bad).
extern "C" int emu_sw_run(void *pairs, int n, const uint8_t *seqbuf, long long seq_bytes,
                          long long stride, int maxlen, int score_lim, const int32_t *params,
                          int warps, int packed, const int32_t *order, long long *bad) {
    sw_packed = packed;
    talsw::SwArgs S;
    std::memset(&S, 0, sizeof(S));
    S.pairs = static_cast<talsw::SwPair *>(pairs);
    S.seq = seqbuf; S.seq_lo = 0; S.seq_hi = seq_bytes; S.stride = stride;
    S.n = n;
    S.order = order;
    int cols = 1;
    for (int k = 0; k < n; k++) cols = std::max<int>(cols, S.pairs[k].len2);
    S.cols_cap = cols;
    S.maxlen = maxlen;
    S.score_lim = score_lim;
    S.match = params[0]; S.mismatch = params[1]; S.open = params[2]; S.ext = params[3];
    int counter = 0, flags = 0;
    long long badi = (long long)INT64_MAX;
    S.work_counter = &counter; S.err_flags = &flags; S.err_index = &badi;
    talbsw::LaunchArgs A;
    std::memset(&A, 0, sizeof(A));
    const int rc = run_launch(A, 1, 4, warps, &S);
    *bad = badi;
    return rc < 0 ? -1 : flags;
}


// The anchor chaining kernel over n_reads reads (anchors 16-byte records, read
// k = [offsets[k], offsets[k+1])).  Returns the kernel's error flags (first
// bad read in *bad), -1 on a divergent exit.
extern "C" int emu_chain_run(const void *anchors, const int64_t *offsets, int n_reads, int bw,
                             int max_iter, int dr, int dq, uint32_t *f, int32_t *p, int32_t *v,
                             int warps, unsigned long long *evals, long long *bad) {
    talchain::ChainArgs C;
    std::memset(&C, 0, sizeof(C));
    C.anchors = static_cast<const talchain::Anchor *>(anchors);
    C.offsets = offsets;
    C.n_reads = n_reads;
    C.bw = bw; C.max_iter = max_iter; C.dr = dr; C.dq = dq;
    std::vector<int2> rq((size_t)std::max<int64_t>(offsets[n_reads], 1));
    C.rq = rq.data();
    C.f = f; C.p = p; C.v = v;
    int counter = 0, flags = 0;
    long long badi = (long long)INT64_MAX;
    *evals = 0;
    C.work_counter = &counter; C.evals = evals; C.err_flags = &flags; C.err_index = &badi;
    talbsw::LaunchArgs A;
    std::memset(&A, 0, sizeof(A));
    const int rc = run_launch(A, 1, 4, warps, nullptr, &C);
    *bad = badi;
    return rc < 0 ? -1 : flags;
}
