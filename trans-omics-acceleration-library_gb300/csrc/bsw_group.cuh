// The reference's SIMD grouping on a warp: getScores16 / getScores8 score
// their pairs in groups of 32 (16-bit) / 64 (8-bit) consecutive pairs, one
// pair per vector lane (AVX-512BW widths, bandedSWA.h:66-67), and every group
// shares one band [beg, end) per row, computed from all of its lanes
// (bandedSWA.cpp:3080-3316 for 16-bit, :2371-2621 for 8-bit).  A lane's
// outputs can depend on the other lanes of its group through that shared
// band: cells outside the lane's own band but inside the group's are still
// evaluated (masked), which zeroes the lane's row entries there, and the
// lane's head / tail re-derivation scans from the group's band edges, so a
// stale non-zero entry past the lane's own end can keep its tail from
// narrowing.  The per-pair kernels score each pair as if it were alone in its
// group, which gives the same outputs on almost all inputs; this kernel gives
// the grouped outputs exactly, for callers that need bit-equality with the
// reference on any input.
//
// One warp is one group: lane l of the group is thread l (16-bit) or threads
// l and l + 32 share a thread (8-bit, two lanes per thread).  Every value is
// kept in the element width the reference computes in (int16 / int8, all
// arithmetic wrapping), so nothing here depends on an exact-range argument.
// The group's row entries (H and F packed in one word, and the query codes)
// live in a per-warp slot of global scratch, column-major with the group's
// lanes contiguous (one column of the group = 128 or 256 bytes, coalesced).
#pragma once

#include "bsw_kernel.cuh"

namespace talbsw {

struct GroupArgs {
    DevPair *pairs;
    const uint8_t *ref, *qer;
    long long ref_lo, ref_hi, qer_lo, qer_hi;
    int n;            // pairs; groups = ceil(n / lanes)
    int w;            // the call's band
    int bits;         // 8 or 16
    int col_cap;      // columns of a scratch slot (>= max len2 + 3)
    int16_t *scratch; // per warp: (H, F) words [col_cap][lanes], then the codes
    size_t slot_elems;  // int16 elements per warp slot
    int *work_counter;
    unsigned long long *cells;
    int *err_flags;
    long long *err_index;
    KernelParams P;
    // member mode (the block-wide kernel of the regroup pass, bsw_regroup.cu,
    // bsw_group_wide.cuh; the one-warp kernel here scores consecutive groups):
    // group g's lane l is the pair with global index members[g * 64 + l]
    // (-1: a padding lane), its band and request are ginfo[g] {w, req,
    // padding lanes' len2, -}, and the groups are 0 .. *ngroups_dev; a
    // global index is the pair's index, or its request's `first` plus its
    // index there when reqs is set (a serving tick's pairs)
    const long long *members = nullptr;
    const int4 *ginfo = nullptr;
    const int *ngroups_dev = nullptr;
    int ngroups_cap = 1 << 30;
    ReqDesc *reqs = nullptr;
    int nreq = 0;
    const unsigned long long *need = nullptr;  // per group, the lanes whose outputs are
                                               // wanted (bit l: lane l; null: all)
    size_t smem_bytes = 0;  // the block-wide kernel's dynamic shared memory per block
    // block-wide kernel in two launches: the first (defer) leaves the groups
    // whose rows do not fit its shared memory, the second skips the groups
    // whose rows need at most skip_upto bytes (the first launch took them)
    bool defer = false;
    size_t skip_upto = 0;
};

// Global pair index -> (request, local index) in a serving tick's pair space.
__device__ __forceinline__ int group_req_of(const ReqDesc *reqs, int nreq, long long gi) {
    int lo = 0, hi = nreq - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (reqs[mid].first <= gi) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Lanes per group: 64 for 8-bit, 32 for 16-bit (AVX-512BW SIMD_WIDTH8/16).
__host__ __device__ inline int group_lanes(int bits) { return bits == 8 ? 64 : 32; }

// int16 elements of one warp's scratch slot: H and F (int16 each, one word
// per lane and column) and the query codes (one byte each, four consecutive
// columns of a lane in one word), rounded to 16 bytes so every slot starts
// aligned.
__host__ __device__ inline size_t group_slot_elems(int col_cap, int bits) {
    const size_t l = (size_t)group_lanes(bits);
    const size_t qbytes = ((((size_t)col_cap + 3) & ~(size_t)3) + 8) * l;  // + two words read ahead
    return ((size_t)col_cap * l * 2 + (qbytes + 1) / 2 + 8 + 7) & ~(size_t)7;
}

// Bytes of a group's rows held in shared memory (block-wide kernel): the
// (H, F) words of col_cap columns and the query codes, as in a scratch slot.
__host__ __device__ inline size_t group_smem_bytes(int col_cap, int bits) {
    const size_t l = (size_t)group_lanes(bits);
    return (size_t)col_cap * l * 4 + ((((size_t)col_cap + 3) & ~(size_t)3) + 8) * l + 16;
}

__host__ __device__ __forceinline__ unsigned umin(unsigned a, unsigned b) { return a < b ? a : b; }

// Element-width helpers: S = 16 or 8 bits; values are held sign-extended.
template <int SB>
struct GE {
    static constexpr int SH = 32 - SB;
    static constexpr unsigned MSK = (1u << SB) - 1u;
    // the low SB bits, sign-extended (one sign-extend instruction)
    __device__ __forceinline__ static int ws(int x) {
        if constexpr (SB == 16) return (int)(int16_t)(uint16_t)(unsigned)x;
        else return (int)(int8_t)(uint8_t)(unsigned)x;
    }
    __device__ __forceinline__ static unsigned us(int x) { return (unsigned)x & MSK; }
};

// 16-bit: at most 40 registers, so 12 blocks (48 warps) fit an SM (196.7 against
// 199.4 ms per 1,000,000 C2 pairs with 52); 8-bit: two lanes per thread need ~90.
template <int SB>
__global__ void __launch_bounds__(128, SB == 16 ? 12 : 5) bsw_group_kernel(GroupArgs A) {
    typedef GE<SB> E;
    constexpr int LPT = SB == 8 ? 2 : 1;  // lanes per thread
    constexpr int W = 32 * LPT;           // lanes per group
    constexpr bool is16 = SB == 16;
    const unsigned full = 0xffffffffu;
    const int t = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // H (low half) and F (high half) of a lane's column in one word
    uint32_t *HF = reinterpret_cast<uint32_t *>(A.scratch + (size_t)gw * A.slot_elems);
    int8_t *Q2 = reinterpret_cast<int8_t *>(HF + (size_t)A.col_cap * W);
    const KernelParams &P = A.P;
    const int ngroups = (A.n + W - 1) / W;

    // scores and constants (bandedSWA.cpp:50-68), wrapped to the element width
    const int w_match = E::ws((int8_t)P.a);
    const int w_mismatch = E::ws((int8_t)(P.b * -1));
    const int e_del = E::ws(P.e_del), oe_del = E::ws(P.o_del + P.e_del);
    const int e_ins = E::ws(P.e_ins), oe_ins = E::ws(P.o_ins + P.e_ins);
    const int o_del = E::ws(P.o_del);
    const int zdropv = E::ws(P.zdrop);
    int maxsc = 0;  // max of the scores (:2779 / :2082)
    if (maxsc < (int8_t)P.a) maxsc = E::ws((int8_t)P.a);
    if (maxsc < (int8_t)(P.b * -1)) maxsc = E::ws((int8_t)(P.b * -1));

    for (;;) {
        int g = 0;
        if (t == 0) g = atomicAdd(A.work_counter, 1);
        g = __shfl_sync(full, g, 0);
        if (g >= ngroups) break;

        // ---- the group's lanes; lanes past n are padded the way the
        // reference pads its array (16-bit: len1 = len2 = 0, :2711-2717;
        // 8-bit: len1 = 0, len2 = the last pair's len2, :2012-2018), h0 = 0
        int len1[LPT], len2[LPT], h0r[LPT];
        long long idr[LPT], idq[LPT];
        DevPair *pp[LPT];
        long long lidx[LPT];  // the pair's index in its caller's array (for errors)
        bool real[LPT];
        bool bad = false;
        const int gw = A.w;
        const uint8_t *Aref = A.ref, *Aqer = A.qer;
        const long long ref_lo = A.ref_lo, ref_hi = A.ref_hi, qer_lo = A.qer_lo, qer_hi = A.qer_hi;
        auto gerr = [&](int flag, long long k) {
            atomicOr(A.err_flags, flag);
            atomicMin(A.err_index, k);
        };
        for (int u = 0; u < LPT; u++) {
            const long long k = (long long)g * W + t + 32 * u;
            real[u] = k < A.n;
            lidx[u] = k;
            pp[u] = real[u] ? A.pairs + k : nullptr;
            if (real[u]) {
                const DevPair &p = *pp[u];
                len1[u] = p.len1; len2[u] = p.len2; h0r[u] = p.h0;
                idr[u] = p.idr; idq[u] = p.idq;
                const int lim = is16 ? 32767 : 127;
                const bool ok = len1[u] >= 0 && len2[u] >= 0 && len1[u] <= lim && len2[u] <= lim &&
                                h0r[u] >= 0 && idr[u] >= ref_lo && idr[u] + len1[u] <= ref_hi &&
                                idq[u] >= qer_lo && idq[u] + len2[u] <= qer_hi &&
                                len2[u] + 3 <= A.col_cap;
                if (!ok) {
                    gerr(ERR_DOMAIN, k);
                    bad = true;
                }
            } else {
                len1[u] = 0;
                len2[u] = is16 ? 0 : A.pairs[A.n - 1].len2;
                h0r[u] = 0;
                idr[u] = idq[u] = -1;
            }
        }
        if (__any_sync(full, bad)) continue;

        // ---- lengths as the wrapper hands them to the kernel
        int m1 = 0, m2 = 0, mq = 0x7fffffff;
        for (int u = 0; u < LPT; u++) {
            m1 = imax(m1, len1[u]);
            m2 = imax(m2, len2[u]);
            mq = imin(mq, len2[u]);
        }
        const int maxLen1 = __reduce_max_sync(full, m1);
        const int maxLen2 = __reduce_max_sync(full, m2);
        const int minq = __reduce_min_sync(full, mq) - 1;
        const int nrow = maxLen1, ncol = maxLen2, wrapRows = maxLen1;
        const int colCap = (ncol > 1 ? ncol : 1) + 3;

        // ---- per-lane set-up: query codes, the first row, band clamp
        int h0[LPT], tlen[LPT], qlen[LPT], myband[LPT];
        int bsz = gw;
        for (int u = 0; u < LPT; u++) {
            const int l = t + 32 * u;
            h0[u] = E::ws((int)E::us(h0r[u]));
            tlen[u] = E::ws((int)E::us(len1[u]));
            qlen[u] = E::ws((int)E::us(len2[u]));
            // a padding lane (8-bit) reads the query bytes at the caller's
            // offset 0, as the reference's zeroed SeqPair does; they only
            // matter where its wrapped first column is non-zero
            const uint8_t *q = real[u] ? Aqer + (idq[u] - qer_lo)
                             : (qer_lo <= 0 && len2[u] <= qer_hi) ? Aqer - qer_lo : nullptr;
            int tt = (h0[u] > oe_ins) ? E::ws(h0[u] - oe_ins) : 0;
            for (int k = 0; k < colCap; k++) {
                int code = 0;
                if (k < len2[u]) {
                    const int b = q ? q[k] : 4;
                    if (b > 4 && real[u]) {
                        gerr(ERR_BASE, lidx[u]);
                        bad = true;
                    }
                    code = b == 4 ? -1 : E::ws(b);
                } else if (k <= maxLen2) {
                    code = 100;  // DUMMY2 (:46)
                }
                Q2[(((size_t)(k >> 2) * W + l) << 2) + (k & 3)] = (int8_t)code;
                int hv = 0;
                if (k == 0) hv = h0[u];
                else if (k == 1) hv = tt;
                else if (k < maxLen2) { tt = E::ws(tt - e_ins); tt = tt > 0 ? tt : 0; hv = tt; }
                HF[(size_t)k * W + l] = (uint16_t)hv;
            }
            // band clamp (:2882-2904 / :2183-2205): integer division, then +1.0
            const int qlenb = E::ws(len2[u] * maxsc);
            const int eb_ins = E::ws(P.end_bonus - P.o_ins), eb_del = E::ws(P.end_bonus - P.o_del);
            int temp = (int)E::us(qlenb + eb_ins);
            int mi = temp / P.e_ins + 1;
            mi = mi > 1 ? mi : 1;
            myband[u] = E::ws((int)E::us(gw > mi ? mi : gw));
            temp = (int)E::us(qlenb + eb_del);
            mi = temp / P.e_del + 1;
            mi = mi > 1 ? mi : 1;
            const int mb = (int)E::us(myband[u]);
            myband[u] = E::ws((int)E::us(mb > mi ? mi : mb));
            bsz = imax(bsz, (int)E::us(myband[u]));
        }
        if (__any_sync(full, bad)) continue;
        const int w = __reduce_max_sync(full, bsz);
        __syncwarp();

        // ---- the kernel proper (:2962-3356 / :2263-2661)
        int head[LPT], tail[LPT], mlen[LPT], maxScore[LPT], x[LPT], y[LPT], gscore[LPT];
        int max_off[LPT], exit0[LPT], max_ie[LPT];
        for (int u = 0; u < LPT; u++) {
            tail[u] = qlen[u];
            head[u] = 0;
            const unsigned ml = E::us(qlen[u] + myband[u]);
            mlen[u] = E::ws((int)umin(ml, E::us(tlen[u])));
            maxScore[u] = h0[u];
            x[u] = y[u] = 0;
            gscore[u] = -1;
            max_off[u] = 0;
            exit0[u] = -1;
            max_ie[u] = 0;
        }
        auto HFa = [&](int c, int u) -> uint32_t & { return HF[(size_t)c * W + t + 32 * u]; };
        auto pack = [](int h, int f) -> uint32_t { return (uint32_t)(uint16_t)h | ((uint32_t)(uint16_t)f << 16); };
        // first column H_v[k]: h0 at k = 0, max(h0 - o_del - k e_del, 0) below
        // (wrapping), DUMMY1 at the wrapper's last row
        auto Hv = [&](int k, int u) -> int {
            if (k == 0) return h0[u];
            if (k < wrapRows) {
                const int v = E::ws(h0[u] - o_del - k * e_del);
                return v > 0 ? v : 0;
            }
            return 99;  // DUMMY1 (:45)
        };
        unsigned long long ncells = 0;
        int tnext[LPT];  // the next row's target base
        for (int u = 0; u < LPT; u++) tnext[u] = len1[u] > 0 ? Aref[idr[u] - ref_lo] : 0;
        int beg = 0, end = ncol, nbeg = 0, nend = ncol;
        for (int i = 0; i < nrow; i++) {
            const int i1 = E::ws(i + 1);
            int e11[LPT], h10[LPT], maxRS1[LPT], y1[LPT], s1[LPT];
            beg = nbeg; end = nend;
            if (beg < i - w) beg = i - w;
            if (end > i + w + 1) end = i + w + 1;
            if (end > ncol) end = ncol;
            bool changed = false;
            for (int u = 0; u < LPT; u++) {
                e11[u] = 0; maxRS1[u] = 0; y1[u] = 0;
                h10[u] = beg == 0 ? Hv(i + 1, u) : 0;
                if (i < len1[u]) {
                    const int b = tnext[u];  // loaded a row ahead
                    if (i + 1 < len1[u]) tnext[u] = Aref[idr[u] - ref_lo + i + 1];
                    s1[u] = b == 4 ? -1 : E::ws(b);
                    if (b > 4) gerr(ERR_BASE, lidx[u]);
                } else {
                    s1[u] = 99;  // DUMMY1
                }
                // per-lane band (:3080-3089)
                const int ph = head[u], pt = tail[u];
                const int c = E::ws(i - myband[u]);
                head[u] = head[u] > c ? head[u] : c;
                unsigned tu = umin(E::us(tail[u]), E::us(i1 + myband[u]));
                tu = umin(tu, E::us(qlen[u]));
                tail[u] = E::ws((int)tu);
                changed |= head[u] != ph || tail[u] != pt;
            }
            // trimming (:3091-3112)
            if (__any_sync(full, changed)) {
                for (int lc = beg; lc < end; lc++) {
                    const int pj = E::ws(lc), jn = E::ws(lc + 1);
                    bool any = false;
                    for (int u = 0; u < LPT; u++) any |= head[u] > pj;
                    if (!__any_sync(full, any)) break;
                    for (int u = 0; u < LPT; u++)
                        if (head[u] > pj || jn > tail[u]) HFa(lc, u) = 0;
                }
            }
            // row exit status (:3119-3129)
            for (int u = 0; u < LPT; u++)
                if (i1 > mlen[u] || tail[u] == head[u] || head[u] > tail[u]) exit0[u] = 0;

            // DP row (:3135-3196), four columns at a time: their (H, F) words and
            // query codes are loaded before the four cells are computed, so
            // the loads overlap
            int j512 = E::ws(beg);
            const uint32_t *Q4 = reinterpret_cast<const uint32_t *>(Q2);
            auto cell = [&](int j, int u, uint32_t hf, int a2) {
                const int pj = E::ws(j);
                const int jn = E::ws(j + 1);
                const int h00 = (int16_t)(hf & 0xffffu), f11 = (int16_t)(hf >> 16);
                int sbt = s1[u] == a2 ? w_match : w_mismatch;
                // the larger code's top bit (as unsigned): an N on either side;
                // codes are held sign-extended, so that is either being negative
                if ((s1[u] | a2) < 0) sbt = -1;
                int m11 = E::ws(h00 + sbt);
                if (h00 == 0) m11 = 0;
                const int h11 = __vimax3_s32(m11, e11[u], f11);
                // E and F are >= 0 throughout: E - e_ins, F - e_del cannot wrap
                e11[u] = __vimax3_s32(E::ws(m11 - oe_ins), 0, e11[u] - e_ins);
                int f21 = __vimax3_s32(E::ws(m11 - oe_del), 0, f11 - e_del);
                const bool cmp2 = head[u] > pj;
                const bool mask = pj > tail[u] || cmp2;
                const int hst = mask ? 0 : h10[u];
                if (mask) f21 = 0;
                const int bmax = maxRS1[u];
                const int nm = maxRS1[u] > h11 ? maxRS1[u] : h11;
                const bool cmpA = nm > bmax || nm == h11;
                if (!(jn > tail[u] || cmp2)) {
                    if (cmpA) y1[u] = jn;
                    maxRS1[u] = nm;
                }
                HFa(j, u) = pack(hst, f21);
                h10[u] = h11;
                // end-to-end score (:3178-3195): the blends there change gscore
                // and max_ie only in the query's last column (j + 1 == qlen,
                // which implies j >= minq), in a live lane, left of the tail,
                // and only where h11 is not below the current gscore
                if (j >= minq && jn == qlen[u] && exit0[u] < 0 && !(jn > tail[u]) && !(gscore[u] > h11)) {
                    gscore[u] = h11;
                    max_ie[u] = i1;
                }
            };
            // four columns per block (eight measured 147 against 150 GCUPS on C2:
            // more registers, fewer resident warps); the next block's words
            // are loaded before this block is computed (blocks never share a
            // column, so the loads see this row's inputs)
            constexpr int CB = 4;
            uint32_t hfb[LPT][CB], qc[LPT];
            auto load_block = [&](int jb, uint32_t (&hv)[LPT][CB], uint32_t (&qv)[LPT]) {
                const int nb = end - jb < CB ? end - jb : CB;
#pragma unroll
                for (int u = 0; u < LPT; u++) {
#pragma unroll
                    for (int k = 0; k < CB; k++) hv[u][k] = k < nb ? HFa(jb + k, u) : 0u;
                    const size_t qi = (size_t)(jb >> 2) * W + t + 32 * u;
                    const uint64_t q2 = (uint64_t)Q4[qi] | ((uint64_t)Q4[qi + W] << 32);
                    qv[u] = (uint32_t)(q2 >> ((jb & 3) * 8));
                }
            };
            if (beg < end) load_block(beg, hfb, qc);
            for (int jb = beg; jb < end; jb += CB) {
                const int nb = end - jb < CB ? end - jb : CB;
                uint32_t hfn[LPT][CB] = {}, qn[LPT] = {};
                if (jb + CB < end) load_block(jb + CB, hfn, qn);
#pragma unroll
                for (int k = 0; k < CB; k++) {
                    if (k < nb) {
#pragma unroll
                        for (int u = 0; u < LPT; u++) cell(jb + k, u, hfb[u][k], (int8_t)(qc[u] >> (8 * k)));
                    }
                }
#pragma unroll
                for (int u = 0; u < LPT; u++) {
                    qc[u] = qn[u];
#pragma unroll
                    for (int k = 0; k < CB; k++) hfb[u][k] = hfn[u][k];
                }
            }
            const int j = beg > end ? beg : end;
            j512 = E::ws(j);
            if (end > beg) ncells += (unsigned long long)(end - beg);
            // the row's last column (:3197-3203); j == max(beg, end) here
            if (j < colCap) {
                for (int u = 0; u < LPT; u++) {
                    const bool m = head[u] > j512 || j512 > tail[u];
                    HFa(j, u) = pack(m ? 0 : h10[u], 0);
                }
            }
            // a zero row in every lane ends the group (:3206-3209)
            bool nz = false;
            for (int u = 0; u < LPT; u++) nz |= maxRS1[u] != 0;
            if (!__any_sync(full, nz)) break;
            for (int u = 0; u < LPT; u++) {
                if (maxRS1[u] == 0) exit0[u] = 0;
                const int bms = maxScore[u];
                const int sc2 = maxScore[u] > maxRS1[u] ? maxScore[u] : maxRS1[u];
                if (exit0[u] < 0) maxScore[u] = sc2;
                if (maxScore[u] > bms) {
                    y[u] = y1[u];
                    x[u] = i1;
                    int ind = E::ws(y1[u] - i1);
                    ind = ind < 0 ? E::ws(-ind) : ind;  // abs (wrapping)
                    max_off[u] = max_off[u] > ind ? max_off[u] : ind;
                }
                // ZSCORE16 / ZSCORE8 (:1868-1881 / :1826-1839)
                const int tmpi = E::ws(i1 - x[u]), tmpj = E::ws(y1[u] - y[u]);
                const int score = E::ws(maxScore[u] - maxRS1[u]);
                const int d = tmpi > tmpj ? E::ws(tmpi - tmpj) : E::ws(tmpj - tmpi);
                if (E::ws(score - d) > zdropv) exit0[u] = 0;
            }
            // band narrowing (:3235-3260): columns zero in every lane
            auto all_zero = [&](int c) {
                bool z = true;
                for (int u = 0; u < LPT; u++) z &= HFa(c, u) == 0;
                return __all_sync(full, z) != 0;
            };
            int lc;
            for (lc = beg; lc < end; lc++) {
                if (all_zero(lc)) nbeg = lc;
                else break;
            }
            for (lc = end; lc >= beg; lc--)
                if (!all_zero(lc)) break;
            nend = lc + 2 < ncol ? lc + 2 : ncol;
            if (is16) { beg = nbeg; end = nend; }
            // per-lane head / tail (:3265-3316 / :2571-2621)
            {
                bool run[LPT];
                auto zero_at = [&](int c, int u) {
                    return exit0[u] != 0 && HFa(c, u) == 0;
                };
                for (int u = 0; u < LPT; u++) run[u] = true;
                int l512 = E::ws(beg);
                for (lc = beg; lc < end; lc++) {
                    bool zl[LPT], any = false;
                    for (int u = 0; u < LPT; u++) { zl[u] = zero_at(lc, u); any |= zl[u]; }
                    if (!__any_sync(full, any)) break;
                    l512 = E::ws(l512 + 1);
                    for (int u = 0; u < LPT; u++) {
                        run[u] = zl[u] && run[u];
                        if (run[u]) head[u] = l512;
                    }
                }
                int index[LPT];
                for (int u = 0; u < LPT; u++) { index[u] = tail[u]; run[u] = true; }
                l512 = E::ws(end);
                for (lc = end; lc >= beg; lc--) {
                    bool zl[LPT], any = false;
                    for (int u = 0; u < LPT; u++) { zl[u] = zero_at(lc, u); any |= zl[u]; }
                    if (!__any_sync(full, any)) break;
                    l512 = E::ws(l512 - 1);
                    for (int u = 0; u < LPT; u++) {
                        run[u] = zl[u] && run[u];
                        if (run[u]) index[u] = l512;
                    }
                }
                for (int u = 0; u < LPT; u++) {
                    const int ix = E::ws(index[u] + 2);
                    tail[u] = ix < qlen[u] ? ix : qlen[u];
                }
            }
            __syncwarp();
        }
        for (int u = 0; u < LPT; u++) {
            if (!real[u]) continue;
            DevPair &p = *pp[u];
            p.score = maxScore[u];
            p.tle = x[u];
            p.qle = y[u];
            p.max_off = max_off[u];
            p.gscore = gscore[u];
            p.gtle = max_ie[u];
        }
        if (A.cells) {
            int nr = 0;
            for (int u = 0; u < LPT; u++) nr += real[u];
            const int nreal = __reduce_add_sync(full, nr);
            if (t == 0) atomicAdd(A.cells, ncells * (unsigned long long)nreal);
        }
        __syncwarp();
    }
}

}  // namespace talbsw
