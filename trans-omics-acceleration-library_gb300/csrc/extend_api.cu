// Caller-side seed extension (include/tal_extend.h): windows and SeqPair
// batches built on the host, the reversed / forward sequence pieces gathered
// on the device, the left batch, the right batch (its h0 set on the device
// from the left results), the regions resolved on the device.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <string>
#include <vector>

#include "../../include/tal_extend.h"
#include "bsw_ctx.h"

static_assert(sizeof(tal_seed) == 24, "tal_seed is 24 bytes");
static_assert(sizeof(tal_region) == 32, "tal_region is 32 bytes");

namespace {

// One sequence piece to place in an arena: src bytes [src, src + len) of the
// reference (or of the reads), reversed or not, to arena offset dst.
struct CopyJob {
    long long src;
    int len;
    int dst;
    int flags;  // bit 0: reverse; bit 1: from the reads, into the query arena
    int pad;
};

// Per seed: its left and right pairs (-1: none) and what the regions need.
struct XSeed {
    long long rbeg;
    int left, right;
    int qbeg, len, L, pad;
};

__global__ void gather_kernel(const CopyJob *jobs, int n, const uint8_t *ref, const uint8_t *reads,
                              uint8_t *tarena, uint8_t *qarena) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += warps) {
        const CopyJob c = jobs[j];
        const uint8_t *src = (c.flags & 2) ? reads : ref;
        uint8_t *dst = ((c.flags & 2) ? qarena : tarena) + c.dst;
        const bool rev = c.flags & 1;
        for (int k = lane; k < c.len; k += 32) dst[k] = src[rev ? c.src + c.len - 1 - k : c.src + k];
    }
}

// The left extension's outcome for seed x: read start qb, reference start rb
// and score sc after the clipping choice.
__device__ __forceinline__ void left_outcome(const XSeed &x, const talbsw::DevPair *lp, int a,
                                             int clip5, int &qb, long long &rb, int &sc) {
    if (x.left < 0) {
        qb = x.qbeg;
        rb = x.rbeg;
        sc = x.len * a;
        return;
    }
    const talbsw::DevPair &p = lp[x.left];
    if (p.gscore <= 0 || p.gscore <= p.score - clip5) {
        qb = x.qbeg - p.qle;
        rb = x.rbeg - p.tle;
        sc = p.score;
    } else {
        qb = 0;
        rb = x.rbeg - p.gtle;
        sc = p.gscore;
    }
}

__global__ void right_h0_kernel(const XSeed *xs, int n, const talbsw::DevPair *lp, talbsw::DevPair *rp,
                                int a, int clip5) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const XSeed x = xs[s];
        if (x.right < 0) continue;
        int qb, sc;
        long long rb;
        left_outcome(x, lp, a, clip5, qb, rb, sc);
        rp[x.right].h0 = sc;
    }
}

__global__ void finalize_kernel(const XSeed *xs, int n, const talbsw::DevPair *lp,
                                const talbsw::DevPair *rp, int a, int clip5, int clip3,
                                tal_region *out) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const XSeed x = xs[s];
        tal_region g;
        int qb, sc;
        long long rb;
        left_outcome(x, lp, a, clip5, qb, rb, sc);
        g.qb = qb;
        g.rb = rb;
        g.left_score = sc;
        const int qe0 = x.qbeg + x.len;
        const long long re0 = x.rbeg + x.len;
        if (x.right < 0) {
            g.qe = qe0;
            g.re = re0;
        } else {
            const talbsw::DevPair &p = rp[x.right];
            if (p.gscore <= 0 || p.gscore <= p.score - clip3) {
                g.qe = qe0 + p.qle;
                g.re = re0 + p.tle;
                sc = p.score;
            } else {
                g.qe = x.L;
                g.re = re0 + p.gtle;
                sc = p.gscore;
            }
        }
        g.score = sc;
        out[s] = g;
    }
}

int xfail(tal_bsw_ctx *h, int code, const std::string &msg) {
    h->last_error = msg;
    return code;
}

// clamp(max((n*a - o_del) / e_del + 1, (n*a - o_ins) / e_ins + 1), 1, 2w)
long long max_gap(const tal_bsw_params &p, long long n, int w) {
    const long long d = (n * p.w_match - p.o_del) / p.e_del + 1;
    const long long i = (n * p.w_match - p.o_ins) / p.e_ins + 1;
    long long l = std::max(d, i);
    l = std::max(l, 1LL);
    return std::min(l, 2LL * w);
}

}  // namespace

extern "C" int tal_bsw_extend_seeds(tal_bsw_handle h, const uint8_t *ref, int64_t ref_len,
                                    const uint8_t *reads, const int64_t *read_off, int32_t n_reads,
                                    const tal_seed *seeds, int32_t n_seeds,
                                    const tal_extend_params *xp, tal_region *out) {
    if (!h) return TAL_EINVAL;
    h->last_error.clear();
    h->last_bad = -1;
    if (!xp || n_reads < 0 || n_seeds < 0 || ref_len < 0 || xp->w < 0 || xp->band_tries < 0 ||
        xp->band_tries > 8 || ((long long)xp->w << std::max(0, xp->band_tries - 1)) > (1LL << 24))
        return xfail(h, TAL_EINVAL, "bad counts or parameters");
    if (n_seeds == 0) return TAL_OK;
    if (!ref || !reads || !read_off || !seeds || !out) return xfail(h, TAL_EINVAL, "NULL buffer");
    const tal_bsw_params &P = h->prm;
    const int a = P.w_match;
    const long long reads_len = read_off[n_reads];
    // windows, copy jobs and SeqPairs (targets in one arena, queries in another)
    std::vector<CopyJob> jobs;
    std::vector<tal_seq_pair> lp, rp;
    std::vector<XSeed> xs((size_t)n_seeds);
    jobs.reserve(4 * (size_t)n_seeds);
    long long tpos = 0, qpos = 0;
    auto piece = [&](long long src, long long len, bool rev, bool from_reads) -> int {
        long long &pos = from_reads ? qpos : tpos;
        const int at = (int)pos;
        jobs.push_back({src, (int)len, at, (rev ? 1 : 0) | (from_reads ? 2 : 0), 0});
        pos += len;
        return at;
    };
    for (int32_t s = 0; s < n_seeds; s++) {
        const tal_seed &sd = seeds[s];
        if (sd.read < 0 || sd.read >= n_reads) {
            h->last_bad = s;
            return xfail(h, TAL_EDOMAIN, "seed " + std::to_string(s) + ": read index out of range");
        }
        const long long r0 = read_off[sd.read], L = read_off[sd.read + 1] - r0;
        if (r0 < 0 || L < 0 || r0 + L > reads_len || L > INT_MAX || sd.qbeg < 0 || sd.len < 0 ||
            sd.qbeg + (long long)sd.len > L || sd.rbeg < 0 || sd.rbeg + sd.len > ref_len) {
            h->last_bad = s;
            return xfail(h, TAL_EDOMAIN, "seed " + std::to_string(s) + " outside its read or the reference");
        }
        XSeed &x = xs[s];
        x.rbeg = sd.rbeg;
        x.qbeg = sd.qbeg;
        x.len = sd.len;
        x.L = (int)L;
        x.pad = 0;
        x.left = x.right = -1;
        if (sd.qbeg > 0) {
            const long long rs = std::max(0LL, sd.rbeg - sd.qbeg - max_gap(P, sd.qbeg, xp->w));
            tal_seq_pair p;
            memset(&p, 0, sizeof(p));
            p.len1 = (int)(sd.rbeg - rs);
            p.len2 = sd.qbeg;
            p.idr = piece(rs, p.len1, true, false);
            p.idq = piece(r0, p.len2, true, true);
            p.id = s;
            p.h0 = sd.len * a;
            p.score = p.tle = p.gtle = p.qle = p.gscore = p.max_off = -1;
            x.left = (int)lp.size();
            lp.push_back(p);
        }
        const long long qe0 = sd.qbeg + (long long)sd.len, re0 = sd.rbeg + sd.len;
        if (qe0 < L) {
            const long long ql = L - qe0;
            const long long re = std::min<long long>(ref_len, re0 + ql + max_gap(P, ql, xp->w));
            tal_seq_pair p;
            memset(&p, 0, sizeof(p));
            p.len1 = (int)(re - re0);
            p.len2 = (int)ql;
            p.idr = piece(re0, p.len1, false, false);
            p.idq = piece(r0 + qe0, p.len2, false, true);
            p.id = s;
            p.h0 = 0;  // set on the device from the left result
            p.score = p.tle = p.gtle = p.qle = p.gscore = p.max_off = -1;
            x.right = (int)rp.size();
            rp.push_back(p);
        }
        if (tpos > INT_MAX || qpos > INT_MAX)
            return xfail(h, TAL_EDOMAIN, "a call's extension windows exceed 2^31 bytes");
    }
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return xfail(h, TAL_ECUDA, "cudaSetDevice");
    const size_t pb = sizeof(tal_seq_pair);
    if ((e = h->xref.ensure((size_t)ref_len + 16)) != cudaSuccess ||
        (e = h->xreads.ensure((size_t)reads_len + 16)) != cudaSuccess ||
        (e = h->xjobs.ensure(sizeof(CopyJob) * jobs.size() + sizeof(XSeed) * xs.size())) != cudaSuccess ||
        (e = h->xpairs.ensure(pb * (lp.size() + rp.size()) + 16)) != cudaSuccess ||
        (e = h->xtarena.ensure((size_t)tpos + 16)) != cudaSuccess ||
        (e = h->xqarena.ensure((size_t)qpos + 16)) != cudaSuccess ||
        (e = h->xout.ensure(sizeof(tal_region) * (size_t)n_seeds)) != cudaSuccess)
        return xfail(h, TAL_ENOMEM, std::string("extension buffers: ") + cudaGetErrorString(e));
    CopyJob *d_jobs = reinterpret_cast<CopyJob *>(h->xjobs.p);
    XSeed *d_xs = reinterpret_cast<XSeed *>(d_jobs + jobs.size());
    tal_seq_pair *d_lp = reinterpret_cast<tal_seq_pair *>(h->xpairs.p);
    tal_seq_pair *d_rp = d_lp + lp.size();
    uint8_t *d_t = reinterpret_cast<uint8_t *>(h->xtarena.p);
    uint8_t *d_q = reinterpret_cast<uint8_t *>(h->xqarena.p);
    tal_region *d_out = reinterpret_cast<tal_region *>(h->xout.p);
    cudaStream_t s = h->stream;
    e = cudaMemcpyAsync(h->xref.p, ref, (size_t)ref_len, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->xreads.p, reads, (size_t)reads_len, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(CopyJob) * jobs.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_xs, xs.data(), sizeof(XSeed) * xs.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !lp.empty()) e = cudaMemcpyAsync(d_lp, lp.data(), pb * lp.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !rp.empty()) e = cudaMemcpyAsync(d_rp, rp.data(), pb * rp.size(), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return xfail(h, TAL_ECUDA, std::string("H2D: ") + cudaGetErrorString(e));
    const int nj = (int)jobs.size();
    if (nj > 0) {
        const int blocks = (int)std::min<long long>(((long long)nj + 7) / 8, 16LL * h->num_sms);
        gather_kernel<<<blocks, 256, 0, s>>>(d_jobs, nj, reinterpret_cast<const uint8_t *>(h->xref.p),
                                             reinterpret_cast<const uint8_t *>(h->xreads.p), d_t, d_q);
        h->launches++;
    }
    const int gb = (int)std::min<long long>(((long long)n_seeds + 255) / 256, 8LL * h->num_sms);
    const int tries = std::max(1, xp->band_tries);
    // One extension batch on the device (its pairs at d_p, host copy hp for
    // the seed ids), with the band retries: pairs whose attempt wants another
    // go again, as a sub-batch, with the doubled band.
    auto run_batch = [&](tal_seq_pair *d_p, std::vector<tal_seq_pair> &hp) -> int {
        const int32_t n = (int32_t)hp.size();
        int rc = tal_bsw_scores_device(h, d_p, d_t, (size_t)tpos + 16, d_q, (size_t)qpos + 16, n, xp->w,
                                       nullptr, TAL_BSW_AUTO);
        if (rc == TAL_OK) rc = tal_bsw_sync(h);
        if (rc != TAL_OK) {
            if (h->last_bad >= 0) h->last_bad = hp[(size_t)h->last_bad].id;
            return rc;
        }
        if (tries <= 1) return TAL_OK;
        cudaError_t e2 = cudaMemcpyAsync(hp.data(), d_p, pb * n, cudaMemcpyDeviceToHost, s);
        if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(s);
        if (e2 != cudaSuccess) return xfail(h, TAL_ECUDA, cudaGetErrorString(e2));
        // prev: the score before the pair's last attempt; idx: the pairs still
        // retrying (all of them before the first check)
        std::vector<int32_t> prev((size_t)n, -1), idx((size_t)n), cur;
        for (int32_t k = 0; k < n; k++) idx[k] = k;
        std::vector<tal_seq_pair> sub;
        for (int i = 1; i < tries; i++) {
            const int wprev = xp->w << (i - 1);
            cur.clear();
            sub.clear();
            for (int32_t k : idx) {
                const tal_seq_pair &p = hp[k];
                if (p.score != prev[k] && p.max_off >= (wprev >> 1) + (wprev >> 2)) {
                    cur.push_back(k);
                    prev[k] = p.score;
                    tal_seq_pair q = p;
                    q.score = q.tle = q.gtle = q.qle = q.gscore = q.max_off = -1;
                    sub.push_back(q);
                }
            }
            idx.swap(cur);
            if (idx.empty()) break;
            if (h->xretry.ensure(pb * sub.size()) != cudaSuccess)
                return xfail(h, TAL_ENOMEM, "band retry buffer");
            tal_seq_pair *d_r = reinterpret_cast<tal_seq_pair *>(h->xretry.p);
            e2 = cudaMemcpyAsync(d_r, sub.data(), pb * sub.size(), cudaMemcpyHostToDevice, s);
            if (e2 != cudaSuccess) return xfail(h, TAL_ECUDA, cudaGetErrorString(e2));
            rc = tal_bsw_scores_device(h, d_r, d_t, (size_t)tpos + 16, d_q, (size_t)qpos + 16,
                                       (int32_t)sub.size(), xp->w << i, nullptr, TAL_BSW_AUTO);
            if (rc == TAL_OK) rc = tal_bsw_sync(h);
            if (rc != TAL_OK) {
                if (h->last_bad >= 0) h->last_bad = sub[(size_t)h->last_bad].id;
                return rc;
            }
            e2 = cudaMemcpyAsync(sub.data(), d_r, pb * sub.size(), cudaMemcpyDeviceToHost, s);
            if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(s);
            if (e2 != cudaSuccess) return xfail(h, TAL_ECUDA, cudaGetErrorString(e2));
            for (size_t m = 0; m < idx.size(); m++) hp[idx[m]] = sub[m];
        }
        e2 = cudaMemcpyAsync(d_p, hp.data(), pb * n, cudaMemcpyHostToDevice, s);
        if (e2 != cudaSuccess) return xfail(h, TAL_ECUDA, cudaGetErrorString(e2));
        return TAL_OK;
    };
    int rc;
    // left batch, then the right batch's h0 from its results, then the right batch
    if (!lp.empty() && (rc = run_batch(d_lp, lp)) != TAL_OK) return rc;
    if (!rp.empty()) {
        right_h0_kernel<<<gb, 256, 0, s>>>(d_xs, n_seeds, reinterpret_cast<const talbsw::DevPair *>(d_lp),
                                           reinterpret_cast<talbsw::DevPair *>(d_rp), a, xp->pen_clip5);
        h->launches++;
        if ((rc = run_batch(d_rp, rp)) != TAL_OK) return rc;
    }
    finalize_kernel<<<gb, 256, 0, s>>>(d_xs, n_seeds, reinterpret_cast<const talbsw::DevPair *>(d_lp),
                                       reinterpret_cast<const talbsw::DevPair *>(d_rp), a, xp->pen_clip5,
                                       xp->pen_clip3, d_out);
    h->launches++;
    e = cudaMemcpyAsync(out, d_out, sizeof(tal_region) * (size_t)n_seeds, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return xfail(h, TAL_ECUDA, cudaGetErrorString(e));
    return TAL_OK;
}
