// Seeded synthetic seed-extension pairs for the benchmark and the tests.
//
// The reference's driver reads pairs from a text file (benchmarks/bench-bsw.cpp
// :117-169: an h0 line, a reference line, a query line, bases '0'..'4').  No
// such file ships with the reference, so the workloads are generated here:
// a random query (bases 0-3, N = 4 at a given rate), a reference derived from
// it by substitutions / insertions / deletions and then padded or truncated
// to len1 = len2 + U[extra_lo, extra_hi], and h0 / band drawn per pair.
//
// Every pair has its own random stream (seed, pair index), so any slice of a
// workload can be generated independently and in parallel, and the same slice
// always holds the same pairs on any machine (lognormal lengths go through
// libm's exp/log/cos, the only place results could differ in the last ulp).
#include <stdint.h>
#include <string.h>
#include <math.h>
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "synth.h"

namespace {

inline uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// xoshiro256** (Blackman & Vigna), one instance per pair and purpose.
struct Rng {
    uint64_t s[4];
    Rng(uint64_t seed, uint64_t index, uint64_t stream) {
        uint64_t x = seed ^ (index * 0xD1B54A32D192ED03ull) ^ (stream * 0x8CB92BA72F3D8DD7ull);
        for (int i = 0; i < 4; i++) s[i] = splitmix64(x);
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    inline uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    inline double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // integer in [lo, hi]
    inline int32_t range(int32_t lo, int32_t hi) {
        if (hi <= lo) return lo;
        uint64_t span = (uint64_t)((int64_t)hi - lo + 1);
        return (int32_t)(lo + (int64_t)(next() % span));
    }
    inline double normal() {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    }
};

enum { STREAM_PLAN = 1, STREAM_QUERY = 2, STREAM_MUTATE = 3 };

void plan_one(const tal_synth_cfg *c, int64_t k, int32_t *len1, int32_t *len2,
              int32_t *h0, int32_t *w) {
    Rng r(c->seed, (uint64_t)k, STREAM_PLAN);
    int32_t l2;
    if (c->len_dist == TAL_SYNTH_LEN_FIXED) {
        l2 = c->len_lo;
    } else if (c->len_dist == TAL_SYNTH_LEN_UNIFORM) {
        l2 = r.range(c->len_lo, c->len_hi);
    } else {
        double v = exp(log(c->len_median) + c->len_sigma * r.normal());
        long lv = lround(v);
        if (lv < c->len_lo) lv = c->len_lo;
        if (lv > c->len_hi) lv = c->len_hi;
        l2 = (int32_t)lv;
    }
    int32_t l1 = l2 + r.range(c->extra_lo, c->extra_hi);
    if (l1 < 0) l1 = 0;
    int32_t hh = r.range(c->h0_lo, c->h0_hi);
    if (c->h0_cap_8bit) {
        int32_t cap = 127 - c->match * std::min(l1, l2);
        if (hh > cap) hh = cap;
        if (hh < 0) hh = 0;
    }
    int32_t ww = c->w_default;
    if (c->n_w_choices > 0) ww = c->w_choices[r.range(0, c->n_w_choices - 1)];
    if (len1) *len1 = l1;
    if (len2) *len2 = l2;
    if (h0) *h0 = hh;
    if (w) *w = ww;
}

void fill_one(const tal_synth_cfg *c, int64_t k, int32_t l1, int32_t l2,
              uint8_t *ref, uint8_t *qer, std::vector<double> &wt) {
    Rng rq(c->seed, (uint64_t)k, STREAM_QUERY);
    for (int32_t j = 0; j < l2; j++) {
        uint8_t b = (uint8_t)(rq.next() >> 62);
        if (c->n_rate > 0 && rq.uniform() < c->n_rate) b = 4;
        qer[j] = b;
    }
    Rng rm(c->seed, (uint64_t)k, STREAM_MUTATE);
    double err = c->err_lo + (c->err_hi - c->err_lo) * rm.uniform();
    double p_sub = err * c->sub_frac, p_ins = err * c->ins_frac, p_del = err * c->del_frac;
    // deletions weighted toward homopolymer runs, keeping the mean rate
    wt.assign((size_t)std::max(l2, 1), 1.0);
    double norm = 1.0;
    if (c->homopolymer_del_bias > 1.0 && l2 > 0) {
        double s = 0;
        for (int32_t j = 0; j < l2; j++) {
            bool hp = (j > 0 && qer[j] == qer[j - 1]) || (j + 1 < l2 && qer[j] == qer[j + 1]);
            wt[j] = hp ? c->homopolymer_del_bias : 1.0;
            s += wt[j];
        }
        norm = s / l2;
    }
    int32_t o = 0;
    for (int32_t j = 0; j < l2 && o < l1; j++) {
        double u = rm.uniform();
        uint8_t b = qer[j];
        if (u < p_sub) {
            uint8_t nb = (uint8_t)(rm.next() >> 62);
            if (b < 4 && nb == b) nb = (uint8_t)((nb + 1 + (rm.next() >> 63)) & 3);
            ref[o++] = nb;
        } else if (u < p_sub + p_ins) {
            ref[o++] = b;
            int32_t L = rm.range(c->indel_lo, c->indel_hi);
            for (int32_t t = 0; t < L && o < l1; t++) ref[o++] = (uint8_t)(rm.next() >> 62);
        } else if (u < p_sub + p_ins + p_del * wt[j] / norm) {
            int32_t L = rm.range(c->indel_lo, c->indel_hi);
            j += L - 1;
        } else {
            ref[o++] = b;
        }
    }
    while (o < l1) ref[o++] = (uint8_t)(rm.next() >> 62);
}

template <typename F>
void parallel_for(int64_t n, int nthreads, F fn) {
    if (nthreads <= 1 || n < 4096) { fn(0, n); return; }
    std::atomic<int64_t> next(0);
    const int64_t chunk = 4096;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&]() {
            for (;;) {
                int64_t s = next.fetch_add(chunk);
                if (s >= n) break;
                fn(s, std::min(n, s + chunk));
            }
        });
    for (auto &t : th) t.join();
}

int hw_threads(int req) {
    if (req > 0) return req;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

}  // namespace

extern "C" {

int tal_synth_plan(const tal_synth_cfg *cfg, int64_t first, int64_t count,
                   int32_t *len1, int32_t *len2, int32_t *h0, int32_t *w,
                   int nthreads) {
    if (!cfg || count < 0) return -1;
    parallel_for(count, hw_threads(nthreads), [&](int64_t s, int64_t e) {
        for (int64_t i = s; i < e; i++)
            plan_one(cfg, first + i, len1 ? len1 + i : nullptr, len2 ? len2 + i : nullptr,
                     h0 ? h0 + i : nullptr, w ? w + i : nullptr);
    });
    return 0;
}

int tal_synth_fill(const tal_synth_cfg *cfg, int64_t first, int64_t count,
                   const int32_t *len1, const int32_t *len2,
                   const int64_t *ref_off, const int64_t *qer_off,
                   uint8_t *ref, uint8_t *qer, int nthreads) {
    if (!cfg || count < 0 || !len1 || !len2 || !ref_off || !qer_off || !ref || !qer) return -1;
    parallel_for(count, hw_threads(nthreads), [&](int64_t s, int64_t e) {
        std::vector<double> wt;
        for (int64_t i = s; i < e; i++)
            fill_one(cfg, first + i, len1[i], len2[i], ref + ref_off[i], qer + qer_off[i], wt);
    });
    return 0;
}

}  // extern "C"
