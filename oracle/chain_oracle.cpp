// ORACLE -- test infrastructure only.  CPU restatement of the reference's
// dynamic-programming anchor chaining, dp_chain::mm_dp_vectorized
// (src/chaining/parallel_chaining_32_bit.h:216-436, the AVX-512 build that
// benchmarks/bench-dp-chaining.cpp drives), one anchor at a time.  Used by
// tests/ and bench.py's CPU leg to check the CUDA kernel; the product library
// never links it.  Pinned against the reference compiled from its own header
// (oracle/ref_chain_shim.cpp) and against golden fixtures made from it.
//
// Per read of n anchors (sorted by r as the reference expects), for each
// anchor i in order:
//   st: the first predecessor with r_i - r_st <= dr (64-bit, unsigned), moved
//       up to i - max_iter when more than max_iter predecessors remain (:231-235)
//   every j in [st, i) with, in 32-bit arithmetic on the low words of r,
//       ddr = r_i - r_j, ddq = q_i - q_j, dd = |ddr - ddq|,
//       not (dd > bw or ddr == 0 or ddq <= 0 or ddq > dq or ddq > dr)
//   scores f_j + min(ddr, ddq, l_i) - gap(dd)
//   f_i = the largest score, at least l_i; p_i = the largest j scoring f_i
//       when f_i > l_i, else -1 (the AVX-512 lane merge :377-388 and the
//       scalar loop :395-428 both pick it); v_i = max(v_{p_i}, f_i) (:432)
// gap(dd) = floor(dd * 0.01 * avg_l) + (floor(log2 dd) >> 1), avg_l = (float)
// (sum of l) / n.  Two roundings exist in the reference, by path:
//   more than six predecessors (:247, the vector loop, :129-150): float
//       product (float)dd * (float)(0.01 * avg_l), rounded down
//   at most six (the scalar loop, :414-415): double product
//       ((double)dd * 0.01) * avg_l, truncated
// Out-of-range conversions give INT_MIN, as the x86 conversions do.
#include <stdint.h>
#include <string.h>

#include <climits>
#include <cmath>
#include <thread>
#include <vector>

namespace {

struct Anchor {  // anchor_t (parallel_chaining_32_bit.h:58-67)
    uint64_t r;
    int32_t q;
    int32_t l;
};

// floor(log2 v) of a nonzero 32-bit value
int floor_log2(uint32_t v) {
    int k = 0;
    while (v >>= 1) k++;
    return k;
}

int32_t to_i32_floor(float x) {  // cvt with round-down; out of range -> INT_MIN
    const double d = std::floor((double)x);
    if (!(d >= -2147483648.0 && d < 2147483648.0)) return INT_MIN;
    return (int32_t)d;
}

int32_t to_i32_trunc(double x) {  // truncating conversion; out of range -> INT_MIN
    const double d = std::trunc(x);
    if (!(d >= -2147483648.0 && d < 2147483648.0)) return INT_MIN;
    return (int32_t)d;
}

int32_t wrap_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
int32_t wrap_sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

// |x| with the two's-complement wrap of the SIMD abs (INT_MIN stays INT_MIN)
int32_t wrap_abs(int32_t x) { return x < 0 ? (int32_t)(0u - (uint32_t)x) : x; }

int32_t gap_float(int32_t dd, float aq) {
    volatile float prod = (float)dd * aq;  // one rounding, no contraction
    const int32_t lg = dd != 0 ? (floor_log2((uint32_t)dd) >> 1) : 0;
    return wrap_add(to_i32_floor(prod), lg);
}

int32_t gap_double(int32_t dd, double avg) {
    volatile double a = (double)dd * 0.01;
    volatile double prod = a * avg;
    const int32_t lg = dd != 0 ? (floor_log2((uint32_t)dd) >> 1) : 0;
    return wrap_add(to_i32_trunc(prod), lg);
}

void chain_read(const Anchor *a, int64_t n, int32_t bw, int32_t max_iter, int32_t dr, int32_t dq,
                uint32_t *f, int32_t *p, int32_t *v) {
    if (n <= 0) return;
    uint64_t sum = 0;
    for (int64_t i = 0; i < n; i++) sum += (uint32_t)a[i].l;
    volatile float avg = (float)sum / (float)n;
    const float aq = (float)(0.01 * (double)avg);
    const double davg = (double)avg;
    int64_t st = 0;
    for (int64_t i = 0; i < n; i++) {
        while (st < i && !(a[i].r - a[st].r <= (uint64_t)(uint32_t)dr)) ++st;
        if (i - st > max_iter) st = i - max_iter;
        const bool vec = (i - 1 - st) > 5;
        const int32_t li = a[i].l, qi = a[i].q;
        const uint32_t ri = (uint32_t)a[i].r;
        int32_t best = li;
        int64_t bj = -1;
        for (int64_t j = i - 1; j >= st; j--) {
            const int32_t ddr = (int32_t)(ri - (uint32_t)a[j].r);
            const int32_t ddq = wrap_sub(qi, a[j].q);
            const int32_t dd = wrap_abs(wrap_sub(ddr, ddq));
            if (dd > bw || ddr == 0 || ddq <= 0 || ddq > dq || ddq > dr) continue;
            int32_t oc = ddr < ddq ? ddr : ddq;
            oc = oc < li ? oc : li;
            const int32_t gc = vec ? gap_float(dd, aq) : gap_double(dd, davg);
            const int32_t sc = wrap_sub(wrap_add((int32_t)f[j], oc), gc);
            if (sc > best) {  // j descends: ties keep the larger j
                best = sc;
                bj = j;
            }
        }
        f[i] = (uint32_t)best;
        p[i] = (int32_t)bj;
        v[i] = (bj >= 0 && v[bj] > best) ? v[bj] : best;
    }
}

}  // namespace

extern "C" {

// anchors: 16-byte anchor_t records; read k = anchors[offsets[k], offsets[k+1]).
// Returns 0, or -1 on malformed offsets.
int oracle_chain(const void *anchors, const int64_t *offsets, int32_t n_reads, int32_t bw,
                 int32_t max_iter, int32_t dr, int32_t dq, uint32_t *f, int32_t *p, int32_t *v,
                 int nthreads) {
    static_assert(sizeof(Anchor) == 16, "anchor_t is 16 bytes");
    for (int32_t k = 0; k < n_reads; k++)
        if (offsets[k + 1] < offsets[k] || offsets[k] < 0) return -1;
    const Anchor *A = static_cast<const Anchor *>(anchors);
    auto work = [&](int t, int nt) {
        for (int32_t k = t; k < n_reads; k += nt) {
            const int64_t o = offsets[k];
            chain_read(A + o, offsets[k + 1] - o, bw, max_iter, dr, dq, f + o, p + o, v + o);
        }
    };
    if (nthreads <= 1) {
        work(0, 1);
        return 0;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++) th.emplace_back(work, t, nthreads);
    for (auto &x : th) x.join();
    return 0;
}

}  // extern "C"
