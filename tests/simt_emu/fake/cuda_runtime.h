// CPU stand-in for the parts of the CUDA runtime / device API that the
// kernels use, so the unchanged kernel source can be compiled for the host
// and run lane-by-lane (one std::thread per lane) by tests/simt_emu/emu.cpp.
// Test infrastructure only.
#pragma once
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <ucontext.h>
#include <cstdint>
#include <cstring>
#include <mutex>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __align__(n) alignas(n)
#define __shared__
#define __restrict__

typedef int cudaError_t;
struct uint2 { unsigned x, y; };
struct uint4 { unsigned x, y, z, w; };
inline uint2 make_uint2(unsigned a, unsigned b) { return uint2{a, b}; }
inline uint4 make_uint4(unsigned a, unsigned b, unsigned c, unsigned d) { return uint4{a, b, c, d}; }

namespace simt {
// The 32 lanes of a warp are fibers (ucontext) run by one host thread; every
// warp-collective is a point where a lane yields until all 32 have arrived.
struct Warp {
    ucontext_t sched;
    ucontext_t lane_ctx[32];
    int64_t slot[2][32];
    int phase[32] = {0};
    bool done[32] = {false};
    bool at_bar[32] = {false};  // waiting at a block barrier (multi-warp blocks)
    void barrier(int l) { swapcontext(&lane_ctx[l], &sched); }
};
struct Dim { unsigned x = 0, y = 0, z = 0; };
extern thread_local Dim tl_threadIdx, tl_blockIdx, tl_blockDim, tl_gridDim;
extern thread_local Warp *tl_warp;
extern thread_local unsigned char *tl_smem;
extern std::mutex atomic_mu;

inline int lane() { return (int)(tl_threadIdx.x & 31); }
// all 32 lanes deposit v, wait, then read the slot of lane src
inline int64_t exchange(int64_t v, int src) {
    Warp *w = tl_warp;
    int l = lane();
    int ph = w->phase[l];
    w->slot[ph][l] = v;
    w->barrier(l);
    int64_t r = w->slot[ph][src];
    w->phase[l] = ph ^ 1;
    return r;
}
inline void gather(int64_t v, int64_t out[32]) {
    Warp *w = tl_warp;
    int l = lane();
    int ph = w->phase[l];
    w->slot[ph][l] = v;
    w->barrier(l);
    for (int i = 0; i < 32; i++) out[i] = w->slot[ph][i];
    w->phase[l] = ph ^ 1;
}
}  // namespace simt

#define threadIdx (simt::tl_threadIdx)
#define blockIdx (simt::tl_blockIdx)
#define blockDim (simt::tl_blockDim)
#define gridDim (simt::tl_gridDim)

template <typename T>
inline T __shfl_sync(unsigned, T v, int src, int width = 32) {
    int l = simt::lane();
    int base = (l / width) * width;
    return (T)simt::exchange((int64_t)v, base + (src % width));
}
template <typename T>
inline T __shfl_up_sync(unsigned, T v, unsigned d, int width = 32) {
    int l = simt::lane();
    int base = (l / width) * width;
    int src = l - (int)d;
    return (T)simt::exchange((int64_t)v, src < base ? l : src);
}
template <typename T>
inline T __shfl_xor_sync(unsigned, T v, int m, int width = 32) {
    int l = simt::lane();
    int base = (l / width) * width;
    int src = l ^ m;
    if (src < base || src >= base + width) src = l;
    return (T)simt::exchange((int64_t)v, src);
}
inline unsigned __ballot_sync(unsigned, int pred) {
    int64_t all[32];
    simt::gather(pred ? 1 : 0, all);
    unsigned m = 0;
    for (int i = 0; i < 32; i++) if (all[i]) m |= 1u << i;
    return m;
}
inline int __any_sync(unsigned m, int pred) { return __ballot_sync(m, pred) != 0; }
inline int __all_sync(unsigned m, int pred) { return __ballot_sync(m, pred) == 0xffffffffu; }
inline unsigned __reduce_max_sync(unsigned, unsigned v) {
    int64_t all[32];
    simt::gather((int64_t)v, all);
    unsigned r = 0;
    for (int i = 0; i < 32; i++) r = (unsigned)all[i] > r ? (unsigned)all[i] : r;
    return r;
}
inline int __reduce_max_sync(unsigned, int v) {
    int64_t all[32];
    simt::gather((int64_t)v, all);
    int r = INT_MIN;
    for (int i = 0; i < 32; i++) r = (int)all[i] > r ? (int)all[i] : r;
    return r;
}
inline int __reduce_add_sync(unsigned, int v) {
    int64_t all[32];
    simt::gather((int64_t)v, all);
    int r = 0;
    for (int i = 0; i < 32; i++) r += (int)all[i];
    return r;
}
inline unsigned __reduce_min_sync(unsigned, unsigned v) {
    int64_t all[32];
    simt::gather((int64_t)v, all);
    unsigned r = 0xffffffffu;
    for (int i = 0; i < 32; i++) r = (unsigned)all[i] < r ? (unsigned)all[i] : r;
    return r;
}
inline int __reduce_min_sync(unsigned, int v) {
    int64_t all[32];
    simt::gather((int64_t)v, all);
    int r = INT_MAX;
    for (int i = 0; i < 32; i++) r = (int)all[i] < r ? (int)all[i] : r;
    return r;
}
inline void __syncwarp(unsigned = 0xffffffffu) { simt::tl_warp->barrier(simt::lane()); }
// A block barrier: the lane waits until every warp of the block has
// arrived (emu.cpp's block scheduler releases them); a one-warp launch
// treats it as a warp barrier.
inline void __syncthreads() {
    simt::Warp *w = simt::tl_warp;
    const int l = simt::lane();
    w->at_bar[l] = true;
    w->barrier(l);
}
inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
inline int __ffs(unsigned x) { return x ? __builtin_ctz(x) + 1 : 0; }
inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
inline int __popc(unsigned x) { return __builtin_popcount(x); }
// CUDA's __byte_perm: result byte n = byte ((s >> 4n) & 7) of {y:x}
inline unsigned __byte_perm(unsigned x, unsigned y, unsigned s) {
    uint64_t v = ((uint64_t)y << 32) | x;
    unsigned r = 0;
    for (int n = 0; n < 4; n++) {
        unsigned sel = (s >> (4 * n)) & 7u;
        r |= (unsigned)((v >> (8 * sel)) & 0xffu) << (8 * n);
    }
    return r;
}
template <typename T, typename V>
inline T atomicAdd(T *p, V vv) { T v = (T)vv; std::lock_guard<std::mutex> g(simt::atomic_mu); T o = *p; *p = o + v; return o; }
template <typename T, typename V>
inline T atomicOr(T *p, V vv) { T v = (T)vv; std::lock_guard<std::mutex> g(simt::atomic_mu); T o = *p; *p = o | v; return o; }
template <typename T, typename V>
inline T atomicMin(T *p, V vv) { T v = (T)vv; std::lock_guard<std::mutex> g(simt::atomic_mu); T o = *p; if (v < o) *p = v; return o; }
template <typename T, typename V>
inline T atomicMax(T *p, V vv) { T v = (T)vv; std::lock_guard<std::mutex> g(simt::atomic_mu); T o = *p; if (v > o) *p = v; return o; }
struct int2 { int x, y; };
struct int4 { int x, y, z, w; };
inline int2 make_int2(int a, int b) { return int2{a, b}; }
inline int4 make_int4(int a, int b, int c, int d) { return int4{a, b, c, d}; }
// DPX integer min/max (sm_90+): semantics per the CUDA math API
inline int __viaddmin_s32(int a, int b, int c) { int s = a + b; return s < c ? s : c; }
inline int __viaddmax_s32(int a, int b, int c) { int s = a + b; return s > c ? s : c; }
inline int __viaddmax_s32_relu(int a, int b, int c) { int s = a + b; int m = s > c ? s : c; return m > 0 ? m : 0; }
inline int __vimax3_s32(int a, int b, int c) { int m = a > b ? a : b; return m > c ? m : c; }
inline int __vimax3_s32_relu(int a, int b, int c) { int m = __vimax3_s32(a, b, c); return m > 0 ? m : 0; }
// Rounded conversions and products as the device intrinsics define them (the
// host computes in IEEE single / double with round-to-nearest, no contraction
// in a single product).
inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
inline float __fdiv_rn(float a, float b) { volatile float r = a / b; return r; }
inline double __dmul_rn(double a, double b) { volatile double r = a * b; return r; }
inline float __int2float_rn(int x) { return (float)x; }
inline float __ull2float_rn(unsigned long long x) { return (float)x; }
inline float __ll2float_rn(long long x) { return (float)x; }
inline float __double2float_rn(double x) { return (float)x; }
inline int __float2int_rd(float x) {  // saturating, like the device conversion
    const double d = std::floor((double)x);
    return d >= 2147483647.0 ? INT_MAX : d <= -2147483648.0 ? INT_MIN : (int)d;
}
inline int __double2int_rz(double x) {
    const double d = std::trunc(x);
    return d >= 2147483647.0 ? INT_MAX : d <= -2147483648.0 ? INT_MIN : (int)d;
}

// 16x2 forms: each 16-bit half on its own
inline int sw_lo16(unsigned v) { return (int)(short)(v & 0xffffu); }
inline int sw_hi16(unsigned v) { return (int)(short)(v >> 16); }
inline unsigned sw_pack16(int lo, int hi) { return ((unsigned)lo & 0xffffu) | ((unsigned)hi << 16); }
inline unsigned __viaddmax_s16x2(unsigned a, unsigned b, unsigned c) {
    auto f = [](int x, int y, int z) { int s = (int)(short)(x + y); return s > z ? s : z; };
    return sw_pack16(f(sw_lo16(a), sw_lo16(b), sw_lo16(c)), f(sw_hi16(a), sw_hi16(b), sw_hi16(c)));
}
inline unsigned __viaddmax_s16x2_relu(unsigned a, unsigned b, unsigned c) {
    auto f = [](int x, int y, int z) { int s = (int)(short)(x + y); s = s > z ? s : z; return s > 0 ? s : 0; };
    return sw_pack16(f(sw_lo16(a), sw_lo16(b), sw_lo16(c)), f(sw_hi16(a), sw_hi16(b), sw_hi16(c)));
}
inline unsigned __vimax3_s16x2_relu(unsigned a, unsigned b, unsigned c) {
    auto f = [](int x, int y, int z) { int m = x > y ? x : y; m = m > z ? m : z; return m > 0 ? m : 0; };
    return sw_pack16(f(sw_lo16(a), sw_lo16(b), sw_lo16(c)), f(sw_hi16(a), sw_hi16(b), sw_hi16(c)));
}
inline unsigned __vimin3_u16x2(unsigned a, unsigned b, unsigned c) {
    auto f = [](unsigned x, unsigned y, unsigned z) { unsigned m = x < y ? x : y; return m < z ? m : z; };
    return (f(a & 0xffffu, b & 0xffffu, c & 0xffffu)) | (f(a >> 16, b >> 16, c >> 16) << 16);
}
