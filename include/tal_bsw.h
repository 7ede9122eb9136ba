/*
 * tal_bsw.h -- C ABI of the GB300 banded Smith-Waterman seed extension.
 *
 * Drop-in replacement for TAL's BandedPairWiseSW (src/alignment/BSW/bandedSWA.h)
 * on one GB300 GPU (sm_103a).  Plain C types only: pointers, sizes, status codes.
 *
 * Semantics follow the reference's inter-task SIMD kernels getScores16 /
 * getScores8 (bandedSWA.cpp:2664-3356 / :1970-2661) bit for bit:
 *   target  seq1 = seqBufRef + idr, length len1   (bandedSWA.cpp:2806)
 *   query   seq2 = seqBufQer + idq, length len2   (bandedSWA.cpp:2848)
 *   bases 0..3, 4 = N; outputs score, tle, gtle, qle, gscore, max_off are
 *   written into the caller's SeqPair records, [0, numPairs) only.
 */
#ifndef TAL_BSW_H
#define TAL_BSW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference's functions return void and exit() or assert()
 * on failure (bandedSWA.cpp:88-93, 2705-2708); every entry point here returns
 * one of these instead. */
enum {
    TAL_OK = 0,
    TAL_EINVAL = 1,   /* bad argument: NULL pointer, negative count, bad bits */
    TAL_EDOMAIN = 2,  /* a pair outside the kernel's exact range (see below) */
    TAL_ENOMEM = 3,   /* device or pinned-host allocation failed */
    TAL_ECUDA = 4,    /* a CUDA runtime call failed */
    TAL_ETIMEOUT = 5, /* a bounded wait ran out */
    TAL_ENODEV = 6,   /* no usable sm_103 device */
    TAL_EBUSY = 7     /* serving queue full / handle in use */
};

/* Precision selector for tal_bsw_scores*. */
enum {
    TAL_BSW_AUTO = 0, /* per pair: 8-bit rules where eligible, else 16-bit */
    TAL_BSW_8 = 8,    /* getScores8  (bandedSWA.h:257-262) */
    TAL_BSW_16 = 16,  /* getScores16 (bandedSWA.h:285-290) */
    /* OR into TAL_BSW_8 / TAL_BSW_16 for tal_bsw_scores and
     * tal_bsw_scores_device (one band per call, no d_w): score every pair in
     * the reference's own SIMD groups -- 64 (8-bit) / 32 (16-bit) consecutive
     * pairs of the array, the AVX-512BW widths, the last group padded as the
     * reference pads it -- one warp per group, every value in the
     * reference's wrapping int8 / int16.  The outputs are the same as
     * without the flag (the default is exact too, see tal_bsw_scores); the
     * flag only changes how they are computed, several times slower: for
     * callers that want the grouped computation for every pair. */
    TAL_BSW_GROUPED = 0x100,
    /* OR into TAL_BSW_8 / TAL_BSW_16 / TAL_BSW_AUTO for tal_bsw_scores and
     * tal_bsw_scores_device: score every pair as if it were alone in its SIMD
     * group (no coupling detector, no group re-scoring) -- the semantics of
     * the reference's scalarBandedSWAWrapper (bandedSWA.cpp:242-260), which
     * scores pairs one at a time; pairs outside the per-pair kernels' exact
     * range give TAL_EDOMAIN. */
    TAL_BSW_PER_PAIR = 0x200
};

/* SeqPair, bandedSWA.h:90-99: 14 x int32 = 56 bytes, fields in this order. */
typedef struct tal_seq_pair {
    int32_t idr, idq, id;
    int32_t len1, len2;
    int32_t h0;
    int32_t seqid, regid;
    int32_t score, tle, gtle, qle;
    int32_t gscore, max_off;
} tal_seq_pair;

/* Constructor arguments of BandedPairWiseSW (bandedSWA.h:118-121).  The
 * reference's vector kernels ignore its scoring matrix and score a match
 * with w_match, a mismatch with -w_mismatch and any N with -1
 * (bandedSWA.cpp:64-68, 1883-1892); so does this library. */
typedef struct tal_bsw_params {
    int32_t o_del, e_del, o_ins, e_ins;
    int32_t zdrop, end_bonus;
    int32_t w_match;    /* a  (int8 in the reference) */
    int32_t w_mismatch; /* b, positive penalty (int8 in the reference) */
} tal_bsw_params;

typedef struct tal_bsw_ctx *tal_bsw_handle;

/* Replaces BandedPairWiseSW::BandedPairWiseSW (bandedSWA.cpp:50-94).  Binds
 * the calling thread's current device (or `device` if >= 0), creates a stream
 * and grow-only device buffers.  Parameters outside the exact range
 * (0 <= o <= 127, 1 <= e <= 127, 0 <= a, b <= 127) give TAL_EINVAL. */
int tal_bsw_create(const tal_bsw_params *params, int device, tal_bsw_handle *out);

/* Replaces ~BandedPairWiseSW (bandedSWA.cpp:97-100). */
int tal_bsw_destroy(tal_bsw_handle h);

/* Replaces getScores8 / getScores16 (bandedSWA.cpp:1970, 2664) on host
 * buffers: copies the pairs and the byte ranges they reference to the
 * device, scores them, and writes the six outputs back into pairs[0, n).
 * bits: TAL_BSW_8, TAL_BSW_16 or TAL_BSW_AUTO.  w: band, per call.
 *
 * Exactness: every output equals the reference's.  The reference scores its
 * array in SIMD groups of 32 (16-bit) / 64 (8-bit) consecutive pairs that
 * share one band per row, and a pair's outputs can depend on the rest of
 * its group (bandedSWA.cpp:3235-3316 re-derive a lane's head and tail from
 * the group's band edges).  The library scores each pair on its own with a
 * detector that flags every pair whose outputs could depend on its group;
 * it then re-scores the groups of the flagged pairs in the reference's
 * grouping, on the device, before the call returns.  With TAL_BSW_AUTO the
 * grouping is that of the reference's caller: the 8-bit-routed pairs form
 * one array and the 16-bit-routed ones another, each in array order; with a
 * band per pair (d_w, wpair) one array per (band, precision).  On the
 * benchmark workloads about 1 pair in 20,000 is flagged; narrow-band
 * seed-extension batches flag a few per cent.
 *
 * Range: lengths up to 127 (8-bit) / 32767 (16-bit) and h0 >= 0, the
 * reference's own limits (bandedSWA.h:82).  Pairs whose int8 / int16 values
 * wrap are scored by the grouped kernel, which wraps as the reference does.
 * A pair outside the range gives TAL_EDOMAIN (for AUTO: the 8-bit rules are
 * used where the pair is inside them), and no outputs are written.
 * Capacity: a pair's rows live in shared memory, as a ring of the band's
 * columns (2w + 12 up to 16,384, any query length) or as whole rows (queries
 * up to ~22,000 bases); a pair that fits neither (a query above ~22,000
 * bases with w above 8,186) is scored with the flagged pairs' groups, its
 * rows in global memory (slowly: ~seconds for a 30,000-base query with a
 * band of 20,000).  With TAL_BSW_PER_PAIR such a pair gives TAL_EDOMAIN. */
int tal_bsw_scores(tal_bsw_handle h, tal_seq_pair *pairs, const uint8_t *seqBufRef,
                   const uint8_t *seqBufQer, int32_t numPairs, int32_t w, int bits);

/* The same on device-resident buffers (cudaMalloc'd), asynchronous on the
 * handle's stream; d_w, if not NULL, gives a band per pair instead of w.
 * ref_bytes / qer_bytes are the allocation sizes of d_ref / d_qer (reads stay
 * inside them).  Call tal_bsw_sync to wait and collect the status. */
int tal_bsw_scores_device(tal_bsw_handle h, tal_seq_pair *d_pairs, const uint8_t *d_ref,
                          size_t ref_bytes, const uint8_t *d_qer, size_t qer_bytes,
                          int32_t numPairs, int32_t w, const int32_t *d_w, int bits);

/* Batched form, no counterpart in the reference (its callers issue one
 * getScores call per batch): scores a large batch of mixed pairs -- uneven
 * lengths, per-pair bands (d_w / wpair, optional), 8/16-bit routing with
 * bits = TAL_BSW_AUTO -- as one CUDA graph: a device-side sort of the pairs
 * into length bins (by query length, then target length) followed by one
 * persistent, work-stealing launch per bin, each with the kernel and tile an
 * autotuner picked for that bin on the handle's first batched call.  Outputs
 * are the same as tal_bsw_scores on the same pairs.  The graph is captured on
 * the first call with a given set of buffers and replayed after that.
 * Device-resident variant; synchronous (returns the status). */
int tal_bsw_scores_batched_device(tal_bsw_handle h, tal_seq_pair *d_pairs, const uint8_t *d_ref,
                                  size_t ref_bytes, const uint8_t *d_qer, size_t qer_bytes,
                                  int32_t numPairs, int32_t w, const int32_t *d_w, int bits);

/* The batched form on host buffers (pairs updated in place); wpair: an
 * optional band per pair. */
int tal_bsw_scores_batched(tal_bsw_handle h, tal_seq_pair *pairs, const uint8_t *seqBufRef,
                           const uint8_t *seqBufQer, int32_t numPairs, int32_t w,
                           const int32_t *wpair, int bits);

/* Forgets the autotuner's choices and the captured graphs (the next batched
 * call tunes again). */
int tal_bsw_autotune_reset(tal_bsw_handle h);

/* The configuration of length bin `bin` (0..20) for bands too wide for a row
 * ring: lanes per pair (1 = the lane-per-pair kernel), columns per lane, and
 * the bin's largest query length. */
int tal_bsw_bin_config(tal_bsw_handle h, int bin, int *lanes_per_pair, int *cols_per_lane,
                       int *max_len2);

/* The configuration of segment `seg` (0..146) of the batched form.  A
 * segment is a length bin x band class (class c < 6: pairs with
 * 2w + 12 <= 64 << c, scored in rings of 64 << c columns; class 6: whole
 * rows); segments 0..10 are the whole-row bins of queries above 384 columns,
 * longest first, then all other segments, bins longest first.  max_len2: the
 * bin's largest query; window: the ring in columns (0: whole rows).  Returns
 * TAL_EINVAL past the last segment. */
int tal_bsw_segment_config(tal_bsw_handle h, int seg, int *lanes_per_pair, int *cols_per_lane,
                           int *max_len2, int *window);

/* Waits for the handle's stream; returns the first error any launch on it
 * reported since the last sync. */
int tal_bsw_sync(tal_bsw_handle h);

/* The handle's CUDA stream (a cudaStream_t), for callers that order their
 * own copies against the scorer. */
void *tal_bsw_stream(tal_bsw_handle h);

/* Human-readable text of the last error on this handle ("" if none). */
const char *tal_bsw_last_error(tal_bsw_handle h);

/* Index of the first pair that gave TAL_EDOMAIN in the last call, or -1. */
int64_t tal_bsw_last_bad_pair(tal_bsw_handle h);

/* Number of kernel launches this handle has issued (for accounting). */
uint64_t tal_bsw_launch_count(tal_bsw_handle h);

/* Device time, in milliseconds, of the scoring kernel of the last collected
 * plain call (tal_bsw_scores / tal_bsw_scores_device + tal_bsw_sync; for a
 * chunked host call, its last chunk's), from CUDA events on the handle's
 * stream around that one launch. */
float tal_bsw_last_kernel_ms(tal_bsw_handle h);

/* DP cells the last collected call computed (sum over rows of the band
 * width the reference's vector kernel visits for each pair).  The reference's
 * own counter, BandedPairWiseSW::SW_cells, is never incremented
 * (bandedSWA.cpp:199). */
uint64_t tal_bsw_last_cells(tal_bsw_handle h);

/* Pairs the last collected call flagged as possibly depending on their
 * SIMD group (or outside the per-pair kernels' exact range), and the groups
 * it re-scored with the reference's grouping for them (see tal_bsw_scores).
 * Accounting only; no counterpart in the reference. */
int tal_bsw_last_regroup(tal_bsw_handle h, int64_t *flagged_pairs, int64_t *groups);

/* Measurement utility, no counterpart in the reference: integer-pipe
 * throughput of `device` in thread-instructions per second, for the
 * roofline -- packed 16x2 add-max (DPX) and plain int32. */
int tal_bsw_probe_int_peak(int device, double *dpx_per_s, double *i32_per_s);

/* Size in bytes of the library's fixed device scratch array used by
 * tal_bsw_scores_device_noalloc (one per device, held until process exit). */
#define TAL_BSW_NOALLOC_SCRATCH_BYTES 256

/* Allocation-free scoring; no counterpart in the reference, which allocates
 * its SIMD scratch inside every call (bandedSWA.cpp:2702-2703).
 *
 * For callers that must not allocate device memory while scoring (device
 * memory owned by their own pool, or hot paths where cudaMalloc/cudaFree
 * would synchronise the device).  Scores numPairs SeqPair records already in
 * device memory, like tal_bsw_scores_device, but needs no handle and calls no
 * allocator: its only scratch is a fixed TAL_BSW_NOALLOC_SCRATCH_BYTES device
 * array inside the library (a control block).  Runs on `stream` (a
 * cudaStream_t, NULL = default stream) of the current device and returns when
 * the scores are in d_pairs; it synchronises `stream` twice (to read the
 * batch's longest sequences, then the status).  The first call on each device
 * resolves the scratch array's device address; make that first call before
 * any stream capture.  All calls on a device share the one array and clear
 * it themselves, so calls that overlap on the GPU (other threads or streams)
 * race: serialise them.
 *
 * Each pair is scored as if alone in its SIMD group: re-scoring the rare
 * pairs whose outputs depend on their group (what the handle entry points
 * do, see tal_bsw_scores) needs device memory that grows with the batch, so
 * this entry point does not; on those pairs its outputs are the pair's own.
 * Status: TAL_EDOMAIN for a pair outside the per-pair kernels' exact range
 * (including wrapping values) or with a base code above 4, TAL_ENOMEM for a
 * pair whose rows do not fit the kernels' shared memory (checked on the
 * device per pair, or for the whole batch before the launch);
 * tal_bsw_noalloc_last_bad_pair names the offending pair. */
int tal_bsw_scores_device_noalloc(const tal_bsw_params *params, tal_seq_pair *d_pairs,
                                  const uint8_t *d_ref, size_t ref_bytes,
                                  const uint8_t *d_qer, size_t qer_bytes, int32_t numPairs,
                                  int32_t w, const int32_t *d_w, int bits, void *stream);

/* The lowest index of a pair that made the last tal_bsw_scores_device_noalloc
 * call on the current device fail (TAL_EDOMAIN, or TAL_ENOMEM found on the
 * device); -1 after a successful call or when the failure names no pair (the
 * batch's longest rows exceed shared memory before any launch), and before
 * the first call.  Reads host memory only; same serialisation rule as the
 * scoring call. */
int64_t tal_bsw_noalloc_last_bad_pair(void);

/* ---------------------------------------------------------------------------
 * Serving loop; no counterpart in the reference, whose callers block in one
 * getScores call per batch (bench-bsw.cpp:216-258).
 *
 * A server takes scoring requests -- SeqPair batches of any size, each with
 * its own sequence buffers, band and precision -- as they arrive, and runs
 * them with continuous batching: a worker thread admits queued requests in
 * arrival order as soon as their pairs and sequences fit the server's device
 * pool (admission by free device memory), copies them in while earlier work
 * runs, and launches every admitted request that is not yet running as one
 * "tick" (a device-side length sort of all their pairs plus one persistent
 * launch per non-empty length bin).  Up to `slots` ticks are on the device at
 * once, on their own streams, so a tick admitted while another runs overlaps
 * with it.  Each request's outputs are those of tal_bsw_scores on the same
 * pairs, alone or in any mix, and one request's bad pair fails only that
 * request.  Caller buffers stay owned by the caller and must stay valid
 * until the request is polled complete; pinned (page-locked) buffers are
 * copied directly, pageable ones through the server's pinned staging. */
typedef struct tal_bsw_server *tal_bsw_server_handle;

typedef struct {
    size_t pool_bytes;      /* device pool for requests' pairs and sequences;
                               0 = min(64 GiB, 85% of the free device memory) */
    size_t staging_bytes;   /* pinned host staging for pageable callers; 0 = 1 GiB */
    int32_t max_tick_pairs; /* most pairs in one tick (and in one request);
                               0 = 8,388,608 */
    int32_t slots;          /* ticks on the device at once, 1..4; 0 = 2 */
    int32_t latency_pairs;  /* ticks with fewer pairs run as a handful of
                               launches with several lanes per pair above 256
                               columns (lower latency per pair); larger ticks
                               run like the batched form, one tuned launch per
                               segment (more cells per second);
                               0 = 131,072, -1 = never */
    int32_t pad_;
} tal_bsw_server_config;

typedef struct {
    int32_t status;          /* TAL_OK, TAL_EDOMAIN (bad_pair names the pair) or TAL_ECUDA */
    int32_t tick_requests;   /* requests in the tick that ran this one */
    int64_t bad_pair;        /* first offending pair of this request, or -1 */
    int64_t tick_pairs;      /* pairs in that tick */
    int64_t submit_ns;       /* steady-clock times (tal_bsw_now_ns): submit call, */
    int64_t admit_ns;        /*   copies issued into the pool, */
    int64_t launch_ns;       /*   its tick launched, */
    int64_t done_ns;         /*   outputs in the caller's SeqPair array */
} tal_bsw_request_info;

typedef struct {
    uint64_t submitted, completed, failed, ticks, pairs, launches;
    uint64_t pool_bytes, pool_used_bytes, pool_peak_bytes;
    int32_t queued, admitted, running;     /* requests in each state now */
    int32_t max_tick_requests;             /* most requests one tick has carried */
    int32_t max_ticks_in_flight;           /* most ticks on the device at once */
    int32_t pad_;
} tal_bsw_server_stats;

/* Steady-clock nanoseconds, the clock of tal_bsw_request_info. */
int64_t tal_bsw_now_ns(void);

/* Creates a server with the scoring parameters of `h` and its length-bin
 * configurations (the autotuner's, when h ran a batched call; else the
 * defaults), on h's device.  h may be destroyed afterwards.  A tick's
 * segment launches run on up to 32 streams: start the process with
 * CUDA_DEVICE_MAX_CONNECTIONS=32 so they do not share CUDA's default 8
 * hardware queues (the same holds for tal_bsw_scores_batched). */
int tal_bsw_server_create(tal_bsw_handle h, const tal_bsw_server_config *cfg,
                          tal_bsw_server_handle *out);

/* Completes every submitted request, then frees the server. */
int tal_bsw_server_destroy(tal_bsw_server_handle s);

/* Queues a request: score pairs[0, numPairs) against seqBufRef / seqBufQer
 * (offsets idr / idq as in tal_bsw_scores) with band w, or wpair[k] per pair
 * when wpair is not NULL, and bits 8 / 16 / TAL_BSW_AUTO.  Returns at once
 * with a ticket.  TAL_EINVAL: bad arguments or numPairs > max_tick_pairs;
 * TAL_ENOMEM: the request can never fit the pool or the staging; TAL_EBUSY:
 * pageable buffers and the staging is full right now (retry later). */
int tal_bsw_submit(tal_bsw_server_handle s, tal_seq_pair *pairs, const uint8_t *seqBufRef,
                   const uint8_t *seqBufQer, int32_t numPairs, int32_t w,
                   const int32_t *wpair, int bits, uint64_t *ticket);

/* Waits up to timeout_us (0: just checks, negative: no limit) for the
 * request.  TAL_OK: it is complete, its outputs are in its SeqPair array,
 * info (optional) holds its status and times, and the ticket is released.
 * TAL_ETIMEOUT: not complete yet.  TAL_EINVAL: unknown ticket. */
int tal_bsw_poll(tal_bsw_server_handle s, uint64_t ticket, int64_t timeout_us,
                 tal_bsw_request_info *info);

int tal_bsw_server_get_stats(tal_bsw_server_handle s, tal_bsw_server_stats *out);

#ifdef __cplusplus
}
#endif

#endif /* TAL_BSW_H */
