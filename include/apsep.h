/*
 * apsep.h -- C ABI of the GB300-native APSE engine (libapsep.so).
 *
 * All Previous Smaller Element: for each key a[i], out[i] is the largest
 * j < i with a[j] < a[i] (APSEP_LT) or a[j] <= a[i] (APSEP_LE), else -1.
 * Keys are int32, float32, int64 or float64 (finite: NaN keys are outside
 * the contract), outputs are int32 indices, so n <= APSEP_MAX_KEYS =
 * 2^31 - 4096.
 *
 * Plain pointers and sizes only: device pointers from any allocator
 * (cudaMalloc, torch), `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  No call exits the process; every failure is an
 * apsep_status.
 *
 * Reference interfaces each entry point replaces (CoderDue/APSEP,
 * src/apsep.cuh):
 *   apsep_plan_create   allocSPTScratch<T,BS,IPT,INCL>(n)   src/apsep.cuh:3014-3040
 *                       allocWSTLScratch<T,BS,IPT>(n)       src/apsep.cuh:2521-2537
 *   apsep_plan_destroy  freeSPTScratch(s)                   src/apsep.cuh:3042-3050
 *                       freeWSTLScratch(s)                  src/apsep.cuh:2539-2546
 *   apsep_run           runSPT<T,BS,IPT,INCL>(d_in,d_out,n,s)  src/apsep.cuh:3052-3067
 *                       runWSTL<T,BS,IPT>(d_in,d_out,n,s)   src/apsep.cuh:2548-2596
 *   apsep_run_cmp       runSPT<...,INCL> with the comparator chosen per call
 *                       (the INCL template argument, src/apsep.cuh:2669-2673)
 *   apsep_launch        launchSPT / launchWSTL: alloc + run + sync + free
 *                       src/apsep.cuh:3069-3076, 2598-2605
 *   apsep_plan_check    gpuAssert after a sync (src/apsep.cuh:39-47), but
 *                       returning a status instead of exit()
 * The C++ shim include/apsep.cuh re-exports the reference template names on
 * top of these.
 */
#ifndef APSEP_H_
#define APSEP_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum apsep_status {
    APSEP_OK = 0,
    APSEP_EINVAL = 1,    /* bad argument: null, n < 0, n > capacity, overlap */
    APSEP_ENOMEM = 2,    /* device allocation failed */
    APSEP_ECUDA = 3,     /* a CUDA runtime/driver call failed */
    APSEP_ETIMEOUT = 4,  /* a bounded device-side wait gave up (see plan_check) */
    APSEP_EINTERNAL = 5, /* a device-side invariant check failed */
    APSEP_ENOTSUP = 6    /* unsupported dtype / device */
} apsep_status;

/* Key types.  8-byte keys (the reference's ApsepInfinity<long long/double>,
 * src/apsep.cuh:62-70) keep int32 positions (n <= APSEP_MAX_KEYS) and run
 * single arrays, segmented batches and the consumers (the histogram takes
 * int32 heights); apsep_run_noalloc refuses them (APSEP_EINVAL), and their
 * plans have one configuration (1). */
typedef enum apsep_dtype { APSEP_INT32 = 0, APSEP_FLOAT32 = 1, APSEP_INT64 = 2, APSEP_FLOAT64 = 3 } apsep_dtype;

typedef enum apsep_cmp {
    APSEP_LT = 0, /* strict previous-smaller (the reference's INCL=false) */
    APSEP_LE = 1  /* previous-smaller-or-equal (INCL=true)                */
} apsep_cmp;

typedef struct apsep_plan apsep_plan;

typedef struct apsep_plan_info {
    int64_t capacity;       /* largest n a run may use                      */
    int64_t scratch_bytes;  /* device scratch owned by the plan             */
    int32_t tile_keys;      /* keys per tile of the selected configuration  */
    int32_t config;         /* index of the selected kernel configuration   */
    int32_t device;         /* CUDA device the plan lives on                */
    int32_t dtype;
    int32_t cmp;
    int32_t reserved;
} apsep_plan_info;

/* Version of this ABI (major*10000 + minor*100 + patch). */
int apsep_version(void);

/* Human-readable name of a status code (static string). */
const char* apsep_status_string(apsep_status s);

/* Create a plan for up to `capacity` keys on the current CUDA device.  Owns
 * all scratch; runs never allocate.  (allocSPTScratch / allocWSTLScratch) */
apsep_status apsep_plan_create(apsep_plan** plan, apsep_dtype dtype, apsep_cmp cmp, int64_t capacity);

/* Free the plan and its scratch.  Null is a no-op.  (freeSPTScratch) */
apsep_status apsep_plan_destroy(apsep_plan* plan);

/* Enqueue one run on `stream`: d_out[0..n) <- APSE(d_in[0..n)).  Asynchronous,
 * no allocation, no synchronisation, so it can be captured in a CUDA graph.
 * n == 0 is a no-op.  d_in/d_out must be 4-byte aligned (else
 * APSEP_EINVAL).  Arrays at the same offset within 16 bytes stream through
 * TMA (off a 16-byte boundary: behind 1-3 virtual keys, in the segmented
 * kernel as one segment); arrays at different offsets take plain loads and
 * stores.  Runs on one plan must not overlap in time (serialise them on one
 * stream).  (runSPT / runWSTL) */
apsep_status apsep_run(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, void* stream);

/* apsep_run with the comparator chosen per call (runSPT<...,INCL>). */
apsep_status apsep_run_cmp(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                           void* stream);

/* Batched segmented run: nseg arrays stored back to back in d_in[0..n),
 * segment s being d_in[d_offsets[s] .. d_offsets[s+1]), all in ONE launch.
 * d_out[i] is the index, relative to the start of i's segment, of the nearest
 * earlier key of the same segment that qualifies (plan comparator), else -1.
 * d_offsets: device array of nseg + 1 int64, 8-byte aligned, d_offsets[0] = 0,
 * non-decreasing, d_offsets[nseg] = n (empty segments allowed); a violation of
 * the end points is detected on the device and reported by apsep_plan_check
 * as APSEP_EINVAL.  Asynchronous, no allocation, graph-capturable, like
 * apsep_run.  No counterpart in the reference (its entry points take one
 * array); it replaces a loop of runSPT calls, one per array. */
apsep_status apsep_run_segmented(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n,
                                 const int64_t* d_offsets, int32_t nseg, void* stream);

/* Synchronise `stream` and report device-side errors of earlier runs on this
 * plan (APSEP_ETIMEOUT / APSEP_EINTERNAL, APSEP_EINVAL for bad segment
 * offsets), clearing them. */
apsep_status apsep_plan_check(apsep_plan* plan, void* stream);

/* Enqueue on `stream` a copy of the plan's sticky device-side error word into
 * *host_word (pinned host memory; nonzero = some earlier run on this plan hit
 * an error), without synchronising.  A caller that keeps many runs in flight
 * reads the word once the stream has passed the copy, and calls
 * apsep_plan_check (which decodes and clears the error) only when it is
 * nonzero, so a failure is tied to the runs before that copy.  No counterpart
 * in the reference (its gpuAssert exits the process). */
apsep_status apsep_plan_error_async(apsep_plan* plan, uint32_t* host_word, void* stream);

/* Plan facts (capacity, scratch bytes, tile size, configuration). */
apsep_status apsep_plan_get_info(const apsep_plan* plan, apsep_plan_info* info);

/* Select a kernel configuration (autotuner hook); 0 <= config < apsep_num_configs(). */
apsep_status apsep_plan_set_config(apsep_plan* plan, int32_t config);
int32_t apsep_num_configs(void);
/* threads per CTA and keys per thread of a configuration */
apsep_status apsep_config_shape(int32_t config, int32_t* threads, int32_t* keys_per_thread);

/* One-shot: plan, run on the legacy default stream, synchronise, free.
 * (launchSPT / launchWSTL) */
apsep_status apsep_launch(const void* d_in, int32_t* d_out, int64_t n, apsep_dtype dtype, apsep_cmp cmp);

/* Largest capacity of a plan (int32 positions, whole tiles below 2^31). */
#define APSEP_MAX_KEYS 2147479552LL

/* Largest n apsep_run_noalloc accepts (2^22 keys). */
#define APSEP_NOALLOC_MAX_KEYS 4194304

/* apsep_run without any device allocation, for callers that cannot allocate
 * device memory at call time (a process that reserved the whole device heap
 * for its own pool, or a path where cudaMalloc/cudaFree and their implicit
 * synchronisation are not allowed).  No counterpart in the reference: its
 * every entry point allocates or takes caller-allocated scratch.
 * The scratch is a static device array sized for APSEP_NOALLOC_MAX_KEYS keys
 * (2,902,272 bytes, held on every GPU that loads the library until exit);
 * n > APSEP_NOALLOC_MAX_KEYS returns APSEP_EINVAL; a device below compute
 * capability 10 returns APSEP_ENOTSUP.  Every call looks up the array's
 * address (a lookup that allocates nothing); the first call in each CUDA
 * context on a device -- the first of the process, and the first after
 * cudaDeviceReset or a switch to another context -- clears the array and
 * initialises it, so make that first call before any stream capture.  All
 * calls share the array: calls whose kernels overlap on the GPU race, so
 * serialise them (e.g. one stream).  Asynchronous on `stream`; device-side
 * errors stay in the array until apsep_noalloc_check reads them. */
apsep_status apsep_run_noalloc(const void* d_in, int32_t* d_out, int64_t n, apsep_dtype dtype, apsep_cmp cmp,
                               void* stream);

/* The device-side error state of apsep_run_noalloc on the current device
 * (the counterpart of apsep_plan_check, and like it no counterpart in the
 * reference): synchronises `stream`, then returns APSEP_ETIMEOUT if a wait
 * of an earlier run gave up, APSEP_EINTERNAL if a search invariant failed,
 * else APSEP_OK, and clears the error (the answers of a run that reported
 * one are not valid).  Allocates nothing. */
apsep_status apsep_noalloc_check(void* stream);

/* ---- Consumers of APSE ------------------------------------------------------
 * The classic callers the reference names for its output (README.md:3,
 * src/bench_spt_le.cu:1-3), each one or two runs on `plan` (whose key type
 * they use; n <= its capacity) -- with 4-byte keys and 16-byte aligned keys
 * and answers the engine flips or reverses the keys as it loads them (next
 * smaller: n a multiple of 32), else memory-bound flip / reverse / mirror
 * passes around plain runs -- asynchronous on `stream` like apsep_run.  d_work: a 16-byte aligned device workspace of
 * apsep_consumer_workspace_bytes(n) bytes, not overlapping the inputs or
 * outputs.  Device-side errors of the inner runs surface through
 * apsep_plan_check. */
int64_t apsep_consumer_workspace_bytes(int64_t n);

/* d_out[i] = the largest j < i with a[j] > a[i] (APSEP_LT) or a[j] >= a[i]
 * (APSEP_LE), else -1: APSE of the order-reversed keys. */
apsep_status apsep_run_prev_greater(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                                    void* d_work, void* stream);

/* d_out[i] = the smallest j > i with a[j] < a[i] (APSEP_LT) or a[j] <= a[i]
 * (APSEP_LE), else -1: APSE of the reversed array, mirrored back. */
apsep_status apsep_run_next_smaller(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, apsep_cmp cmp,
                                    void* d_work, void* stream);

/* Stock span: d_out[i] = i - (the largest j < i with a[j] > a[i], else -1),
 * the number of consecutive keys ending at i that are <= a[i]. */
apsep_status apsep_stock_span(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, void* d_work,
                              void* stream);

/* Largest rectangle in a histogram of int32 heights >= 0 (an int32 plan):
 * *d_area (device int64) = max over i of h[i] * (R - L - 1), L the previous
 * and R the next strictly smaller index (-1 / n when none); 0 for n == 0. */
apsep_status apsep_largest_rectangle(apsep_plan* plan, const int32_t* d_heights, int64_t n, int64_t* d_area,
                                     void* d_work, void* stream);

/* Min-rooted Cartesian tree: d_out[i] = the parent of i (-1 at the root),
 * ties as the stack construction makes them (a later equal key becomes the
 * right child of an earlier one).  The parent is, of the previous
 * smaller-or-equal and the next strictly smaller key, the larger one (the
 * next on a tie). */
apsep_status apsep_cartesian_parents(apsep_plan* plan, const void* d_in, int32_t* d_out, int64_t n, void* d_work,
                                     void* stream);

/* ---- 64-bit positions: arrays of any length -------------------------------
 * d_out[i] (int64) = the largest j < i with a[j] < a[i] (APSEP_LT) or
 * a[j] <= a[i] (APSEP_LE), else -1, for n up to APSEP_MAX_KEYS64 keys of the
 * plan's type: the reference's entry points take `int n`
 * (src/apsep.cuh:3052-3076) while its key types anticipate longer arrays
 * (src/apsep.cuh:62-70).  The array runs as consecutive pieces of the plan's
 * capacity (rounded down to whole 32-key groups; the whole array when
 * n <= capacity), one engine run each writing b0 + answer as int64; keys
 * that no key of their own piece answers are answered from a hierarchy of
 * minima over the keys before the piece.  d_work: a 16-byte aligned device workspace of
 * apsep_run64_workspace_bytes(plan, n) bytes (-1: n out of range, or a plan
 * with capacity < 32 for n > capacity), not overlapping the keys or d_out
 * (8-byte aligned).  Asynchronous on `stream` and graph-capturable like
 * apsep_run; device-side errors surface through apsep_plan_check. */
#define APSEP_MAX_KEYS64 1099511627776LL /* 2^40 */
int64_t apsep_run64_workspace_bytes(const apsep_plan* plan, int64_t n);
apsep_status apsep_run64(apsep_plan* plan, const void* d_in, int64_t* d_out, int64_t n, apsep_cmp cmp,
                         void* d_work, void* stream);

/* Copy nspans byte spans, src[i] -> dst[i] (bytes[i] bytes each; device
 * memory, or host memory the device can address; spans must not overlap),
 * in one kernel launch per 256 spans, asynchronously on `stream`.  The
 * serving layer's gather of admitted requests' keys into its device pool
 * and scatter of their answers: one call instead of one memcpy per request.
 * No counterpart in the reference (it has no serving layer). */
apsep_status apsep_copy_spans(const void* const* src, void* const* dst, const int64_t* bytes, int32_t nspans,
                              void* stream);

/* Fault injection for failure-detection tests: in the next run, range `range`
 * (the contiguous block of tiles one persistent warp sweeps) never publishes
 * its look-back status, and every device wait gives up after `spin_limit`
 * polls, so its successors report APSEP_ETIMEOUT through apsep_plan_check
 * instead of hanging.  range = -1 restores normal runs (spin_limit 0 =
 * default).  plan = NULL arms the next apsep_run_noalloc call instead
 * (reported by apsep_noalloc_check). */
apsep_status apsep_debug_inject(apsep_plan* plan, int32_t range, uint32_t spin_limit);

#ifdef __cplusplus
}
#endif

#endif /* APSEP_H_ */
