/*
 * xss_gpu.h -- C ABI of the GB300 sort/select library (libxss_gb300.so).
 *
 * Every entry point takes plain pointers and sizes.  Device-pointer entry
 * points (xss_gpu_*) run asynchronously on the caller's stream; host-pointer
 * entry points (xss_*) stage through device memory and return when the
 * result is back in the caller's buffers.
 *
 * Semantics follow the reference library intel/x86-simd-sort:
 *   - ordering: integers by value; floats with NaN after +inf (ascending) or
 *     before it (descending), -0.0 and +0.0 adjacent (utils/custom-compare.h:11-34);
 *   - qsort with hasnan writes the canonical quiet NaN into the NaN slots
 *     (src/xss-common-qsort.h:107-135; _Float16 uses bits 0x7c01,
 *     src/xss-custom-float.h:81-85);
 *   - keyvalue / argsort / select keep NaN payload bits;
 *   - k counts from the front of the requested order (descending included).
 * Sorts are unstable, as in the reference.
 */
#ifndef XSS_GPU_H
#define XSS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same handle type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st *xss_stream_t;

/* Status codes returned by every int-returning entry point. */
enum {
    XSS_OK = 0,
    XSS_EINVAL = 1,      /* bad dtype / k >= n / null pointer with n > 1 */
    XSS_ENOMEM = 2,      /* workspace too small or device allocation failed */
    XSS_ETIMEOUT = 3,    /* a bounded device-side wait gave up (result invalid) */
    XSS_ECUDA = 4,       /* a CUDA runtime call failed */
    XSS_EUNSUPPORTED = 5,/* type combination the reference does not offer */
    XSS_ETOOBIG = 6,     /* n above the library limit (XSS_MAX_N) */
    XSS_EBUSY = 7,       /* server queue full or stopping: request refused */
    XSS_EAGAIN = 8       /* server request not finished yet */
};

/* Largest array the library accepts.  The reference has no ceiling (size_t
 * lengths, lib/x86simdsort.h:16-18); this bound only keeps byte counts far
 * from overflow and lies beyond any device's memory.  Arrays above 2^30 - 1
 * keys are sorted in chunks of up to that size and merged; segments of a
 * batched segmented sort are each limited to XSS_SEGMENT_MAX_N keys. */
#define XSS_MAX_N ((size_t)1 << 40)
#define XSS_SEGMENT_MAX_N ((size_t)((1u << 30) - 1))

/* Key / value element types (the reference's nine key types). */
enum {
    XSS_DT_U16 = 0, XSS_DT_I16 = 1, XSS_DT_F16 = 2,
    XSS_DT_U32 = 3, XSS_DT_I32 = 4, XSS_DT_F32 = 5,
    XSS_DT_U64 = 6, XSS_DT_I64 = 7, XSS_DT_F64 = 8
};

/* Operation ids for xss_gpu_workspace_size. */
enum {
    XSS_OP_QSORT = 0, XSS_OP_QSELECT = 1, XSS_OP_PARTIAL_QSORT = 2,
    XSS_OP_ARGSORT = 3, XSS_OP_ARGSELECT = 4,
    XSS_OP_KV_QSORT = 5, XSS_OP_KV_SELECT = 6, XSS_OP_KV_PARTIAL_SORT = 7
};

const char *xss_strerror(int status);
/* Library version string. */
const char *xss_version(void);

/*
 * Bytes of device scratch the call (op, key dtype, value dtype, n, k) needs.
 * val_dtype is ignored for ops without values.  Passing d_ws = NULL to a
 * device entry point makes the library use its own cached per-stream
 * workspace instead (grown on demand, never shrunk).
 */
size_t xss_gpu_workspace_size(int op, int key_dtype, int val_dtype, size_t n, size_t k);

/*
 * Frees the device memory the library keeps between calls on the current
 * device: the cached workspaces of every stream (device-pointer calls given
 * d_ws = NULL, and the device record sort), and the calling thread's staging
 * and pipeline buffers of host-pointer calls (each thread that makes
 * host-pointer calls holds its own, up to about twice the bytes of its
 * largest array).  Waits for all work on the device first.  Buffers of other
 * threads' host-pointer calls stay: each thread releases its own, e.g. before
 * it exits.  Later calls allocate again as needed.  Not to be called while
 * another thread is inside a call of this library on the same device.
 * Returns XSS_OK or XSS_ECUDA.  No counterpart in the reference library (a CPU
 * library keeps no device memory).
 */
int xss_release_cached(void);

/*
 * Device-pointer calls are asynchronous.  Kernels that give up a bounded wait
 * latch an error word on the device; this call synchronises `stream`, reads
 * and clears that word and returns XSS_OK, XSS_ETIMEOUT or XSS_ECUDA.
 */
int xss_gpu_stream_status(xss_stream_t stream);

/*
 * Self test of the device-side bounded waits: runs the look-back spin
 * (which = 0) or the bulk-copy mbarrier wait (which = 1) against a condition
 * that never becomes true, with the given spin limit.  Returns XSS_ETIMEOUT
 * when the wait gave up as designed (synchronises `stream`).  Diagnostic
 * only; no counterpart in the reference library.
 */
int xss_gpu_selftest_bounded_wait(int which, unsigned spin_limit, xss_stream_t stream);

/*
 * Self test of the hardware property the radix pass's ranking relies on (no
 * counterpart in the reference): shared-memory atomic adds that lanes of one
 * warp instruction make to one address return their results in lane order.
 * Runs about 300 million such adds of many collision patterns on the current
 * device and stores the number that broke lane order in *violations (0 on
 * every GB300 measured).  Synchronous.
 */
int xss_gpu_selftest_rank_order(unsigned long long *violations, xss_stream_t stream);

/* ------------------------------------------------------------------ */
/* Device-pointer entry points.  Arrays live in device memory; work is   */
/* enqueued on `stream` and the call returns without synchronising      */
/* (except when the cached workspace grows).  A bounded wait that gave  */
/* up is reported later by xss_gpu_stream_status.                       */
/* ------------------------------------------------------------------ */

/* x86simdsort::qsort (lib/x86simdsort.h:15-18) */
int xss_gpu_qsort(int dtype, void *d_arr, size_t n, int hasnan, int descending,
                  void *d_ws, size_t ws_bytes, xss_stream_t stream);
/* x86simdsort::qselect (lib/x86simdsort.h:20-26) */
int xss_gpu_qselect(int dtype, void *d_arr, size_t k, size_t n, int hasnan,
                    int descending, void *d_ws, size_t ws_bytes, xss_stream_t stream);
/* x86simdsort::partial_qsort (lib/x86simdsort.h:28-34) */
int xss_gpu_partial_qsort(int dtype, void *d_arr, size_t k, size_t n, int hasnan,
                          int descending, void *d_ws, size_t ws_bytes,
                          xss_stream_t stream);
/* x86simdsort::argsort (lib/x86simdsort.h:36-39); d_arg receives n indices. */
int xss_gpu_argsort(int dtype, const void *d_arr, uint64_t *d_arg, size_t n,
                    int hasnan, int descending, void *d_ws, size_t ws_bytes,
                    xss_stream_t stream);
/* x86simdsort::argselect (lib/x86simdsort.h:41-44); no descending form. */
int xss_gpu_argselect(int dtype, const void *d_arr, uint64_t *d_arg, size_t k,
                      size_t n, int hasnan, void *d_ws, size_t ws_bytes,
                      xss_stream_t stream);
/* x86simdsort::keyvalue_qsort (lib/x86simdsort.h:46-52); 32/64-bit keys and values. */
int xss_gpu_keyvalue_qsort(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                           size_t n, int hasnan, int descending, void *d_ws,
                           size_t ws_bytes, xss_stream_t stream);
/* x86simdsort::keyvalue_select (lib/x86simdsort.h:54-61) */
int xss_gpu_keyvalue_select(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                            size_t k, size_t n, int hasnan, int descending,
                            void *d_ws, size_t ws_bytes, xss_stream_t stream);
/* x86simdsort::keyvalue_partial_sort (lib/x86simdsort.h:63-70) */
int xss_gpu_keyvalue_partial_sort(int key_dtype, int val_dtype, void *d_keys,
                                  void *d_vals, size_t k, size_t n, int hasnan,
                                  int descending, void *d_ws, size_t ws_bytes,
                                  xss_stream_t stream);

/*
 * Allocation-free device qsort.  No counterpart in the reference library.
 *
 * For callers that cannot allocate device memory when they sort: code running
 * inside a memory allocator or an out-of-memory handler, plugins whose host
 * application owns every device allocation, fixed-budget real-time loops.
 * Same semantics as xss_gpu_qsort, but it never calls cudaMalloc / cudaFree or
 * any allocating routine: its scratch is a fixed 12 MiB array compiled into
 * the library's device image (held on every GPU that loads the library until
 * the process exits), which limits n to XSS_NOALLOC_MAX_N keys of any type;
 * larger n returns XSS_ETOOBIG without touching the array.
 *
 * The call is synchronous: it returns once the sort on `stream` is done, with
 * XSS_OK or XSS_ETIMEOUT from the device-side checks.  The first call on each
 * device is its set-up: it looks up the array's device address and loads onto
 * that device every kernel a call can launch (CUDA loads kernel code lazily,
 * and that load does allocate device memory), by sorting small arrays inside
 * the array itself.  Make that first call once per device, outside the code
 * that must not allocate; every later call on the device allocates nothing.
 * No call can be made while its stream is being captured (into a CUDA graph):
 * each one copies its status word to the host and synchronises the stream.
 * All calls share the one array and find the
 * previous call's data in it: calls whose GPU work could overlap (other
 * streams, other host threads) race on it and must be serialised by the caller.
 */
#define XSS_NOALLOC_MAX_N ((size_t)1 << 20)
int xss_gpu_qsort_noalloc(int dtype, void *d_arr, size_t n, int hasnan, int descending,
                          xss_stream_t stream);

/*
 * Batched segmented sort: sorts each segment [offsets[i], offsets[i+1]) of
 * d_keys (and d_vals when non-NULL) independently, in one launch sequence.
 * d_offsets holds num_segments+1 non-decreasing uint64 offsets in device
 * memory; h_offsets is the same array in host memory (used to bin segments
 * by size on the host; may be NULL, then it is read back from the device).
 */
int xss_gpu_segmented_sort(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                           const uint64_t *d_offsets, const uint64_t *h_offsets,
                           size_t num_segments, int hasnan, int descending,
                           void *d_ws, size_t ws_bytes, xss_stream_t stream);
size_t xss_gpu_segmented_workspace_size(int key_dtype, int val_dtype,
                                        const uint64_t *h_offsets,
                                        size_t num_segments);

/*
 * Batched segmented top-k (no counterpart in the reference, which has no
 * segmented form): for every segment, its min(k, length) smallest keys
 * (largest when descending) in order at the segment's front, with their
 * values; the rest of the segment holds its other keys in any order -- a
 * partial_qsort per segment, with the reference's partial_qsort semantics
 * (lib/x86simdsort.h:27-29).  Runs in the batched segmented launch: segments
 * up to 4096 keys are sorted on chip whole (which costs no more than their
 * top k).  For k <= 2048 each longer segment is read once by one CTA, which
 * keeps the best k so far on chip and merges in only the keys below the
 * current k-th (their places in the segment take the keys they displace);
 * for a larger k the longer segments are sorted by the segmented radix sort.
 * k == 0: no-op.  Workspace: xss_gpu_segmented_workspace_size is enough.
 */
int xss_gpu_segmented_topk(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                           const uint64_t *d_offsets, const uint64_t *h_offsets,
                           size_t num_segments, size_t k, int hasnan, int descending,
                           void *d_ws, size_t ws_bytes, xss_stream_t stream);

/*
 * Reusable plan for a fixed segment layout.  The segments are binned by size
 * once (<= 32 keys: a warp each; <= 4096: a CTA each; larger: one segmented
 * radix sort over all of them).  xss_seg_plan_run enqueues the whole batch on
 * `stream`; with use_graph != 0 the launch sequence is captured into a CUDA
 * graph on the first run and replayed while keys, values, offsets and
 * workspace stay the same pointers.  val_dtype < 0: keys only.  A plan is not
 * safe to run from two host threads at once.
 */
typedef struct xss_seg_plan_s *xss_seg_plan;
int xss_seg_plan_create(xss_seg_plan *out, int key_dtype, int val_dtype,
                        const uint64_t *h_offsets, size_t num_segments, int hasnan,
                        int descending);
size_t xss_seg_plan_workspace_size(const struct xss_seg_plan_s *plan);
int xss_seg_plan_run(xss_seg_plan plan, void *d_keys, void *d_vals, const uint64_t *d_offsets,
                     void *d_ws, size_t ws_bytes, xss_stream_t stream, int use_graph);
void xss_seg_plan_destroy(xss_seg_plan plan);

/* The same batch sorted by one single-array call per segment (the baseline
 * the batched form is measured against). */
int xss_gpu_segmented_sort_percall(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                                   const uint64_t *h_offsets, size_t num_segments, int hasnan,
                                   int descending, xss_stream_t stream);

/*
 * Record sort on the device: sorts n records of rec_bytes bytes each in
 * d_recs by the 32- or 64-bit key of type key_dtype stored at byte offset
 * key_offset inside every record.  Device form of object_qsort
 * (lib/x86simdsort.h:73-106) for keys that are a member of the record: the
 * keys are read out on the GPU, sorted with the records' positions
 * (key-value sort) and the records are gathered into sorted order.  Equal
 * keys keep their input order.  Workspace: xss_gpu_object_workspace_size
 * (holds a copy of the records), or NULL for the library's cached one.
 */
int xss_gpu_object_qsort(void *d_recs, size_t n, size_t rec_bytes, size_t key_offset,
                         int key_dtype, int hasnan, int descending, void *d_ws,
                         size_t ws_bytes, xss_stream_t stream);
size_t xss_gpu_object_workspace_size(size_t n, size_t rec_bytes, int key_dtype);

/* ------------------------------------------------------------------ */
/* Instrumentation: per-kernel-kind launch counts (always on) and       */
/* optional CUDA-event timing of every launch on its own stream.        */
/* Kinds: 0 hist, 1 onesweep pass, 2 fixup, 3 small sort, 4 select      */
/* histogram, 5 select find, 6 partition collect, 7 partition place,    */
/* 8 segmented small, 9 segmented block, 10 segmented bookkeeping,      */
/* 11 record key extraction / gather.                                   */
/* ------------------------------------------------------------------ */
void xss_prof_enable(int on);
void xss_prof_reset(void);
int xss_prof_read(int kind, double *total_ms, unsigned long long *timed_launches);
unsigned long long xss_prof_launches(int kind);
const char *xss_prof_kind_name(int kind);

/* ------------------------------------------------------------------ */
/* Serving loop: a scheduler thread that takes sort / select / argsort / */
/* key-value requests on host buffers, admits them as device memory for */
/* their data and scratch frees up (continuous batching), coalesces     */
/* small same-kind requests into one segmented sort, runs large ones on */
/* a pool of streams so their copies and kernels overlap, and keeps     */
/* arrival-to-completion latencies.  Host buffers should be pinned for  */
/* the copies to overlap.  No counterpart in the reference library.     */
/* ------------------------------------------------------------------ */
typedef struct xss_serve_request {
    int op;                 /* XSS_OP_* */
    int key_dtype, val_dtype;
    const void *keys_in;    /* n keys (host) */
    void *keys_out;         /* result keys (may equal keys_in); unused for arg ops */
    const void *vals_in;    /* key-value ops */
    void *vals_out;
    uint64_t *arg_out;      /* argsort / argselect: n indices */
    size_t n, k;
    int hasnan, descending;
} xss_serve_request;

typedef struct xss_server_config {
    int device;
    size_t hbm_budget_bytes;  /* device pool for data + scratch; 0: half of free memory */
    int streams;              /* streams for large requests; 0: 4 */
    size_t small_max;         /* requests up to this size are coalesced; 0: 65536 */
    size_t max_batch;         /* requests per coalesced launch; 0: 4096 */
    size_t max_queue;         /* queued requests before submissions are refused; 0: 1024 */
} xss_server_config;

typedef struct xss_server_stats {
    uint64_t submitted, shed, completed, failed, batches, batched_requests;
    double keys;              /* keys in completed requests */
    double wall_s;            /* since creation or the last reset */
    double p50_us, p99_us, max_us;  /* arrival -> completion */
    size_t pool_bytes;
} xss_server_stats;

typedef struct xss_server_s *xss_server;
int xss_server_create(xss_server *out, const xss_server_config *cfg);
/* XSS_OK and a ticket, or XSS_EBUSY when the queue is full (request shed). */
int xss_server_submit(xss_server s, const xss_serve_request *req, uint64_t *ticket);
/* Block until the request is done; *status is its result code. */
int xss_server_wait(xss_server s, uint64_t ticket, int *status);
/* XSS_OK with *status when done, XSS_EAGAIN while pending. */
int xss_server_poll(xss_server s, uint64_t ticket, int *status);
int xss_server_get_stats(xss_server s, xss_server_stats *out);
int xss_server_reset_stats(xss_server s);
/* Stop admitting; drain != 0 finishes queued work, else refuses it (XSS_EBUSY). */
void xss_server_destroy(xss_server s, int drain);

/* ------------------------------------------------------------------ */
/* Host-pointer entry points: copy in, run on the device, copy back.     */
/* ------------------------------------------------------------------ */
int xss_qsort(int dtype, void *arr, size_t n, int hasnan, int descending);
int xss_qselect(int dtype, void *arr, size_t k, size_t n, int hasnan, int descending);
int xss_partial_qsort(int dtype, void *arr, size_t k, size_t n, int hasnan,
                      int descending);
int xss_argsort(int dtype, const void *arr, uint64_t *arg, size_t n, int hasnan,
                int descending);
int xss_argselect(int dtype, const void *arr, uint64_t *arg, size_t k, size_t n,
                  int hasnan);
int xss_keyvalue_qsort(int key_dtype, int val_dtype, void *keys, void *vals,
                       size_t n, int hasnan, int descending);
int xss_keyvalue_select(int key_dtype, int val_dtype, void *keys, void *vals,
                        size_t k, size_t n, int hasnan, int descending);
int xss_keyvalue_partial_sort(int key_dtype, int val_dtype, void *keys, void *vals,
                              size_t k, size_t n, int hasnan, int descending);

/* ------------------------------------------------------------------ */
/* The reference's own C symbols (lib/x86simdsort.cpp:298-339): host    */
/* pointers, ascending, hasnan = true.  Errors abort with a message, as */
/* the reference has no error channel here.                             */
/* ------------------------------------------------------------------ */
void keyvalue_qsort_float_uint32(float *key, uint32_t *val, size_t size);
void keyvalue_qsort_float_uint64(float *key, uint64_t *val, size_t size);
void keyvalue_qsort_uint64_uint32(uint64_t *key, uint32_t *val, size_t size);
void keyvalue_qsort_uint64_uint64(uint64_t *key, uint64_t *val, size_t size);
void keyvalue_qsort_int32_uint32(int32_t *key, uint32_t *val, size_t size);
void keyvalue_qsort_int32_uint64(int32_t *key, uint64_t *val, size_t size);
void keyvalue_qsort_uint32_uint32(uint32_t *key, uint32_t *val, size_t size);
void keyvalue_qsort_uint32_uint64(uint32_t *key, uint64_t *val, size_t size);

#ifdef __cplusplus
}
#endif

#endif /* XSS_GPU_H */
