// xss_internal.cuh -- declarations shared by the kernel translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include "xss_keys.cuh"
#include "xss_prof.cuh"
#include "../../include/xss_gpu.h"

namespace xss {

// Value type of a keys-only sort.
struct NoVal {};

// Operation families understood by the sort engine.
enum SortOp : int { SOP_KEYS = 0, SOP_KV = 1, SOP_ARG = 2 };

constexpr int RADIX_BITS = 8;
constexpr int RADIX = 1 << RADIX_BITS;
constexpr int MAX_PASSES = 8;
constexpr uint32_t FLAG_AGG = 1u << 30;     // tile aggregate published
constexpr uint32_t FLAG_PRE = 2u << 30;     // inclusive prefix published
constexpr uint32_t FLAG_MASK = 3u << 30;
constexpr uint32_t COUNT_MASK = (1u << 30) - 1;

// Keys one radix sort takes: its look-back words hold a 30-bit count and its
// tile arithmetic is 32-bit.  Larger arrays are sorted in chunks of at most
// this size and merged (xss_merge.cu).
constexpr size_t XSS_RADIX_MAX_N = (size_t(1) << 30) - 1;

// Inputs up to this size are sorted by one CTA in shared memory.
constexpr size_t SMALL_SORT_MAX = 4096;

// Per-pass plan written on the device by the histogram kernel.
struct PassDesc {
    int active;      // 0: every key has the same digit -> pass skipped
    int src, dst;    // key buffer ids (0 = caller array, 1/2 = scratch)
    int vsrc, vdst;  // value buffer ids
    int first;       // load applies the key transform
    int last;        // store applies the inverse transform
    int gen_idx;     // values are the element index (argsort, first pass)
    int skip_keys;   // keys are not stored (argsort, last pass)
    int out_idx;     // values go to the 64-bit index output (argsort, last pass)
    int tie_free;    // keys only, first pass: ties need no order (unstable ranking)
};

enum FixupMode : int { FIX_NONE = 0, FIX_COPY = 1, FIX_CANON = 2, FIX_IOTA = 3 };

struct RadixHeader {
    uint32_t hist[MAX_PASSES][RADIX];
    uint32_t start[MAX_PASSES][RADIX];
    PassDesc desc[MAX_PASSES];
    uint32_t tile_ctr[MAX_PASSES];
    uint32_t done_ctr;
    int fixup;
    int num_active;
    int pad;
};

struct RadixArgs {
    void *kbuf[3];
    void *vbuf[3];
    uint64_t *out_idx;
    size_t n;
    uint32_t num_tiles;
    int passes;
    int op;
    KeyXform xf;
    RadixHeader *hdr;
    uint32_t *status;      // [passes][num_tiles][RADIX]
    unsigned *err;         // device-visible error word
};

constexpr size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Device-visible error word (mapped pinned host memory); see xss_capi.cu.
unsigned *device_error_word();

// ---- launchers (defined in the .cu files) --------------------------------
size_t radix_workspace_bytes(int op, int kbytes, int vbytes, size_t n);
int radix_sort(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
               uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s);

// Chunked sorts of arrays above XSS_RADIX_MAX_N keys (xss_merge.cu): chunks
// radix-sorted in place, then merged pairwise.  radix_sort / radix_select and
// radix_workspace_bytes route there by size.
bool big_sort_needed(size_t n);
size_t big_sort_workspace_bytes(int op, int kbytes, int vbytes, size_t n);
int big_sort(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
             uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s);

// Host-pointer sorts from PIPE_MIN_N keys on: chunk copies overlapped with
// chunk sorts, merged, copied back slice by slice (xss_merge.cu).  hk / hv /
// hidx are host pointers; the call returns once the results are on the host.
constexpr size_t PIPE_MIN_N = size_t(1) << 22;
bool host_pipeline_wanted(size_t n);
// One CPU read per page of a host range, right before a copy reads it
// (xss_capi.cu explains why).
void touch_host_pages(const void *p, size_t bytes);
int host_pipelined_sort(int op, int kbytes, KeyXform xf, void *hk, void *hv, int vbytes,
                        uint64_t *hidx, size_t n);
// Free the calling thread's pipeline buffer on the current device (its
// streams stay); the caller has synchronised the device.  False if the free
// failed.
bool release_pipeline_buffer();

// Keys-only sorts of 16-bit keys above COUNT16_MIN_N keys count every code
// instead of radix sorting (xss_count16.cu); radix_sort, radix_select and
// their workspace sizes route there.  canon_end: sorted positions below it
// get canonical NaNs when xf.canon is set.
constexpr size_t COUNT16_MIN_N = size_t(1) << 15;
bool count16_wanted(int op, int kbytes, size_t n);
size_t count16_workspace_bytes(size_t n);
int count16_sort(KeyXform xf, void *keys, size_t n, size_t canon_end, void *ws, size_t ws_bytes,
                 cudaStream_t s);

// Workspace of radix_sort_chunk (a radix sort of at most XSS_RADIX_MAX_N keys,
// never the counting form).
size_t radix_chunk_workspace_bytes(int op, int kbytes, int vbytes, size_t n);

size_t select_workspace_bytes(int op, int kbytes, int vbytes, size_t n);
// Partition so that position k holds the k-th element in code order,
// smaller codes before it and larger after.  keys are modified in place for
// SOP_KEYS / SOP_KV; for SOP_ARG keys are read-only and out_idx receives the
// partitioned index permutation.
int radix_select(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
                 uint64_t *out_idx, size_t k, size_t n, void *ws, size_t ws_bytes,
                 cudaStream_t s);

int num_sms();

// Raise a kernel's dynamic shared-memory limit to `bytes`, once per (kernel,
// device); thread-safe.  Returns XSS_OK or XSS_ECUDA.
int set_max_dyn_smem(const void *kernel, size_t bytes);

// Per host thread: sort arrays of every size with the mid-size pass lines
// (several CTAs per SM), so kernels of concurrent requests on other streams
// share the SMs.  The serving loop's scheduler thread sets it.
void set_prefer_shared_sm(bool on);

// Library-owned scratch for (current device, stream), grown on demand.
int cached_workspace(cudaStream_t s, size_t bytes, void **out);

}  // namespace xss

// Launch bracketed by the profiler hooks (launch count, optional event timing).
#define XSS_LAUNCH(kind, stream, ...)      \
    do {                                    \
        ::xss::prof_begin(stream, kind);    \
        __VA_ARGS__;                        \
        ::xss::prof_end(stream, kind);      \
    } while (0)

#define XSS_CUDA_TRY(expr)                                  \
    do {                                                    \
        cudaError_t _e = (expr);                            \
        if (_e != cudaSuccess) return XSS_ECUDA;            \
    } while (0)
