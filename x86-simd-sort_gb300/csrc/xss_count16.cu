// xss_count16.cu -- keys-only sorts of 16-bit keys (uint16, int16, _Float16)
// by counting.  A 16-bit key has only 65,536 possible codes, so one read of
// the array gives the count of every code, a scan of those counts gives each
// code's first position, and one write expands the codes back into the array
// in order.  Two memory passes (read 2 bytes, write 2 bytes per key) replace
// the up-front histogram and two 8-bit radix passes (10 bytes per key).
//
// Serves qsort, and qselect / partial_qsort too: a sorted array satisfies
// their contract (the k-th element in place, nothing larger before it,
// nothing smaller after it).  The output holds exactly the input's bit
// patterns -- codes are a bijection of the key bits -- except that the sorted
// positions below `canon_end` write the canonical quiet NaN for every NaN
// when the sort canonicalises (qsort with hasnan, and the sorted prefix of
// partial_qsort), as the reference's qsort does (src/xss-common-qsort.h:107-135,
// src/xss-custom-float.h:81-85).  Replaces, for 16-bit keys:
//   src/avx512-16bit-qsort.hpp:583-670    (qsort / qselect / partial_qsort, fp16)
//   src/avx512fp16-16bit-qsort.hpp:172-199 (NaN handling of native _Float16)
#include <algorithm>
#include "xss_internal.cuh"

namespace xss {

constexpr int C16_BINS = 1 << 16;
constexpr int C16_WORDS = C16_BINS / 2;                // two 16-bit counters per word
constexpr int C16_HIST_BLOCK = 1024;
constexpr size_t C16_SMEM = size_t(C16_WORDS) * 4;     // 128 KiB of counters per CTA
constexpr int C16_EXPAND_BLOCK = 256;
constexpr int C16_GROUP = 8;                           // keys per thread per step (16 bytes)

struct C16Args {
    uint16_t *keys;
    size_t n;
    size_t canon_end;            // sorted positions below this canonicalise NaNs
    KeyXform xf;
    uint32_t *part;              // [grid][C16_WORDS] per-CTA packed counts
    unsigned long long *over;    // [C16_BINS] counts moved out of the shared counters
    unsigned long long *start;   // [C16_BINS + 1] first position of each code; start[BINS] = n
};

// Elements before the first 16-byte boundary of the array (keys are 2-byte aligned).
__device__ __forceinline__ size_t c16_head(const uint16_t *p, size_t n)
{
    const size_t mis = (reinterpret_cast<uintptr_t>(p) & 15) / 2;
    return min(n, mis ? (size_t)(8 - mis) : (size_t)0);
}

// Counts of every code.  Each CTA keeps 16-bit counters in shared memory, two
// per word.  A counter that reaches 0x8000 is moved out: the thread whose
// increment took it there (exactly one, since increments are atomic and by
// one) subtracts 0x8000 from the word and adds it to the code's 64-bit global
// overflow count.  Fewer than 0x8000 further increments can reach the word
// before that subtraction lands (at most one in flight per thread), so a
// counter never carries into its neighbour.  At the end each CTA stores its
// counters as they are; the reduce kernel adds every CTA's and the overflow.
__global__ void __launch_bounds__(C16_HIST_BLOCK, 1) c16_hist_kernel(C16Args a)
{
    extern __shared__ __align__(16) uint32_t sh[];
    const int tid = threadIdx.x;
    for (int i = tid; i < C16_WORDS; i += C16_HIST_BLOCK) sh[i] = 0;
    __syncthreads();
    const Codec<uint16_t> cx(a.xf);
    auto count = [&](uint16_t b) {
        const uint32_t c = cx.to(b);
        const uint32_t s16 = (c & 1u) << 4;
        const uint32_t old = atomicAdd(&sh[c >> 1], 1u << s16);
        if (((old >> s16) & 0xFFFFu) == 0x7FFFu) {
            atomicSub(&sh[c >> 1], 0x8000u << s16);
            atomicAdd(&a.over[c], 0x8000ull);
        }
    };
    const uint16_t *src = a.keys;
    const size_t n = a.n;
    const size_t head = c16_head(src, n);
    const size_t gtid = (size_t)blockIdx.x * C16_HIST_BLOCK + tid;
    const size_t stride = (size_t)gridDim.x * C16_HIST_BLOCK;
    if (gtid < head) count(src[gtid]);
    const size_t nvec = (n - head) / C16_GROUP;
    const uint4 *vsrc = reinterpret_cast<const uint4 *>(src + head);
    constexpr int U = 4;   // 16-byte loads per thread in flight
    for (size_t v0 = gtid; v0 < nvec; v0 += U * stride) {
        uint4 q[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const size_t v = v0 + (size_t)u * stride;
            q[u] = v < nvec ? vsrc[v] : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (v0 + (size_t)u * stride >= nvec) continue;
            const uint32_t w[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                count((uint16_t)(w[j] & 0xFFFFu));
                count((uint16_t)(w[j] >> 16));
            }
        }
    }
    const size_t tail0 = head + nvec * C16_GROUP;
    if (tail0 + gtid < n) count(src[tail0 + gtid]);
    __syncthreads();
    uint4 *dst = reinterpret_cast<uint4 *>(a.part + (size_t)blockIdx.x * C16_WORDS);
    const uint4 *s4 = reinterpret_cast<const uint4 *>(sh);
    for (int i = tid; i < C16_WORDS / 4; i += C16_HIST_BLOCK) dst[i] = s4[i];
}

// Total of every code (the CTAs' counters plus the overflow) and its first
// position within its block of 1024 codes; one CTA per block, one counter
// word (two codes) per thread.  The block totals go to bsum.
constexpr int C16_SCAN_BLOCK = 256;                        // words per block
constexpr int C16_SCAN_CODES = 2 * C16_SCAN_BLOCK;         // codes per block
constexpr int C16_NBLK = C16_BINS / C16_SCAN_CODES;        // 128
__global__ void __launch_bounds__(C16_SCAN_BLOCK) c16_reduce_kernel(C16Args a, int parts,
                                                                     unsigned long long *bsum)
{
    __shared__ unsigned long long s_warp[C16_SCAN_BLOCK / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int w = blockIdx.x * C16_SCAN_BLOCK + tid;
    unsigned long long lo = a.over[2 * w], hi = a.over[2 * w + 1];
#pragma unroll 8
    for (int c = 0; c < parts; ++c) {
        const uint32_t v = a.part[(size_t)c * C16_WORDS + w];
        lo += v & 0xFFFFu;
        hi += v >> 16;
    }
    const unsigned long long sum = lo + hi;
    unsigned long long x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long t = lane < C16_SCAN_BLOCK / 32 ? s_warp[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < C16_SCAN_BLOCK / 32) s_warp[lane] = t;
    }
    __syncthreads();
    const unsigned long long ex = (warp ? s_warp[warp - 1] : 0ull) + x - sum;
    a.start[2 * w] = ex;
    a.start[2 * w + 1] = ex + lo;
    if (tid == C16_SCAN_BLOCK - 1) bsum[blockIdx.x] = ex + sum;
}

// Add every block's offset (exclusive scan of the 128 block totals); start[BINS] = n.
__global__ void __launch_bounds__(1024) c16_offsets_kernel(C16Args a,
                                                           const unsigned long long *bsum)
{
    __shared__ unsigned long long s_off[C16_NBLK];
    const int tid = threadIdx.x, lane = tid & 31;
    constexpr int PER = C16_NBLK / 32;   // blocks per lane
    static_assert(C16_NBLK % 32 == 0, "whole blocks per lane");
    if (tid < 32) {
        unsigned long long b[PER], x = 0;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            b[i] = bsum[PER * lane + i];
            x += b[i];
        }
        const unsigned long long tot = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        unsigned long long ex = x - tot;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            s_off[PER * lane + i] = ex;
            ex += b[i];
        }
    }
    __syncthreads();
    for (int i = tid; i < C16_BINS; i += 1024) a.start[i] += s_off[i / C16_SCAN_CODES];
    if (tid == 0) a.start[C16_BINS] = a.n;
}

// The code at sorted position p (0 <= p < n): the last code whose first
// position is <= p, by binary search of start[lo .. hi] (start[lo] <= p,
// and p < start[hi + 1]).
__device__ __forceinline__ uint32_t c16_search(const unsigned long long *start, size_t p,
                                               uint32_t lo, uint32_t hi)
{
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (start[mid] <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Output chunks: C16_CHUNK positions from the first 16-byte boundary on
// (positions before it, fewer than eight, belong to chunk 0's first CTA).
constexpr int C16_EXPAND_ITERS = 4;                                      // 16-byte stores per thread
constexpr size_t C16_CHUNK = (size_t)C16_EXPAND_BLOCK * C16_GROUP * C16_EXPAND_ITERS;  // 8192
constexpr int C16_RANGE_MAX = 2047;   // codes per chunk held in shared memory

// first[q] = the code at the chunk's first position (q < chunks), and
// first[chunks] = the code at position n - 1; one search per thread.
__global__ void __launch_bounds__(256) c16_chunk_kernel(C16Args a, uint32_t *first,
                                                        size_t chunks, size_t head)
{
    const size_t q = (size_t)blockIdx.x * 256 + threadIdx.x;
    if (q > chunks) return;
    const size_t p = q < chunks ? head + q * C16_CHUNK : a.n - 1;
    first[q] = c16_search(a.start, p, 0, C16_BINS - 1);
}

// Write the sorted keys, one chunk per CTA: the starts of the chunk's codes
// come into shared memory (or, for a chunk spanning more codes than fit,
// are searched in place), then each thread writes 8 consecutive positions
// per 16-byte store, stepping to the next code where one ends.
__global__ void __launch_bounds__(C16_EXPAND_BLOCK) c16_expand_kernel(C16Args a,
                                                                      const uint32_t *first,
                                                                      size_t chunks, size_t head)
{
    __shared__ unsigned long long s_start[C16_RANGE_MAX + 2];
    const size_t q = blockIdx.x;
    const Codec<uint16_t> cx(a.xf);
    uint16_t *dst = a.keys;
    const size_t n = a.n;
    const uint32_t c0 = first[q], c1 = first[q + 1];
    const bool local = c1 - c0 <= (uint32_t)C16_RANGE_MAX;
    if (local)
        for (uint32_t i = threadIdx.x; i <= c1 - c0 + 1; i += C16_EXPAND_BLOCK)
            s_start[i] = a.start[c0 + i];
    __syncthreads();
    auto start_of = [&](uint32_t c) -> unsigned long long {
        return local ? s_start[c - c0] : a.start[c];
    };
    auto code_at = [&](size_t p, uint32_t lo) -> uint32_t {
        uint32_t hi = c1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (start_of(mid) <= p) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    };
    auto key_at = [&](size_t p, uint32_t c) -> uint16_t {
        return p < a.canon_end ? cx.from_canon((uint16_t)c) : cx.from((uint16_t)c);
    };
    if (q == 0 && threadIdx.x < head) {
        const size_t p = threadIdx.x;
        dst[p] = key_at(p, c16_search(a.start, p, 0, c0));
    }
    const size_t base = head + q * C16_CHUNK;
    uint32_t c = c0;
#pragma unroll 1
    for (int it = 0; it < C16_EXPAND_ITERS; ++it) {
        const size_t p0 = base + ((size_t)it * C16_EXPAND_BLOCK + threadIdx.x) * C16_GROUP;
        if (p0 >= n) break;
        const size_t p1 = min(n, p0 + C16_GROUP);
        c = code_at(p0, c);
        unsigned long long next = start_of(c + 1);
        if (p1 - p0 == C16_GROUP && p1 <= next && (p1 <= a.canon_end || p0 >= a.canon_end)) {
            // the common case: eight copies of one key
            const uint32_t k = key_at(p0, c);
            const uint32_t kk = k | (k << 16);
            *reinterpret_cast<uint4 *>(dst + p0) = make_uint4(kk, kk, kk, kk);
            continue;
        }
        uint16_t out[C16_GROUP];
#pragma unroll
        for (int j = 0; j < C16_GROUP; ++j) {
            const size_t p = p0 + j;
            out[j] = 0;
            if (p < p1) {
                if (p >= next) {
                    c = code_at(p, c + 1);
                    next = start_of(c + 1);
                }
                out[j] = key_at(p, c);
            }
        }
        if (p1 - p0 == C16_GROUP) {
            uint4 v;
            v.x = out[0] | ((uint32_t)out[1] << 16);
            v.y = out[2] | ((uint32_t)out[3] << 16);
            v.z = out[4] | ((uint32_t)out[5] << 16);
            v.w = out[6] | ((uint32_t)out[7] << 16);
            *reinterpret_cast<uint4 *>(dst + p0) = v;
        } else {
            for (int j = 0; j < C16_GROUP; ++j)
                if (p0 + j < p1) dst[p0 + j] = out[j];
        }
    }
}

// Host side --------------------------------------------------------------------
static int c16_grid(size_t n)
{
    // about 2^16 keys or more per CTA; at most one CTA per SM (128 KiB counters)
    return (int)std::max<size_t>(1, std::min<size_t>((size_t)num_sms(), n >> 16));
}

struct C16Layout {
    size_t part, over, start, bsum, first, total;
};

static size_t c16_chunks(size_t n) { return (n + C16_CHUNK - 1) / C16_CHUNK; }

static C16Layout c16_layout(size_t n)
{
    C16Layout L{};
    size_t off = 0;
    L.part = off;  off = align_up(off + (size_t)c16_grid(n) * C16_SMEM, 256);
    L.over = off;  off = align_up(off + sizeof(unsigned long long) * C16_BINS, 256);
    L.start = off; off = align_up(off + sizeof(unsigned long long) * (C16_BINS + 1), 256);
    L.bsum = off;  off = align_up(off + sizeof(unsigned long long) * C16_NBLK, 256);
    L.first = off; off = align_up(off + sizeof(uint32_t) * (c16_chunks(n) + 1), 256);
    L.total = off;
    return L;
}

bool count16_wanted(int op, int kbytes, size_t n)
{
    return op == SOP_KEYS && kbytes == 2 && n > COUNT16_MIN_N;
}

size_t count16_workspace_bytes(size_t n) { return c16_layout(n).total; }

int count16_sort(KeyXform xf, void *keys, size_t n, size_t canon_end, void *ws, size_t ws_bytes,
                 cudaStream_t s)
{
    if (n <= 1) return XSS_OK;
    const C16Layout L = c16_layout(n);
    if (ws == nullptr || ws_bytes < L.total) return XSS_ENOMEM;
    char *base = static_cast<char *>(ws);
    C16Args a{};
    a.keys = static_cast<uint16_t *>(keys);
    a.n = n;
    a.canon_end = canon_end;
    a.xf = xf;
    a.part = reinterpret_cast<uint32_t *>(base + L.part);
    a.over = reinterpret_cast<unsigned long long *>(base + L.over);
    a.start = reinterpret_cast<unsigned long long *>(base + L.start);
    const int grid = c16_grid(n);
    int rc = set_max_dyn_smem((const void *)c16_hist_kernel, C16_SMEM);
    if (rc) return rc;
    XSS_CUDA_TRY(cudaMemsetAsync(a.over, 0, sizeof(unsigned long long) * C16_BINS, s));
    XSS_LAUNCH(PK_COUNT16, s, (c16_hist_kernel<<<grid, C16_HIST_BLOCK, C16_SMEM, s>>>(a)));
    XSS_CUDA_TRY(cudaGetLastError());
    unsigned long long *bsum = reinterpret_cast<unsigned long long *>(base + L.bsum);
    uint32_t *first = reinterpret_cast<uint32_t *>(base + L.first);
    XSS_LAUNCH(PK_COUNT16, s,
               (c16_reduce_kernel<<<C16_NBLK, C16_SCAN_BLOCK, 0, s>>>(a, grid, bsum)));
    XSS_CUDA_TRY(cudaGetLastError());
    XSS_LAUNCH(PK_COUNT16, s, (c16_offsets_kernel<<<1, 1024, 0, s>>>(a, bsum)));
    XSS_CUDA_TRY(cudaGetLastError());
    // chunks of the aligned part; the head (< 8 positions) rides with chunk 0
    const size_t head = std::min(n, (size_t)((16 - (reinterpret_cast<uintptr_t>(keys) & 15)) & 15) / 2);
    const size_t chunks = std::max<size_t>(1, c16_chunks(n - head));
    XSS_LAUNCH(PK_COUNT16, s,
               (c16_chunk_kernel<<<(unsigned)((chunks + 1 + 255) / 256), 256, 0, s>>>(
                   a, first, chunks, head)));
    XSS_CUDA_TRY(cudaGetLastError());
    XSS_LAUNCH(PK_COUNT16, s,
               (c16_expand_kernel<<<(unsigned)chunks, C16_EXPAND_BLOCK, 0, s>>>(a, first, chunks,
                                                                               head)));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

}  // namespace xss
