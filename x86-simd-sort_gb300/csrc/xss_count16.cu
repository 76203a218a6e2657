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

// Total count of every code: the CTAs' counters plus the overflow (written
// into `over`, which then holds the totals).
__global__ void __launch_bounds__(256) c16_reduce_kernel(C16Args a, int parts)
{
    const int w = blockIdx.x * 256 + threadIdx.x;
    if (w >= C16_WORDS) return;
    unsigned long long lo = 0, hi = 0;
    for (int c = 0; c < parts; ++c) {
        const uint32_t v = a.part[(size_t)c * C16_WORDS + w];
        lo += v & 0xFFFFu;
        hi += v >> 16;
    }
    a.over[2 * w] += lo;
    a.over[2 * w + 1] += hi;
}

// Exclusive scan of the totals into the first position of every code (one
// CTA, 64 codes per thread).
__global__ void __launch_bounds__(1024) c16_scan_kernel(C16Args a)
{
    constexpr int PER = C16_BINS / 1024;
    __shared__ unsigned long long s_warp[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned long long sum = 0;
    for (int i = 0; i < PER; ++i) sum += a.over[tid * PER + i];
    unsigned long long x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long t = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        s_warp[lane] = t;
    }
    __syncthreads();
    unsigned long long run = (warp ? s_warp[warp - 1] : 0ull) + x - sum;
    for (int i = 0; i < PER; ++i) {
        a.start[tid * PER + i] = run;
        run += a.over[tid * PER + i];
    }
    if (tid == 0) a.start[C16_BINS] = a.n;
}

// The code at sorted position p (0 <= p < n): the last code whose first
// position is <= p.  Two levels: the block's shared copy of every 32nd
// code's first position picks the block of 32 codes, then five probes of
// start[] (L1/L2) pick the code in it.
constexpr int C16_COARSE = 32;                               // codes per coarse entry
constexpr int C16_NCOARSE = C16_BINS / C16_COARSE;           // 2048
__device__ __forceinline__ uint32_t c16_code_at(const unsigned long long *s_coarse,
                                                const unsigned long long *start, size_t p)
{
    uint32_t lo = 0, hi = C16_NCOARSE - 1;   // s_coarse[0] = 0 <= p
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (s_coarse[mid] <= p) lo = mid;
        else hi = mid - 1;
    }
    uint32_t c = lo * C16_COARSE;
    uint32_t top = c + C16_COARSE - 1;
    while (c < top) {
        const uint32_t mid = (c + top + 1) >> 1;
        if (start[mid] <= p) c = mid;
        else top = mid - 1;
    }
    return c;
}

// Write the sorted keys: each thread 8 consecutive positions (one 16-byte
// store where aligned), stepping to the next code inside its eight positions
// when it crosses a code's end.
__global__ void __launch_bounds__(C16_EXPAND_BLOCK) c16_expand_kernel(C16Args a)
{
    __shared__ unsigned long long s_coarse[C16_NCOARSE];
    for (int i = threadIdx.x; i < C16_NCOARSE; i += C16_EXPAND_BLOCK)
        s_coarse[i] = a.start[(size_t)i * C16_COARSE];
    __syncthreads();
    const Codec<uint16_t> cx(a.xf);
    const unsigned long long *start = a.start;
    uint16_t *dst = a.keys;
    const size_t n = a.n;
    const size_t head = c16_head(dst, n);
    // group 0 = the unaligned head; group g >= 1 = [head + 8(g-1), head + 8g)
    const size_t groups = 1 + (n - head + C16_GROUP - 1) / C16_GROUP;
    const size_t stride = (size_t)gridDim.x * C16_EXPAND_BLOCK;
    for (size_t g = (size_t)blockIdx.x * C16_EXPAND_BLOCK + threadIdx.x; g < groups; g += stride) {
        const size_t p0 = g == 0 ? 0 : head + (g - 1) * C16_GROUP;
        const size_t p1 = g == 0 ? head : min(n, p0 + C16_GROUP);
        if (p0 >= p1) continue;
        uint32_t c = c16_code_at(s_coarse, start, p0);
        unsigned long long next = start[c + 1];
        uint16_t out[C16_GROUP];
#pragma unroll
        for (int j = 0; j < C16_GROUP; ++j) {
            const size_t p = p0 + j;
            out[j] = 0;
            if (p < p1) {
                if (p >= next) {
                    c = c16_code_at(s_coarse, start, p);
                    next = start[c + 1];
                }
                out[j] = p < a.canon_end ? cx.from_canon((uint16_t)c) : cx.from((uint16_t)c);
            }
        }
        if (p1 - p0 == C16_GROUP && g != 0) {
            uint4 q;
            q.x = out[0] | ((uint32_t)out[1] << 16);
            q.y = out[2] | ((uint32_t)out[3] << 16);
            q.z = out[4] | ((uint32_t)out[5] << 16);
            q.w = out[6] | ((uint32_t)out[7] << 16);
            *reinterpret_cast<uint4 *>(dst + p0) = q;
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
    size_t part, over, start, total;
};

static C16Layout c16_layout(size_t n)
{
    C16Layout L{};
    size_t off = 0;
    L.part = off;  off = align_up(off + (size_t)c16_grid(n) * C16_SMEM, 256);
    L.over = off;  off = align_up(off + sizeof(unsigned long long) * C16_BINS, 256);
    L.start = off; off = align_up(off + sizeof(unsigned long long) * (C16_BINS + 1), 256);
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
    XSS_LAUNCH(PK_COUNT16, s, (c16_reduce_kernel<<<C16_WORDS / 256, 256, 0, s>>>(a, grid)));
    XSS_CUDA_TRY(cudaGetLastError());
    XSS_LAUNCH(PK_COUNT16, s, (c16_scan_kernel<<<1, 1024, 0, s>>>(a)));
    XSS_CUDA_TRY(cudaGetLastError());
    const size_t groups = 1 + (n + C16_GROUP - 1) / C16_GROUP;
    const int eg = (int)std::max<size_t>(
        1, std::min<size_t>((groups + C16_EXPAND_BLOCK - 1) / C16_EXPAND_BLOCK,
                            (size_t)num_sms() * 16));
    XSS_LAUNCH(PK_COUNT16, s, (c16_expand_kernel<<<eg, C16_EXPAND_BLOCK, 0, s>>>(a)));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

}  // namespace xss
