// xss_radix.cu -- full sorts: one-CTA bitonic sort for small inputs and an
// LSD "onesweep" radix sort (one up-front histogram, then one kernel per
// 8-bit digit with a decoupled look-back prefix, xss_onesweep.cuh) for large ones.
//
// Replaces, for the reference's qsort / keyvalue_qsort / argsort:
//   src/xss-common-qsort.h:529-605   (qsort_ recursion, partition sweeps)
//   src/xss-common-keyvaluesort.hpp:419-653 (kvsort_, kv partition)
//   src/xss-common-argsort.h:470-669 (argsort_, argpartition)
//   src/xss-network-qsort.hpp, src/xss-network-keyvaluesort.hpp (small-n networks)
// The reference's quicksort is in-place and unstable; an LSD radix sort is
// stable per pass and yields one of the orders the reference may produce.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>
#include "xss_blocksort.cuh"
#include "xss_onesweep.cuh"

namespace xss {

// ---------------------------------------------------------------------------
// Up-front histogram of every digit of every key (one read of the input),
// fused with clearing the look-back status words.  The last CTA to finish
// turns the histograms into per-pass bucket starts and writes the pass plan:
// a pass whose digit is the same for every key is skipped.
// 64-bit keys (eight digits per key): every lane counts into its own column of
// 16-bit counters: word
// ((p * RADIX + d) / 2) * 32 + lane holds digits d and d + 1 (d even) of pass
// p in its two halves, so the 32 lanes of a warp always touch 32 different
// banks -- random digits and a digit every key shares (the top byte of
// floats, small-range integers) alike cost one shared-memory wavefront per
// warp and digit.  The HIST_BLOCK / 32 warps of a CTA share the columns, so
// a CTA flushes its counters into the global histograms before any half
// could pass 65535 (every HIST_FLUSH_KEYS keys per thread), and once at the
// end.  The counters take sizeof(C) * 16 KiB of dynamic shared memory.
constexpr int HIST_BLOCK = 512;
constexpr int HIST_VEC_IN_FLIGHT = 8;          // 16-byte loads per thread per step
constexpr uint32_t HIST_FLUSH_KEYS = 65535u / (HIST_BLOCK / 32);
template <typename C> constexpr size_t hist_cols_smem_bytes()
{
    return sizeof(C) * (RADIX / 2) * 32 * sizeof(uint32_t);
}

// The last CTA to finish turns the histograms into per-pass bucket starts
// and writes the pass plan (a pass whose digit every key shares is skipped).
template <int BLOCK>
__device__ __forceinline__ void hist_finish(const RadixArgs &a, uint32_t *s_scan, int *s_active)
{
    __shared__ int s_last;
    const int tid = threadIdx.x;
    const int P = a.passes;
    const size_t n = a.n;
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = (atomicAdd(&a.hdr->done_ctr, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();

    for (int p = 0; p < P; ++p) {
        const uint32_t h = tid < RADIX ? ld_relaxed_u32(&a.hdr->hist[p][tid]) : 0u;
        const int trivial = __syncthreads_or(tid < RADIX && h == (uint32_t)n);
        uint32_t total;
        const uint32_t ex = block_excl_scan<BLOCK>(h, s_scan, total);
        if (tid < RADIX) a.hdr->start[p][tid] = ex;
        if (tid == 0) s_active[p] = !trivial;
    }
    __syncthreads();
    if (tid != 0) return;

    int m = 0;
    for (int p = 0; p < P; ++p) m += s_active[p];
    int cur = 0, seen = 0;
    for (int p = 0; p < P; ++p) {
        PassDesc d = {};
        if (s_active[p]) {
            d.active = 1;
            d.first = (seen == 0);
            d.last = (seen == m - 1);
            d.src = cur;
            d.vsrc = cur;
            // a keys-only sort's first pass may order ties arbitrarily: equal
            // codes are the same key and nothing is ordered yet
            d.tie_free = a.op == SOP_KEYS && d.first;
            if (a.op == SOP_ARG) {
                d.dst = (cur == 1) ? 2 : 1;
                d.vdst = d.dst;
                d.gen_idx = d.first;
                d.skip_keys = d.last;
                d.out_idx = d.last;
            } else {
                d.dst = 1 - cur;
                d.vdst = d.dst;
            }
            cur = d.dst;
            ++seen;
        }
        a.hdr->desc[p] = d;
    }
    int fix = FIX_NONE;
    if (m == 0) {
        if (a.op == SOP_ARG) fix = FIX_IOTA;
        else if (a.op == SOP_KEYS && a.xf.canon && a.xf.kind == XK_FLOAT) fix = FIX_CANON;
    } else if (a.op != SOP_ARG && cur == 1) {
        fix = FIX_COPY;
    }
    a.hdr->fixup = fix;
    a.hdr->num_active = m;
}

template <typename C>
__device__ __forceinline__ void hist_count(uint32_t *col, C c)
{
#pragma unroll
    for (int p = 0; p < (int)sizeof(C); ++p) {
        const uint32_t d = uint32_t(c >> (p * RADIX_BITS)) & (RADIX - 1);
        atomicAdd(col + (p * (RADIX / 2) + (d >> 1)) * 32, 1u << ((d & 1u) << 4));
    }
}

template <typename C>
__global__ void __launch_bounds__(HIST_BLOCK) hist_cols_kernel(RadixArgs a)
{
    extern __shared__ __align__(16) uint32_t sh_all[];
    __shared__ uint32_t s_scan[HIST_BLOCK / 32];
    __shared__ int s_active[MAX_PASSES];
    const int tid = threadIdx.x, lane = tid & 31;
    const int P = a.passes;
    constexpr int ROWS = (int)sizeof(C) * (RADIX / 2);   // 32 words each
    // the passes sort codes of the keys as they are (NaN payloads included);
    // the last pass writes canonical NaNs where the sort asks for them.  (The
    // branched transform measured faster here than the passes' codec.)
    const KeyXform xnc{a.xf.kind, a.xf.desc, 0};
    for (int i = tid; i < ROWS * 32; i += HIST_BLOCK) sh_all[i] = 0;
    __syncthreads();
    uint32_t *const col = sh_all + lane;

    // add every row's 32 columns (lanes read rotated columns: distinct banks)
    // into the global histograms and clear them
    auto flush = [&]() {
        __syncthreads();
        for (int r = tid; r < ROWS; r += HIST_BLOCK) {
            uint32_t lo = 0, hi = 0;
#pragma unroll 8
            for (int i = 0; i < 32; ++i) {
                uint32_t *w = sh_all + r * 32 + ((i + tid) & 31);
                const uint32_t v = *w;
                *w = 0;
                lo += v & 0xFFFFu;
                hi += v >> 16;
            }
            uint32_t *g = &a.hdr->hist[0][0] + 2 * r;
            if (lo) atomicAdd(g, lo);
            if (hi) atomicAdd(g + 1, hi);
        }
        __syncthreads();
    };

    const C *src = static_cast<const C *>(a.kbuf[0]);
    const size_t n = a.n;
    const size_t gtid = (size_t)blockIdx.x * HIST_BLOCK + tid;
    const size_t stride = (size_t)gridDim.x * HIST_BLOCK;
    constexpr int VEC = 16 / sizeof(C);
    constexpr int U = HIST_VEC_IN_FLIGHT;
    const bool aligned = (reinterpret_cast<uintptr_t>(src) & 15) == 0;
    const size_t nvec = aligned ? n / VEC : 0;
    // the same number of steps in every thread of the grid, so the flushes
    // (barriers) are reached by all threads of a CTA
    const size_t vsteps = (nvec + (size_t)U * stride - 1) / ((size_t)U * stride);
    uint32_t since = 0;   // keys per thread since the last flush (bound)
    for (size_t st = 0; st < vsteps; ++st) {
        uint4 q[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const size_t v = st * U * stride + (size_t)u * stride + gtid;
            q[u] = v < nvec ? reinterpret_cast<const uint4 *>(src)[v] : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const size_t v = st * U * stride + (size_t)u * stride + gtid;
            if (v < nvec) {
                C e[VEC];
                memcpy(e, &q[u], 16);
#pragma unroll
                for (int k = 0; k < VEC; ++k) hist_count<C>(col, to_code(e[k], xnc));
            }
        }
        since += U * VEC;
        if (since + U * VEC > HIST_FLUSH_KEYS) {
            flush();
            since = 0;
        }
    }
    const size_t rest = n - nvec * VEC;
    const size_t ssteps = (rest + stride - 1) / stride;
    for (size_t st = 0; st < ssteps; ++st) {
        const size_t i = nvec * VEC + st * stride + gtid;
        if (i < n) hist_count<C>(col, to_code(src[i], xnc));
        if (++since + 1 > HIST_FLUSH_KEYS) {
            flush();
            since = 0;
        }
    }

    // clear the look-back words of every pass (multiple of 4 words, 16B aligned)
    const size_t nst4 = (size_t)P * a.num_tiles * RADIX / 4;
    uint4 *st4 = reinterpret_cast<uint4 *>(a.status);
    for (size_t i = gtid; i < nst4; i += stride) st4[i] = make_uint4(0, 0, 0, 0);

    flush();
    hist_finish<HIST_BLOCK>(a, s_scan, s_active);
}

// 16- and 32-bit keys (measured faster this way than with lane columns, which
// hold fewer resident warps): lanes count into eight interleaved copies of the
// histograms -- counter (pass p, digit d, copy c) is word (p * RADIX + d) * 8
// + c and lane l uses copy l & 7.  A copy's words all lie in the four banks c,
// c+8, c+16, c+24, which only the four lanes of that copy touch: random digits
// meet at most 4-way bank conflicts, and a digit every key shares costs a
// 4-way same-address conflict instead of 32-way.  sizeof(C) * 8 KiB of
// dynamic shared memory, 256-thread CTAs.
constexpr int HIST_COPIES = 8;
template <typename C> constexpr size_t hist_copies_smem_bytes()
{
    return sizeof(C) * RADIX * HIST_COPIES * sizeof(uint32_t);
}
template <typename C>
__global__ void __launch_bounds__(256) hist_copies_kernel(RadixArgs a)
{
    extern __shared__ __align__(16) uint32_t sh_all[];
    __shared__ uint32_t s_scan[8];
    __shared__ int s_active[MAX_PASSES];
    const int tid = threadIdx.x;
    const int P = a.passes;
    constexpr int NW = (int)sizeof(C) * RADIX * HIST_COPIES;
    const KeyXform xnc{a.xf.kind, a.xf.desc, 0};   // codes as in hist_cols_kernel
    for (int i = tid; i < NW; i += 256) sh_all[i] = 0;
    __syncthreads();
    uint32_t *const sh = sh_all + (tid & (HIST_COPIES - 1));

    const C *src = static_cast<const C *>(a.kbuf[0]);
    const size_t n = a.n;
    const size_t gtid = (size_t)blockIdx.x * 256 + tid;
    const size_t stride = (size_t)gridDim.x * 256;
    constexpr int VEC = 16 / sizeof(C);
    const bool aligned = (reinterpret_cast<uintptr_t>(src) & 15) == 0;
    const size_t nvec = aligned ? n / VEC : 0;
    for (size_t v = gtid; v < nvec; v += stride) {
        const uint4 q = reinterpret_cast<const uint4 *>(src)[v];
        C e[VEC];
        memcpy(e, &q, 16);
#pragma unroll
        for (int u = 0; u < VEC; ++u) {
            const C c = to_code(e[u], xnc);
#pragma unroll
            for (int p = 0; p < (int)sizeof(C); ++p)
                atomicAdd(&sh[(p * RADIX + (uint32_t(c >> (p * RADIX_BITS)) & (RADIX - 1))) *
                              HIST_COPIES], 1u);
        }
    }
    for (size_t i = nvec * VEC + gtid; i < n; i += stride) {
        const C c = to_code(src[i], xnc);
#pragma unroll
        for (int p = 0; p < (int)sizeof(C); ++p)
            atomicAdd(&sh[(p * RADIX + (uint32_t(c >> (p * RADIX_BITS)) & (RADIX - 1))) *
                          HIST_COPIES], 1u);
    }

    // clear the look-back words of every pass (multiple of 4 words, 16B aligned)
    const size_t nst4 = (size_t)P * a.num_tiles * RADIX / 4;
    uint4 *st4 = reinterpret_cast<uint4 *>(a.status);
    for (size_t i = gtid; i < nst4; i += stride) st4[i] = make_uint4(0, 0, 0, 0);

    __syncthreads();
    for (int i = tid; i < P * RADIX; i += 256) {
        const uint4 *w = reinterpret_cast<const uint4 *>(sh_all + i * HIST_COPIES);
        const uint4 x = w[0], y = w[1];
        const uint32_t t = x.x + x.y + x.z + x.w + y.x + y.y + y.z + y.w;
        if (t) atomicAdd(&a.hdr->hist[0][0] + i, t);
    }
    hist_finish<256>(a, s_scan, s_active);
}

// ---------------------------------------------------------------------------
// Finishing step after the passes: copy back when an odd number of passes
// ran, canonicalise NaNs when no pass ran, or write the identity permutation.
template <typename C, typename V>
__global__ void fixup_kernel(RadixArgs a)
{
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    const int mode = a.hdr->fixup;
    if (mode == FIX_NONE) return;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        if (mode == FIX_COPY) {
            static_cast<C *>(a.kbuf[0])[i] = static_cast<const C *>(a.kbuf[1])[i];
            if constexpr (HAS_V)
                static_cast<V *>(a.vbuf[0])[i] = static_cast<const V *>(a.vbuf[1])[i];
        } else if (mode == FIX_CANON) {
            C *k = static_cast<C *>(a.kbuf[0]);
            k[i] = canon_bits(k[i], a.xf);
        } else if (mode == FIX_IOTA) {
            a.out_idx[i] = i;
        }
    }
}

// ---------------------------------------------------------------------------
// Host side.
struct RadixLayout {
    size_t hdr, status, k1, k2, v1, v2, total;
};

static constexpr RadixLayout radix_layout(int op, int kbytes, int vbytes, size_t n, size_t tile)
{
    RadixLayout L{};
    const int passes = kbytes;  // 8-bit digits
    const size_t tiles = (n + tile - 1) / tile;
    const int vb = (op == SOP_ARG) ? 4 : vbytes;
    size_t off = 0;
    L.hdr = off;    off = align_up(off + sizeof(RadixHeader), 256);
    L.status = off; off = align_up(off + (size_t)passes * tiles * RADIX * 4, 256);
    L.k1 = off;     off = align_up(off + n * kbytes, 256);
    L.k2 = off;     if (op == SOP_ARG) off = align_up(off + n * kbytes, 256);
    L.v1 = off;     if (vb) off = align_up(off + n * vb, 256);
    L.v2 = off;     if (op == SOP_ARG) off = align_up(off + n * vb, 256);
    L.total = off;
    return L;
}

static thread_local bool t_prefer_shared_sm = false;
void set_prefer_shared_sm(bool on) { t_prefer_shared_sm = on; }

static bool use_mid_lines(size_t n) { return n <= XSS_MID_N || t_prefer_shared_sm; }

// Tile of the lines a sort of n keys may use: for n above XSS_MID_N both
// classes are possible (see set_prefer_shared_sm), so the workspace is sized
// for the smaller tile, which needs the larger look-back array.
template <typename C, typename V> static constexpr size_t tile_of(size_t n)
{
    return n <= XSS_MID_N ? pass_tile_size_mid<C, V>()
                          : std::min(pass_tile_size_mid<C, V>(), pass_tile_size<C, V>());
}

static size_t tile_for_bytes(int op, int kbytes, int vbytes, size_t n)
{
    const int vb = (op == SOP_ARG) ? 4 : (op == SOP_KV ? vbytes : 0);
    switch (kbytes) {
    case 2: return vb == 0 ? tile_of<uint16_t, NoVal>(n) : vb == 2 ? tile_of<uint16_t, uint16_t>(n) : vb == 4 ? tile_of<uint16_t, uint32_t>(n) : tile_of<uint16_t, uint64_t>(n);
    case 4: return vb == 0 ? tile_of<uint32_t, NoVal>(n) : vb == 2 ? tile_of<uint32_t, uint16_t>(n) : vb == 4 ? tile_of<uint32_t, uint32_t>(n) : tile_of<uint32_t, uint64_t>(n);
    default: return vb == 0 ? tile_of<uint64_t, NoVal>(n) : vb == 2 ? tile_of<uint64_t, uint16_t>(n) : vb == 4 ? tile_of<uint64_t, uint32_t>(n) : tile_of<uint64_t, uint64_t>(n);
    }
}

size_t radix_chunk_workspace_bytes(int op, int kbytes, int vbytes, size_t n)
{
    if (n <= SMALL_SORT_MAX) return 0;
    return radix_layout(op, kbytes, vbytes, n, tile_for_bytes(op, kbytes, vbytes, n)).total;
}

size_t radix_workspace_bytes(int op, int kbytes, int vbytes, size_t n)
{
    if (n <= SMALL_SORT_MAX) return 0;
    if (count16_wanted(op, kbytes, n)) return count16_workspace_bytes(n);
    if (big_sort_needed(n)) return big_sort_workspace_bytes(op, kbytes, vbytes, n);
    return radix_chunk_workspace_bytes(op, kbytes, vbytes, n);
}

// How a sort is launched: where device-side errors go and whether launches
// go through the profiler hooks (which may create CUDA events).
struct LaunchOpts {
    unsigned *err;
    bool instrument;
};

#define XSS_LAUNCH_OPT(opts, kind, stream, ...) \
    do {                                        \
        if ((opts).instrument) {                \
            XSS_LAUNCH(kind, stream, __VA_ARGS__); \
        } else {                                \
            __VA_ARGS__;                        \
        }                                       \
    } while (0)

template <typename C, typename V>
static int small_sort_launch(int op, KeyXform xf, void *keys, void *vals,
                             uint64_t *out_idx, size_t n, cudaStream_t s, const LaunchOpts &o)
{
    SmallArgs a{};
    a.keys_in = keys;
    a.keys_out = (op == SOP_ARG) ? nullptr : keys;
    a.vals_in = vals;
    a.vals_out = vals;
    a.out_idx = (op == SOP_ARG) ? out_idx : nullptr;
    a.n = (uint32_t)n;
    uint32_t npad = 2;
    while (npad < n) npad <<= 1;
    a.npad = npad;
    a.xf = xf;
    const size_t smem = align_up(sizeof(C) * npad, 16) + 2 * npad;  // <= 40 KiB
    XSS_LAUNCH_OPT(o, PK_SMALL, s,
                   (small_sort_kernel<C, V, SMALL_BLOCK, SMALL_SORT_MAX><<<1, SMALL_BLOCK, smem, s>>>(a)));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

// Launch every active pass with resident CTAs (grid = what fits on the SMs).
template <typename C, typename V, int BLOCK, int ITEMS, int MINB, int LB, int RANK, int DPT,
          bool PF>
static int resident_passes(const RadixArgs &a, int sms, cudaStream_t s, const LaunchOpts &o)
{
    constexpr size_t TILE = (size_t)BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    const size_t smem = (PF ? 2 : 1) * TILE * (sizeof(C) + (HAS_V ? sizeof(V) : 0));
    auto kern = onesweep_persist_kernel<C, V, BLOCK, ITEMS, MINB, LB, RANK, DPT, PF>;
    int rc = set_max_dyn_smem((const void *)kern, smem);
    if (rc) return rc;
    static std::atomic<int> per_sm_cached{0};   // same GPU model on every device
    int per_sm = per_sm_cached.load(std::memory_order_relaxed);
    if (!per_sm) {
        int v = 0;
        XSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, BLOCK, smem));
        per_sm = std::max(v, 1);
        per_sm_cached.store(per_sm, std::memory_order_relaxed);
    }
    const uint32_t grid = (uint32_t)std::min<size_t>(a.num_tiles, (size_t)per_sm * sms);
    for (int p = 0; p < a.passes; ++p) {
        XSS_LAUNCH_OPT(o, PK_ONESWEEP, s, kern<<<grid, BLOCK, smem, s>>>(a, p));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    return XSS_OK;
}

// Pipelined resident CTAs (two tiles held per CTA) for every active pass.
template <typename C, typename V, int BLOCK, int ITEMS, int MINB, int LB>
static int pipe_passes(const RadixArgs &a, int sms, cudaStream_t s, const LaunchOpts &o)
{
    constexpr size_t TILE = (size_t)BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    const size_t smem = 2 * TILE * (sizeof(C) + (HAS_V ? sizeof(V) : 0));
    auto kern = onesweep_pipe_kernel<C, V, BLOCK, ITEMS, MINB, LB>;
    int rc = set_max_dyn_smem((const void *)kern, smem);
    if (rc) return rc;
    static std::atomic<int> per_sm_cached{0};   // same GPU model on every device
    int per_sm = per_sm_cached.load(std::memory_order_relaxed);
    if (!per_sm) {
        int v = 0;
        XSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, BLOCK, smem));
        per_sm = std::max(v, 1);
        per_sm_cached.store(per_sm, std::memory_order_relaxed);
    }
    const uint32_t grid = (uint32_t)std::min<size_t>(a.num_tiles, (size_t)per_sm * sms);
    for (int p = 0; p < a.passes; ++p) {
        XSS_LAUNCH_OPT(o, PK_ONESWEEP, s, kern<<<grid, BLOCK, smem, s>>>(a, p));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    return XSS_OK;
}

// One CTA per tile for every active pass.
template <typename C, typename V, int BLOCK, int ITEMS, int MINB, int LB, int RANK, int DPT>
static int tile_passes(const RadixArgs &a, cudaStream_t s, const LaunchOpts &o)
{
    constexpr size_t TILE = (size_t)BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    const size_t smem = TILE * (sizeof(C) + (HAS_V ? sizeof(V) : 0));
    auto kern = onesweep_kernel<C, V, BLOCK, ITEMS, MINB, LB, RANK, DPT>;
    const int rc = set_max_dyn_smem((const void *)kern, smem);
    if (rc) return rc;
    for (int p = 0; p < a.passes; ++p) {
        XSS_LAUNCH_OPT(o, PK_ONESWEEP, s, kern<<<a.num_tiles, BLOCK, smem, s>>>(a, p));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    return XSS_OK;
}

// LARGE: the large-array lines, else the mid-size lines; each in its tuned
// launch form only.
template <typename C, typename V, bool LARGE>
static int onesweep_launch_cls(int op, KeyXform xf, void *keys, void *vals, uint64_t *out_idx,
                               size_t n, void *ws, size_t ws_bytes, cudaStream_t s,
                               const LaunchOpts &o)
{
    using Cfg = typename std::conditional<LARGE, PassCfg<C, V>, PassCfgMid<C, V>>::type;
    constexpr int BLOCK = Cfg::BLOCK, ITEMS = Cfg::ITEMS, MINB = Cfg::MINB, LB = Cfg::LB,
                  RANK = Cfg::RANK, DPT = Cfg::DPT;
    constexpr size_t TILE = (size_t)BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    const int kbytes = sizeof(C);
    const int vbytes = HAS_V ? (int)sizeof(V) : 0;
    const RadixLayout L = radix_layout(op, kbytes, op == SOP_ARG ? 4 : vbytes, n, TILE);
    if (ws == nullptr || ws_bytes < L.total) return XSS_ENOMEM;
    char *base = static_cast<char *>(ws);

    RadixArgs a{};
    a.kbuf[0] = keys;
    a.kbuf[1] = base + L.k1;
    a.kbuf[2] = base + L.k2;
    a.vbuf[0] = vals;
    a.vbuf[1] = base + L.v1;
    a.vbuf[2] = base + L.v2;
    a.out_idx = out_idx;
    a.n = n;
    a.num_tiles = (uint32_t)((n + TILE - 1) / TILE);
    a.passes = kbytes;
    a.op = op;
    a.xf = xf;
    a.hdr = reinterpret_cast<RadixHeader *>(base + L.hdr);
    a.status = reinterpret_cast<uint32_t *>(base + L.status);
    a.err = o.err;
    if (!a.err) return XSS_ECUDA;

    XSS_CUDA_TRY(cudaMemsetAsync(a.hdr, 0, sizeof(RadixHeader), s));
    const int sms = num_sms();
    if constexpr (sizeof(C) == 8) {
        constexpr size_t HSMEM = hist_cols_smem_bytes<C>();
        {
            const int rc = set_max_dyn_smem((const void *)hist_cols_kernel<C>, HSMEM);
            if (rc) return rc;
        }
        // resident CTAs per SM of the histogram kernel (measured once)
        static std::atomic<int> hist_per_sm{0};
        int per_sm = hist_per_sm.load(std::memory_order_relaxed);
        if (per_sm == 0) {
            XSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, hist_cols_kernel<C>, HIST_BLOCK, HSMEM));
            per_sm = std::max(per_sm, 1);
            hist_per_sm.store(per_sm, std::memory_order_relaxed);
        }
        constexpr size_t PER_CTA = (size_t)HIST_BLOCK * HIST_VEC_IN_FLIGHT * (16 / sizeof(C));
        const size_t want = (n + PER_CTA - 1) / PER_CTA;
        const int hist_grid =
            (int)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * (size_t)per_sm));
        XSS_LAUNCH_OPT(o, PK_HIST, s,
                       hist_cols_kernel<C><<<hist_grid, HIST_BLOCK, HSMEM, s>>>(a));
    } else {
        const size_t want = (n + 256 * 16 - 1) / (256 * 16);
        const int hist_grid = (int)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * 8));
        constexpr size_t HSMEM = hist_copies_smem_bytes<C>();
        {
            const int rc = set_max_dyn_smem((const void *)hist_copies_kernel<C>, HSMEM);
            if (rc) return rc;
        }
        XSS_LAUNCH_OPT(o, PK_HIST, s, hist_copies_kernel<C><<<hist_grid, 256, HSMEM, s>>>(a));
    }
    XSS_CUDA_TRY(cudaGetLastError());

    int rc = XSS_OK;
    if constexpr (Cfg::PERSIST == 3) {
        static_assert(RANK == 2, "the pipelined form ranks by the count atomic");
        rc = pipe_passes<C, V, BLOCK, ITEMS, MINB, LB>(a, sms, s, o);
    } else if constexpr (Cfg::PERSIST == 1)
        rc = resident_passes<C, V, BLOCK, ITEMS, MINB, LB, RANK, DPT, true>(a, sms, s, o);
    else if constexpr (Cfg::PERSIST == 2)
        rc = resident_passes<C, V, BLOCK, ITEMS, MINB, LB, RANK, DPT, false>(a, sms, s, o);
    else
        rc = tile_passes<C, V, BLOCK, ITEMS, MINB, LB, RANK, DPT>(a, s, o);
    if (rc) return rc;
    XSS_LAUNCH_OPT(o, PK_FIXUP, s, fixup_kernel<C, V><<<sms * 2, 256, 0, s>>>(a));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

template <typename C, typename V>
static int onesweep_launch(int op, KeyXform xf, void *keys, void *vals, uint64_t *out_idx,
                           size_t n, void *ws, size_t ws_bytes, cudaStream_t s,
                           const LaunchOpts &o)
{
    return use_mid_lines(n)
               ? onesweep_launch_cls<C, V, false>(op, xf, keys, vals, out_idx, n, ws, ws_bytes, s, o)
               : onesweep_launch_cls<C, V, true>(op, xf, keys, vals, out_idx, n, ws, ws_bytes, s, o);
}

template <typename C>
static int radix_sort_c(int op, KeyXform xf, void *keys, void *vals, int vbytes,
                        uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s,
                        const LaunchOpts &o)
{
    const bool small = n <= SMALL_SORT_MAX;
    if (op == SOP_ARG) {
        return small ? small_sort_launch<C, NoVal>(op, xf, keys, nullptr, out_idx, n, s, o)
                     : onesweep_launch<C, uint32_t>(op, xf, keys, nullptr, out_idx, n, ws,
                                                    ws_bytes, s, o);
    }
    if (op == SOP_KEYS || vbytes == 0) {
        return small ? small_sort_launch<C, NoVal>(op, xf, keys, nullptr, nullptr, n, s, o)
                     : onesweep_launch<C, NoVal>(op, xf, keys, nullptr, nullptr, n, ws, ws_bytes,
                                                 s, o);
    }
    if (vbytes == 2)
        return small ? small_sort_launch<C, uint16_t>(op, xf, keys, vals, nullptr, n, s, o)
                     : onesweep_launch<C, uint16_t>(op, xf, keys, vals, nullptr, n, ws, ws_bytes,
                                                    s, o);
    if (vbytes == 4)
        return small ? small_sort_launch<C, uint32_t>(op, xf, keys, vals, nullptr, n, s, o)
                     : onesweep_launch<C, uint32_t>(op, xf, keys, vals, nullptr, n, ws, ws_bytes,
                                                    s, o);
    return small ? small_sort_launch<C, uint64_t>(op, xf, keys, vals, nullptr, n, s, o)
                 : onesweep_launch<C, uint64_t>(op, xf, keys, vals, nullptr, n, ws, ws_bytes, s,
                                                o);
}

static int radix_sort_opts(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
                           uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes,
                           cudaStream_t s, const LaunchOpts &o)
{
    if (n == 0) return XSS_OK;
    if (n == 1) {
        // the reference returns early for arrsize <= 1 (src/xss-common-qsort.h:660);
        // argsort of one element is the index 0
        if (op == SOP_ARG) XSS_CUDA_TRY(cudaMemsetAsync(out_idx, 0, sizeof(uint64_t), s));
        return XSS_OK;
    }
    if (n > XSS_RADIX_MAX_N) return XSS_ETOOBIG;
    switch (kbytes) {
    case 2: return radix_sort_c<uint16_t>(op, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s, o);
    case 4: return radix_sort_c<uint32_t>(op, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s, o);
    case 8: return radix_sort_c<uint64_t>(op, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s, o);
    default: return XSS_EINVAL;
    }
}

// One radix sort of at most XSS_RADIX_MAX_N keys (also a chunk of a larger sort).
int radix_sort_chunk(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
                     uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s)
{
    if (n <= 1 || n > XSS_RADIX_MAX_N)
        return radix_sort_opts(op, kbytes, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s,
                               LaunchOpts{nullptr, true});
    const LaunchOpts o{device_error_word(), true};
    return radix_sort_opts(op, kbytes, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s, o);
}

int radix_sort(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
               uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s)
{
    if (n > XSS_MAX_N) return XSS_ETOOBIG;
    if (count16_wanted(op, kbytes, n)) return count16_sort(xf, keys, n, n, ws, ws_bytes, s);
    if (big_sort_needed(n))
        return big_sort(op, kbytes, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s);
    return radix_sort_chunk(op, kbytes, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s);
}

}  // namespace xss

// ---------------------------------------------------------------------------
// Allocation-free qsort: xss_gpu_qsort_noalloc.
//
// For callers that must not allocate device memory at call time -- code that
// runs inside a memory allocator or an out-of-memory handler, plugins whose
// host process owns every device allocation, fixed-budget real-time loops.
// Its scratch is this file-scope device array instead of a cudaMalloc'd or
// caller-provided workspace.  The array is part of the library's device image,
// so every GPU that loads the library holds these bytes until the process
// exits.  Every call uses the same array and finds the previous call's data
// in it; the header and error word are cleared at the start of each call.
// Calls whose work overlaps on the GPU (different streams, or different host
// threads) race on the array and must be serialised by the caller.
namespace xss {

constexpr size_t NOALLOC_MAX_N = size_t(1) << 20;               // keys per call
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(12) << 20;      // 12 MiB
constexpr size_t NOALLOC_ERR_BYTES = 256;                       // error word slot

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// The scratch layout of the largest call fits the array for every key width
// with the tuned tile sizes (a tuning line that breaks this fails the build).
constexpr size_t NOALLOC_WS_BYTES = NOALLOC_SCRATCH_BYTES - NOALLOC_ERR_BYTES;
static_assert(NOALLOC_MAX_N <= XSS_MID_N, "calls up to the limit use the mid-size lines");
static_assert(radix_layout(SOP_KEYS, 2, 0, NOALLOC_MAX_N,
                           tile_of<uint16_t, NoVal>(NOALLOC_MAX_N)).total <= NOALLOC_WS_BYTES,
              "16-bit scratch layout exceeds the static array");
static_assert(radix_layout(SOP_KEYS, 4, 0, NOALLOC_MAX_N,
                           tile_of<uint32_t, NoVal>(NOALLOC_MAX_N)).total <= NOALLOC_WS_BYTES,
              "32-bit scratch layout exceeds the static array");
static_assert(radix_layout(SOP_KEYS, 8, 0, NOALLOC_MAX_N,
                           tile_of<uint64_t, NoVal>(NOALLOC_MAX_N)).total <= NOALLOC_WS_BYTES,
              "64-bit scratch layout exceeds the static array");

// Device address of g_noalloc_scratch, looked up once per device.  In host
// code the symbol itself is only a host-side stand-in, never a device address.
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_addr[64];

// Per-device set-up of the first call, with that device current: look up the
// array's device address, then load every kernel a call can launch.  CUDA
// loads a kernel's code onto a device when it is first used (lazy loading),
// and that load allocates device memory; so the set-up sorts, inside the
// array itself, a small (one-CTA) and a mid-size (radix) array of each key
// width, synchronously.  Later calls on the device allocate nothing.
static int noalloc_prepare(unsigned char *scratch, cudaStream_t s)
{
    const LaunchOpts o{reinterpret_cast<unsigned *>(scratch), false};
    XSS_CUDA_TRY(cudaMemsetAsync(scratch, 0, NOALLOC_ERR_BYTES, s));
    for (int kbytes : {2, 4, 8}) {
        for (size_t n : {size_t(64), SMALL_SORT_MAX + 904}) {
            const size_t wsb = align_up(radix_chunk_workspace_bytes(SOP_KEYS, kbytes, 0, n), 256);
            unsigned char *ws = scratch + NOALLOC_ERR_BYTES;
            unsigned char *keys = ws + wsb;
            if (wsb + n * kbytes > NOALLOC_WS_BYTES) return XSS_ENOMEM;
            XSS_CUDA_TRY(cudaMemsetAsync(keys, 0, n * kbytes, s));
            const int rc = radix_sort_opts(SOP_KEYS, kbytes, KeyXform{XK_UINT, 0, 0}, keys,
                                           nullptr, 0, nullptr, n, ws, wsb, s, o);
            if (rc) return rc;
        }
    }
    XSS_CUDA_TRY(cudaStreamSynchronize(s));
    return XSS_OK;
}

static int noalloc_scratch(cudaStream_t s, unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return XSS_ECUDA;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return XSS_ECUDA;
        }
        const int rc = noalloc_prepare(static_cast<unsigned char *>(p), s);
        if (rc) return rc;
        g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_noalloc_addr[dev];
    return XSS_OK;
}

}  // namespace xss

extern "C" int xss_gpu_qsort_noalloc(int dtype, void *d_arr, size_t n, int hasnan,
                                     int descending, xss_stream_t stream)
{
    using namespace xss;
    int kbytes, kind;
    switch (dtype) {
    case XSS_DT_U16: kbytes = 2; kind = XK_UINT; break;
    case XSS_DT_I16: kbytes = 2; kind = XK_INT; break;
    case XSS_DT_F16: kbytes = 2; kind = XK_FLOAT; break;
    case XSS_DT_U32: kbytes = 4; kind = XK_UINT; break;
    case XSS_DT_I32: kbytes = 4; kind = XK_INT; break;
    case XSS_DT_F32: kbytes = 4; kind = XK_FLOAT; break;
    case XSS_DT_U64: kbytes = 8; kind = XK_UINT; break;
    case XSS_DT_I64: kbytes = 8; kind = XK_INT; break;
    case XSS_DT_F64: kbytes = 8; kind = XK_FLOAT; break;
    default: return XSS_EINVAL;
    }
    if (n > NOALLOC_MAX_N) return XSS_ETOOBIG;
    if (n > 1 && d_arr == nullptr) return XSS_EINVAL;
    if (n <= 1) return XSS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *scratch = nullptr;
    int rc = noalloc_scratch(s, &scratch);
    if (rc) return rc;
    XSS_CUDA_TRY(cudaMemsetAsync(scratch, 0, NOALLOC_ERR_BYTES, s));
    const KeyXform xf{kind, descending ? 1 : 0, hasnan ? 1 : 0};
    const LaunchOpts o{reinterpret_cast<unsigned *>(scratch), false};
    rc = radix_sort_opts(SOP_KEYS, kbytes, xf, d_arr, nullptr, 0, nullptr, n,
                         scratch + NOALLOC_ERR_BYTES, NOALLOC_WS_BYTES, s, o);
    if (rc) return rc;
    unsigned h = 0;
    XSS_CUDA_TRY(cudaMemcpyAsync(&h, scratch, sizeof(h), cudaMemcpyDeviceToHost, s));
    XSS_CUDA_TRY(cudaStreamSynchronize(s));
    return h ? XSS_ETIMEOUT : XSS_OK;
}
