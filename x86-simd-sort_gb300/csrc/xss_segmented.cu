// xss_segmented.cu -- batched sort of many independent segments.
//
// The reference sorts one array per call; a caller with many arrays calls it
// once per array.  Here all segments of a batch are sorted by a fixed handful
// of launches, whatever their number:
//   * segments of <= 32 keys: one warp each, bitonic network in registers;
//   * <= 256 keys: one CTA each, bitonic network in shared memory
//     (xss_blocksort.cuh);
//   * <= 4096 keys: one CTA each, stable LSD radix sort in shared memory
//     (xss_blockradix.cuh);
//   * larger segments: one segmented LSD radix sort -- the onesweep pass of
//     xss_onesweep.cuh over the tiles of every large segment at once, with
//     per-segment bucket starts and a look-back that stops at the first tile
//     of the tile's segment.
// The small-segment classes run on a side stream so they overlap the radix
// passes.  A plan (xss_seg_plan_*) bins the segments once; its launch
// sequence can be captured into a CUDA graph and replayed.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>
#include "xss_blockradix.cuh"
#include "xss_blocksort.cuh"
#include "xss_onesweep.cuh"

namespace xss {
int stream_status(cudaStream_t s);

constexpr uint32_t SEG_WARP_MAX = 32;
constexpr uint32_t SEG_SMALL_MAX = 256;
constexpr uint32_t SEG_MED_MAX = (uint32_t)SMALL_SORT_MAX;  // 4096
constexpr int SEG_SMALL_BLOCK = 128;
constexpr int SEG_MED_BLOCK = 256;
constexpr int SEG_MED_ITEMS = (int)SEG_MED_MAX / SEG_MED_BLOCK;
// mid-size segments up to this many keys take a 4-keys-per-thread CTA (fewer
// registers and less shared memory: more CTAs per SM)
constexpr uint32_t SEG_MED1_MAX = 1024;
constexpr int SEG_MED1_ITEMS = (int)SEG_MED1_MAX / SEG_MED_BLOCK;

struct SegArgs {
    void *keys;
    void *vals;
    void *tkeys;                 // scratch mirrors of keys / vals (large class)
    void *tvals;
    const uint64_t *offsets;     // num_segments + 1, device
    const uint32_t *list;        // segment ids of one class
    uint32_t count;              // entries in list
    KeyXform xf;
    // large class
    const uint32_t *large_ids;   // [L] segment id
    const uint32_t *large_tile0; // [L] first tile
    const uint32_t *tile_large;  // [T] large-list index of each tile
    uint32_t *seg_hist;          // [L][P][RADIX]
    uint32_t *seg_start;         // [L][P][RADIX]
    uint32_t *status;            // [2][T][RADIX]
    uint32_t *tile_ctr;          // [P]
    uint32_t L, T;
    int passes;
    unsigned *err;
    uint32_t topk;               // top-k plans: k (segments above 4096 keys)
};

// ---- <= 32 keys: one warp per segment -------------------------------------
template <typename C, typename V>
__global__ void __launch_bounds__(256) seg_warp_kernel(SegArgs a)
{
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    const uint32_t w = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= a.count) return;  // whole warps leave together
    const uint32_t s = a.list[w];
    const uint64_t off = a.offsets[s];
    const uint32_t len = (uint32_t)(a.offsets[s + 1] - off);
    C *keys = static_cast<C *>(a.keys) + off;
    C code = lane < (int)len ? to_code(keys[lane], a.xf) : C(~C(0));
    uint32_t idx = lane;
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const C oc = __shfl_xor_sync(0xffffffffu, code, j);
            const uint32_t oi = __shfl_xor_sync(0xffffffffu, idx, j);
            const bool other_less = (oc < code) || (oc == code && oi < idx);
            const bool lower = (lane & j) == 0;
            const bool up = (lane & k) == 0;
            if (lower == up ? other_less : !other_less) {
                code = oc;
                idx = oi;
            }
        }
    }
    V v{};
    if constexpr (HAS_V) {
        V *vals = static_cast<V *>(a.vals) + off;
        if (lane < (int)len) v = vals[idx];
        __syncwarp();
        if (lane < (int)len) vals[lane] = v;
    }
    if (lane < (int)len) keys[lane] = from_code(code, a.xf);
}

// ---- <= MAXN keys: one CTA per segment --------------------------------------
template <typename C, typename V, int BLOCK, int MAXN>
__global__ void __launch_bounds__(BLOCK) seg_block_kernel(SegArgs a)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    const uint32_t s = a.list[blockIdx.x];
    const uint64_t off = a.offsets[s];
    const uint32_t len = (uint32_t)(a.offsets[s + 1] - off);
    uint32_t npad = 2;
    while (npad < len) npad <<= 1;
    C *keys = static_cast<C *>(a.keys) + off;
    V *vals = nullptr;
    if constexpr (!std::is_same<V, NoVal>::value) vals = static_cast<V *>(a.vals) + off;
    block_bitonic_sort<C, V, BLOCK, MAXN>(keys, keys, vals, vals, nullptr, len, npad, a.xf,
                                          s_raw);
}

// ---- <= 4096 keys: one CTA per segment, radix sort in shared memory --------
template <typename C, typename V, int ITEMS>
__global__ void __launch_bounds__(SEG_MED_BLOCK) seg_radix_kernel(SegArgs a)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    const uint32_t s = a.list[blockIdx.x];
    const uint64_t off = a.offsets[s];
    const uint32_t len = (uint32_t)(a.offsets[s + 1] - off);
    C *keys = static_cast<C *>(a.keys) + off;
    V *vals = nullptr;
    if constexpr (!std::is_same<V, NoVal>::value) vals = static_cast<V *>(a.vals) + off;
    block_radix_sort<C, V, SEG_MED_BLOCK, ITEMS>(keys, vals, len, (int)sizeof(C), a.xf, s_raw);
}

// ---- top-k of a segment longer than 4096 keys: one CTA streams it once ------
// For k <= SEG_TOPK_MAX (the segment's k smallest codes, in order, at its
// front; the other keys anywhere in the rest of it).  The CTA sorts the
// segment's first SEG_MED_MAX keys on chip (block_radix_sort) and writes them
// back: the first k are the best k so far, and thr (the code of the k-th)
// bounds what can still enter.  It then reads the rest in windows of
// SEG_TOPK_W positions; a key whose code is below thr is staged, raw, in the
// block sort's own tile after the best k (its position kept in `cpos`), and
// every other key stays where it is.  When the stage would overflow, and at
// the end, the best k are read back in front of the staged keys, the tile is
// sorted (stable), the first k go back to the segment's front and the rest
// into the positions the staged keys came from; thr tightens.  Each key is
// read once and written only if it was staged, so the pass is bound by
// reading the segment, not by four radix passes.  Keys equal to thr are not
// staged: any of the tied keys completes the k smallest.
constexpr uint32_t SEG_TOPK_MAX = SEG_MED_MAX / 2;   // 2048: a stage of >= one window
constexpr int SEG_TOPK_WI = 8;                        // window items per thread
constexpr uint32_t SEG_TOPK_W = SEG_MED_BLOCK * SEG_TOPK_WI;   // 2048 positions

template <typename C, typename V> constexpr size_t seg_topk_smem()
{
    return block_radix_smem<C, V, SEG_MED_BLOCK, SEG_MED_ITEMS>() +
           (size_t)SEG_MED_MAX * sizeof(uint32_t) + 32 * sizeof(uint32_t);
}

template <typename C, typename V>
__global__ void __launch_bounds__(SEG_MED_BLOCK) seg_topk_kernel(SegArgs a)
{
    constexpr int BLOCK = SEG_MED_BLOCK, ITEMS = SEG_MED_ITEMS, WI = SEG_TOPK_WI;
    constexpr uint32_t TILE = SEG_MED_MAX;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    using VS = typename std::conditional<HAS_V, V, uint8_t>::type;
    static_assert((uint32_t)BLOCK * ITEMS == TILE, "the tile is the block sort's capacity");
    static_assert(SEG_TOPK_W <= TILE - SEG_TOPK_MAX, "a window's keys always fit the stage");
    extern __shared__ __align__(16) unsigned char s_raw[];
    C *s_k = reinterpret_cast<C *>(s_raw);   // the block sort's key tile
    VS *s_v = reinterpret_cast<VS *>(s_raw + round16((size_t)TILE * sizeof(C)));
    uint32_t *cpos = reinterpret_cast<uint32_t *>(
        s_raw + block_radix_smem<C, V, BLOCK, ITEMS>());   // [TILE - k] staged positions
    uint32_t *s_scan = cpos + TILE;                          // [32]

    const uint32_t s = a.list[blockIdx.x];
    const uint64_t off = a.offsets[s];
    const uint32_t len = (uint32_t)(a.offsets[s + 1] - off);   // > TILE by the plan
    const uint32_t K = a.topk;                                   // 1 .. SEG_TOPK_MAX
    C *keys = static_cast<C *>(a.keys) + off;
    VS *vals = nullptr;
    if constexpr (HAS_V) vals = static_cast<V *>(a.vals) + off;
    const int tid = threadIdx.x;
    if (len <= TILE || K == 0 || K > SEG_TOPK_MAX) return;   // the plan never sends these

    // the first TILE keys, sorted on chip and written back
    for (uint32_t e = tid; e < TILE; e += BLOCK) {
        s_k[e] = keys[e];
        if constexpr (HAS_V) s_v[e] = vals[e];
    }
    __syncthreads();
    block_radix_sort<C, V, BLOCK, ITEMS>(s_k, reinterpret_cast<V *>(s_v), TILE, (int)sizeof(C),
                                         a.xf, s_raw);
    __syncthreads();
    for (uint32_t e = tid; e < TILE; e += BLOCK) {
        keys[e] = s_k[e];
        if constexpr (HAS_V) vals[e] = s_v[e];
    }
    C thr = to_code(s_k[K - 1], a.xf);
    __syncthreads();   // the stage below reuses s_k beyond the best k

    const uint32_t cap = TILE - K;
    uint32_t cnt = 0;   // staged keys (uniform across the CTA)
    // merge the stage into the best k; the evicted keys fill the stage's holes
    auto flush = [&]() {
        __syncthreads();   // every staged key and position is in shared memory
        for (uint32_t e = tid; e < K; e += BLOCK) {
            s_k[e] = keys[e];
            if constexpr (HAS_V) s_v[e] = vals[e];
        }
        __syncthreads();
        block_radix_sort<C, V, BLOCK, ITEMS>(s_k, reinterpret_cast<V *>(s_v), K + cnt,
                                             (int)sizeof(C), a.xf, s_raw);
        __syncthreads();
        for (uint32_t e = tid; e < K; e += BLOCK) {
            keys[e] = s_k[e];
            if constexpr (HAS_V) vals[e] = s_v[e];
        }
        for (uint32_t i = tid; i < cnt; i += BLOCK) {
            const uint32_t p = cpos[i];
            if (p < len) {
                keys[p] = s_k[K + i];
                if constexpr (HAS_V) vals[p] = s_v[K + i];
            }
        }
        thr = to_code(s_k[K - 1], a.xf);
        __syncthreads();   // s_k and cpos are restaged next
        cnt = 0;
    };

    for (uint32_t p0 = TILE; p0 < len; p0 += SEG_TOPK_W) {
        C raw[WI], code[WI];
#pragma unroll
        for (int j = 0; j < WI; ++j) {
            const uint32_t p = p0 + (uint32_t)j * BLOCK + tid;
            raw[j] = p < len ? keys[p] : C(0);
            code[j] = to_code(raw[j], a.xf);
        }
        uint32_t mine = 0;
#pragma unroll
        for (int j = 0; j < WI; ++j)
            mine += (p0 + (uint32_t)j * BLOCK + tid < len && code[j] < thr) ? 1u : 0u;
        uint32_t tot;
        uint32_t at = block_excl_scan<BLOCK>(mine, s_scan, tot);
        if (cnt + tot > cap) {   // uniform: merge first, then stage against the new bound
            flush();
            mine = 0;
#pragma unroll
            for (int j = 0; j < WI; ++j)
                mine += (p0 + (uint32_t)j * BLOCK + tid < len && code[j] < thr) ? 1u : 0u;
            at = block_excl_scan<BLOCK>(mine, s_scan, tot);
        }
        at += cnt;
#pragma unroll
        for (int j = 0; j < WI; ++j) {
            const uint32_t p = p0 + (uint32_t)j * BLOCK + tid;
            if (p < len && code[j] < thr && at < cap) {
                s_k[K + at] = raw[j];
                if constexpr (HAS_V) s_v[K + at] = vals[p];
                cpos[at] = p;
                ++at;
            }
        }
        cnt += tot;
    }
    if (cnt) flush();
}

// ---- large segments: histogram of every pass per segment ---------------------
template <typename C, int TILE>
__global__ void __launch_bounds__(256) seg_hist_kernel(SegArgs a)
{
    // Each CTA takes a contiguous run of tiles.  Tiles of one segment are
    // contiguous, so the CTA accumulates in shared memory and adds to the
    // segment's global histograms only when the segment changes (once per
    // segment it touches, not once per tile).
    __shared__ uint32_t sh[MAX_PASSES * RADIX];
    const int tid = threadIdx.x;
    const int P = a.passes;
    const uint32_t per = (a.T + gridDim.x - 1) / gridDim.x;
    const uint32_t t0 = blockIdx.x * per;
    const uint32_t t1 = min(a.T, t0 + per);
    for (int i = tid; i < P * RADIX; i += 256) sh[i] = 0;
    uint32_t cur = 0xffffffffu;   // large-segment index being accumulated
    auto flush = [&]() {
        __syncthreads();
        if (cur != 0xffffffffu) {
            uint32_t *gh = a.seg_hist + (size_t)cur * P * RADIX;
            for (int i = tid; i < P * RADIX; i += 256) {
                if (sh[i]) atomicAdd(&gh[i], sh[i]);
                sh[i] = 0;
            }
        }
        __syncthreads();
    };
    for (uint32_t t = t0; t < t1; ++t) {
        const uint32_t l = a.tile_large[t];
        if (l != cur) {
            flush();
            cur = l;
        }
        const uint32_t s = a.large_ids[l];
        const uint64_t off = a.offsets[s];
        const uint32_t len = (uint32_t)(a.offsets[s + 1] - off);
        const uint32_t base = (t - a.large_tile0[l]) * (uint32_t)TILE;
        const uint32_t end = min(len, base + (uint32_t)TILE);
        // the first pass's look-back row of this tile starts cleared
        for (int i = tid; i < RADIX; i += 256) a.status[(size_t)t * RADIX + i] = 0;
        const C *keys = static_cast<const C *>(a.keys) + off;
        for (uint32_t i = base + tid; i < end; i += 256) {
            const C c = to_code(keys[i], a.xf);
#pragma unroll
            for (int p = 0; p < (int)sizeof(C); ++p)
                if (p < P)
                    atomicAdd(&sh[p * RADIX + (uint32_t(c >> (p * RADIX_BITS)) & (RADIX - 1))], 1u);
        }
    }
    flush();
}

// ---- large segments: bucket starts (per segment, per pass) -------------------
__global__ void __launch_bounds__(256) seg_scan_kernel(SegArgs a)
{
    __shared__ uint32_t s_scan[8];
    const uint32_t l = blockIdx.x;
    for (int p = 0; p < a.passes; ++p) {
        const size_t row = ((size_t)l * a.passes + p) * RADIX;
        uint32_t total;
        const uint32_t ex = block_excl_scan<256>(a.seg_hist[row + threadIdx.x], s_scan, total);
        a.seg_start[row + threadIdx.x] = ex;
    }
}

// ---- large segments: one LSD pass over every large segment's tiles ----------
template <typename C, typename V, int BLOCK, int ITEMS, int MINB, int LB, int RANK, int DPT>
__global__ void __launch_bounds__(BLOCK, MINB) seg_pass_kernel(SegArgs a, int pass)
{
    constexpr int TILE = BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    using VS = typename std::conditional<HAS_V, V, uint8_t>::type;
    __shared__ PassSmem<BLOCK, RANK> ps;
    __shared__ uint32_t s_tile;
    extern __shared__ __align__(128) unsigned char s_dyn[];
    C *s_k = reinterpret_cast<C *>(s_dyn);
    VS *s_v = reinterpret_cast<VS *>(s_dyn + TILE * sizeof(C));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < PassSmem<BLOCK, RANK>::WORDS; i += BLOCK) ps.wm[i] = 0;
    if (tid == 0) s_tile = atomicAdd(&a.tile_ctr[pass], 1u);
    __syncthreads();
    const uint32_t t = s_tile;
    const uint32_t l = a.tile_large[t];
    const uint32_t s = a.large_ids[l];
    const uint64_t off = a.offsets[s];
    const uint32_t len = (uint32_t)(a.offsets[s + 1] - off);
    const uint32_t base = (t - a.large_tile0[l]) * (uint32_t)TILE;

    PassDesc pd{};
    pd.active = 1;
    pd.first = pass == 0;
    pd.last = pass == a.passes - 1;
    const bool even = (pass & 1) == 0;
    const C *ksrc = static_cast<const C *>(even ? a.keys : a.tkeys) + off;
    C *kdst = static_cast<C *>(even ? a.tkeys : a.keys) + off;

    // clear this tile's rows of the next pass's look-back buffer (the pass
    // that used it last has finished)
    if (pass + 1 < a.passes)
        for (int i = tid; i < RADIX; i += BLOCK)
            a.status[((size_t)((pass + 1) & 1) * a.T + t) * RADIX + i] = 0;

    const uint32_t first_idx = base + (uint32_t)warp * (ITEMS * 32) + lane;
    C key[ITEMS];
    VS val[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint32_t idx = first_idx + j * 32;
        if (idx < len) {
            const C b = ksrc[idx];
            key[j] = pd.first ? to_code(b, a.xf) : b;
        } else {
            key[j] = C(~C(0));
        }
    }
    V *vdst = nullptr;
    if constexpr (HAS_V) {
        const V *vsrc = static_cast<const V *>(even ? a.vals : a.tvals) + off;
        vdst = static_cast<V *>(even ? a.tvals : a.vals) + off;
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t idx = first_idx + j * 32;
            val[j] = idx < len ? vsrc[idx] : VS(0);
        }
    }
    RadixArgs ra{};
    ra.xf = a.xf;
    ra.err = a.err;
    ra.num_tiles = a.T;
    const TileJob job{t, a.large_tile0[l], base, len,
                      a.seg_start + ((size_t)l * a.passes + pass) * RADIX,
                      a.status + (size_t)(pass & 1) * a.T * RADIX};
    const Codec<C> cx(a.xf);   // unused with ROLE_RUNTIME (from_code decides)
    // s_dyn holds TILE keys then TILE values: the layout pair staging needs
    pass_tile<C, V, BLOCK, ITEMS, LB, RANK, DPT, ROLE_RUNTIME, pair_staged<C, VS, RANK>()>(
        ra, pd, pass, job, key, val, s_k, s_v, ps, kdst, vdst, cx, NoAfterRank{});
}

// ---------------------------------------------------------------------------
// Host side: plan = segments binned by size, tile map of the large class.
struct SegLayout {
    size_t warp, small, med, lids, ltile0, tlarge, hist, start, status, ctr, tkeys, tvals, tk,
        total;
};

struct SegPlan {
    int key_dtype, val_dtype, kb, vb, kind;
    int hasnan, desc;
    size_t nseg, total_n;
    size_t tile;
    std::vector<uint32_t> warp, small, med, lids, ltile0, tlarge;
    size_t med1 = 0;    // the first med1 entries of med hold <= SEG_MED1_MAX keys
    // top-k plans (1 <= topk <= SEG_TOPK_MAX): segments above SEG_MED_MAX keys
    // go to `tk` (seg_topk_kernel) instead of the segmented radix sort
    uint32_t topk = 0;
    std::vector<uint32_t> tk;
    SegLayout lay;
    // graph cache for one (keys, vals, offsets, workspace) binding
    cudaGraphExec_t exec = nullptr;
    const void *gk = nullptr, *gv = nullptr, *goff = nullptr, *gws = nullptr;
    const void *uploaded_to = nullptr;  // workspace that holds this plan's lists
    unsigned long long graph_launches[PK_COUNT] = {};  // kernels per graph replay, by kind
};

// Pass lines (BLOCK, ITEMS, MINB, LB, RANK, PERSIST, DPT) of the large
// class.  Its tiles run one CTA per tile across many segments, so it keeps
// lines measured for that form (two CTAs per SM) instead of the resident
// lines tuned for one whole array.  Ranking by the count atomic (RANK 2) and
// larger tiles took the 200,000-segment batch (4.2e9 keys) from 123.3 to
// 93.5 ms (int32 -> uint32) and from 127.7 to 99.4 ms (float32); three CTAs
// per SM of 384 x 12 then to 89.5 / 94.6 ms (512 x 12 x 2: 93.9 / 99.7;
// 256 x 12 x 4: 93.1 / 98.9; 256 x 16 x 3: 96.4 / 102.9; 512 x 8 x 3:
// 97.9 / 100.7 ms).  A resident form (CTAs claiming tiles in order, the next
// tile claimed once the current one is ranked and bulk-copied when it is
// full and 16-byte aligned) measured slower on the literal batch: 99.5 ms
// (512 x 10, 2 CTAs per SM), 105.9 (256 x 14 x 3), 107.0 (384 x 12 x 2),
// 120.0 (512 x 24 x 1) against 89.4 ms, and 1.6 s with 4 CTAs per SM of
// 256 x 10.  Only segments whose first key sits on a 16-byte boundary can be
// bulk-copied, the second buffer costs a CTA per SM, and a tile claimed
// ahead publishes its counts a tile later, so its successors' look-backs
// poll longer (with many small tiles in flight the polling fills L2).
#ifndef XSS_SEGCFG_KEYS
#define XSS_SEGCFG_KEYS 512, 16, 2, 16, 2, 0, 0
#endif
#ifndef XSS_SEGCFG_K32V32
#define XSS_SEGCFG_K32V32 384, 12, 3, 16, 2, 0, 0
#endif
#ifndef XSS_SEGCFG_DEFAULT
#define XSS_SEGCFG_DEFAULT 256, 16, 2, 16, 2, 0, 0
#endif
template <typename C, typename V> struct SegPassCfg : CfgT<XSS_SEGCFG_DEFAULT> {};
template <> struct SegPassCfg<uint16_t, NoVal> : CfgT<XSS_SEGCFG_KEYS> {};
template <> struct SegPassCfg<uint32_t, NoVal> : CfgT<XSS_SEGCFG_KEYS> {};
template <> struct SegPassCfg<uint32_t, uint32_t> : CfgT<XSS_SEGCFG_K32V32> {};

template <typename C, typename V> constexpr size_t seg_tile()
{
    return (size_t)SegPassCfg<C, V>::BLOCK * SegPassCfg<C, V>::ITEMS;
}

static size_t seg_tile_size(int kb, int vb)
{
    switch (kb) {
    case 2: return vb == 0 ? seg_tile<uint16_t, NoVal>() : vb == 2 ? seg_tile<uint16_t, uint16_t>() : vb == 4 ? seg_tile<uint16_t, uint32_t>() : seg_tile<uint16_t, uint64_t>();
    case 4: return vb == 0 ? seg_tile<uint32_t, NoVal>() : vb == 2 ? seg_tile<uint32_t, uint16_t>() : vb == 4 ? seg_tile<uint32_t, uint32_t>() : seg_tile<uint32_t, uint64_t>();
    default: return vb == 0 ? seg_tile<uint64_t, NoVal>() : vb == 2 ? seg_tile<uint64_t, uint16_t>() : vb == 4 ? seg_tile<uint64_t, uint32_t>() : seg_tile<uint64_t, uint64_t>();
    }
}

static int plan_build(SegPlan &p, const uint64_t *off, size_t nseg)
{
    p.nseg = nseg;
    p.total_n = nseg ? off[nseg] : 0;
    p.tile = seg_tile_size(p.kb, p.vb);
    p.warp.clear(); p.small.clear(); p.med.clear(); p.lids.clear(); p.ltile0.clear(); p.tlarge.clear();
    p.tk.clear();
    std::vector<uint32_t> med2;
    for (size_t i = 0; i < nseg; ++i) {
        if (off[i + 1] < off[i]) return XSS_EINVAL;
        const uint64_t len = off[i + 1] - off[i];
        if (len > XSS_SEGMENT_MAX_N) return XSS_ETOOBIG;
        if (len <= 1) continue;
        if (len <= SEG_WARP_MAX) p.warp.push_back((uint32_t)i);
        else if (len <= SEG_SMALL_MAX) p.small.push_back((uint32_t)i);
        else if (len <= SEG_MED1_MAX) p.med.push_back((uint32_t)i);
        else if (len <= SEG_MED_MAX) med2.push_back((uint32_t)i);
        else if (p.topk) p.tk.push_back((uint32_t)i);
        else {
            p.ltile0.push_back((uint32_t)p.tlarge.size());
            const uint32_t l = (uint32_t)p.lids.size();
            p.lids.push_back((uint32_t)i);
            const size_t tiles = (len + p.tile - 1) / p.tile;
            if (p.tlarge.size() + tiles > 0xffffffffull) return XSS_ETOOBIG;
            p.tlarge.insert(p.tlarge.end(), tiles, l);
        }
    }
    p.med1 = p.med.size();
    p.med.insert(p.med.end(), med2.begin(), med2.end());
    const size_t L = p.lids.size(), T = p.tlarge.size(), P = p.kb;
    SegLayout &y = p.lay;
    size_t o = 0;
    auto take = [&](size_t bytes) { const size_t at = o; o = align_up(o + bytes, 256); return at; };
    y.warp = take(p.warp.size() * 4);
    y.small = take(p.small.size() * 4);
    y.med = take(p.med.size() * 4);
    y.lids = take(L * 4);
    y.ltile0 = take(L * 4);
    y.tlarge = take(T * 4);
    y.hist = take(L * P * RADIX * 4);
    y.start = take(L * P * RADIX * 4);
    y.status = take(2 * T * RADIX * 4);
    y.ctr = take(MAX_PASSES * 4);
    // the large class ping-pongs through mirrors of the whole batch
    y.tkeys = take(L ? p.total_n * p.kb : 0);
    y.tvals = take(L && p.vb ? p.total_n * p.vb : 0);
    y.tk = take(p.tk.size() * 4);
    y.total = o;
    return XSS_OK;
}

// Side stream + fork/join events for overlapping the small classes.
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
static std::mutex g_side_mu;
static SideStream g_side[64];

static int side_stream(SideStream *&out)
{
    int d = 0;
    cudaGetDevice(&d);
    if (d < 0 || d >= 64) return XSS_ECUDA;
    std::lock_guard<std::mutex> lk(g_side_mu);
    SideStream &ss = g_side[d];
    if (!ss.s) {
        if (cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming) != cudaSuccess)
            return XSS_ECUDA;
    }
    out = &ss;
    return XSS_OK;
}

template <typename C, typename V>
static int seg_launch(const SegPlan &p, SegArgs a, cudaStream_t s)
{
    using Cfg = SegPassCfg<C, V>;
    constexpr int BLOCK = Cfg::BLOCK, ITEMS = Cfg::ITEMS, MINB = Cfg::MINB, LB = Cfg::LB,
                  RANK = Cfg::RANK, DPT = Cfg::DPT;
    constexpr size_t TILE = (size_t)BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    const bool any_small = !p.warp.empty() || !p.small.empty() || !p.med.empty();
    const bool any_large = !p.lids.empty() || !p.tk.empty();
    SideStream *side = nullptr;
    cudaStream_t ss = s;
    if (any_small && any_large) {
        int rc = side_stream(side);
        if (rc) return rc;
        ss = side->s;
        XSS_CUDA_TRY(cudaEventRecord(side->fork, s));
        XSS_CUDA_TRY(cudaStreamWaitEvent(ss, side->fork, 0));
    }
    char *ws = static_cast<char *>(const_cast<void *>(p.uploaded_to));
    if (!p.warp.empty()) {
        SegArgs b = a;
        b.list = reinterpret_cast<const uint32_t *>(ws + p.lay.warp);
        b.count = (uint32_t)p.warp.size();
        XSS_LAUNCH(PK_SEG_SMALL, ss,
                   (seg_warp_kernel<C, V><<<(b.count + 7) / 8, 256, 0, ss>>>(b)));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    if (!p.small.empty()) {
        SegArgs b = a;
        b.list = reinterpret_cast<const uint32_t *>(ws + p.lay.small);
        b.count = (uint32_t)p.small.size();
        const size_t smem = align_up(sizeof(C) * SEG_SMALL_MAX, 16) + 2 * SEG_SMALL_MAX;
        XSS_LAUNCH(PK_SEG_BLOCK, ss,
                   (seg_block_kernel<C, V, SEG_SMALL_BLOCK, SEG_SMALL_MAX>
                    <<<b.count, SEG_SMALL_BLOCK, smem, ss>>>(b)));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    if (p.med1 > 0) {
        SegArgs b = a;
        b.list = reinterpret_cast<const uint32_t *>(ws + p.lay.med);
        b.count = (uint32_t)p.med1;
        const size_t smem = block_radix_smem<C, V, SEG_MED_BLOCK, SEG_MED1_ITEMS>();
        auto kern = seg_radix_kernel<C, V, SEG_MED1_ITEMS>;
        {
            const int rc = set_max_dyn_smem((const void *)kern, smem);
            if (rc) return rc;
        }
        XSS_LAUNCH(PK_SEG_BLOCK, ss, (kern<<<b.count, SEG_MED_BLOCK, smem, ss>>>(b)));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    if (p.med.size() > p.med1) {
        SegArgs b = a;
        b.list = reinterpret_cast<const uint32_t *>(ws + p.lay.med) + p.med1;
        b.count = (uint32_t)(p.med.size() - p.med1);
        const size_t smem = block_radix_smem<C, V, SEG_MED_BLOCK, SEG_MED_ITEMS>();
        auto kern = seg_radix_kernel<C, V, SEG_MED_ITEMS>;
        {
            const int rc = set_max_dyn_smem((const void *)kern, smem);
            if (rc) return rc;
        }
        XSS_LAUNCH(PK_SEG_BLOCK, ss, (kern<<<b.count, SEG_MED_BLOCK, smem, ss>>>(b)));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    if (!p.tk.empty()) {
        SegArgs b = a;
        b.list = reinterpret_cast<const uint32_t *>(ws + p.lay.tk);
        b.count = (uint32_t)p.tk.size();
        b.topk = p.topk;
        const size_t smem = seg_topk_smem<C, V>();
        auto kern = seg_topk_kernel<C, V>;
        {
            const int rc = set_max_dyn_smem((const void *)kern, smem);
            if (rc) return rc;
        }
        XSS_LAUNCH(PK_SEG_BLOCK, s, (kern<<<b.count, SEG_MED_BLOCK, smem, s>>>(b)));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    if (!p.lids.empty()) {
        SegArgs b = a;
        b.large_ids = reinterpret_cast<const uint32_t *>(ws + p.lay.lids);
        b.large_tile0 = reinterpret_cast<const uint32_t *>(ws + p.lay.ltile0);
        b.tile_large = reinterpret_cast<const uint32_t *>(ws + p.lay.tlarge);
        b.seg_hist = reinterpret_cast<uint32_t *>(ws + p.lay.hist);
        b.seg_start = reinterpret_cast<uint32_t *>(ws + p.lay.start);
        b.status = reinterpret_cast<uint32_t *>(ws + p.lay.status);
        b.tile_ctr = reinterpret_cast<uint32_t *>(ws + p.lay.ctr);
        b.tkeys = ws + p.lay.tkeys;
        b.tvals = ws + p.lay.tvals;
        b.L = (uint32_t)p.lids.size();
        b.T = (uint32_t)p.tlarge.size();
        XSS_CUDA_TRY(cudaMemsetAsync(b.seg_hist, 0, (size_t)b.L * b.passes * RADIX * 4, s));
        XSS_CUDA_TRY(cudaMemsetAsync(b.tile_ctr, 0, MAX_PASSES * 4, s));
        const uint32_t hgrid = (uint32_t)std::max<size_t>(1, std::min<size_t>(b.T, (size_t)num_sms() * 8));
        XSS_LAUNCH(PK_SEG_MISC, s, (seg_hist_kernel<C, TILE><<<hgrid, 256, 0, s>>>(b)));
        XSS_CUDA_TRY(cudaGetLastError());
        XSS_LAUNCH(PK_SEG_MISC, s, (seg_scan_kernel<<<b.L, 256, 0, s>>>(b)));
        XSS_CUDA_TRY(cudaGetLastError());
        const size_t smem = TILE * (sizeof(C) + (HAS_V ? sizeof(V) : 0));
        auto kern = seg_pass_kernel<C, V, BLOCK, ITEMS, MINB, LB, RANK, DPT>;
        {
            const int rc = set_max_dyn_smem((const void *)kern, smem);
            if (rc) return rc;
        }
        for (int pass = 0; pass < b.passes; ++pass) {
            XSS_LAUNCH(PK_ONESWEEP, s, (kern<<<b.T, BLOCK, smem, s>>>(b, pass)));
            XSS_CUDA_TRY(cudaGetLastError());
        }
    }
    if (side) {
        XSS_CUDA_TRY(cudaEventRecord(side->join, ss));
        XSS_CUDA_TRY(cudaStreamWaitEvent(s, side->join, 0));
    }
    return XSS_OK;
}

template <typename C>
static int seg_launch_v(const SegPlan &p, SegArgs a, cudaStream_t s)
{
    if (p.vb == 0) return seg_launch<C, NoVal>(p, a, s);
    if (p.vb == 2) return seg_launch<C, uint16_t>(p, a, s);
    if (p.vb == 4) return seg_launch<C, uint32_t>(p, a, s);
    return seg_launch<C, uint64_t>(p, a, s);
}

static int dtype_kind(int dt, int &kb, int &kind)
{
    switch (dt) {
    case XSS_DT_U16: kb = 2; kind = XK_UINT; return XSS_OK;
    case XSS_DT_I16: kb = 2; kind = XK_INT; return XSS_OK;
    case XSS_DT_F16: kb = 2; kind = XK_FLOAT; return XSS_OK;
    case XSS_DT_U32: kb = 4; kind = XK_UINT; return XSS_OK;
    case XSS_DT_I32: kb = 4; kind = XK_INT; return XSS_OK;
    case XSS_DT_F32: kb = 4; kind = XK_FLOAT; return XSS_OK;
    case XSS_DT_U64: kb = 8; kind = XK_UINT; return XSS_OK;
    case XSS_DT_I64: kb = 8; kind = XK_INT; return XSS_OK;
    case XSS_DT_F64: kb = 8; kind = XK_FLOAT; return XSS_OK;
    default: return XSS_EINVAL;
    }
}

static int plan_init(SegPlan &p, int key_dtype, int val_dtype, const uint64_t *h_offsets,
                     size_t nseg, int hasnan, int descending, uint32_t topk = 0)
{
    p.topk = topk;
    int rc = dtype_kind(key_dtype, p.kb, p.kind);
    if (rc) return rc;
    p.key_dtype = key_dtype;
    p.val_dtype = val_dtype;
    p.vb = 0;
    if (val_dtype >= 0) {
        if (val_dtype < XSS_DT_U16 || val_dtype > XSS_DT_F64) return XSS_EUNSUPPORTED;
        p.vb = val_dtype >= XSS_DT_U64 ? 8 : (val_dtype >= XSS_DT_U32 ? 4 : 2);
    }
    p.hasnan = hasnan;
    p.desc = descending;
    if (nseg && !h_offsets) return XSS_EINVAL;
    return plan_build(p, h_offsets, nseg);
}

static int plan_upload(SegPlan &p, char *ws, cudaStream_t s)
{
    auto up = [&](size_t at, const std::vector<uint32_t> &v) -> int {
        if (v.empty()) return XSS_OK;
        XSS_CUDA_TRY(cudaMemcpyAsync(ws + at, v.data(), v.size() * 4, cudaMemcpyHostToDevice, s));
        return XSS_OK;
    };
    int rc;
    if ((rc = up(p.lay.warp, p.warp)) || (rc = up(p.lay.small, p.small)) ||
        (rc = up(p.lay.med, p.med)) || (rc = up(p.lay.lids, p.lids)) ||
        (rc = up(p.lay.ltile0, p.ltile0)) || (rc = up(p.lay.tlarge, p.tlarge)) ||
        (rc = up(p.lay.tk, p.tk)))
        return rc;
    // pageable copies: make sure they are done before the vectors can change
    XSS_CUDA_TRY(cudaStreamSynchronize(s));
    p.uploaded_to = ws;
    return XSS_OK;
}

static int plan_enqueue(SegPlan &p, void *d_keys, void *d_vals, const uint64_t *d_offsets,
                        cudaStream_t s)
{
    SegArgs a{};
    a.keys = d_keys;
    a.vals = d_vals;
    a.offsets = d_offsets;
    a.xf = KeyXform{p.kind, p.desc ? 1 : 0, (p.vb == 0 && p.hasnan) ? 1 : 0};
    a.passes = p.kb;
    a.err = device_error_word();
    if (!a.err) return XSS_ECUDA;
    switch (p.kb) {
    case 2: return seg_launch_v<uint16_t>(p, a, s);
    case 4: return seg_launch_v<uint32_t>(p, a, s);
    default: return seg_launch_v<uint64_t>(p, a, s);
    }
}

}  // namespace xss

using namespace xss;

struct xss_seg_plan_s {
    SegPlan p;
};

extern "C" {

int xss_seg_plan_create(xss_seg_plan_s **out, int key_dtype, int val_dtype,
                        const uint64_t *h_offsets, size_t num_segments, int hasnan,
                        int descending)
{
    if (!out) return XSS_EINVAL;
    *out = nullptr;
    auto *pl = new (std::nothrow) xss_seg_plan_s();
    if (!pl) return XSS_ENOMEM;
    const int rc = plan_init(pl->p, key_dtype, val_dtype, h_offsets, num_segments, hasnan,
                             descending);
    if (rc) {
        delete pl;
        return rc;
    }
    // allocate the error word now, outside any stream capture
    if (!device_error_word()) {
        delete pl;
        return XSS_ECUDA;
    }
    *out = pl;
    return XSS_OK;
}

size_t xss_seg_plan_workspace_size(const xss_seg_plan_s *plan)
{
    return plan ? plan->p.lay.total : 0;
}

int xss_seg_plan_run(xss_seg_plan_s *plan, void *d_keys, void *d_vals, const uint64_t *d_offsets,
                     void *d_ws, size_t ws_bytes, xss_stream_t stream, int use_graph)
{
    if (!plan) return XSS_EINVAL;
    SegPlan &p = plan->p;
    if (p.nseg == 0 || p.total_n == 0) return XSS_OK;
    if (!d_keys || !d_offsets || (p.vb && !d_vals)) return XSS_EINVAL;
    if (!d_ws || ws_bytes < p.lay.total) return XSS_ENOMEM;
    cudaStream_t s = (cudaStream_t)stream;
    if (p.uploaded_to != d_ws) {
        const int rc = plan_upload(p, static_cast<char *>(d_ws), s);
        if (rc) return rc;
        if (p.exec) {
            cudaGraphExecDestroy(p.exec);
            p.exec = nullptr;
        }
    }
    if (!use_graph) return plan_enqueue(p, d_keys, d_vals, d_offsets, s);
    if (!p.exec || p.gk != d_keys || p.gv != d_vals || p.goff != d_offsets || p.gws != d_ws) {
        if (p.exec) {
            cudaGraphExecDestroy(p.exec);
            p.exec = nullptr;
        }
        // capture on a private stream so the caller's stream is never in capture mode
        cudaStream_t cs;
        XSS_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        int rc = XSS_OK;
        if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            rc = XSS_ECUDA;
        } else {
            // launches issued while capturing did not run: move them from the
            // counters into the per-replay count
            unsigned long long before[PK_COUNT], after[PK_COUNT];
            prof_snapshot(before);
            rc = plan_enqueue(p, d_keys, d_vals, d_offsets, cs);
            prof_snapshot(after);
            for (int k = 0; k < PK_COUNT; ++k) p.graph_launches[k] = after[k] - before[k];
            prof_sub(p.graph_launches);
            if (cudaStreamEndCapture(cs, &g) != cudaSuccess) rc = rc ? rc : XSS_ECUDA;
        }
        if (rc == XSS_OK && cudaGraphInstantiate(&p.exec, g, 0) != cudaSuccess) rc = XSS_ECUDA;
        if (g) cudaGraphDestroy(g);
        cudaStreamDestroy(cs);
        if (rc) {
            cudaGetLastError();
            p.exec = nullptr;
            return rc;
        }
        p.gk = d_keys;
        p.gv = d_vals;
        p.goff = d_offsets;
        p.gws = d_ws;
    }
    XSS_CUDA_TRY(cudaGraphLaunch(p.exec, s));
    prof_add(p.graph_launches);
    return XSS_OK;
}

void xss_seg_plan_destroy(xss_seg_plan_s *plan)
{
    if (!plan) return;
    if (plan->p.exec) cudaGraphExecDestroy(plan->p.exec);
    delete plan;
}

size_t xss_gpu_segmented_workspace_size(int key_dtype, int val_dtype, const uint64_t *h_offsets,
                                        size_t num_segments)
{
    SegPlan p;
    if (plan_init(p, key_dtype, val_dtype, h_offsets, num_segments, 0, 0)) return 0;
    return p.lay.total;
}

int xss_gpu_segmented_sort(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                           const uint64_t *d_offsets, const uint64_t *h_offsets,
                           size_t num_segments, int hasnan, int descending, void *d_ws,
                           size_t ws_bytes, xss_stream_t stream)
{
    if (num_segments == 0) return XSS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<uint64_t> off;
    if (!h_offsets) {
        if (!d_offsets) return XSS_EINVAL;
        off.resize(num_segments + 1);
        XSS_CUDA_TRY(cudaMemcpyAsync(off.data(), d_offsets, off.size() * 8,
                                     cudaMemcpyDeviceToHost, s));
        XSS_CUDA_TRY(cudaStreamSynchronize(s));
        h_offsets = off.data();
    }
    SegPlan p;
    int rc = plan_init(p, key_dtype, d_vals ? val_dtype : -1, h_offsets, num_segments, hasnan,
                       descending);
    if (rc) return rc;
    if (!d_ws) {
        rc = cached_workspace(s, p.lay.total, &d_ws);
        if (rc) return rc;
        ws_bytes = p.lay.total;
    }
    if (ws_bytes < p.lay.total) return XSS_ENOMEM;
    rc = plan_upload(p, static_cast<char *>(d_ws), s);
    if (rc) return rc;
    return plan_enqueue(p, d_keys, d_vals, d_offsets, s);
}

// Segmented top-k.  For k <= SEG_TOPK_MAX the plan sorts segments of up to
// SEG_MED_MAX keys whole on chip (no more work than their top k) and streams
// each longer segment once through seg_topk_kernel; a larger k sorts the
// batch (a sorted segment meets the contract for every k).
int xss_gpu_segmented_topk(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                           const uint64_t *d_offsets, const uint64_t *h_offsets,
                           size_t num_segments, size_t k, int hasnan, int descending,
                           void *d_ws, size_t ws_bytes, xss_stream_t stream)
{
    if (k == 0 || num_segments == 0) return XSS_OK;
    if (k > SEG_TOPK_MAX)
        return xss_gpu_segmented_sort(key_dtype, val_dtype, d_keys, d_vals, d_offsets, h_offsets,
                                      num_segments, hasnan, descending, d_ws, ws_bytes, stream);
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<uint64_t> off;
    if (!h_offsets) {
        if (!d_offsets) return XSS_EINVAL;
        off.resize(num_segments + 1);
        XSS_CUDA_TRY(cudaMemcpyAsync(off.data(), d_offsets, off.size() * 8,
                                     cudaMemcpyDeviceToHost, s));
        XSS_CUDA_TRY(cudaStreamSynchronize(s));
        h_offsets = off.data();
    }
    SegPlan p;
    int rc = plan_init(p, key_dtype, d_vals ? val_dtype : -1, h_offsets, num_segments, hasnan,
                       descending, (uint32_t)k);
    if (rc) return rc;
    if (!d_ws) {
        rc = cached_workspace(s, p.lay.total, &d_ws);
        if (rc) return rc;
        ws_bytes = p.lay.total;
    }
    if (ws_bytes < p.lay.total) return XSS_ENOMEM;
    rc = plan_upload(p, static_cast<char *>(d_ws), s);
    if (rc) return rc;
    return plan_enqueue(p, d_keys, d_vals, d_offsets, s);
}

// The same batch sorted by one call of the single-array entry point per
// segment: the baseline the batched form is measured against.
int xss_gpu_segmented_sort_percall(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                                   const uint64_t *h_offsets, size_t num_segments, int hasnan,
                                   int descending, xss_stream_t stream)
{
    int kb, kind;
    if (dtype_kind(key_dtype, kb, kind)) return XSS_EINVAL;
    const int vb = d_vals ? (val_dtype >= XSS_DT_U64 ? 8 : (val_dtype >= XSS_DT_U32 ? 4 : 2)) : 0;
    for (size_t i = 0; i < num_segments; ++i) {
        const uint64_t b = h_offsets[i], e = h_offsets[i + 1];
        if (e < b) return XSS_EINVAL;
        void *k = static_cast<char *>(d_keys) + b * kb;
        int rc;
        if (vb)
            rc = xss_gpu_keyvalue_qsort(key_dtype, val_dtype, k, static_cast<char *>(d_vals) + b * vb,
                                        e - b, hasnan, descending, nullptr, 0, stream);
        else
            rc = xss_gpu_qsort(key_dtype, k, e - b, hasnan, descending, nullptr, 0, stream);
        if (rc) return rc;
    }
    return XSS_OK;
}

}  // extern "C"
