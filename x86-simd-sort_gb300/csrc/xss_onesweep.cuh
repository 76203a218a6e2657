// xss_onesweep.cuh -- the LSD radix pass ("onesweep": one read and one write
// of keys and values per 8-bit digit, tile offsets by decoupled look-back).
//
// Two launch forms share the per-tile body `pass_tile`:
//   onesweep_kernel          one CTA per tile, keys read with ordinary loads;
//   onesweep_persist_kernel  resident CTAs that keep claiming tiles and
//                            prefetch the next tile with a bulk copy (TMA).
// Replaces the reference's vectorised partition sweeps
// (src/xss-common-qsort.h:252-524, src/xss-common-keyvaluesort.hpp:109-379,
// src/xss-common-argsort.h:174-422): each pass is a counting scatter instead
// of an unstable in-place partition, stable wherever ties can be told apart
// (every pass but a keys-only sort's first).
#pragma once
#include <type_traits>
#include "xss_internal.cuh"
#include "xss_tma.cuh"

namespace xss {

// Block-wide exclusive scan of one 32-bit value per thread.
template <int BLOCK>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *s_warp,
                                                    uint32_t &total)
{
    constexpr int WARPS = BLOCK / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < WARPS ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < WARPS) s_warp[lane] = w;
    }
    __syncthreads();
    const uint32_t pre = warp > 0 ? s_warp[warp - 1] : 0u;
    total = s_warp[WARPS - 1];
    __syncthreads();
    return pre + x - v;
}

// Buffer id -> pointer without dynamically indexing the parameter array
// (which would force a local-memory copy of it).
__device__ __forceinline__ void *pick3(void *const (&b)[3], int i)
{
    return i == 0 ? b[0] : (i == 1 ? b[1] : b[2]);
}

// Tuning of one (key width, value width) instance.
//   BLOCK, ITEMS: threads and keys per thread (tile = BLOCK * ITEMS)
//   MINB:         CTAs per SM the register budget is cut for
//   LB:           predecessors probed per look-back round trip
//   RANK:         1 = peer masks from eight ballots, 0 = from shared atomicOr,
//                 2 = the count atomic's return value is the key's rank in its
//                 warp (shared atomics that meet at one address within a warp
//                 instruction return in lane order; see rank_order_verified)
//   PERSIST:      0 = one CTA per tile, 1 = resident CTAs with TMA prefetch,
//                 2 = resident CTAs with ordinary loads (one staging buffer),
//                 3 = resident CTAs holding two tiles, the next one counted
//                 and published before the current one's look-back
//                 (onesweep_pipe_kernel; RANK must be 2, DPT is unused)
//   DPT:          look-back placement.  0: after ranking, one digit per
//                 thread; 1, 2, 4: right after the counts, by 256 / DPT
//                 threads with DPT digits each while the other warps rank;
//                 12, 14: after ranking, by 128 / 64 threads with 2 / 4
//                 digits each (fewer walking warps, vector status loads)
// Each line can be overridden at build time (a pre-included header defining
// XSS_CFG_K32 etc.) for tuning; xss_tuning.h, written by autotune.py, holds
// the lines it measured fastest and takes precedence over the defaults below.
template <int B, int I, int M, int L, int R, int P, int D = 0> struct CfgT {
    static constexpr int BLOCK = B, ITEMS = I, MINB = M, LB = L, RANK = R, PERSIST = P, DPT = D;
};
#if __has_include("xss_tuning.h")
#include "xss_tuning.h"
#endif
#ifndef XSS_CFG_DEFAULT
#define XSS_CFG_DEFAULT 256, 12, 2, 16, 1, 0
#endif
#ifndef XSS_CFG_K16
#define XSS_CFG_K16 512, 16, 2, 16, 0, 1
#endif
#ifndef XSS_CFG_K32
#define XSS_CFG_K32 512, 16, 2, 16, 0, 1, 1
#endif
#ifndef XSS_CFG_K64
#define XSS_CFG_K64 256, 16, 2, 16, 1, 1
#endif
#ifndef XSS_CFG_K32V32
#define XSS_CFG_K32V32 512, 10, 2, 16, 1, 0
#endif
#ifndef XSS_CFG_K64V64
#define XSS_CFG_K64V64 512, 6, 2, 16, 1, 0, 1
#endif
template <typename C, typename V> struct PassCfg : CfgT<XSS_CFG_DEFAULT> {};
template <> struct PassCfg<uint16_t, NoVal> : CfgT<XSS_CFG_K16> {};
template <> struct PassCfg<uint32_t, NoVal> : CfgT<XSS_CFG_K32> {};
template <> struct PassCfg<uint64_t, NoVal> : CfgT<XSS_CFG_K64> {};
template <> struct PassCfg<uint32_t, uint32_t> : CfgT<XSS_CFG_K32V32> {};
template <> struct PassCfg<uint64_t, uint64_t> : CfgT<XSS_CFG_K64V64> {};

// Size class: arrays of at most XSS_MID_N keys use the XSS_CFGM_* lines.
// Those keep several CTAs per SM in the tile or resident form, so a grid of
// one or two waves stays busy and sorts on other streams (a serving loop)
// can run beside them; the lines above are for large arrays, where one
// resident CTA per SM with a prefetched tile moves the most bytes.
#ifndef XSS_MID_N
#define XSS_MID_N (size_t(1) << 24)
#endif
#ifndef XSS_CFGM_DEFAULT
#define XSS_CFGM_DEFAULT 256, 12, 2, 16, 1, 0, 0
#endif
#ifndef XSS_CFGM_K16
#define XSS_CFGM_K16 512, 16, 2, 16, 0, 1, 0
#endif
#ifndef XSS_CFGM_K32
#define XSS_CFGM_K32 512, 16, 2, 16, 0, 1, 0
#endif
#ifndef XSS_CFGM_K64
#define XSS_CFGM_K64 256, 16, 2, 16, 1, 1, 0
#endif
#ifndef XSS_CFGM_K32V32
#define XSS_CFGM_K32V32 512, 10, 2, 16, 1, 0, 0
#endif
#ifndef XSS_CFGM_K64V64
#define XSS_CFGM_K64V64 256, 12, 2, 16, 1, 0, 0
#endif
template <typename C, typename V> struct PassCfgMid : CfgT<XSS_CFGM_DEFAULT> {};
template <> struct PassCfgMid<uint16_t, NoVal> : CfgT<XSS_CFGM_K16> {};
template <> struct PassCfgMid<uint32_t, NoVal> : CfgT<XSS_CFGM_K32> {};
template <> struct PassCfgMid<uint64_t, NoVal> : CfgT<XSS_CFGM_K64> {};
template <> struct PassCfgMid<uint32_t, uint32_t> : CfgT<XSS_CFGM_K32V32> {};
template <> struct PassCfgMid<uint64_t, uint64_t> : CfgT<XSS_CFGM_K64V64> {};

template <typename C, typename V> constexpr size_t pass_tile_size()
{
    return (size_t)PassCfg<C, V>::BLOCK * PassCfg<C, V>::ITEMS;
}
template <typename C, typename V> constexpr size_t pass_tile_size_mid()
{
    return (size_t)PassCfgMid<C, V>::BLOCK * PassCfgMid<C, V>::ITEMS;
}

// Exclusive prefixes of DPT consecutive digits d0.. over tiles [first, tile)
// by decoupled look-back: probe LB predecessors per round trip (one vector
// load of DPT status words each), add aggregates until each digit meets its
// first inclusive prefix; a row with an unpublished word of a digit still
// walking is probed again (bounded).
#ifndef XSS_LOOKBACK_FIRST
#define XSS_LOOKBACK_FIRST 16
#endif
template <int LB, int DPT>
__device__ __forceinline__ void lookback_excl(const uint32_t *st_pass, uint32_t tile,
                                              uint32_t first, int d0, unsigned *err,
                                              uint32_t (&excl)[DPT],
                                              uint32_t spin_limit = XSS_SPIN_LIMIT)
{
#pragma unroll
    for (int j = 0; j < DPT; ++j) excl[j] = 0;
    uint32_t pending = (1u << DPT) - 1u;   // digits still walking
    int p = (int)tile - 1;
    const int lo = (int)first;
    uint32_t spins = 0;
    // the first round probes only the nearest predecessors; later rounds LB
    int width = XSS_LOOKBACK_FIRST < LB ? XSS_LOOKBACK_FIRST : LB;
    while (p >= lo) {
        uint32_t v[LB][DPT];
#pragma unroll
        for (int w = 0; w < LB; ++w) {
            if (w < width && p - w >= lo) {
                ld_relaxed_vec<DPT>(st_pass + (size_t)(p - w) * RADIX + d0, v[w]);
            } else {
#pragma unroll
                for (int j = 0; j < DPT; ++j) v[w][j] = p - w >= lo ? 0u : FLAG_PRE;
            }
        }
        int used = 0;
#pragma unroll
        for (int w = 0; w < LB; ++w) {
            if (pending == 0u || used != w) break;
            bool ready = true;
#pragma unroll
            for (int j = 0; j < DPT; ++j)
                if (((pending >> j) & 1u) && (v[w][j] & FLAG_MASK) == 0u) ready = false;
            if (!ready) break;
#pragma unroll
            for (int j = 0; j < DPT; ++j) {
                if ((pending >> j) & 1u) {
                    excl[j] += v[w][j] & COUNT_MASK;
                    if ((v[w][j] & FLAG_MASK) == FLAG_PRE) pending &= ~(1u << j);
                }
            }
            ++used;
        }
        if (pending == 0u) return;
        if (used == 0 && ++spins > spin_limit) {
            atomicOr(err, XSS_DEVERR_TIMEOUT);
            return;
        }
        p -= used;
        width = LB;
    }
}

// Shared-memory scratch of the per-tile body (static part).
template <int BLOCK, int RANK> struct PassSmem {
    // Per-warp words per digit: 32-bit digit counts, then running offsets;
    // with RANK 0 followed by as many lane masks.  Zero between tiles.
    static constexpr int WORDS = (BLOCK / 32) * RADIX * (RANK == 0 ? 2 : 1);
    uint32_t wm[WORDS];
    int32_t off[RADIX];                     // global offset - local start, per digit
    uint32_t cnt[RADIX];                    // tile count per digit
    uint32_t lstart[RADIX];                 // tile-local start per digit
    uint32_t scan[BLOCK / 32];
};

// Where a tile sits: its row in the look-back status array, the first tile
// of its segment (a whole-array sort has one segment), its first element and
// the segment's size, and this pass's bucket starts relative to the segment.
struct TileJob {
    uint32_t tile;
    uint32_t first;
    uint32_t base;
    uint32_t n;
    const uint32_t *start;
    uint32_t *st_pass;      // this pass's look-back status rows
};

// Rank, publish, look up offsets and scatter one tile whose keys (codes) and
// values are in registers.  s_k / s_v: TILE-sized staging buffers that no
// thread reads any more once the first barrier here is passed.
// after_rank() runs on every thread once the tile is staged (the persistent
// form claims and prefetches its next tile there).
// Pre: ps.wm is zero.  Post: zero again after the caller's next barrier.
// ROLE: what the pass does to keys on store, known at compile time --
// ROLE_MID (codes stay codes), ROLE_LAST (codes back to keys through the
// codec, canonical NaNs where asked) -- or ROLE_RUNTIME (pd.last decides,
// through from_code; the segmented passes use this form).
constexpr int ROLE_RUNTIME = -1, ROLE_MID = 0, ROLE_FIRST = 1, ROLE_LAST = 2;

// PAIRS: keys and values of the same width (4 or 8 bytes) are staged as
// (key, value) pairs in the 2 * TILE * sizeof(C) bytes starting at s_k (s_v
// unused): one shared store per key when staging and one shared load when
// scattering, instead of two each.
template <typename C, typename V, int BLOCK, int ITEMS, int LB, int RANK, int DPT, int ROLE,
          bool PAIRS = false, typename VS, typename AfterRank>
__device__ __forceinline__ void pass_tile(const RadixArgs &a, const PassDesc &pd, int pass,
                                          const TileJob &job, const C (&key)[ITEMS],
                                          const VS (&val)[ITEMS], C *s_k, VS *s_v,
                                          PassSmem<BLOCK, RANK> &ps, C *kdst, V *vdst,
                                          const Codec<C> &cx, AfterRank after_rank)
{
    constexpr int WARPS = BLOCK / 32;
    constexpr int TILE = BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    static_assert(!PAIRS || (HAS_V && RANK == 2 && sizeof(C) == sizeof(VS) &&
                             (sizeof(C) == 8 || sizeof(C) == 4)),
                  "pair staging: 4- or 8-byte keys and values ranked by the count atomic");
    using PairT = typename std::conditional<sizeof(C) == 8, ulonglong2, uint2>::type;
    PairT *const s_kv = reinterpret_cast<PairT *>(s_k);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n = job.n;
    const uint32_t tile = job.tile;
    const int shift = pass * RADIX_BITS;
    const uint32_t tile_base = job.base;
    uint32_t *const hist32 = ps.wm;
    uint32_t *wh = hist32 + warp * RADIX;

    // Keys-only first pass (pd.tie_free): equal codes are the same key and no
    // earlier pass has ordered the tile, so ties need no order.  The tile then
    // counts into one set of counters and each key claims its staging slot
    // with one shared atomic, instead of the per-warp counts and lane masks
    // that keep ties stable.
    // Keys past the end of a partial tile (padding) are left out there: they
    // would take slots among the real keys of the top digit.
    const bool tie_free = !HAS_V && pd.tie_free;
    const uint32_t valid = min((uint32_t)TILE, n - tile_base);
    const uint32_t local0 = (uint32_t)warp * (ITEMS * 32) + lane;

    // ---- digit counts (independent shared atomics): per warp, or per tile.
    // RANK 2 keeps each count atomic's result: the number of keys of the same
    // digit before this one in its warp (program order across items, lane
    // order within one; the warp barrier orders the items' atomics).
    // The ranks are below 32 * ITEMS, so two share a register.
    constexpr bool KEEP_RANK = RANK == 2;
    static_assert(!KEEP_RANK || 32 * ITEMS < 65536, "ranks fit 16 bits");
    uint32_t wrank[KEEP_RANK ? (ITEMS + 1) / 2 : 1];
    if (tie_free) {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j)
            if (local0 + j * 32 < valid)
                atomicAdd(&hist32[uint32_t(key[j] >> shift) & (RADIX - 1)], 1u);
    } else if constexpr (KEEP_RANK) {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t r = atomicAdd(&wh[uint32_t(key[j] >> shift) & (RADIX - 1)], 1u);
            if (j & 1) wrank[j >> 1] |= r << 16;
            else wrank[j >> 1] = r;
            __syncwarp();
        }
    } else {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) atomicAdd(&wh[uint32_t(key[j] >> shift) & (RADIX - 1)], 1u);
    }
    __syncthreads();

    // ---- tile counts published at once, so successors' look-backs can pass
    // this tile; then each warp's exclusive offset per digit
    uint32_t *st_tile = job.st_pass + (size_t)tile * RADIX;
    uint32_t cnt = 0;
    if (tid < RADIX) {
        if (tie_free) {
            cnt = hist32[tid];
        } else {
#pragma unroll
            for (int w = 0; w < WARPS; ++w) cnt += hist32[w * RADIX + tid];
        }
        st_relaxed_u32(st_tile + tid, (tile == job.first ? FLAG_PRE : FLAG_AGG) | cnt);
    }
    uint32_t total;
    const uint32_t local_start = block_excl_scan<BLOCK>(cnt, ps.scan, total);
    if (tid < RADIX) {
        if (tie_free) {
            hist32[tid] = local_start;
        } else {
            uint32_t run = local_start;
#pragma unroll
            for (int w = 0; w < WARPS; ++w) {
                const uint32_t c = hist32[w * RADIX + tid];
                hist32[w * RADIX + tid] = run;
                run += c;
            }
        }
        ps.cnt[tid] = cnt;
        ps.lstart[tid] = local_start;
    }
    __syncthreads();

    // ---- look-back for this tile's global offsets.  DPT > 0: as soon as the
    // counts are out, RADIX / DPT threads (the first warps) walk back, DPT
    // digits each, while the other warps already rank; the walkers rank
    // afterwards.  DPT 0: after ranking, one digit per thread.
    static_assert(DPT == 0 || DPT == 1 || DPT == 2 || DPT == 4 || DPT == 12 || DPT == 14,
                  "look-back placement");
    constexpr bool LATE = DPT == 0 || DPT >= 10;            // walk after ranking
    constexpr int DW = DPT == 0 ? 1 : (DPT >= 10 ? (DPT == 12 ? 2 : 4) : DPT);
    auto walk = [&]() {
        const int d0 = tid * DW;
        uint32_t excl[DW];
#pragma unroll
        for (int j = 0; j < DW; ++j) excl[j] = 0;
        if (tile > job.first) {
            lookback_excl<LB, DW>(job.st_pass, tile, job.first, d0, a.err, excl);
            uint32_t pre[DW];
#pragma unroll
            for (int j = 0; j < DW; ++j) pre[j] = FLAG_PRE | ((excl[j] + ps.cnt[d0 + j]) & COUNT_MASK);
            st_relaxed_vec<DW>(st_tile + d0, pre);
        }
#pragma unroll
        for (int j = 0; j < DW; ++j)
            ps.off[d0 + j] = (int32_t)(job.start[d0 + j] + excl[j]) - (int32_t)ps.lstart[d0 + j];
    };
    if (!LATE && tid < RADIX / DW) walk();

    // ---- stable rank (digit, warp, item, lane) and stage in digit order.
    // The lanes sharing a digit find each other either by eight ballots, one
    // per digit bit (RANK 1: no shared memory, consecutive items overlap), or
    // through a per-warp word per digit that each lane sets its bit in and
    // reads back (RANK 0: fewer instructions, the leader clears the word).
    // (The warp match instruction measured 1.8x slower than either.)
    // The highest such lane advances the warp's running offset for the digit.
    if (tie_free) {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j)
            if (local0 + j * 32 < valid)
                s_k[atomicAdd(&hist32[uint32_t(key[j] >> shift) & (RADIX - 1)], 1u)] = key[j];
    } else if constexpr (KEEP_RANK) {
        // staging slot = the warp's start for the digit + the kept rank; the
        // starts are only read here, so the items are independent
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t p = wh[uint32_t(key[j] >> shift) & (RADIX - 1)] +
                               ((wrank[j >> 1] >> (16 * (j & 1))) & 0xFFFFu);
            if constexpr (PAIRS) {
                PairT kv;
                kv.x = key[j];
                kv.y = val[j];
                s_kv[p] = kv;
            } else {
                s_k[p] = key[j];
                if constexpr (HAS_V) s_v[p] = val[j];
            }
        }
    } else {
        const uint32_t lt_mask = (1u << lane) - 1u;
        uint32_t *mt = hist32 + (WARPS + warp) * RADIX;   // RANK 0 only
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t d = uint32_t(key[j] >> shift) & (RADIX - 1);
            uint32_t peers = 0xffffffffu;
            if constexpr (RANK == 1) {
#pragma unroll
                for (int b = 0; b < RADIX_BITS; ++b) {
                    const bool set = (d >> b) & 1u;
                    const uint32_t m = __ballot_sync(0xffffffffu, set);
                    peers &= set ? m : ~m;
                }
            } else {
                atomicOr(&mt[d], 1u << lane);
                __syncwarp();
                peers = mt[d];
                __syncwarp();
            }
            const int leader = 31 - __clz(peers);
            uint32_t base = 0;
            if (lane == leader) {
                if constexpr (RANK == 0) {
                    // one shared atomic instead of a load and a store (measured
                    // faster with shared-memory masks, slower with ballots)
                    base = atomicAdd(&wh[d], (uint32_t)__popc(peers));
                    mt[d] = 0;
                } else {
                    base = wh[d];
                    wh[d] = base + __popc(peers);
                }
            }
            base = __shfl_sync(0xffffffffu, base, leader);
            const uint32_t p = base + __popc(peers & lt_mask);
            s_k[p] = key[j];
            if constexpr (HAS_V) s_v[p] = val[j];
            __syncwarp();
        }
    }
    after_rank();
    if (LATE && tid < RADIX / DW) walk();
    __syncthreads();

    // ---- scatter runs of equal digits to consecutive global addresses
#pragma unroll
    for (int m = 0; m < ITEMS; ++m) {
        const uint32_t i = tid + m * BLOCK;
        if (i < valid) {
            C c;
            VS v{};
            if constexpr (PAIRS) {
                const PairT kv = s_kv[i];
                c = (C)kv.x;
                v = (VS)kv.y;
            } else {
                c = s_k[i];
            }
            const uint32_t d = uint32_t(c >> shift) & (RADIX - 1);
            const uint32_t g = (uint32_t)(ps.off[d] + (int32_t)i);
            if (g < n) {
                if (!pd.skip_keys) {
                    if constexpr (ROLE == ROLE_RUNTIME) kdst[g] = pd.last ? from_code(c, a.xf) : c;
                    else if constexpr ((ROLE & ROLE_LAST) != 0) kdst[g] = cx.from_canon(c);
                    else kdst[g] = c;
                }
                if constexpr (HAS_V) {
                    if constexpr (!PAIRS) v = s_v[i];
                    if (pd.out_idx) a.out_idx[g] = (uint64_t)v;
                    else vdst[g] = v;
                }
            } else {
                atomicOr(a.err, XSS_DEVERR_BOUNDS);  // only after a look-back timeout
            }
        }
    }
    const int dirty = tie_free ? RADIX : PassSmem<BLOCK, RANK>::WORDS;
    for (int i = tid; i < dirty; i += BLOCK) ps.wm[i] = 0;
}

struct NoAfterRank {
    __device__ void operator()() const {}
};

// Whether a pass of (C, value type VS) ranked by RANK stages (key, value)
// pairs (pass_tile's PAIRS).  The tile and resident forms then lay each tile
// buffer out as TILE keys followed by TILE values, so one buffer's bytes hold
// the tile's pairs once its keys and values are in registers.  Measured on
// 2^28 keys: 64/64 15.82 -> 15.71 ms (2^21: 1% faster passes); 32/32 pairs
// measured slower (4.99 -> 5.02 ms; 200,000-segment batch 89.4 -> 89.6 ms),
// so 4-byte pairs stay off.
#ifndef XSS_PAIR_STAGING
#define XSS_PAIR_STAGING 1
#endif
template <typename C, typename VS, int RANK> constexpr bool pair_staged()
{
    return XSS_PAIR_STAGING && RANK == 2 && sizeof(C) == 8 && sizeof(VS) == 8;
}

// ---------------------------------------------------------------------------
// One CTA per tile; the tile id comes from an in-order atomic counter, so a
// tile only waits on tiles whose CTAs are already running.
template <typename C, typename V, int BLOCK, int ITEMS, int LB, int RANK, int DPT, int ROLE>
__device__ __forceinline__ void onesweep_tile_body(const RadixArgs &a, int pass,
                                                   const PassDesc &pd,
                                                   PassSmem<BLOCK, RANK> &ps, uint32_t &s_tile,
                                                   unsigned char *s_dyn)
{
    constexpr int TILE = BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    using VS = typename std::conditional<HAS_V, V, uint8_t>::type;
    C *s_k = reinterpret_cast<C *>(s_dyn);
    VS *s_v = reinterpret_cast<VS *>(s_dyn + TILE * sizeof(C));
    const Codec<C> cx(a.xf);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < PassSmem<BLOCK, RANK>::WORDS; i += BLOCK) ps.wm[i] = 0;
    if (tid == 0) s_tile = atomicAdd(&a.hdr->tile_ctr[pass], 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t n = (uint32_t)a.n;
    const uint32_t first_idx = tile * (uint32_t)TILE + (uint32_t)warp * (ITEMS * 32) + lane;
    const C *ksrc = static_cast<const C *>(pick3(a.kbuf, pd.src));
    C key[ITEMS];
    VS val[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint32_t idx = first_idx + j * 32;
        if (idx < n) {
            const C b = ksrc[idx];
            key[j] = (ROLE & ROLE_FIRST) ? cx.to(b) : b;
        } else {
            key[j] = C(~C(0));
        }
    }
    V *vdst = nullptr;
    if constexpr (HAS_V) {
        const V *vsrc = static_cast<const V *>(pick3(a.vbuf, pd.vsrc));
        vdst = static_cast<V *>(pick3(a.vbuf, pd.vdst));
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t idx = first_idx + j * 32;
            val[j] = pd.gen_idx ? VS(idx) : (idx < n ? vsrc[idx] : VS(0));
        }
    }
    const TileJob job{tile, 0u, tile * (uint32_t)TILE, n, a.hdr->start[pass],
                      a.status + (size_t)pass * a.num_tiles * RADIX};
    // s_dyn holds TILE keys then TILE values: the layout pair staging needs
    pass_tile<C, V, BLOCK, ITEMS, LB, RANK, DPT, ROLE, pair_staged<C, VS, RANK>()>(
        a, pd, pass, job, key, val, s_k, s_v, ps, static_cast<C *>(pick3(a.kbuf, pd.dst)), vdst,
        cx, NoAfterRank{});
}

// The pass's role (does it load keys, store keys?) is read from the device
// plan and dispatched to a body compiled for it.
template <typename C, typename V, int BLOCK, int ITEMS, int MINB, int LB, int RANK, int DPT>
__global__ void __launch_bounds__(BLOCK, MINB) onesweep_kernel(RadixArgs a, int pass)
{
    static_assert(BLOCK >= RADIX, "one thread per digit");
    const PassDesc pd = a.hdr->desc[pass];
    if (!pd.active) return;
    __shared__ PassSmem<BLOCK, RANK> ps;
    __shared__ uint32_t s_tile;
    extern __shared__ __align__(128) unsigned char s_dyn[];
    if (pd.first) {
        if (pd.last)
            onesweep_tile_body<C, V, BLOCK, ITEMS, LB, RANK, DPT, ROLE_FIRST | ROLE_LAST>(
                a, pass, pd, ps, s_tile, s_dyn);
        else
            onesweep_tile_body<C, V, BLOCK, ITEMS, LB, RANK, DPT, ROLE_FIRST>(a, pass, pd, ps,
                                                                              s_tile, s_dyn);
    } else {
        if (pd.last)
            onesweep_tile_body<C, V, BLOCK, ITEMS, LB, RANK, DPT, ROLE_LAST>(a, pass, pd, ps,
                                                                             s_tile, s_dyn);
        else
            onesweep_tile_body<C, V, BLOCK, ITEMS, LB, RANK, DPT, ROLE_MID>(a, pass, pd, ps,
                                                                            s_tile, s_dyn);
    }
}

// ---------------------------------------------------------------------------
// Resident CTAs that keep claiming tiles from the same in-order counter.
// Once a tile is ranked and staged, the CTA claims its next tile and (PF)
// starts its bulk copy (TMA) into the other buffer, so the load overlaps the
// current tile's scatter.  Without PF the CTA keeps one staging buffer and
// reads each tile with ordinary loads: less shared memory per CTA, more CTAs
// per SM, and no per-tile CTA launch.  Claims are in increasing order per CTA,
// which keeps the look-back free of deadlock: the lowest unfinished tile is
// always the current tile of the CTA holding it, and every tile below it is
// finished.  Partial tiles and sources that are not 16-byte aligned are read
// with ordinary loads.
template <typename C, typename V, int BLOCK, int ITEMS, int LB, int RANK, int DPT, bool PF,
          int ROLE>
__device__ __forceinline__ void onesweep_persist_body(const RadixArgs &a, int pass,
                                                      const PassDesc &pd,
                                                      PassSmem<BLOCK, RANK> &ps,
                                                      uint32_t (&s_tile)[2],
                                                      uint64_t (&s_bar)[2],
                                                      unsigned char *s_dyn)
{
    constexpr int TILE = BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    using VS = typename std::conditional<HAS_V, V, uint8_t>::type;
    constexpr size_t VSZ = HAS_V ? sizeof(V) : 0;
    const Codec<C> cx(a.xf);
    constexpr int NBUF = PF ? 2 : 1;
    // Buffer b: its TILE keys at kbuf(b), values at vbuf(b).  Pair staging
    // keeps each buffer's keys and values together (b * TILE pairs in);
    // otherwise all keys come first, then all values.
    constexpr bool PAIRS = pair_staged<C, VS, RANK>();
    auto kbuf = [&](int b) -> C * {
        return PAIRS ? reinterpret_cast<C *>(s_dyn + (size_t)b * TILE * (sizeof(C) + VSZ))
                     : reinterpret_cast<C *>(s_dyn) + b * TILE;
    };
    auto vbuf = [&](int b) -> VS * {
        return PAIRS ? reinterpret_cast<VS *>(s_dyn + (size_t)b * TILE * (sizeof(C) + VSZ) +
                                              TILE * sizeof(C))
                     : reinterpret_cast<VS *>(s_dyn + NBUF * TILE * sizeof(C)) + b * TILE;
    };

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n = (uint32_t)a.n;
    const uint32_t num_tiles = a.num_tiles;
    const C *ksrc = static_cast<const C *>(pick3(a.kbuf, pd.src));
    C *kdst = static_cast<C *>(pick3(a.kbuf, pd.dst));
    const V *vsrc = nullptr;
    V *vdst = nullptr;
    if constexpr (HAS_V) {
        vsrc = static_cast<const V *>(pick3(a.vbuf, pd.vsrc));
        vdst = static_cast<V *>(pick3(a.vbuf, pd.vdst));
    }
    const bool load_vals = HAS_V && !pd.gen_idx;
    const bool tma = PF && (reinterpret_cast<uintptr_t>(ksrc) & 15) == 0 &&
                     (!load_vals || (reinterpret_cast<uintptr_t>(vsrc) & 15) == 0);
    const uint32_t tile_bytes = TILE * (uint32_t)(sizeof(C) + (load_vals ? VSZ : 0));

    auto issue = [&](uint32_t t, int b) {
        const size_t base = (size_t)t * TILE;
        mbar_arrive_expect_tx(&s_bar[b], tile_bytes);
        bulk_load(kbuf(b), ksrc + base, TILE * sizeof(C), &s_bar[b]);
        if constexpr (HAS_V)
            if (load_vals) bulk_load(vbuf(b), vsrc + base, TILE * sizeof(VS), &s_bar[b]);
    };
    auto by_tma = [&](uint32_t t) { return tma && t < num_tiles && (size_t)t * TILE + TILE <= n; };

    for (int i = tid; i < PassSmem<BLOCK, RANK>::WORDS; i += BLOCK) ps.wm[i] = 0;
    if (tid == 0) {
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
        fence_mbar_init();
        const uint32_t t0 = atomicAdd(&a.hdr->tile_ctr[pass], 1u);
        s_tile[0] = t0;
        if (by_tma(t0)) issue(t0, 0);
    }
    __syncthreads();

    uint32_t parity[2] = {0u, 0u};
    for (uint32_t it = 0;; ++it) {
        const int cur = it & 1;
        const uint32_t tile = s_tile[cur];
        if (tile >= num_tiles) break;
        const uint32_t tile_base = tile * (uint32_t)TILE;
        const uint32_t local0 = (uint32_t)warp * (ITEMS * 32) + lane;
        C *s_k = kbuf(PF ? cur : 0);
        VS *s_v = vbuf(PF ? cur : 0);
        C key[ITEMS];
        VS val[ITEMS];
        if (by_tma(tile)) {
            // a copy that never landed (the error word is already set): this
            // CTA neither reads nor reuses that buffer and claims no further
            // tile; its successors' look-backs give up with the same flag
            const bool landed = mbar_wait_bounded(&s_bar[cur], parity[cur], a.err);
            if (__syncthreads_or(!landed)) break;
            parity[cur] ^= 1u;
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) {
                const C b = s_k[local0 + j * 32];
                key[j] = (ROLE & ROLE_FIRST) ? cx.to(b) : b;
            }
            if constexpr (HAS_V) {
#pragma unroll
                for (int j = 0; j < ITEMS; ++j)
                    val[j] = pd.gen_idx ? VS(tile_base + local0 + j * 32) : s_v[local0 + j * 32];
            }
        } else {
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) {
                const uint32_t idx = tile_base + local0 + j * 32;
                if (idx < n) {
                    const C b = ksrc[idx];
                    key[j] = (ROLE & ROLE_FIRST) ? cx.to(b) : b;
                } else {
                    key[j] = C(~C(0));
                }
            }
            if constexpr (HAS_V) {
#pragma unroll
                for (int j = 0; j < ITEMS; ++j) {
                    const uint32_t idx = tile_base + local0 + j * 32;
                    val[j] = pd.gen_idx ? VS(idx) : (idx < n ? vsrc[idx] : VS(0));
                }
            }
        }
        // pass_tile's first barrier orders these reads before the buffer is
        // reused for staging; the other buffer was released by the previous
        // iteration's final barrier, so the next tile may land there.
        auto claim_next = [&]() {
            if (tid == 0) {
                const uint32_t t1 = atomicAdd(&a.hdr->tile_ctr[pass], 1u);
                s_tile[cur ^ 1] = t1;
                if (by_tma(t1)) {
                    fence_proxy_async_smem();
                    issue(t1, cur ^ 1);
                }
            }
        };
        const TileJob job{tile, 0u, tile_base, n, a.hdr->start[pass],
                          a.status + (size_t)pass * num_tiles * RADIX};
        pass_tile<C, V, BLOCK, ITEMS, LB, RANK, DPT, ROLE, PAIRS>(a, pd, pass, job, key, val, s_k,
                                                                  s_v, ps, kdst, vdst, cx,
                                                                  claim_next);
        __syncthreads();
    }
}

template <typename C, typename V, int BLOCK, int ITEMS, int MINB, int LB, int RANK, int DPT,
          bool PF>
__global__ void __launch_bounds__(BLOCK, MINB) onesweep_persist_kernel(RadixArgs a, int pass)
{
    static_assert(BLOCK >= RADIX, "one thread per digit");
    const PassDesc pd = a.hdr->desc[pass];
    if (!pd.active) return;
    __shared__ PassSmem<BLOCK, RANK> ps;
    __shared__ uint32_t s_tile[2];
    __shared__ __align__(8) uint64_t s_bar[2];
    extern __shared__ __align__(128) unsigned char s_dyn[];
    if (pd.first) {
        if (pd.last)
            onesweep_persist_body<C, V, BLOCK, ITEMS, LB, RANK, DPT, PF, ROLE_FIRST | ROLE_LAST>(
                a, pass, pd, ps, s_tile, s_bar, s_dyn);
        else
            onesweep_persist_body<C, V, BLOCK, ITEMS, LB, RANK, DPT, PF, ROLE_FIRST>(
                a, pass, pd, ps, s_tile, s_bar, s_dyn);
    } else {
        if (pd.last)
            onesweep_persist_body<C, V, BLOCK, ITEMS, LB, RANK, DPT, PF, ROLE_LAST>(
                a, pass, pd, ps, s_tile, s_bar, s_dyn);
        else
            onesweep_persist_body<C, V, BLOCK, ITEMS, LB, RANK, DPT, PF, ROLE_MID>(
                a, pass, pd, ps, s_tile, s_bar, s_dyn);
    }
}

// ---------------------------------------------------------------------------
// Pipelined resident form (PERSIST 3).  A CTA holds two tiles: the current
// one, ranked and staged in the staging buffer, and the next one, landing in
// the landing buffer.  Each iteration reads the next tile into registers,
// counts it, starts the copy of the tile after it into the landing buffer
// (now free), publishes the next tile's aggregate, and only then walks back
// for the current tile; it scatters the current tile and stages the next.  The walk thus starts a
// count and a scan later than in pass_tile (its predecessors are further
// along, so it needs fewer round trips), and a tile's aggregate goes out
// soon after its data lands instead of after the previous tile's walk and
// scatter.  Ranks come from the count atomics (RANK 2) in every pass.
// Deadlock-free as the other forms: tiles are claimed in increasing order,
// and the CTA holding the lowest unfinished tile has every predecessor's
// inclusive prefix available.
template <int BLOCK> struct PipeSmem {
    uint32_t wh[(BLOCK / 32) * RADIX];   // per-warp counts, then per-warp offsets
    uint32_t cl[2][RADIX];               // per held tile: count | local start << 16
    int32_t off[RADIX];                  // global offset - local start, current tile
    uint32_t scan[BLOCK / 32];
};

template <typename C, typename V, int BLOCK, int ITEMS, int LB, int ROLE>
__device__ __forceinline__ void onesweep_pipe_body(const RadixArgs &a, int pass,
                                                   const PassDesc &pd, PipeSmem<BLOCK> &ps,
                                                   uint32_t (&s_tile)[2], uint64_t (&s_bar)[2],
                                                   unsigned char *s_dyn)
{
    constexpr int WARPS = BLOCK / 32;
    constexpr int TILE = BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    using VS = typename std::conditional<HAS_V, V, uint8_t>::type;
    constexpr size_t VSZ = HAS_V ? sizeof(V) : 0;
    static_assert(TILE < 65536, "ranks, counts and local starts fit 16 bits");
    const Codec<C> cx(a.xf);
    C *const s_k0 = reinterpret_cast<C *>(s_dyn);
    VS *const s_v0 = reinterpret_cast<VS *>(s_dyn + 2 * TILE * sizeof(C));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n = (uint32_t)a.n;
    const uint32_t num_tiles = a.num_tiles;
    const int shift = pass * RADIX_BITS;
    const C *ksrc = static_cast<const C *>(pick3(a.kbuf, pd.src));
    C *kdst = static_cast<C *>(pick3(a.kbuf, pd.dst));
    const V *vsrc = nullptr;
    V *vdst = nullptr;
    if constexpr (HAS_V) {
        vsrc = static_cast<const V *>(pick3(a.vbuf, pd.vsrc));
        vdst = static_cast<V *>(pick3(a.vbuf, pd.vdst));
    }
    const bool load_vals = HAS_V && !pd.gen_idx;
    const bool tma = (reinterpret_cast<uintptr_t>(ksrc) & 15) == 0 &&
                     (!load_vals || (reinterpret_cast<uintptr_t>(vsrc) & 15) == 0);
    const uint32_t tile_bytes = TILE * (uint32_t)(sizeof(C) + (load_vals ? VSZ : 0));
    uint32_t *const st_pass = a.status + (size_t)pass * num_tiles * RADIX;
    const uint32_t *const gstart = a.hdr->start[pass];
    uint32_t *const wh = ps.wh + warp * RADIX;
    const uint32_t local0 = (uint32_t)warp * (ITEMS * 32) + lane;

    auto issue = [&](uint32_t t, int b) {
        const size_t base = (size_t)t * TILE;
        mbar_arrive_expect_tx(&s_bar[b], tile_bytes);
        bulk_load(s_k0 + b * TILE, ksrc + base, TILE * sizeof(C), &s_bar[b]);
        if constexpr (HAS_V)
            if (load_vals) bulk_load(s_v0 + b * TILE, vsrc + base, TILE * sizeof(VS), &s_bar[b]);
    };
    auto by_tma = [&](uint32_t t) { return tma && t < num_tiles && (size_t)t * TILE + TILE <= n; };
    // claim a tile and start its copy into the landing buffer (0)
    auto claim_next = [&]() {
        if (tid == 0) {
            const uint32_t t1 = atomicAdd(&a.hdr->tile_ctr[pass], 1u);
            s_tile[0] = t1;
            if (by_tma(t1)) {
                fence_proxy_async_smem();
                issue(t1, 0);
            }
        }
    };

    uint32_t parity[2] = {0u, 0u};
    C key[ITEMS];
    VS val[ITEMS];
    uint32_t wrank[(ITEMS + 1) / 2];
    // tile t (data in buffer b) into registers; false: its copy never landed
    // (the error word is set), and the CTA stops
    auto load_tile = [&](uint32_t t, int b) -> bool {
        const uint32_t tile_base = t * (uint32_t)TILE;
        if (by_tma(t)) {
            const bool landed = mbar_wait_bounded(&s_bar[b], parity[b], a.err);
            if (__syncthreads_or(!landed)) return false;
            parity[b] ^= 1u;
            const C *sk = s_k0 + b * TILE;
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) {
                const C x = sk[local0 + j * 32];
                key[j] = (ROLE & ROLE_FIRST) ? cx.to(x) : x;
            }
            if constexpr (HAS_V) {
                const VS *sv = s_v0 + b * TILE;
#pragma unroll
                for (int j = 0; j < ITEMS; ++j)
                    val[j] = pd.gen_idx ? VS(tile_base + local0 + j * 32) : sv[local0 + j * 32];
            }
        } else {
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) {
                const uint32_t idx = tile_base + local0 + j * 32;
                if (idx < n) {
                    const C x = ksrc[idx];
                    key[j] = (ROLE & ROLE_FIRST) ? cx.to(x) : x;
                } else {
                    key[j] = C(~C(0));
                }
            }
            if constexpr (HAS_V) {
#pragma unroll
                for (int j = 0; j < ITEMS; ++j) {
                    const uint32_t idx = tile_base + local0 + j * 32;
                    val[j] = pd.gen_idx ? VS(idx) : (idx < n ? vsrc[idx] : VS(0));
                }
            }
        }
        return true;
    };
    // per-warp digit counts; each key keeps its rank in its warp
    auto count = [&]() {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t r = atomicAdd(&wh[uint32_t(key[j] >> shift) & (RADIX - 1)], 1u);
            if (j & 1) wrank[j >> 1] |= r << 16;
            else wrank[j >> 1] = r;
            __syncwarp();
        }
    };
    // (after a barrier) publish tile t's counts, scan them, per-warp offsets
    auto publish_scan = [&](uint32_t t, int slot) {
        uint32_t c = 0;
        if (tid < RADIX) {
#pragma unroll
            for (int w = 0; w < WARPS; ++w) c += ps.wh[w * RADIX + tid];
            st_relaxed_u32(st_pass + (size_t)t * RADIX + tid, (t == 0 ? FLAG_PRE : FLAG_AGG) | c);
        }
        uint32_t total;
        const uint32_t ls = block_excl_scan<BLOCK>(c, ps.scan, total);
        if (tid < RADIX) {
            uint32_t run = ls;
#pragma unroll
            for (int w = 0; w < WARPS; ++w) {
                const uint32_t x = ps.wh[w * RADIX + tid];
                ps.wh[w * RADIX + tid] = run;
                run += x;
            }
            ps.cl[slot][tid] = c | (ls << 16);
        }
    };
    // (tid < RADIX) tile t's global offsets; its inclusive prefixes go out
    auto walk = [&](uint32_t t, int slot) {
        uint32_t excl[1] = {0};
        const uint32_t cl = ps.cl[slot][tid];
        if (t > 0) {
            lookback_excl<LB, 1>(st_pass, t, 0u, tid, a.err, excl);
            st_relaxed_u32(st_pass + (size_t)t * RADIX + tid,
                           FLAG_PRE | ((excl[0] + (cl & 0xFFFFu)) & COUNT_MASK));
        }
        ps.off[tid] = (int32_t)(gstart[tid] + excl[0]) - (int32_t)(cl >> 16);
    };
    auto stage = [&](int b) {
        C *sk = s_k0 + b * TILE;
        VS *sv = s_v0 + b * TILE;
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t p = wh[uint32_t(key[j] >> shift) & (RADIX - 1)] +
                               ((wrank[j >> 1] >> (16 * (j & 1))) & 0xFFFFu);
            sk[p] = key[j];
            if constexpr (HAS_V) sv[p] = val[j];
        }
    };
    auto scatter = [&](uint32_t t, int b) {
        const C *sk = s_k0 + b * TILE;
        const VS *sv = s_v0 + b * TILE;
        const uint32_t valid = min((uint32_t)TILE, n - t * (uint32_t)TILE);
#pragma unroll
        for (int m = 0; m < ITEMS; ++m) {
            const uint32_t i = tid + m * BLOCK;
            if (i < valid) {
                const C c = sk[i];
                const uint32_t d = uint32_t(c >> shift) & (RADIX - 1);
                const uint32_t g = (uint32_t)(ps.off[d] + (int32_t)i);
                if (g < n) {
                    if (!pd.skip_keys) {
                        if constexpr ((ROLE & ROLE_LAST) != 0) kdst[g] = cx.from_canon(c);
                        else kdst[g] = c;
                    }
                    if constexpr (HAS_V) {
                        if (pd.out_idx) a.out_idx[g] = (uint64_t)sv[i];
                        else vdst[g] = sv[i];
                    }
                } else {
                    atomicOr(a.err, XSS_DEVERR_BOUNDS);  // only after a look-back timeout
                }
            }
        }
    };
    auto clear_wh = [&]() {
        for (int i = tid; i < WARPS * RADIX; i += BLOCK) ps.wh[i] = 0;
    };

    // ---- prologue: the first tile counted, published, staged
    clear_wh();
    if (tid == 0) {
        mbar_init(&s_bar[0], 1);
        fence_mbar_init();
        const uint32_t t0 = atomicAdd(&a.hdr->tile_ctr[pass], 1u);
        s_tile[0] = t0;
        if (by_tma(t0)) issue(t0, 0);
    }
    __syncthreads();
    int slot = 0;                             // count / start slot of the current tile
    uint32_t t = s_tile[0];
    if (t >= num_tiles) return;
    if (!load_tile(t, 0)) return;
    count();
    __syncthreads();                          // the landing buffer is read
    claim_next();
    publish_scan(t, slot);
    __syncthreads();
    stage(1);
    __syncthreads();

    for (;;) {
        const uint32_t nxt = s_tile[0];
        const bool have_next = nxt < num_tiles;   // uniform across the CTA
        clear_wh();
        __syncthreads();
        if (have_next) {
            if (!load_tile(nxt, 0)) {
                // the next tile's copy never landed: finish the current tile
                // (its walk may give up too; the error word is already set)
                if (tid < RADIX) walk(t, slot);
                __syncthreads();
                scatter(t, 1);
                return;
            }
            count();
        }
        __syncthreads();                      // the landing buffer is read
        if (have_next) {
            claim_next();
            publish_scan(nxt, slot ^ 1);
        }
        if (tid < RADIX) walk(t, slot);
        __syncthreads();
        scatter(t, 1);
        __syncthreads();
        if (!have_next) break;
        stage(1);
        __syncthreads();
        t = nxt;
        slot ^= 1;
    }
}

template <typename C, typename V, int BLOCK, int ITEMS, int MINB, int LB>
__global__ void __launch_bounds__(BLOCK, MINB) onesweep_pipe_kernel(RadixArgs a, int pass)
{
    static_assert(BLOCK >= RADIX, "one thread per digit");
    const PassDesc pd = a.hdr->desc[pass];
    if (!pd.active) return;
    __shared__ PipeSmem<BLOCK> ps;
    __shared__ uint32_t s_tile[2];
    __shared__ __align__(8) uint64_t s_bar[2];
    extern __shared__ __align__(128) unsigned char s_dyn[];
    if (pd.first) {
        if (pd.last)
            onesweep_pipe_body<C, V, BLOCK, ITEMS, LB, ROLE_FIRST | ROLE_LAST>(a, pass, pd, ps,
                                                                              s_tile, s_bar, s_dyn);
        else
            onesweep_pipe_body<C, V, BLOCK, ITEMS, LB, ROLE_FIRST>(a, pass, pd, ps, s_tile, s_bar,
                                                                   s_dyn);
    } else {
        if (pd.last)
            onesweep_pipe_body<C, V, BLOCK, ITEMS, LB, ROLE_LAST>(a, pass, pd, ps, s_tile, s_bar,
                                                                  s_dyn);
        else
            onesweep_pipe_body<C, V, BLOCK, ITEMS, LB, ROLE_MID>(a, pass, pd, ps, s_tile, s_bar,
                                                                 s_dyn);
    }
}

}  // namespace xss
