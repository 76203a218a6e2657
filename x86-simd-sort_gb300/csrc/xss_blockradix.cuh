// xss_blockradix.cuh -- one-CTA stable LSD radix sort of a segment of up to
// BLOCK * ITEMS keys (and values) held in registers, ranked through shared
// memory: per 8-bit digit, per-warp digit counts, a (digit, warp) scan, and
// the lane-mask ranking of the onesweep pass (xss_onesweep.cuh) writing each
// key to its place in a shared buffer, read back in element order for the
// next digit.  A bitonic network costs O(n log^2 n) compare-exchanges; this
// costs a few shared-memory operations per key and digit, which wins from a
// few hundred keys up.  Replaces the reference's network sorts for its
// mid-size arrays (src/xss-network-qsort.hpp:171-234,
// src/xss-network-keyvaluesort.hpp:209-388) in the segmented batch.
#pragma once
#include <type_traits>
#include "xss_onesweep.cuh"

namespace xss {

__host__ __device__ constexpr size_t round16(size_t x) { return (x + 15) / 16 * 16; }

// Dynamic shared memory of block_radix_sort: keys, values, per-warp words.
template <typename C, typename V, int BLOCK, int ITEMS>
constexpr size_t block_radix_smem()
{
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    return round16((size_t)BLOCK * ITEMS * sizeof(C)) +
           (HAS_V ? round16((size_t)BLOCK * ITEMS * sizeof(V)) : 0) +
           (size_t)(BLOCK / 32) * RADIX * 2 * sizeof(uint32_t) + 32 * sizeof(uint32_t);
}

// Sort keys[0, len) (and vals) in place, len <= BLOCK * ITEMS; `passes` digit
// passes from the lowest.  Element e lives in warp e / (32 * ITEMS), item
// (e / 32) % ITEMS, lane e % 32, so loads and stores are coalesced and the
// (digit, warp, item, lane) rank order is element order: stable.
template <typename C, typename V, int BLOCK, int ITEMS>
__device__ __forceinline__ void block_radix_sort(C *keys, V *vals, uint32_t len, int passes,
                                                 const KeyXform &xf, unsigned char *s_raw)
{
    constexpr int WARPS = BLOCK / 32;
    constexpr int TILE = BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    using VS = typename std::conditional<HAS_V, V, uint8_t>::type;
    static_assert(BLOCK == RADIX, "one thread per digit in the scan");
    C *s_k = reinterpret_cast<C *>(s_raw);
    unsigned char *p = s_raw + round16((size_t)TILE * sizeof(C));
    VS *s_v = reinterpret_cast<VS *>(p);
    if constexpr (HAS_V) p += round16((size_t)TILE * sizeof(V));
    uint32_t *wm = reinterpret_cast<uint32_t *>(p);   // [WARPS][RADIX] counts/offsets, then masks
    uint32_t *s_scan = wm + 2 * WARPS * RADIX;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t local0 = (uint32_t)warp * (ITEMS * 32) + lane;
    // items of this warp that hold elements (uniform across the warp)
    const uint32_t wbase = (uint32_t)warp * (ITEMS * 32);
    const int witems = wbase >= len ? 0 : (int)min((uint32_t)ITEMS, (len - wbase + 31) / 32);

    C key[ITEMS];
    VS val[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint32_t e = local0 + j * 32;
        if (e < len) {
            key[j] = to_code(keys[e], xf);
            if constexpr (HAS_V) val[j] = vals[e];
        }
    }
    for (int i = tid; i < 2 * WARPS * RADIX; i += BLOCK) wm[i] = 0;
    __syncthreads();

    uint32_t *wh = wm + warp * RADIX;
    uint32_t *mt = wm + (WARPS + warp) * RADIX;
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = pass * RADIX_BITS;
#pragma unroll
        for (int j = 0; j < ITEMS; ++j)
            if (j < witems && local0 + j * 32 < len)
                atomicAdd(&wh[uint32_t(key[j] >> shift) & (RADIX - 1)], 1u);
        __syncthreads();

        // (digit, warp) exclusive offsets; a digit every key shares leaves
        // the order as it is
        uint32_t cnt = 0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) cnt += wm[w * RADIX + tid];
        if (__syncthreads_or(cnt == len)) {
#pragma unroll
            for (int w = 0; w < WARPS; ++w) wm[w * RADIX + tid] = 0;
            __syncthreads();
            continue;
        }
        uint32_t total;
        uint32_t run = block_excl_scan<BLOCK>(cnt, s_scan, total);
#pragma unroll
        for (int w = 0; w < WARPS; ++w) {
            const uint32_t c = wm[w * RADIX + tid];
            wm[w * RADIX + tid] = run;
            run += c;
        }
        __syncthreads();

        // stable rank: lanes sharing a digit set their bit in the warp's word
        // for it and read it back; the highest advances the warp's offset
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            if (j >= witems) break;
            const bool ok = local0 + j * 32 < len;
            const uint32_t d = uint32_t(key[j] >> shift) & (RADIX - 1);
            if (ok) atomicOr(&mt[d], 1u << lane);
            __syncwarp();
            const uint32_t peers = ok ? mt[d] : (1u << lane);
            __syncwarp();
            const int leader = 31 - __clz(peers);
            uint32_t base = 0;
            if (ok && lane == leader) {
                base = atomicAdd(&wh[d], (uint32_t)__popc(peers));
                mt[d] = 0;
            }
            base = __shfl_sync(0xffffffffu, base, leader);
            if (ok) {
                const uint32_t pos = base + __popc(peers & lt_mask);
                s_k[pos] = key[j];
                if constexpr (HAS_V) s_v[pos] = val[j];
            }
            __syncwarp();
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t e = local0 + j * 32;
            if (e < len) {
                key[j] = s_k[e];
                if constexpr (HAS_V) val[j] = s_v[e];
            }
        }
#pragma unroll
        for (int w = 0; w < WARPS; ++w) wm[w * RADIX + tid] = 0;
        __syncthreads();
    }

#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint32_t e = local0 + j * 32;
        if (e < len) {
            keys[e] = from_code(key[j], xf);
            if constexpr (HAS_V) vals[e] = val[j];
        }
    }
}

}  // namespace xss
