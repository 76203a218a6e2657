// xss_blocksort.cuh -- one-CTA sort of a small array (or segment) in shared
// memory: a bitonic network over (code, index) pairs.  The index tie-break
// makes the network stable and lets values and argsort indices follow the
// keys by one gather.  Replaces the reference's register networks for
// n <= network_sort_threshold (src/xss-network-qsort.hpp:171-234,
// src/xss-network-keyvaluesort.hpp:209-388).
#pragma once
#include <type_traits>
#include "xss_internal.cuh"

namespace xss {

struct SmallArgs {
    const void *keys_in;
    void *keys_out;      // nullptr: keys not written (argsort)
    const void *vals_in;
    void *vals_out;
    uint64_t *out_idx;   // argsort output
    uint32_t n, npad;
    KeyXform xf;
};

constexpr int SMALL_BLOCK = 1024;

// Sort n <= MAXN keys with the calling CTA of BLOCK threads.  s_raw holds
// npad codes followed by npad 16-bit indices (npad: power of two >= n).
// Keys and values may be sorted in place (kin == kout, vin == vout).
template <typename C, typename V, int BLOCK, int MAXN>
__device__ __forceinline__ void block_bitonic_sort(const C *kin, C *kout, const V *vin, V *vout,
                                                   uint64_t *out_idx, uint32_t n, uint32_t npad,
                                                   const KeyXform &xf, unsigned char *s_raw)
{
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    static_assert(MAXN <= 65536, "16-bit indices");
    C *s_code = reinterpret_cast<C *>(s_raw);
    uint16_t *s_idx = reinterpret_cast<uint16_t *>(s_raw + sizeof(C) * npad);
    const int tid = threadIdx.x;
    for (uint32_t i = tid; i < npad; i += BLOCK) {
        s_code[i] = i < n ? to_code(kin[i], xf) : C(~C(0));
        s_idx[i] = (uint16_t)i;
    }
    __syncthreads();
    for (uint32_t k = 2; k <= npad; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = tid; t < npad / 2; t += BLOCK) {
                const uint32_t i = 2 * t - (t & (j - 1));
                const uint32_t ixj = i + j;
                const C ca = s_code[i], cb = s_code[ixj];
                const uint16_t ia = s_idx[i], ib = s_idx[ixj];
                const bool a_gt_b = (ca > cb) || (ca == cb && ia > ib);
                const bool up = (i & k) == 0;
                if (a_gt_b == up) {
                    s_code[i] = cb; s_code[ixj] = ca;
                    s_idx[i] = ib;  s_idx[ixj] = ia;
                }
            }
            __syncthreads();
        }
    }
    if (kout) {
        for (uint32_t i = tid; i < n; i += BLOCK) kout[i] = from_code(s_code[i], xf);
    }
    if (out_idx) {
        for (uint32_t i = tid; i < n; i += BLOCK) out_idx[i] = s_idx[i];
    }
    if constexpr (HAS_V) {
        constexpr int R = (MAXN + BLOCK - 1) / BLOCK;
        V tmp[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t i = tid + r * BLOCK;
            if (i < n) tmp[r] = vin[s_idx[i]];
        }
        __syncthreads();  // every value read before any is overwritten
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t i = tid + r * BLOCK;
            if (i < n) vout[i] = tmp[r];
        }
    }
}

template <typename C, typename V, int BLOCK, int MAXN>
__global__ void __launch_bounds__(BLOCK) small_sort_kernel(SmallArgs a)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    block_bitonic_sort<C, V, BLOCK, MAXN>(
        static_cast<const C *>(a.keys_in), static_cast<C *>(a.keys_out),
        static_cast<const V *>(a.vals_in), static_cast<V *>(a.vals_out), a.out_idx, a.n, a.npad,
        a.xf, s_raw);
}

}  // namespace xss
