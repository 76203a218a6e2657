// xss_radix.cu -- full sorts: one-CTA bitonic sort for small inputs and an
// LSD "onesweep" radix sort (one up-front histogram, then one kernel per
// 8-bit digit with a decoupled look-back prefix) for large ones.
//
// Replaces, for the reference's qsort / keyvalue_qsort / argsort:
//   src/xss-common-qsort.h:529-605   (qsort_ recursion, partition sweeps)
//   src/xss-common-keyvaluesort.hpp:419-653 (kvsort_, kv partition)
//   src/xss-common-argsort.h:470-669 (argsort_, argpartition)
//   src/xss-network-qsort.hpp, src/xss-network-keyvaluesort.hpp (small-n networks)
// The reference's quicksort is in-place and unstable; an LSD radix sort is
// stable per pass and yields one of the orders the reference may produce.
#include <algorithm>
#include <mutex>
#include <type_traits>
#include "xss_internal.cuh"

namespace xss {

struct NoVal {};

// ---------------------------------------------------------------------------
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

// ---------------------------------------------------------------------------
// Up-front histogram of every digit of every key (one read of the input),
// fused with clearing the look-back status words.  The last CTA to finish
// turns the histograms into per-pass bucket starts and writes the pass plan:
// a pass whose digit is the same for every key is skipped.
template <typename C>
__global__ void __launch_bounds__(256) hist_kernel(RadixArgs a)
{
    __shared__ uint32_t sh[MAX_PASSES * RADIX];
    __shared__ uint32_t s_scan[8];
    __shared__ int s_last;
    __shared__ int s_active[MAX_PASSES];
    const int tid = threadIdx.x;
    const int P = a.passes;
    for (int i = tid; i < P * RADIX; i += 256) sh[i] = 0;
    __syncthreads();

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
            const C c = to_code(e[u], a.xf);
            for (int p = 0; p < P; ++p)
                atomicAdd(&sh[p * RADIX + (uint32_t(c >> (p * RADIX_BITS)) & (RADIX - 1))], 1u);
        }
    }
    for (size_t i = nvec * VEC + gtid; i < n; i += stride) {
        const C c = to_code(src[i], a.xf);
        for (int p = 0; p < P; ++p)
            atomicAdd(&sh[p * RADIX + (uint32_t(c >> (p * RADIX_BITS)) & (RADIX - 1))], 1u);
    }

    // clear the look-back words of every pass (multiple of 4 words, 16B aligned)
    const size_t nst4 = (size_t)P * a.num_tiles * RADIX / 4;
    uint4 *st4 = reinterpret_cast<uint4 *>(a.status);
    for (size_t i = gtid; i < nst4; i += stride) st4[i] = make_uint4(0, 0, 0, 0);

    __syncthreads();
    for (int i = tid; i < P * RADIX; i += 256)
        if (sh[i]) atomicAdd(&a.hdr->hist[0][0] + i, sh[i]);
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = (atomicAdd(&a.hdr->done_ctr, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();

    for (int p = 0; p < P; ++p) {
        const uint32_t h = ld_relaxed_u32(&a.hdr->hist[p][tid]);
        const int trivial = __syncthreads_or(h == (uint32_t)n);
        uint32_t total;
        const uint32_t ex = block_excl_scan<256>(h, s_scan, total);
        a.hdr->start[p][tid] = ex;
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

// Buffer id -> pointer without dynamically indexing the parameter array
// (which would force a local-memory copy of it).
__device__ __forceinline__ void *pick3(void *const (&b)[3], int i)
{
    return i == 0 ? b[0] : (i == 1 ? b[1] : b[2]);
}

// ---------------------------------------------------------------------------
// One LSD pass over 8 bits.  Each CTA takes the next tile id from an atomic
// counter (so a tile only waits on tiles already running), ranks its keys by
// digit with warp match + per-warp counters (stable: digit, warp, item, lane),
// publishes its digit counts, resolves its global offsets by decoupled
// look-back, stages the tile in digit order in shared memory and scatters
// runs of equal digits to consecutive global addresses.
template <typename C, typename V, int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) onesweep_kernel(RadixArgs a, int pass)
{
    constexpr int WARPS = BLOCK / 32;
    constexpr int TILE = BLOCK * ITEMS;
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    static_assert(BLOCK >= RADIX, "one thread per digit");

    const PassDesc pd = a.hdr->desc[pass];
    if (!pd.active) return;

    __shared__ uint32_t s_whist[WARPS * RADIX];
    __shared__ int32_t s_off[RADIX];
    __shared__ uint32_t s_scan[WARPS];
    __shared__ uint32_t s_tile;
    extern __shared__ __align__(16) unsigned char s_stage[];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n = (uint32_t)a.n;
    const int shift = pass * RADIX_BITS;

    for (int i = tid; i < WARPS * RADIX; i += BLOCK) s_whist[i] = 0;
    if (tid == 0) s_tile = atomicAdd(&a.hdr->tile_ctr[pass], 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t tile_base = tile * (uint32_t)TILE;
    const uint32_t wbase = tile_base + (uint32_t)warp * (ITEMS * 32) + lane;

    C key[ITEMS];
    {
        const C *ksrc = static_cast<const C *>(pick3(a.kbuf, pd.src));
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t idx = wbase + j * 32;
            if (idx < n) {
                const C b = ksrc[idx];
                key[j] = pd.first ? to_code(b, a.xf) : b;
            } else {
                key[j] = C(~C(0));
            }
        }
    }
    typename std::conditional<HAS_V, V, uint8_t>::type val[ITEMS];
    if constexpr (HAS_V) {
        const V *vsrc = static_cast<const V *>(pick3(a.vbuf, pd.vsrc));
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t idx = wbase + j * 32;
            if (pd.gen_idx) val[j] = V(idx);
            else val[j] = idx < n ? vsrc[idx] : V(0);
        }
    }

    // ---- stable rank within the tile
    uint32_t pos[ITEMS];
    {
        uint32_t *wh = s_whist + warp * RADIX;
        const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const uint32_t d = uint32_t(key[j] >> shift) & (RADIX - 1);
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            const int leader = 31 - __clz(peers);
            uint32_t base = 0;
            if (lane == leader) {
                base = wh[d];
                wh[d] = base + __popc(peers);
            }
            base = __shfl_sync(0xffffffffu, base, leader);
            pos[j] = base + __popc(peers & lt_mask);
            __syncwarp();
        }
    }
    __syncthreads();

    // ---- tile digit counts, publish, local scan, look-back
    uint32_t cnt = 0;
    uint32_t *st_tile = a.status + ((size_t)pass * a.num_tiles + tile) * RADIX;
    if (tid < RADIX) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) {
            const uint32_t c = s_whist[w * RADIX + tid];
            s_whist[w * RADIX + tid] = run;
            run += c;
        }
        cnt = run;
        st_relaxed_u32(st_tile + tid, (tile == 0 ? FLAG_PRE : FLAG_AGG) | cnt);
    }
    uint32_t total;
    const uint32_t local_start = block_excl_scan<BLOCK>(cnt, s_scan, total);
    if (tid < RADIX) {
        uint32_t excl = 0;
        if (tile > 0) {
            const uint32_t *st_pass = a.status + (size_t)pass * a.num_tiles * RADIX;
            int p = (int)tile - 1;
            uint32_t spins = 0;
            while (p >= 0) {
                const uint32_t v = ld_relaxed_u32(st_pass + (size_t)p * RADIX + tid);
                const uint32_t f = v & FLAG_MASK;
                if (f == 0u) {
                    if (++spins > XSS_SPIN_LIMIT) {
                        atomicOr(a.err, XSS_DEVERR_TIMEOUT);
                        break;
                    }
                    continue;
                }
                excl += v & COUNT_MASK;
                if (f == FLAG_PRE) break;
                --p;
            }
            st_relaxed_u32(st_tile + tid, FLAG_PRE | ((excl + cnt) & COUNT_MASK));
        }
        s_off[tid] = (int32_t)(a.hdr->start[pass][tid] + excl) - (int32_t)local_start;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) s_whist[w * RADIX + tid] += local_start;
    }
    __syncthreads();

    // ---- stage keys in digit order
    C *s_keys = reinterpret_cast<C *>(s_stage);
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        const uint32_t d = uint32_t(key[j] >> shift) & (RADIX - 1);
        pos[j] += s_whist[warp * RADIX + d];
        s_keys[pos[j]] = key[j];
    }
    __syncthreads();

    // ---- scatter: consecutive threads write consecutive slots of a digit run
    const uint32_t valid = min((uint32_t)TILE, n - tile_base);
    uint32_t gdst[HAS_V ? ITEMS : 1];
    {
        C *kdst = static_cast<C *>(pick3(a.kbuf, pd.dst));
#pragma unroll
        for (int m = 0; m < ITEMS; ++m) {
            const uint32_t i = tid + m * BLOCK;
            if (i < valid) {
                const C c = s_keys[i];
                const uint32_t d = uint32_t(c >> shift) & (RADIX - 1);
                uint32_t g = (uint32_t)(s_off[d] + (int32_t)i);
                if (g >= n) {  // only reachable after a look-back timeout
                    atomicOr(a.err, XSS_DEVERR_BOUNDS);
                    g = n;     // marks the slot as not to be written
                }
                if constexpr (HAS_V) gdst[m] = g;
                if (!pd.skip_keys && g < n) kdst[g] = pd.last ? from_code(c, a.xf) : c;
            }
        }
    }
    if constexpr (HAS_V) {
        __syncthreads();
        V *s_vals = reinterpret_cast<V *>(s_stage);
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) s_vals[pos[j]] = val[j];
        __syncthreads();
        if (pd.out_idx) {
#pragma unroll
            for (int m = 0; m < ITEMS; ++m) {
                const uint32_t i = tid + m * BLOCK;
                if (i < valid && gdst[m] < n) a.out_idx[gdst[m]] = (uint64_t)s_vals[i];
            }
        } else {
            V *vdst = static_cast<V *>(pick3(a.vbuf, pd.vdst));
#pragma unroll
            for (int m = 0; m < ITEMS; ++m) {
                const uint32_t i = tid + m * BLOCK;
                if (i < valid && gdst[m] < n) vdst[gdst[m]] = s_vals[i];
            }
        }
    }
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
// Small inputs: one CTA, bitonic network in shared memory over (code, index)
// pairs.  The index tie-break makes the network stable and lets values and
// argsort indices follow the keys by one gather.  Replaces the reference's
// register networks for n <= network_sort_threshold
// (src/xss-network-qsort.hpp:171-234, src/xss-network-keyvaluesort.hpp:209-388).
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

template <typename C, typename V>
__global__ void __launch_bounds__(SMALL_BLOCK) small_sort_kernel(SmallArgs a)
{
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    extern __shared__ __align__(16) unsigned char s_raw[];
    C *s_code = reinterpret_cast<C *>(s_raw);
    uint16_t *s_idx = reinterpret_cast<uint16_t *>(s_raw + sizeof(C) * a.npad);
    const int tid = threadIdx.x;
    const uint32_t n = a.n, npad = a.npad;
    const C *kin = static_cast<const C *>(a.keys_in);
    for (uint32_t i = tid; i < npad; i += SMALL_BLOCK) {
        s_code[i] = i < n ? to_code(kin[i], a.xf) : C(~C(0));
        s_idx[i] = (uint16_t)i;
    }
    __syncthreads();
    for (uint32_t k = 2; k <= npad; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = tid; t < npad / 2; t += SMALL_BLOCK) {
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
    if (a.keys_out) {
        C *kout = static_cast<C *>(a.keys_out);
        for (uint32_t i = tid; i < n; i += SMALL_BLOCK) kout[i] = from_code(s_code[i], a.xf);
    }
    if (a.out_idx) {
        for (uint32_t i = tid; i < n; i += SMALL_BLOCK) a.out_idx[i] = s_idx[i];
    }
    if constexpr (HAS_V) {
        constexpr int R = (int)(SMALL_SORT_MAX * 2 / SMALL_BLOCK);
        const V *vin = static_cast<const V *>(a.vals_in);
        V tmp[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t i = tid + r * SMALL_BLOCK;
            if (i < n) tmp[r] = vin[s_idx[i]];
        }
        __syncthreads();
        V *vout = static_cast<V *>(a.vals_out);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t i = tid + r * SMALL_BLOCK;
            if (i < n) vout[i] = tmp[r];
        }
    }
}

// ---------------------------------------------------------------------------
// Host side.
template <typename C, typename V> struct TileCfg {
    static constexpr int BLOCK = 256;
    static constexpr int ITEMS = (sizeof(C) + sizeof(V) > 8) ? 8 : 16;
};
template <typename C> struct TileCfg<C, NoVal> {
    static constexpr int BLOCK = 256;
    static constexpr int ITEMS = sizeof(C) == 8 ? 12 : 16;
};

template <typename C, typename V> constexpr size_t tile_size()
{
    return (size_t)TileCfg<C, V>::BLOCK * TileCfg<C, V>::ITEMS;
}

struct RadixLayout {
    size_t hdr, status, k1, k2, v1, v2, total;
};

static RadixLayout radix_layout(int op, int kbytes, int vbytes, size_t n, size_t tile)
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

template <typename C, typename V> static size_t tile_for()
{
    return tile_size<C, V>();
}

static size_t tile_for_bytes(int op, int kbytes, int vbytes)
{
    const int vb = (op == SOP_ARG) ? 4 : (op == SOP_KV ? vbytes : 0);
    switch (kbytes) {
    case 2: return vb == 0 ? tile_for<uint16_t, NoVal>() : vb == 4 ? tile_for<uint16_t, uint32_t>() : tile_for<uint16_t, uint64_t>();
    case 4: return vb == 0 ? tile_for<uint32_t, NoVal>() : vb == 4 ? tile_for<uint32_t, uint32_t>() : tile_for<uint32_t, uint64_t>();
    default: return vb == 0 ? tile_for<uint64_t, NoVal>() : vb == 4 ? tile_for<uint64_t, uint32_t>() : tile_for<uint64_t, uint64_t>();
    }
}

size_t radix_workspace_bytes(int op, int kbytes, int vbytes, size_t n)
{
    if (n <= SMALL_SORT_MAX) return 0;
    return radix_layout(op, kbytes, vbytes, n, tile_for_bytes(op, kbytes, vbytes)).total;
}

template <typename C, typename V>
static int small_sort_launch(int op, KeyXform xf, void *keys, void *vals,
                             uint64_t *out_idx, size_t n, cudaStream_t s)
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
    const size_t smem = align_up(sizeof(C) * npad, 16) + 2 * npad;
    auto kern = small_sort_kernel<C, V>;
    static bool attr_set = false;
    if (!attr_set) {
        XSS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(align_up(sizeof(C) * SMALL_SORT_MAX * 2, 16) + 4 * SMALL_SORT_MAX)));
        attr_set = true;
    }
    XSS_LAUNCH(PK_SMALL, s, kern<<<1, SMALL_BLOCK, smem, s>>>(a));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

template <typename C, typename V>
static int onesweep_launch(int op, KeyXform xf, void *keys, void *vals,
                           uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes,
                           cudaStream_t s)
{
    constexpr int BLOCK = TileCfg<C, V>::BLOCK, ITEMS = TileCfg<C, V>::ITEMS;
    constexpr size_t TILE = (size_t)BLOCK * ITEMS;
    const int kbytes = sizeof(C);
    const int vbytes = std::is_same<V, NoVal>::value ? 0 : (int)sizeof(V);
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
    a.err = device_error_word();

    XSS_CUDA_TRY(cudaMemsetAsync(a.hdr, 0, sizeof(RadixHeader), s));
    const int sms = num_sms();
    const size_t want = (n + 256 * 16 - 1) / (256 * 16);
    const int hist_grid = (int)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * 8));
    XSS_LAUNCH(PK_HIST, s, hist_kernel<C><<<hist_grid, 256, 0, s>>>(a));
    XSS_CUDA_TRY(cudaGetLastError());

    const size_t smem = TILE * std::max(sizeof(C), std::is_same<V, NoVal>::value ? (size_t)0 : sizeof(V));
    auto kern = onesweep_kernel<C, V, BLOCK, ITEMS>;
    static bool attr_set = false;
    if (!attr_set) {
        XSS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    for (int p = 0; p < a.passes; ++p) {
        XSS_LAUNCH(PK_ONESWEEP, s, kern<<<a.num_tiles, BLOCK, smem, s>>>(a, p));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    XSS_LAUNCH(PK_FIXUP, s, fixup_kernel<C, V><<<sms * 2, 256, 0, s>>>(a));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

template <typename C>
static int radix_sort_c(int op, KeyXform xf, void *keys, void *vals, int vbytes,
                        uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s)
{
    const bool small = n <= SMALL_SORT_MAX;
    if (op == SOP_ARG) {
        return small ? small_sort_launch<C, NoVal>(op, xf, keys, nullptr, out_idx, n, s)
                     : onesweep_launch<C, uint32_t>(op, xf, keys, nullptr, out_idx, n, ws, ws_bytes, s);
    }
    if (op == SOP_KEYS || vbytes == 0) {
        return small ? small_sort_launch<C, NoVal>(op, xf, keys, nullptr, nullptr, n, s)
                     : onesweep_launch<C, NoVal>(op, xf, keys, nullptr, nullptr, n, ws, ws_bytes, s);
    }
    if (vbytes == 4)
        return small ? small_sort_launch<C, uint32_t>(op, xf, keys, vals, nullptr, n, s)
                     : onesweep_launch<C, uint32_t>(op, xf, keys, vals, nullptr, n, ws, ws_bytes, s);
    return small ? small_sort_launch<C, uint64_t>(op, xf, keys, vals, nullptr, n, s)
                 : onesweep_launch<C, uint64_t>(op, xf, keys, vals, nullptr, n, ws, ws_bytes, s);
}

int radix_sort(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
               uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s)
{
    if (n == 0) return XSS_OK;
    if (n == 1) {
        // the reference returns early for arrsize <= 1 (src/xss-common-qsort.h:660);
        // argsort of one element is the index 0
        if (op == SOP_ARG) XSS_CUDA_TRY(cudaMemsetAsync(out_idx, 0, sizeof(uint64_t), s));
        return XSS_OK;
    }
    if (n > XSS_MAX_N) return XSS_ETOOBIG;
    switch (kbytes) {
    case 2: return radix_sort_c<uint16_t>(op, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s);
    case 4: return radix_sort_c<uint32_t>(op, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s);
    case 8: return radix_sort_c<uint64_t>(op, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s);
    default: return XSS_EINVAL;
    }
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

// Device address of g_noalloc_scratch, looked up once per device.  In host
// code the symbol itself is only a host-side stand-in, never a device address.
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_addr[64];

static int noalloc_scratch(unsigned char **out)
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
        g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_noalloc_addr[dev];
    return XSS_OK;
}

template <typename C>
static int qsort_noalloc_c(KeyXform xf, void *keys, size_t n, unsigned char *scratch,
                           cudaStream_t s)
{
    unsigned *err = reinterpret_cast<unsigned *>(scratch);
    if (n <= SMALL_SORT_MAX) {
        SmallArgs a{};
        a.keys_in = keys;
        a.keys_out = keys;
        a.n = (uint32_t)n;
        uint32_t npad = 2;
        while (npad < n) npad <<= 1;
        a.npad = npad;
        a.xf = xf;
        const size_t smem = align_up(sizeof(C) * npad, 16) + 2 * npad;  // <= 40 KiB
        small_sort_kernel<C, NoVal><<<1, SMALL_BLOCK, smem, s>>>(a);
        XSS_CUDA_TRY(cudaGetLastError());
        return XSS_OK;
    }
    constexpr int BLOCK = TileCfg<C, NoVal>::BLOCK, ITEMS = TileCfg<C, NoVal>::ITEMS;
    constexpr size_t TILE = (size_t)BLOCK * ITEMS;
    const RadixLayout L = radix_layout(SOP_KEYS, sizeof(C), 0, n, TILE);
    if (L.total > NOALLOC_SCRATCH_BYTES - NOALLOC_ERR_BYTES) return XSS_ENOMEM;
    unsigned char *base = scratch + NOALLOC_ERR_BYTES;
    RadixArgs a{};
    a.kbuf[0] = keys;
    a.kbuf[1] = base + L.k1;
    a.kbuf[2] = base + L.k2;
    a.n = n;
    a.num_tiles = (uint32_t)((n + TILE - 1) / TILE);
    a.passes = sizeof(C);
    a.op = SOP_KEYS;
    a.xf = xf;
    a.hdr = reinterpret_cast<RadixHeader *>(base + L.hdr);
    a.status = reinterpret_cast<uint32_t *>(base + L.status);
    a.err = err;
    XSS_CUDA_TRY(cudaMemsetAsync(a.hdr, 0, sizeof(RadixHeader), s));
    const int sms = num_sms();
    const size_t want = (n + 256 * 16 - 1) / (256 * 16);
    const int hist_grid = (int)std::max<size_t>(1, std::min<size_t>(want, (size_t)sms * 8));
    hist_kernel<C><<<hist_grid, 256, 0, s>>>(a);
    XSS_CUDA_TRY(cudaGetLastError());
    const size_t smem = TILE * sizeof(C);  // <= 24 KiB, no opt-in needed
    for (int p = 0; p < a.passes; ++p) {
        onesweep_kernel<C, NoVal, BLOCK, ITEMS><<<a.num_tiles, BLOCK, smem, s>>>(a, p);
        XSS_CUDA_TRY(cudaGetLastError());
    }
    fixup_kernel<C, NoVal><<<sms * 2, 256, 0, s>>>(a);
    XSS_CUDA_TRY(cudaGetLastError());
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
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    XSS_CUDA_TRY(cudaMemsetAsync(scratch, 0, NOALLOC_ERR_BYTES, s));
    const KeyXform xf{kind, descending ? 1 : 0, hasnan ? 1 : 0};
    switch (kbytes) {
    case 2: rc = qsort_noalloc_c<uint16_t>(xf, d_arr, n, scratch, s); break;
    case 4: rc = qsort_noalloc_c<uint32_t>(xf, d_arr, n, scratch, s); break;
    default: rc = qsort_noalloc_c<uint64_t>(xf, d_arr, n, scratch, s); break;
    }
    if (rc) return rc;
    unsigned h = 0;
    XSS_CUDA_TRY(cudaMemcpyAsync(&h, scratch, sizeof(h), cudaMemcpyDeviceToHost, s));
    XSS_CUDA_TRY(cudaStreamSynchronize(s));
    return h ? XSS_ETIMEOUT : XSS_OK;
}
