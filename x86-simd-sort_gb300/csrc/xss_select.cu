// xss_select.cu -- radix select and in-place partition.
//
// Replaces the reference's quickselect family:
//   src/xss-common-qsort.h:607-649, 712-762     (qselect_, xss_qselect, xss_partial_qsort)
//   src/xss-common-argsort.h:551-585, 694-731   (argselect_, xss_argselect)
//   src/xss-common-keyvaluesort.hpp:519-562, 655-738 (kvselect_, select/partial kv)
//
// Method: find the exact k-th code by histogramming 11-bit digits from the
// top (round 0 reads every key; round 1 reads every key again and compacts
// the keys that share the chosen top digit; later rounds read only those
// candidates).  With the k-th code K and the counts of codes < K and == K
// known, the array is partitioned in place: every element whose class
// (<, ==, > K) does not match the region its position falls in is appended
// to a per-class list, its position to the per-region hole list, and a
// second kernel moves list entries into holes.  Only misplaced elements are
// written, as in an in-place quickselect partition.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include "xss_internal.cuh"

namespace xss {

constexpr int SEL_DIGIT = 11;
constexpr int SEL_BINS = 1 << SEL_DIGIT;

struct SelState {
    unsigned long long k_rem;
    unsigned long long cnt_less;
    unsigned long long cand_n;
    unsigned long long prefix;
    unsigned long long mask;
    unsigned long long cl;
    unsigned long long ce;
    unsigned int nmis[3];
    unsigned int nhole[3];
    unsigned int hist[SEL_BINS];
};

struct SelArgs {
    void *keys;
    void *vals;
    uint64_t *out_idx;
    size_t n;
    KeyXform xf;
    int op;
    SelState *st;
    void *cand;
    void *mis_k;
    void *mis_v;
    uint32_t *holes;
};

template <int BLOCK>
__device__ __forceinline__ uint32_t sel_block_excl_scan(uint32_t v, uint32_t *s_warp)
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
    __syncthreads();
    return pre + x - v;
}

// Warp-aggregated append: returns this lane's slot among lanes with `pred`.
__device__ __forceinline__ uint32_t warp_append(bool pred, unsigned int *counter)
{
    const uint32_t m = __ballot_sync(0xffffffffu, pred);
    if (m == 0) return 0;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// One histogram round over every key (rounds 0, 1) or over the compacted
// candidates (rounds >= 2).  16-byte vector loads, four per thread in
// flight, keep enough bytes moving to cover memory latency; an unaligned
// array takes the scalar loop.  Every loop bound is uniform across a warp so
// the ballots of the round-1 compaction see all 32 lanes.
template <typename C>
__global__ void __launch_bounds__(256) sel_hist_kernel(SelArgs a, int round, int lo, int bits)
{
    constexpr int VW = 16 / sizeof(C);   // keys per vector
    constexpr int U = 4;                 // vectors per thread in flight
    __shared__ uint32_t sh[SEL_BINS];
    const int nb = 1 << bits;
    for (int i = threadIdx.x; i < nb; i += 256) sh[i] = 0;
    __syncthreads();
    const C prefix = (C)a.st->prefix, mask = (C)a.st->mask;
    const size_t count = round <= 1 ? a.n : (size_t)a.st->cand_n;
    const C *src = round <= 1 ? static_cast<const C *>(a.keys) : static_cast<const C *>(a.cand);
    C *cand = static_cast<C *>(a.cand);
    const int lane = threadIdx.x & 31;
    const size_t stride = (size_t)gridDim.x * 256;
    const size_t wbase = (size_t)blockIdx.x * 256 + threadIdx.x - lane;   // warp's first thread

    auto visit = [&](C b, bool active) {
        C c = 0;
        if (active) c = round <= 1 ? to_code(b, a.xf) : b;
        const bool match = active && ((C)(c & mask) == prefix);
        if (match) atomicAdd(&sh[uint32_t(c >> lo) & (uint32_t)(nb - 1)], 1u);
        if (round == 1) {
            const uint32_t slot = warp_append(match, (unsigned int *)&a.st->cand_n);
            if (match) cand[slot] = c;
        }
    };

    size_t head = 0;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        const size_t nvec = count / VW;
        const uint4 *vsrc = reinterpret_cast<const uint4 *>(src);
        for (size_t v0 = wbase; v0 < nvec; v0 += U * stride) {
            uint4 w[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const size_t v = v0 + lane + u * stride;
                w[u] = v < nvec ? vsrc[v] : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool act = v0 + lane + u * stride < nvec;
                const C *e = reinterpret_cast<const C *>(&w[u]);
#pragma unroll
                for (int j = 0; j < VW; ++j) visit(e[j], act);
            }
        }
        head = nvec * VW;
    }
    for (size_t i0 = head + wbase; i0 < count; i0 += stride) {
        const size_t i = i0 + lane;
        visit(i < count ? src[i] : C(0), i < count);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += 256)
        if (sh[i]) atomicAdd(&a.st->hist[i], sh[i]);
}

// One CTA: locate the bin holding rank k_rem, extend the prefix, reset the
// histogram for the next round.
template <typename C>
__global__ void __launch_bounds__(1024) sel_find_kernel(SelArgs a, int round, int lo, int bits,
                                                        int last, unsigned long long k0)
{
    __shared__ uint32_t s_warp[32];
    const int nb = 1 << bits;
    const int per = (nb + 1023) / 1024;
    const int t = threadIdx.x;
    uint32_t sum = 0;
    for (int b = t * per; b < min(nb, (t + 1) * per); ++b) sum += a.st->hist[b];
    const uint32_t ex = sel_block_excl_scan<1024>(sum, s_warp);
    const unsigned long long krem = round == 0 ? k0 : a.st->k_rem;
    if ((unsigned long long)ex <= krem && krem < (unsigned long long)ex + sum) {
        uint32_t cum = ex;
        for (int b = t * per; b < min(nb, (t + 1) * per); ++b) {
            const uint32_t h = a.st->hist[b];
            if (krem < (unsigned long long)cum + h) {
                a.st->cnt_less += cum;
                a.st->k_rem = krem - cum;
                a.st->prefix |= (unsigned long long)b << lo;
                a.st->mask |= (unsigned long long)(nb - 1) << lo;
                if (last) {
                    a.st->cl = a.st->cnt_less;
                    a.st->ce = h;
                }
                break;
            }
            cum += h;
        }
    }
    __syncthreads();
    for (int b = t; b < nb; b += 1024) a.st->hist[b] = 0;
    if (round == 0 && t == 0) a.st->cand_n = 0;
}

// Block-wide exclusive scan of three 32-bit words per thread (each word
// packs two 16-bit counters that cannot overflow within one chunk).
__device__ __forceinline__ void sel_scan3(uint32_t (&v)[3], uint32_t (*s_w)[3], uint32_t (&tot)[3])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x[3] = {v[0], v[1], v[2]};
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x[q], o);
            if (lane >= o) x[q] += y;
        }
    }
    if (lane == 31)
        for (int q = 0; q < 3; ++q) s_w[warp][q] = x[q];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        uint32_t pre = 0, t = 0;
        for (int w = 0; w < 8; ++w) {
            const uint32_t c = s_w[w][q];
            if (w < warp) pre += c;
            t += c;
        }
        tot[q] = t;
        v[q] = pre + x[q] - v[q];
    }
    __syncthreads();
}

// Partition bookkeeping: every element whose class (<, ==, > K) differs from
// the region its position lies in goes to its class's list, its position to
// its region's hole list.  A CTA takes chunks of 256 * IPT elements, each
// thread IPT consecutive ones (8 16-bit or 32 bytes of wider keys; 16-byte
// vector loads when the array is aligned), so the lists come out in position
// order and the placing kernel's writes are coalesced.  Per element the work
// is 32-bit: region bounds relative to the thread's first element, six list
// counters in 4-bit fields of one word.  List slots are reserved with one
// global atomic per list per chunk, and a chunk without misplaced elements
// skips that step.  The next chunk's keys are loaded before the current
// chunk's scan, so reads stay in flight across the chunk's barriers.
template <typename C, typename V>
__global__ void __launch_bounds__(256) sel_collect_kernel(SelArgs a)
{
    constexpr int IPT = sizeof(C) >= 4 ? 32 / (int)sizeof(C) : 8, CH = 256 * IPT;
    constexpr int NV = IPT * (int)sizeof(C) / 16;   // 16-byte vectors per thread
    __shared__ uint32_t s_w[8][3];
    __shared__ unsigned long long s_base[6];
    const C K = (C)a.st->prefix;
    const size_t cl = a.st->cl, ce = a.st->ce;
    const C *keys = static_cast<const C *>(a.keys);
    const V *vals = static_cast<const V *>(a.vals);
    C *mis_k = static_cast<C *>(a.mis_k);
    V *mis_v = static_cast<V *>(a.mis_v);
    const size_t n = a.n;
    const int tid = threadIdx.x;
    const size_t gstride = (size_t)gridDim.x * CH;
    const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15) == 0;
    C nxt[IPT];
    auto load_chunk = [&](size_t c0) {
        const size_t p0 = c0 + (size_t)tid * IPT;
        if (vec && p0 + IPT <= n) {
            uint4 q[NV];
            const uint4 *src = reinterpret_cast<const uint4 *>(keys + p0);
#pragma unroll
            for (int v = 0; v < NV; ++v) q[v] = src[v];
            memcpy(nxt, q, sizeof(nxt));
        } else {
#pragma unroll
            for (int j = 0; j < IPT; ++j) nxt[j] = p0 + j < n ? keys[p0 + j] : C(0);
        }
    };
    load_chunk((size_t)blockIdx.x * CH);
    for (size_t c0 = (size_t)blockIdx.x * CH; c0 < n; c0 += gstride) {
        C raw[IPT];
#pragma unroll
        for (int j = 0; j < IPT; ++j) raw[j] = nxt[j];
        if (c0 + gstride < n) load_chunk(c0 + gstride);
        const size_t p0 = c0 + (size_t)tid * IPT;
        // region boundaries relative to this thread's first element, clamped
        // to [0, IPT], so the per-element region test is 32-bit
        const uint32_t r1 = (uint32_t)(cl > p0 ? min(cl - p0, (size_t)IPT) : 0);
        const uint32_t r2 = (uint32_t)(cl + ce > p0 ? min(cl + ce - p0, (size_t)IPT) : 0);
        const uint32_t valid = (uint32_t)(n > p0 ? min(n - p0, (size_t)IPT) : 0);
        uint32_t tags = 0;                      // 4 bits per element: list class, hole region
        uint32_t cnt4 = 0;                      // 4-bit counters: lists 0..2, holes 0..2
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            uint32_t t = 0xF;
            if ((uint32_t)j < valid) {
                const C c = to_code(raw[j], a.xf);
                const uint32_t cls = (uint32_t)(c >= K) + (uint32_t)(c > K);
                const uint32_t reg = (uint32_t)((uint32_t)j >= r1) + (uint32_t)((uint32_t)j >= r2);
                if (a.op == SOP_ARG) a.out_idx[p0 + j] = p0 + j;
                if (cls != reg) {
                    const bool rec = a.op != SOP_KEYS || cls != 1;
                    t = (rec ? cls : 3u) | (reg << 2);
                    cnt4 += (rec ? (1u << (4 * cls)) : 0u) + (1u << (4 * (3 + reg)));
                }
            }
            tags |= t << (4 * j);
        }
        if (!__syncthreads_or(cnt4 != 0u)) continue;
        // two 16-bit counters per scanned word
        uint32_t w[3];
#pragma unroll
        for (int q = 0; q < 3; ++q)
            w[q] = ((cnt4 >> (8 * q)) & 0xFu) | (((cnt4 >> (8 * q + 4)) & 0xFu) << 16);
        uint32_t tot[3];
        sel_scan3(w, s_w, tot);
        if (tid < 6) {
            const uint32_t t = (tot[tid >> 1] >> ((tid & 1) * 16)) & 0xFFFFu;
            unsigned int *ctr = tid < 3 ? &a.st->nmis[tid] : &a.st->nhole[tid - 3];
            const size_t rs = (tid % 3) == 0 ? 0 : ((tid % 3) == 1 ? cl : cl + ce);
            // a list that would run past the array (never, with consistent
            // counts) is not written for this chunk
            const size_t at = rs + (t ? atomicAdd(ctr, t) : 0u);
            s_base[tid] = at + t <= n ? at : ~0ull;
        }
        __syncthreads();
        // this thread's first slot in each list: chunk base + exclusive prefix
        size_t slot[6];
        bool ok[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const unsigned long long b0 = s_base[q];
            ok[q] = b0 != ~0ull;
            slot[q] = b0 + ((w[q >> 1] >> ((q & 1) * 16)) & 0xFFFFu);
        }
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            const size_t p = p0 + j;
            const uint32_t X = (tags >> (4 * j)) & 3u, R = (tags >> (4 * j + 2)) & 3u;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (X == (uint32_t)q) {
                    if (ok[q]) {
                        const size_t at = slot[q];
                        if (a.op == SOP_ARG) {
                            reinterpret_cast<uint32_t *>(a.mis_v)[at] = (uint32_t)p;
                        } else {
                            mis_k[at] = raw[j];
                            if constexpr (!std::is_same<V, uint8_t>::value)
                                if (a.op == SOP_KV) mis_v[at] = vals[p];
                        }
                    }
                    ++slot[q];
                }
                if (R == (uint32_t)q) {
                    if (ok[3 + q]) a.holes[slot[3 + q]] = (uint32_t)p;
                    ++slot[3 + q];
                }
            }
        }
        __syncthreads();   // s_base is rewritten by the next chunk
    }
}

template <typename C, typename V>
__global__ void __launch_bounds__(256) sel_place_kernel(SelArgs a)
{
    const C K = (C)a.st->prefix;
    const size_t cl = a.st->cl, ce = a.st->ce;
    const size_t regstart[3] = {0, cl, cl + ce};
    C *keys = static_cast<C *>(a.keys);
    V *vals = static_cast<V *>(a.vals);
    const C *mis_k = static_cast<const C *>(a.mis_k);
    const V *mis_v = static_cast<const V *>(a.mis_v);
    const C kraw = from_code(K, a.xf);
    const size_t stride = (size_t)gridDim.x * 256;
    for (int X = 0; X < 3; ++X) {
        // counts are consistent by construction; clamp so a broken state can
        // never index past the lists
        const size_t cnt = min((size_t)a.st->nhole[X], a.n - regstart[X]);
        // four list entries per thread in flight
        constexpr int U = 4;
        for (size_t j0 = (size_t)blockIdx.x * 256 + threadIdx.x; j0 < cnt; j0 += U * stride) {
            uint32_t pos[U];
            C mk[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const size_t j = j0 + u * stride;
                pos[u] = j < cnt ? a.holes[regstart[X] + j] : 0xffffffffu;
                mk[u] = (j < cnt && a.op == SOP_KEYS && X != 1) ? mis_k[regstart[X] + j] : C(0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const size_t j = j0 + u * stride;
                if (j >= cnt || pos[u] >= a.n) continue;
                const size_t at = regstart[X] + j;
                if (a.op == SOP_ARG) {
                    a.out_idx[pos[u]] = reinterpret_cast<const uint32_t *>(a.mis_v)[at];
                } else if (a.op == SOP_KEYS) {
                    keys[pos[u]] = X == 1 ? kraw : mk[u];
                } else {
                    keys[pos[u]] = mis_k[at];
                    if constexpr (!std::is_same<V, uint8_t>::value)
                        if (a.op == SOP_KV) vals[pos[u]] = mis_v[at];
                }
            }
        }
    }
}

struct SelLayout {
    size_t st, cand, mis_k, mis_v, holes, total;
};

static SelLayout sel_layout(int op, int kbytes, int vbytes, size_t n)
{
    SelLayout L{};
    const int vb = op == SOP_ARG ? 4 : (op == SOP_KV ? vbytes : 0);
    size_t off = 0;
    L.st = off;    off = align_up(off + sizeof(SelState), 256);
    L.cand = off;  off = align_up(off + n * kbytes, 256);
    L.mis_k = off; if (op != SOP_ARG) off = align_up(off + n * kbytes, 256);
    L.mis_v = off; if (vb) off = align_up(off + n * vb, 256);
    L.holes = off; off = align_up(off + n * 4, 256);
    L.total = off;
    return L;
}

size_t select_workspace_bytes(int op, int kbytes, int vbytes, size_t n)
{
    if (n <= SMALL_SORT_MAX) return 0;
    return sel_layout(op, kbytes, vbytes, n).total;
}

template <typename C, typename V>
static int select_launch(int op, KeyXform xf, void *keys, void *vals, uint64_t *out_idx,
                         size_t k, size_t n, void *ws, size_t ws_bytes, cudaStream_t s)
{
    const int vbytes = std::is_same<V, uint8_t>::value ? 0 : (int)sizeof(V);
    const SelLayout L = sel_layout(op, sizeof(C), vbytes, n);
    if (ws == nullptr || ws_bytes < L.total) return XSS_ENOMEM;
    char *base = static_cast<char *>(ws);
    SelArgs a{};
    a.keys = keys;
    a.vals = vals;
    a.out_idx = out_idx;
    a.n = n;
    a.xf = xf;
    a.op = op;
    a.st = reinterpret_cast<SelState *>(base + L.st);
    a.cand = base + L.cand;
    a.mis_k = base + L.mis_k;
    a.mis_v = base + L.mis_v;
    a.holes = reinterpret_cast<uint32_t *>(base + L.holes);
    XSS_CUDA_TRY(cudaMemsetAsync(a.st, 0, sizeof(SelState), s));

    const int sms = num_sms();
    const int grid = (int)std::max<size_t>(1, std::min<size_t>((n + 2047) / 2048, (size_t)sms * 8));
    const int W = 8 * (int)sizeof(C);
    const int rounds = (W + SEL_DIGIT - 1) / SEL_DIGIT;
    for (int r = 0; r < rounds; ++r) {
        const int hi = W - SEL_DIGIT * r;
        const int lo = std::max(0, hi - SEL_DIGIT);
        const int bits = hi - lo;
        // rounds >= 2 scan only the compacted candidates; a smaller grid does
        const int g = r >= 2 ? std::max(1, grid / 4) : grid;
        XSS_LAUNCH(PK_SEL_HIST, s, sel_hist_kernel<C><<<g, 256, 0, s>>>(a, r, lo, bits));
        XSS_CUDA_TRY(cudaGetLastError());
        XSS_LAUNCH(PK_SEL_FIND, s,
                   sel_find_kernel<C><<<1, 1024, 0, s>>>(a, r, lo, bits, r == rounds - 1,
                                                         (unsigned long long)k));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    XSS_LAUNCH(PK_SEL_COLLECT, s, sel_collect_kernel<C, V><<<grid, 256, 0, s>>>(a));
    XSS_CUDA_TRY(cudaGetLastError());
    XSS_LAUNCH(PK_SEL_PLACE, s, sel_place_kernel<C, V><<<grid, 256, 0, s>>>(a));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

template <typename C>
static int select_c(int op, KeyXform xf, void *keys, void *vals, int vbytes,
                    uint64_t *out_idx, size_t k, size_t n, void *ws, size_t ws_bytes,
                    cudaStream_t s)
{
    if (op == SOP_KV && vbytes == 4)
        return select_launch<C, uint32_t>(op, xf, keys, vals, out_idx, k, n, ws, ws_bytes, s);
    if (op == SOP_KV && vbytes == 8)
        return select_launch<C, uint64_t>(op, xf, keys, vals, out_idx, k, n, ws, ws_bytes, s);
    return select_launch<C, uint8_t>(op, xf, keys, vals, out_idx, k, n, ws, ws_bytes, s);
}

int radix_select(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
                 uint64_t *out_idx, size_t k, size_t n, void *ws, size_t ws_bytes,
                 cudaStream_t s)
{
    if (n <= SMALL_SORT_MAX) {
        // a full sort satisfies the select contract
        return radix_sort(op, kbytes, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s);
    }
    if (n > XSS_MAX_N) return XSS_ETOOBIG;
    switch (kbytes) {
    case 2: return select_c<uint16_t>(op, xf, keys, vals, vbytes, out_idx, k, n, ws, ws_bytes, s);
    case 4: return select_c<uint32_t>(op, xf, keys, vals, vbytes, out_idx, k, n, ws, ws_bytes, s);
    case 8: return select_c<uint64_t>(op, xf, keys, vals, vbytes, out_idx, k, n, ws, ws_bytes, s);
    default: return XSS_EINVAL;
    }
}

}  // namespace xss
