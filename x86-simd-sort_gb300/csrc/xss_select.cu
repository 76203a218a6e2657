// xss_select.cu -- radix select and in-place partition.
//
// Replaces the reference's quickselect family:
//   src/xss-common-qsort.h:607-649, 712-762     (qselect_, xss_qselect, xss_partial_qsort)
//   src/xss-common-argsort.h:551-585, 694-731   (argselect_, xss_argselect)
//   src/xss-common-keyvaluesort.hpp:519-562, 655-738 (kvselect_, select/partial kv)
//
// Method: find the exact k-th code by histogramming 11-bit digits from the
// top.  Round 0 reads every key and picks the bucket B of the top digit that
// holds rank k: keys below B (class L) belong in [0, b_lo), keys of B in
// [b_lo, b_lo + b_n), keys above (G) after that.  One more read of every key
// (the split kernel) does three things at once: it compacts B's keys (with
// their values or positions) into a candidate list, histograms their next
// digit for round 1, and records every L or G element that lies outside its
// region in a per-class list and every L/G-region position holding a
// foreign element in a per-region hole list.  Later rounds read only the
// candidates.  With the exact k-th code K known, the candidates are written
// back into B's region partitioned around K, and a last kernel moves the
// listed L/G elements into the holes.  Only misplaced elements move, as in
// an in-place quickselect partition, and the array is read twice.  When k
// is far from both ends (about half of each side's keys misplaced) round 0's
// read also copies the array to scratch, and the split reads that copy and
// writes every key once into the array -- L to its front, G to its back
// (select_launch chooses).
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
    unsigned long long b_lo;   // keys whose top digit is below the round-0 bucket
    unsigned long long b_n;    // keys in the round-0 bucket (the candidates)
    unsigned int nmis[3];
    unsigned int nhole[3];
    unsigned int nbpart[3];    // candidates placed per class (< K, == K, > K)
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
    void *cand;            // candidate codes
    void *cand_p;          // candidate values (key-value) or positions (argselect)
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

// dst[i] = src[i] for i in [s, e) by every thread of the grid (global thread
// gtid of `stride`): 16-byte vectors, four per thread in flight, over the part
// of the range that starts on a 16-byte boundary in both arrays; single
// elements before and after it, and everywhere if the arrays' alignments differ.
template <typename T>
__device__ __forceinline__ void copy_range(T *dst, const T *src, size_t s, size_t e, size_t gtid,
                                           size_t stride)
{
    constexpr size_t VW = 16 / sizeof(T);
    constexpr int U = 4;
    if (s >= e) return;
    const bool al = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0;
    const size_t a0 = al ? std::min(e, (s + VW - 1) / VW * VW) : e;   // first vector element
    const size_t a1 = al ? std::max(a0, e / VW * VW) : e;             // end of the vectors
    for (size_t i = s + gtid; i < a0; i += stride) dst[i] = src[i];
    for (size_t i = a1 + gtid; i < e; i += stride) dst[i] = src[i];
    const uint4 *vs = reinterpret_cast<const uint4 *>(src);
    uint4 *vd = reinterpret_cast<uint4 *>(dst);
    const size_t j1 = a1 / VW;
    for (size_t j0 = a0 / VW + gtid; j0 < j1; j0 += U * stride) {
        uint4 q[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (j0 + u * stride < j1) q[u] = vs[j0 + u * stride];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (j0 + u * stride < j1) vd[j0 + u * stride] = q[u];
    }
}

// One histogram round over every key (round 0) or over the compacted
// candidates (rounds >= 2; round 1 is the split pass).  16-byte vector
// loads, four per thread in flight, keep enough bytes moving to cover memory
// latency; an unaligned array takes the scalar loop.  (Issuing each step's
// loads before the previous step's keys are counted, and interleaved copies
// of the bins, measured no faster.)  With `copy` set (round 0 of an
// out-of-place select) the same read also copies the keys into the scratch
// copy a.mis_k, and a key-value select's values (copy_vb bytes each) into
// a.mis_v: the split pass then reads the copy and writes the outer classes
// straight into the caller's arrays, so no copy-back pass is needed.
template <typename C>
__global__ void __launch_bounds__(256) sel_hist_kernel(SelArgs a, int round, int lo, int bits,
                                                       int from_keys, int copy = 0,
                                                       int copy_vb = 0)
{
    constexpr int VW = 16 / sizeof(C);   // keys per vector
    constexpr int U = 4;                 // vectors per thread in flight
    __shared__ uint32_t sh[SEL_BINS];
    const int nb = 1 << bits;
    for (int i = threadIdx.x; i < nb; i += 256) sh[i] = 0;
    __syncthreads();
    const C prefix = (C)a.st->prefix, mask = (C)a.st->mask;
    const Codec<C> cx(a.xf);
    const size_t count = from_keys ? a.n : (size_t)a.st->cand_n;
    const C *src = from_keys ? static_cast<const C *>(a.keys) : static_cast<const C *>(a.cand);
    const int lane = threadIdx.x & 31;
    const size_t stride = (size_t)gridDim.x * 256;
    const size_t wbase = (size_t)blockIdx.x * 256 + threadIdx.x - lane;   // warp's first thread

    auto visit = [&](C b, bool active) {
        C c = 0;
        if (active) c = from_keys ? cx.to(b) : b;
        const bool match = active && ((C)(c & mask) == prefix);
        if (match) atomicAdd(&sh[uint32_t(c >> lo) & (uint32_t)(nb - 1)], 1u);
    };

    C *dst = copy ? static_cast<C *>(a.mis_k) : nullptr;   // 256-byte aligned scratch
    size_t head = 0;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        const size_t nvec = count / VW;
        const uint4 *vsrc = reinterpret_cast<const uint4 *>(src);
        uint4 *vdst = reinterpret_cast<uint4 *>(dst);
        for (size_t v0 = wbase; v0 < nvec; v0 += U * stride) {
            uint4 w[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const size_t v = v0 + lane + u * stride;
                w[u] = v < nvec ? vsrc[v] : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const size_t v = v0 + lane + u * stride;
                const bool act = v < nvec;
                if (copy && act) vdst[v] = w[u];
                const C *e = reinterpret_cast<const C *>(&w[u]);
#pragma unroll
                for (int j = 0; j < VW; ++j) visit(e[j], act);
            }
        }
        head = nvec * VW;
    }
    for (size_t i0 = head + wbase; i0 < count; i0 += stride) {
        const size_t i = i0 + lane;
        const C b = i < count ? src[i] : C(0);
        if (copy && i < count) dst[i] = b;
        visit(b, i < count);
    }
    if (copy && a.op == SOP_KV && copy_vb) {
        const size_t gtid = (size_t)blockIdx.x * 256 + threadIdx.x;
        if (copy_vb == 2)
            copy_range<uint16_t>(static_cast<uint16_t *>(a.mis_v),
                                 static_cast<const uint16_t *>(a.vals), 0, count, gtid, stride);
        else if (copy_vb == 4)
            copy_range<uint32_t>(static_cast<uint32_t *>(a.mis_v),
                                 static_cast<const uint32_t *>(a.vals), 0, count, gtid, stride);
        else if (copy_vb == 8)
            copy_range<uint64_t>(static_cast<uint64_t *>(a.mis_v),
                                 static_cast<const uint64_t *>(a.vals), 0, count, gtid, stride);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += 256)
        if (sh[i]) atomicAdd(&a.st->hist[i], sh[i]);
}

// One CTA: locate the bin holding rank k_rem, extend the prefix, reset the
// histogram for the next round.
template <typename C>
__global__ void __launch_bounds__(1024) sel_find_kernel(SelArgs a, int round, int lo, int bits,
                                                        int last, int exact,
                                                        unsigned long long k0)
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
                if (round == 0) {
                    a.st->b_lo = a.st->cnt_less;
                    a.st->b_n = h;
                }
                if (last) {
                    a.st->cl = a.st->cnt_less;
                    a.st->ce = h;
                    if (exact) {        // the partition's middle class is the code K
                        a.st->b_lo = a.st->cnt_less;
                        a.st->b_n = h;
                    }
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

// Block-wide exclusive scan of NW 32-bit words per thread (each word packs
// two 16-bit counters that cannot overflow within one chunk); tot = block sums.
template <int NW>
__device__ __forceinline__ void sel_scan(uint32_t (&v)[NW], uint32_t (*s_w)[NW], uint32_t (&tot)[NW])
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x[NW];
#pragma unroll
    for (int q = 0; q < NW; ++q) x[q] = v[q];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x[q], o);
            if (lane >= o) x[q] += y;
        }
    }
    if (lane == 31)
        for (int q = 0; q < NW; ++q) s_w[warp][q] = x[q];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NW; ++q) {
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

// Keys per thread per chunk: 8 16-bit keys or 32 bytes of wider keys, read
// with 16-byte vector loads when the array is aligned.
template <typename C> struct SelChunk {
    static constexpr int IPT = sizeof(C) >= 4 ? 32 / (int)sizeof(C) : 8;
    static constexpr int NV = IPT * (int)sizeof(C) / 16;
    static constexpr int CH = 256 * IPT;
};

template <typename C>
__device__ __forceinline__ void sel_load_chunk(const C *keys, size_t n, size_t p0, bool vec,
                                               C (&out)[SelChunk<C>::IPT])
{
    constexpr int IPT = SelChunk<C>::IPT, NV = SelChunk<C>::NV;
    if (vec && p0 + IPT <= n) {
        uint4 q[NV];
        const uint4 *src = reinterpret_cast<const uint4 *>(keys + p0);
#pragma unroll
        for (int v = 0; v < NV; ++v) q[v] = src[v];
        memcpy(out, q, sizeof(out));
    } else {
#pragma unroll
        for (int j = 0; j < IPT; ++j) out[j] = p0 + j < n ? keys[p0 + j] : C(0);
    }
}

// The split pass (see the file comment).  Classes of an element by its code
// against the round-0 bucket B: 0 = L (below), 1 = B, 2 = G (above); regions
// of a position: 0 = [0, b_lo), 1 = [b_lo, b_hi), 2 = [b_hi, n).  An element
// whose class differs from its region's is listed (list X = its class) and
// its position is a hole of its region (hole list R).  With candidates
// (EXACT false), B's elements are compacted instead of listed and B's region
// is rewritten whole later, so neither list 1 nor hole list 1 is kept; with
// EXACT (B is the single code K, known exactly: the 16-bit path) every class
// is listed and the place pass moves all three.
//
// Each warp takes super-chunks of S chunks of 32 * IPT consecutive elements,
// IPT per thread (16-byte vector loads).  It classifies all S chunks first
// (a 4-bit tag per element kept in registers; a candidate is tagged as list
// 1, which the candidate form does not keep), and a warp with nothing to
// record in a super-chunk moves on after one vote.  Otherwise it scans its
// per-thread counts with shuffles and reserves every list's slots with one
// global atomic per list -- S chunks per reservation keep the contention on
// the few list counters low -- then reloads the chunks holding records
// (still in L2) and writes them, so lists are in position order within a
// super-chunk and no barrier is needed.  List X's slots start at its
// region's first position (the number of misplaced elements of a class is at
// most its region's size).  Keys-only exact partitions list no element equal
// to K: the place pass writes K into the holes of K's region instead.
template <typename C, typename V, bool EXACT>
__global__ void __launch_bounds__(256) sel_split_kernel(SelArgs a, int lo, int bits)
{
    constexpr int IPT = SelChunk<C>::IPT, WCH = 32 * IPT, S = 8;
    constexpr bool HAS_V = !std::is_same<V, uint8_t>::value;
    __shared__ uint32_t sh[EXACT ? 1 : SEL_BINS];
    const int tid = threadIdx.x, lane = tid & 31;
    const int nb = 1 << bits;
    if constexpr (!EXACT) {
        for (int i = tid; i < nb; i += 256) sh[i] = 0;
        __syncthreads();
    }
    const Codec<C> cx(a.xf);
    const C pre = (C)a.st->prefix, msk = (C)a.st->mask;
    const size_t b_lo = a.st->b_lo, b_hi = a.st->b_lo + a.st->b_n;
    const C *keys = static_cast<const C *>(a.keys);
    const V *vals = static_cast<const V *>(a.vals);
    C *mis_k = static_cast<C *>(a.mis_k);
    V *mis_v = static_cast<V *>(a.mis_v);
    C *cand = static_cast<C *>(a.cand);
    const size_t n = a.n;
    const size_t warps = (size_t)gridDim.x * 8;
    const size_t gw = (size_t)blockIdx.x * 8 + (tid >> 5);
    const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15) == 0;
    const bool keys_only_exact = EXACT && a.op == SOP_KEYS;
    for (size_t s0 = gw * (S * WCH); s0 < n; s0 += warps * (S * WCH)) {
        uint32_t tags[S];
        unsigned long long lists = 0, holes = 0;   // 16-bit fields per list / hole list
        uint32_t ncand = 0;
#pragma unroll
        for (int q = 0; q < S; ++q) {
            const size_t p0 = s0 + (size_t)q * WCH + (size_t)lane * IPT;
            tags[q] = 0xFFFFFFFFu;
            if (p0 >= n) continue;
            C raw[IPT];
            sel_load_chunk<C>(keys, n, p0, vec, raw);
            const uint32_t r1 = (uint32_t)(b_lo > p0 ? min(b_lo - p0, (size_t)IPT) : 0);
            const uint32_t r2 = (uint32_t)(b_hi > p0 ? min(b_hi - p0, (size_t)IPT) : 0);
            const uint32_t valid = (uint32_t)min(n - p0, (size_t)IPT);
            uint32_t t4 = 0;
#pragma unroll
            for (int j = 0; j < IPT; ++j) {
                uint32_t t = 0xF;
                if ((uint32_t)j < valid) {
                    const C c = cx.to(raw[j]);
                    const C top = EXACT ? c : (C)(c & msk);
                    const uint32_t cls = (uint32_t)(top >= pre) + (uint32_t)(top > pre);
                    const uint32_t reg = (uint32_t)((uint32_t)j >= r1) + (uint32_t)((uint32_t)j >= r2);
                    if (a.op == SOP_ARG && (EXACT || reg != 1)) a.out_idx[p0 + j] = p0 + j;
                    uint32_t X = 3u, R = 3u;
                    if (!EXACT && cls == 1) {
                        X = 1u;                  // candidate
                        ++ncand;
                        atomicAdd(&sh[uint32_t(c >> lo) & (uint32_t)(nb - 1)], 1u);
                    }
                    if (cls != reg) {
                        if (EXACT && !(keys_only_exact && cls == 1)) X = cls;
                        else if (!EXACT && cls != 1) X = cls;
                        if (EXACT || reg != 1) R = reg;
                    }
                    if (X != 3u && !(!EXACT && X == 1u)) lists += 1ull << (16 * X);
                    if (R != 3u) holes += 1ull << (16 * R);
                    t = X | (R << 2);
                }
                t4 |= t << (4 * j);
            }
            tags[q] = t4;
        }
        if (!__any_sync(0xffffffffu, (lists | holes | ncand) != 0ull)) continue;
        // warp-inclusive scans of the packed counts
        unsigned long long il = lists, ih = holes;
        uint32_t ic = ncand;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long yl = __shfl_up_sync(0xffffffffu, il, o);
            const unsigned long long yh = __shfl_up_sync(0xffffffffu, ih, o);
            const uint32_t yc = __shfl_up_sync(0xffffffffu, ic, o);
            if (lane >= o) {
                il += yl;
                ih += yh;
                ic += yc;
            }
        }
        // lane 31 holds the warp's totals: reserve slots, one atomic per list
        const unsigned long long tl = __shfl_sync(0xffffffffu, il, 31);
        const unsigned long long th = __shfl_sync(0xffffffffu, ih, 31);
        const uint32_t tc = __shfl_sync(0xffffffffu, ic, 31);
        size_t base = 0;
        if (lane < 7) {
            uint32_t t = 0;
            if (lane < 3) t = (uint32_t)(tl >> (16 * lane)) & 0xFFFFu;
            else if (lane < 6) t = (uint32_t)(th >> (16 * (lane - 3))) & 0xFFFFu;
            else t = tc;
            if (t) {
                const int q = lane < 3 ? lane : lane - 3;
                const size_t rs = q == 0 ? 0 : (q == 1 ? b_lo : b_hi);
                if (lane < 3) base = rs + atomicAdd(&a.st->nmis[q], t);
                else if (lane < 6) base = rs + atomicAdd(&a.st->nhole[q], t);
                else base = (size_t)atomicAdd(&a.st->cand_n, (unsigned long long)t);
                // a list that would run past its space (never, with consistent
                // counts) is not written for this super-chunk
                if (base + t > n) base = ~size_t(0);
            }
        }
        size_t slot[7];
        bool ok[7];
#pragma unroll
        for (int q = 0; q < 7; ++q) {
            const size_t b0 = __shfl_sync(0xffffffffu, base, q);
            ok[q] = b0 != ~size_t(0);
            const uint32_t excl = q < 3 ? (uint32_t)((il - lists) >> (16 * q)) & 0xFFFFu
                                : q < 6 ? (uint32_t)((ih - holes) >> (16 * (q - 3))) & 0xFFFFu
                                        : ic - ncand;
            slot[q] = b0 + excl;
        }
#pragma unroll 1
        for (int q = 0; q < S; ++q) {
            const uint32_t t4 = tags[q];
            // 0xF per element: nothing to record
            bool any = false;
#pragma unroll
            for (int j = 0; j < IPT; ++j) any |= ((t4 >> (4 * j)) & 0xFu) != 0xFu;
            if (!any) continue;
            const size_t p0 = s0 + (size_t)q * WCH + (size_t)lane * IPT;
            C raw[IPT];
            sel_load_chunk<C>(keys, n, p0, vec, raw);
#pragma unroll
            for (int j = 0; j < IPT; ++j) {
                const size_t p = p0 + j;
                const uint32_t X = (t4 >> (4 * j)) & 3u, R = (t4 >> (4 * j + 2)) & 3u;
                if (!EXACT && X == 1u) {           // candidate
                    if (ok[6]) {
                        const size_t at = slot[6];
                        cand[at] = cx.to(raw[j]);
                        if (a.op == SOP_ARG) {
                            static_cast<uint32_t *>(a.cand_p)[at] = (uint32_t)p;
                        } else if constexpr (HAS_V) {
                            if (a.op == SOP_KV) static_cast<V *>(a.cand_p)[at] = vals[p];
                        }
                    }
                    ++slot[6];
                } else if (X != 3u) {
#pragma unroll
                    for (int x = 0; x < 3; ++x) {
                        if (X != (uint32_t)x) continue;
                        if (ok[x]) {
                            const size_t at = slot[x];
                            if (a.op == SOP_ARG) {
                                reinterpret_cast<uint32_t *>(a.mis_v)[at] = (uint32_t)p;
                            } else {
                                mis_k[at] = raw[j];
                                if constexpr (HAS_V)
                                    if (a.op == SOP_KV) mis_v[at] = vals[p];
                            }
                        }
                        ++slot[x];
                    }
                }
                if (R != 3u) {
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        if (R != (uint32_t)r) continue;
                        if (ok[3 + r]) a.holes[slot[3 + r]] = (uint32_t)p;
                        ++slot[3 + r];
                    }
                }
            }
        }
    }
    if constexpr (!EXACT) {
        __syncthreads();
        for (int i = tid; i < nb; i += 256)
            if (sh[i]) atomicAdd(&a.st->hist[i], sh[i]);
    }
}

// Shape of the out-of-place split (below): CTAs of SPL_BLOCK threads, each
// lane loading 16-byte vectors of consecutive keys, SPL_SUB sub-steps per
// slot reservation.
constexpr int SPL_BLOCK = 256;
constexpr int SPL_WARPS = SPL_BLOCK / 32;
constexpr int SPL_SUB = 8;                                // sub-steps per reservation
template <typename C> struct SplShape {
    static constexpr int VEC = 16 / (int)sizeof(C);     // keys per 16-byte vector
    static constexpr int VECS = sizeof(C) == 8 ? 4 : 2;  // vectors per lane per sub-step
    static constexpr int E = VEC * VECS;                  // keys per lane per sub-step (8)
    static constexpr int WSUB = 32 * E;                   // keys per warp per sub-step
    static constexpr int SUB = SPL_WARPS * WSUB;          // keys per CTA per sub-step
    static constexpr int STEP = SPL_SUB * SUB;            // keys per reservation
};

template <typename C>
__device__ __forceinline__ void spl_load(const C *keys, uint32_t n, uint32_t w0, int lane,
                                         bool vec_ok, C (&raw)[SplShape<C>::E])
{
    using S = SplShape<C>;
#pragma unroll
    for (int v = 0; v < S::VECS; ++v) {
        const uint32_t p0 = w0 + ((uint32_t)v * 32 + (uint32_t)lane) * S::VEC;
        if (vec_ok && p0 + S::VEC <= n) {
            const uint4 q = *reinterpret_cast<const uint4 *>(keys + p0);
            memcpy(&raw[v * S::VEC], &q, 16);
        } else {
#pragma unroll
            for (int i = 0; i < S::VEC; ++i)
                raw[v * S::VEC + i] = p0 + i < n ? keys[p0 + i] : C(0);
        }
    }
}

// Sparse in-place split for k near either end of the array (32- and 64-bit
// keys): few keys need recording -- the candidates (class B), the L / G keys
// outside their regions and the holes they leave -- so each warp classifies
// a 16-byte vector row per lane with a few instructions per key and moves on
// unless some lane holds a key to record.  Only then does it vote the five
// output masks of each key slot and reserve slots with one global atomic per
// non-empty output (rare, so the counters see little contention).  Output
// layout as the tag split above (lists and holes start at their region's
// first position); argselect writes the identity of every position outside
// B's region.
// Identity positions of a full row (every lane's VEC consecutive keys) into
// the index output, 16 bytes per store where the output is 16-byte aligned.
template <typename C>
__device__ __forceinline__ void spl_iota(uint64_t *out, uint32_t w0, uint32_t lane0, bool vec)
{
    using S = SplShape<C>;
#pragma unroll
    for (int v = 0; v < S::VECS; ++v) {
        const uint32_t p = w0 + (uint32_t)v * (32 * S::VEC) + lane0;
        if (vec) {
#pragma unroll
            for (int i = 0; i < S::VEC; i += 2)
                *reinterpret_cast<ulonglong2 *>(out + p + i) = make_ulonglong2(p + i, p + i + 1);
        } else {
#pragma unroll
            for (int i = 0; i < S::VEC; ++i) out[p + i] = p + i;
        }
    }
}

template <typename C, typename V>
__global__ void __launch_bounds__(256) sel_split_sparse_kernel(SelArgs a, int lo, int bits)
{
    using S = SplShape<C>;
    constexpr int E = S::E, VEC = S::VEC;
    constexpr bool HAS_V = !std::is_same<V, uint8_t>::value;
    __shared__ uint32_t sh[SEL_BINS];
    const int tid = threadIdx.x, lane = tid & 31;
    const int nb = 1 << bits;
    for (int i = tid; i < nb; i += 256) sh[i] = 0;
    __syncthreads();
    const Codec<C> cx(a.xf);
    const C pre = (C)a.st->prefix, msk = (C)a.st->mask;
    const uint32_t n = (uint32_t)a.n;
    const uint32_t b_lo = (uint32_t)a.st->b_lo, b_hi = (uint32_t)(a.st->b_lo + a.st->b_n);
    const uint32_t rs[3] = {0u, b_lo, b_hi};
    const C *keys = static_cast<const C *>(a.keys);
    const V *vals = static_cast<const V *>(a.vals);
    C *mis_k = static_cast<C *>(a.mis_k);
    V *mis_v = static_cast<V *>(a.mis_v);
    C *cand = static_cast<C *>(a.cand);
    const bool vec_ok = (reinterpret_cast<uintptr_t>(keys) & 15) == 0;
    const uint32_t lt = (1u << lane) - 1u, bit = 1u << lane;
    const uint32_t lane0 = (uint32_t)lane * VEC;
    const uint32_t wstride = gridDim.x * 8u * (uint32_t)S::WSUB;
    const bool idx_vec = (reinterpret_cast<uintptr_t>(a.out_idx) & 15) == 0;
    for (uint32_t w0 = (blockIdx.x * 8u + (uint32_t)(tid >> 5)) * (uint32_t)S::WSUB; w0 < n;
         w0 += wstride) {
        C raw[E];
        spl_load<C>(keys, n, w0, lane, vec_ok, raw);
        const uint32_t wend = w0 + (uint32_t)S::WSUB;     // the warp's keys: [w0, wend)
        if (w0 >= b_hi && wend <= n) {
            // the whole row lies in region 2 (the common case for k near 0):
            // a key needs recording only if it is not of class G
            bool any2 = false;
#pragma unroll
            for (int e = 0; e < E; ++e) any2 |= (C)(cx.to(raw[e]) & msk) <= pre;
            if (a.op == SOP_ARG) spl_iota<C>(a.out_idx, w0, lane0, idx_vec);
            if (!__any_sync(0xffffffffu, any2)) continue;
        } else if (wend <= b_lo) {
            // the whole row lies in region 0 (k near n - 1): record non-L keys
            bool any0 = false;
#pragma unroll
            for (int e = 0; e < E; ++e) any0 |= (C)(cx.to(raw[e]) & msk) >= pre;
            if (a.op == SOP_ARG) spl_iota<C>(a.out_idx, w0, lane0, idx_vec);
            if (!__any_sync(0xffffffffu, any0)) continue;
        }
        uint32_t cls4 = 0, reg4 = 0;   // 2 bits per key slot
        bool any = false;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t p = w0 + (uint32_t)(e / VEC) * (32 * VEC) + lane0 + (e % VEC);
            const C top = (C)(cx.to(raw[e]) & msk);
            const uint32_t cls = (uint32_t)(top >= pre) + (uint32_t)(top > pre);
            const uint32_t reg = (uint32_t)(p >= b_lo) + (uint32_t)(p >= b_hi);
            cls4 |= cls << (2 * e);
            reg4 |= reg << (2 * e);
            if (p < n) {
                any |= cls != reg || cls == 1u;
                if (a.op == SOP_ARG && reg != 1u) a.out_idx[p] = p;
            }
        }
        if (!__any_sync(0xffffffffu, any)) continue;
#pragma unroll 1
        for (int e = 0; e < E; ++e) {
            const uint32_t p = w0 + (uint32_t)(e / VEC) * (32 * VEC) + lane0 + (e % VEC);
            const bool in = p < n;
            const uint32_t cls = (cls4 >> (2 * e)) & 3u, reg = (reg4 >> (2 * e)) & 3u;
            // outputs: 0 list L, 1 list G, 2 candidates, 3 holes of region 0, 4 of region 2
            uint32_t m[5];
            m[0] = __ballot_sync(0xffffffffu, in && cls == 0u && reg != 0u);
            m[1] = __ballot_sync(0xffffffffu, in && cls == 2u && reg != 2u);
            m[2] = __ballot_sync(0xffffffffu, in && cls == 1u);
            m[3] = __ballot_sync(0xffffffffu, in && reg == 0u && cls != 0u);
            m[4] = __ballot_sync(0xffffffffu, in && reg == 2u && cls != 2u);
            if ((m[0] | m[1] | m[2] | m[3] | m[4]) == 0u) continue;
            uint32_t base = 0;
            if (lane < 5) {
                const uint32_t c = __popc(lane == 0 ? m[0] : lane == 1 ? m[1] : lane == 2 ? m[2] : lane == 3 ? m[3] : m[4]);
                if (c) {
                    if (lane == 2) base = (uint32_t)atomicAdd(&a.st->cand_n, (unsigned long long)c);
                    else if (lane < 2) base = rs[lane == 0 ? 0 : 2] + atomicAdd(&a.st->nmis[lane == 0 ? 0 : 2], c);
                    else base = rs[lane == 3 ? 0 : 2] + atomicAdd(&a.st->nhole[lane == 3 ? 0 : 2], c);
                }
            }
            uint32_t b[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) b[q] = __shfl_sync(0xffffffffu, base, q);
            if (!in) continue;
            if (m[2] & bit) {
                const C c = cx.to(raw[e]);
                atomicAdd(&sh[uint32_t(c >> lo) & (uint32_t)(nb - 1)], 1u);
                const uint32_t at = b[2] + __popc(m[2] & lt);
                if (at < n) {
                    cand[at] = c;
                    if (a.op == SOP_ARG) static_cast<uint32_t *>(a.cand_p)[at] = p;
                    else if constexpr (HAS_V)
                        if (a.op == SOP_KV) static_cast<V *>(a.cand_p)[at] = vals[p];
                }
            }
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                if (m[x] & bit) {
                    const uint32_t at = b[x] + __popc(m[x] & lt);
                    if (at < n) {
                        if (a.op == SOP_ARG) {
                            reinterpret_cast<uint32_t *>(a.mis_v)[at] = p;
                        } else {
                            mis_k[at] = raw[e];
                            if constexpr (HAS_V)
                                if (a.op == SOP_KV) mis_v[at] = vals[p];
                        }
                    }
                }
                if (m[3 + x] & bit) {
                    const uint32_t at = b[3 + x] + __popc(m[3 + x] & lt);
                    if (at < n) a.holes[at] = p;
                }
            }
        }
    }
    __syncthreads();
    for (int i = tid; i < nb; i += 256)
        if (sh[i]) atomicAdd(&a.st->hist[i], sh[i]);
}

// Out-of-place three-way split for 32- and 64-bit keys.  Round 0's histogram
// read left a scratch copy of the keys (and of a key-value select's values);
// this pass reads the copy and writes every key of class L to the front of
// the caller's array ([0, b_lo)) and every key of class G to its back
// ([b_hi, n)); B's keys become candidates (codes, with values or positions).
// Argselect leaves the array alone: it reads the array itself and writes the
// positions of L and G straight into its output.  For each key slot the warp
// votes two masks (class L, class G; class B is the rest); a CTA votes
// SPL_SUB sub-steps (masks kept in shared memory), adds its warps' counts and
// reserves each output's slots with one global atomic per output, then
// reloads the keys (from L2) and writes each once, slot = warp base + the
// warp's count of that class before the key slot (stored with the masks) +
// rank among the lanes of the vote.  No hole lists are kept, and nothing is
// copied back.
// The values of the keys spl_load read (same key slots), with vector loads
// where the value array is aligned to a row of VEC values.
template <typename C, typename V>
__device__ __forceinline__ void spl_load_vals(const V *vals, uint32_t n, uint32_t w0, int lane,
                                              bool vec_ok, V (&out)[SplShape<C>::E])
{
    using S = SplShape<C>;
    constexpr int VB = S::VEC * (int)sizeof(V);   // bytes of one row: 4 .. 32
#pragma unroll
    for (int v = 0; v < S::VECS; ++v) {
        const uint32_t p0 = w0 + ((uint32_t)v * 32 + (uint32_t)lane) * S::VEC;
        if (vec_ok && p0 + S::VEC <= n && VB >= 4) {
            if constexpr (VB == 32) {
                const uint4 *q = reinterpret_cast<const uint4 *>(vals + p0);
                const uint4 x = q[0], y = q[1];
                memcpy(&out[v * S::VEC], &x, 16);
                memcpy(reinterpret_cast<char *>(&out[v * S::VEC]) + 16, &y, 16);
            } else if constexpr (VB == 16) {
                const uint4 x = *reinterpret_cast<const uint4 *>(vals + p0);
                memcpy(&out[v * S::VEC], &x, 16);
            } else if constexpr (VB == 8) {
                const uint2 x = *reinterpret_cast<const uint2 *>(vals + p0);
                memcpy(&out[v * S::VEC], &x, 8);
            } else {
                const uint32_t x = *reinterpret_cast<const uint32_t *>(vals + p0);
                memcpy(&out[v * S::VEC], &x, 4);
            }
        } else {
#pragma unroll
            for (int i = 0; i < S::VEC; ++i)
                out[v * S::VEC + i] = p0 + i < n ? vals[p0 + i] : V(0);
        }
    }
}

template <typename C, typename V>
__global__ void __launch_bounds__(SPL_BLOCK, 2) sel_split3_kernel(SelArgs a, int lo, int bits)
{
    using S = SplShape<C>;
    constexpr int E = S::E, VEC = S::VEC;
    constexpr bool HAS_V = !std::is_same<V, uint8_t>::value;
    __shared__ uint32_t sh[SEL_BINS];
    // per key slot of a warp: class L mask, class G mask, and the warp's L and G
    // counts before the slot within the step (16 bits each: a warp's step holds
    // SPL_SUB * WSUB = 2048 keys)
    __shared__ uint4 s_ent[SPL_SUB][SPL_WARPS][E];
    __shared__ uint32_t s_cnt[SPL_WARPS][3];
    __shared__ uint32_t s_base[SPL_WARPS][3];
    static_assert(SPL_SUB * S::WSUB < 65536, "step counts must fit 16 bits");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb = 1 << bits;
    for (int i = tid; i < nb; i += SPL_BLOCK) sh[i] = 0;
    __syncthreads();
    const Codec<C> cx(a.xf);
    const C pre = (C)a.st->prefix, msk = (C)a.st->mask;
    // positions and slots fit 32 bits: selects above XSS_RADIX_MAX_N keys sort
    const uint32_t n = (uint32_t)a.n;
    const uint32_t b_hi = (uint32_t)(a.st->b_lo + a.st->b_n);
    // read the scratch copy (argselect: the array), write the array
    const C *keys = a.op == SOP_ARG ? static_cast<const C *>(a.keys)
                                    : static_cast<const C *>(a.mis_k);
    const V *vals = static_cast<const V *>(a.mis_v);
    C *out_k = static_cast<C *>(a.keys);
    V *out_v = static_cast<V *>(a.vals);
    C *cand = static_cast<C *>(a.cand);
    uint32_t *cand_pos = static_cast<uint32_t *>(a.cand_p);
    V *cand_val = static_cast<V *>(a.cand_p);
    const bool vec_ok = (reinterpret_cast<uintptr_t>(keys) & 15) == 0;
    const bool vals_vec = HAS_V && vals != nullptr &&
                          (reinterpret_cast<uintptr_t>(vals) % (VEC * sizeof(V))) == 0;
    const uint32_t lt = (1u << lane) - 1u, bit = 1u << lane;
    const uint32_t lane0 = (uint32_t)lane * VEC;   // lane's first key in a vector row
    for (uint32_t s0 = blockIdx.x * (uint32_t)S::STEP; s0 < n; s0 += gridDim.x * (uint32_t)S::STEP) {
        uint32_t tL = 0, tG = 0, tIn = 0;   // the warp's L, G and in-range keys so far
        C raw[E], nxt[E];
        spl_load<C>(keys, n, s0 + (uint32_t)warp * S::WSUB, lane, vec_ok, nxt);
#pragma unroll 1
        for (int sub = 0; sub < SPL_SUB; ++sub) {
            const uint32_t w0 = s0 + (uint32_t)sub * S::SUB + (uint32_t)warp * S::WSUB;
#pragma unroll
            for (int e = 0; e < E; ++e) raw[e] = nxt[e];
            if (sub + 1 < SPL_SUB) spl_load<C>(keys, n, w0 + S::SUB, lane, vec_ok, nxt);
            const bool full = w0 + (uint32_t)S::WSUB <= n;   // uniform across the warp
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const uint32_t p = w0 + (uint32_t)(e / VEC) * (32 * VEC) + lane0 + (e % VEC);
                const bool in = full || p < n;
                const C c = cx.to(raw[e]);
                const C top = (C)(c & msk);
                const bool isL = in && top < pre, isG = in && top > pre;
                const uint32_t mL = __ballot_sync(0xffffffffu, isL);
                const uint32_t mG = __ballot_sync(0xffffffffu, isG);
                const uint32_t mIn = full ? 0xffffffffu : __ballot_sync(0xffffffffu, in);
                if (lane == 0) s_ent[sub][warp][e] = make_uint4(mL, mG, tL | (tG << 16), 0u);
                if ((mL | mG) != mIn) {   // uniform: some lane holds a class-B key
                    if (in && !isL && !isG)
                        atomicAdd(&sh[uint32_t(c >> lo) & (uint32_t)(nb - 1)], 1u);
                }
                tL += __popc(mL);
                tG += __popc(mG);
                tIn += full ? 32u : __popc(mIn);
            }
        }
        if (lane < 3) s_cnt[warp][lane] = lane == 0 ? tL : (lane == 1 ? tG : tIn - tL - tG);
        __syncthreads();
        if (tid < 3) {
            uint32_t sum = 0;
            for (int w = 0; w < SPL_WARPS; ++w) sum += s_cnt[w][tid];
            uint32_t b = 0;
            if (sum) {
                if (tid == 2) b = (uint32_t)atomicAdd(&a.st->cand_n, (unsigned long long)sum);
                else b = atomicAdd(&a.st->nmis[tid == 0 ? 0 : 2], sum);
            }
            if (tid == 1) b += b_hi;
            for (int w = 0; w < SPL_WARPS; ++w) {
                s_base[w][tid] = b;
                b += s_cnt[w][tid];
            }
        }
        __syncthreads();
        const uint32_t bL = s_base[warp][0], bG = s_base[warp][1], bC = s_base[warp][2];
        uint32_t inBefore = 0;   // the warp's in-range keys of the step before this slot
#pragma unroll 1
        for (int sub = 0; sub < SPL_SUB; ++sub) {
            const uint32_t w0 = s0 + (uint32_t)sub * S::SUB + (uint32_t)warp * S::WSUB;
            if (w0 >= n) break;
            spl_load<C>(keys, n, w0, lane, vec_ok, raw);
            V vv[E];
            if constexpr (HAS_V)
                if (a.op == SOP_KV) spl_load_vals<C, V>(vals, n, w0, lane, vals_vec, vv);
            const bool full = w0 + (uint32_t)S::WSUB <= n;   // uniform across the warp
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const uint32_t p = w0 + (uint32_t)(e / VEC) * (32 * VEC) + lane0 + (e % VEC);
                const uint32_t act = full ? 0xffffffffu : __ballot_sync(0xffffffffu, p < n);
                const uint4 ent = s_ent[sub][warp][e];
                const uint32_t mL = ent.x, mG = ent.y;
                const uint32_t pL = ent.z & 0xFFFFu, pG = ent.z >> 16;
                const uint32_t mC = act & ~(mL | mG);
                // this key's class mask and slot; one store path per output kind
                const bool inL = mL & bit, inG = mG & bit;
                const uint32_t m = inL ? mL : (inG ? mG : mC);
                const uint32_t at = (inL ? bL + pL : (inG ? bG + pG : bC + inBefore - pL - pG)) +
                                    __popc(m & lt);
                inBefore += full ? 32u : __popc(act);
                if ((act & bit) && at < n) {
                    if (!inL && !inG) {
                        cand[at] = cx.to(raw[e]);
                        if (a.op == SOP_ARG) cand_pos[at] = p;
                        else if constexpr (HAS_V)
                            if (a.op == SOP_KV) cand_val[at] = vv[e];
                    } else if (a.op == SOP_ARG) {
                        a.out_idx[at] = p;
                    } else {
                        out_k[at] = raw[e];
                        if constexpr (HAS_V)
                            if (a.op == SOP_KV) out_v[at] = vv[e];
                    }
                }
            }
        }
        __syncthreads();   // s_ent / s_cnt / s_base are rewritten by the next step
    }
    __syncthreads();
    for (int i = tid; i < nb; i += SPL_BLOCK)
        if (sh[i]) atomicAdd(&a.st->hist[i], sh[i]);
}

// B's region rewritten from the candidates, partitioned around K:
// [b_lo, cl) < K, [cl, cl + ce) == K, [cl + ce, b_lo + b_n) > K.  Same chunk
// and slot reservation scheme as the split pass, over the candidate list.
template <typename C, typename V>
__global__ void __launch_bounds__(256) sel_bpart_kernel(SelArgs a)
{
    constexpr int IPT = SelChunk<C>::IPT, CH = SelChunk<C>::CH;
    __shared__ uint32_t s_w[8][2];
    __shared__ unsigned long long s_base[3];
    const int tid = threadIdx.x;
    const C K = (C)a.st->prefix;
    const size_t cl = a.st->cl, ce = a.st->ce;
    const size_t b_lo = a.st->b_lo, b_n = a.st->b_n;
    const size_t m = min((size_t)a.st->cand_n, b_n);
    const size_t rstart[3] = {b_lo, cl, cl + ce};
    const size_t rend[3] = {cl, cl + ce, b_lo + b_n};
    const C *cand = static_cast<const C *>(a.cand);
    C *keys = static_cast<C *>(a.keys);
    V *vals = static_cast<V *>(a.vals);
    for (size_t c0 = (size_t)blockIdx.x * CH; c0 < m; c0 += (size_t)gridDim.x * CH) {
        const size_t p0 = c0 + (size_t)tid * IPT;
        const uint32_t valid = (uint32_t)(m > p0 ? min(m - p0, (size_t)IPT) : 0);
        C cc[IPT];
        uint32_t cls4 = 0, cnt4 = 0;
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            cc[j] = (uint32_t)j < valid ? cand[p0 + j] : C(0);
            const uint32_t cls = (uint32_t)(cc[j] >= K) + (uint32_t)(cc[j] > K);
            if ((uint32_t)j < valid) {
                cls4 |= cls << (2 * j);
                cnt4 += 1u << (4 * cls);
            }
        }
        uint32_t w[2] = {(cnt4 & 0xFu) | (((cnt4 >> 4) & 0xFu) << 16), (cnt4 >> 8) & 0xFu};
        uint32_t tot[2];
        sel_scan<2>(w, s_w, tot);
        if (tid < 3) {
            const uint32_t t = tid < 2 ? (tot[0] >> (16 * tid)) & 0xFFFFu : tot[1];
            const size_t at = rstart[tid] + (t ? atomicAdd(&a.st->nbpart[tid], t) : 0u);
            s_base[tid] = at + t <= rend[tid] ? at : ~0ull;
        }
        __syncthreads();
        size_t slot[3];
        bool ok[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            ok[q] = s_base[q] != ~0ull;
            slot[q] = s_base[q] + (q < 2 ? (w[0] >> (16 * q)) & 0xFFFFu : w[1]);
        }
#pragma unroll
        for (int j = 0; j < IPT; ++j) {
            if ((uint32_t)j >= valid) continue;
            const uint32_t cls = (cls4 >> (2 * j)) & 3u;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (cls == (uint32_t)q) {
                    if (ok[q] && slot[q] < a.n) {
                        const size_t at = slot[q];
                        if (a.op == SOP_ARG) {
                            a.out_idx[at] = static_cast<const uint32_t *>(a.cand_p)[p0 + j];
                        } else {
                            keys[at] = from_code(cc[j], a.xf);
                            if constexpr (!std::is_same<V, uint8_t>::value)
                                if (a.op == SOP_KV) vals[at] = static_cast<const V *>(a.cand_p)[p0 + j];
                        }
                    }
                    ++slot[q];
                }
            }
        }
        __syncthreads();   // s_base is rewritten by the next chunk
    }
}

// Listed L / G elements into the holes of their regions.
template <typename C, typename V>
__global__ void __launch_bounds__(256) sel_place_kernel(SelArgs a, int exact)
{
    const size_t b_hi = a.st->b_lo + a.st->b_n;
    C *keys = static_cast<C *>(a.keys);
    V *vals = static_cast<V *>(a.vals);
    const C *mis_k = static_cast<const C *>(a.mis_k);
    const V *mis_v = static_cast<const V *>(a.mis_v);
    const size_t stride = (size_t)gridDim.x * 256;
    // keys-only exact partitions list no element equal to K: its region's
    // holes get K itself
    const C kval = from_code((C)a.st->prefix, a.xf);
    const bool fill_k = exact && a.op == SOP_KEYS;
    for (int X = 0; X < 3; X += exact ? 1 : 2) {
        const size_t rs = X == 0 ? 0 : (X == 1 ? a.st->b_lo : b_hi);
        // counts are consistent by construction; clamp so a broken state can
        // never index past the lists
        const size_t cnt = min((size_t)a.st->nhole[X], a.n - min(rs, a.n));
        // four list entries per thread in flight
        constexpr int U = 4;
        for (size_t j0 = (size_t)blockIdx.x * 256 + threadIdx.x; j0 < cnt; j0 += U * stride) {
            uint32_t pos[U];
            C mk[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const size_t j = j0 + u * stride;
                pos[u] = j < cnt ? a.holes[rs + j] : 0xffffffffu;
                mk[u] = (j < cnt && a.op != SOP_ARG) ? (X == 1 && fill_k ? kval : mis_k[rs + j])
                                                      : C(0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const size_t j = j0 + u * stride;
                if (j >= cnt || pos[u] >= a.n) continue;
                const size_t at = rs + j;
                if (a.op == SOP_ARG) {
                    a.out_idx[pos[u]] = reinterpret_cast<const uint32_t *>(a.mis_v)[at];
                } else {
                    keys[pos[u]] = mk[u];
                    if constexpr (!std::is_same<V, uint8_t>::value)
                        if (a.op == SOP_KV) vals[pos[u]] = mis_v[at];
                }
            }
        }
    }
}

struct SelLayout {
    size_t st, cand, cand_p, mis_k, mis_v, holes, total;
};

static SelLayout sel_layout(int op, int kbytes, int vbytes, size_t n)
{
    SelLayout L{};
    const int vb = op == SOP_ARG ? 4 : (op == SOP_KV ? vbytes : 0);
    size_t off = 0;
    L.st = off;    off = align_up(off + sizeof(SelState), 256);
    L.cand = off;  off = align_up(off + n * kbytes, 256);
    L.cand_p = off; if (vb) off = align_up(off + n * vb, 256);
    L.mis_k = off; if (op != SOP_ARG) off = align_up(off + n * kbytes, 256);
    L.mis_v = off; if (vb) off = align_up(off + n * vb, 256);
    L.holes = off; off = align_up(off + n * 4, 256);
    L.total = off;
    return L;
}

size_t select_workspace_bytes(int op, int kbytes, int vbytes, size_t n)
{
    if (n <= SMALL_SORT_MAX) return 0;
    if (count16_wanted(op, kbytes, n)) return count16_workspace_bytes(n);
    // beyond one radix sort's size the select is a full (chunked) sort
    if (big_sort_needed(n)) return radix_workspace_bytes(op, kbytes, vbytes, n);
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
    a.cand_p = base + L.cand_p;
    a.mis_k = base + L.mis_k;
    a.mis_v = base + L.mis_v;
    a.holes = reinterpret_cast<uint32_t *>(base + L.holes);
    XSS_CUDA_TRY(cudaMemsetAsync(a.st, 0, sizeof(SelState), s));

    const int sms = num_sms();
    const int grid = (int)std::max<size_t>(1, std::min<size_t>((n + 2047) / 2048, (size_t)sms * 8));
    const unsigned long long kk = (unsigned long long)k;
    if constexpr (sizeof(C) == 2) {
        // 16-bit keys: two 8-bit histogram reads of the keys give the exact
        // k-th code K; one pass lists every element outside its class's
        // region (< K, == K, > K) and the place pass moves all three classes
        for (int r = 0; r < 2; ++r) {
            const int lo = r == 0 ? 8 : 0;
            XSS_LAUNCH(PK_SEL_HIST, s, sel_hist_kernel<C><<<grid, 256, 0, s>>>(a, r, lo, 8, 1));
            XSS_CUDA_TRY(cudaGetLastError());
            XSS_LAUNCH(PK_SEL_FIND, s,
                       sel_find_kernel<C><<<1, 1024, 0, s>>>(a, r, lo, 8, r == 1, 1, kk));
            XSS_CUDA_TRY(cudaGetLastError());
        }
        XSS_LAUNCH(PK_SEL_COLLECT, s, (sel_split_kernel<C, V, true><<<grid, 256, 0, s>>>(a, 0, 0)));
        XSS_CUDA_TRY(cudaGetLastError());
        XSS_LAUNCH(PK_SEL_PLACE, s, (sel_place_kernel<C, V><<<grid, 256, 0, s>>>(a, 1)));
        XSS_CUDA_TRY(cudaGetLastError());
        return XSS_OK;
    }
    const int W = 8 * (int)sizeof(C);
    const int rounds = (W + SEL_DIGIT - 1) / SEL_DIGIT;   // 3 (32-bit) or 6 (64-bit)
    // Where k is not near either end, a good share of the keys on each side
    // of the bucket lie in the other side's region: copying the array to
    // scratch during round 0's read and writing every key once from the copy
    // costs less than listing and moving the misplaced ones (qselect float32
    // 2^27, k = 2^26: 0.60 ms; 0.76 against 1.38 ms with a copy-back of the
    // outer regions after the split, which the copy during round 0 replaced).
    // Within n / 4096 of an end only a few keys are recorded, and the sparse
    // in-place split reads the array at little more than memory speed.
    const bool out_of_place = std::min(k, n - 1 - k) >= n / 4096;
    for (int r = 0; r < rounds; ++r) {
        const int hi = W - SEL_DIGIT * r;
        const int lo = std::max(0, hi - SEL_DIGIT);
        const int bits = hi - lo;
        if (r == 1 && out_of_place) {
            // one read of every key: candidates and their next-digit
            // histogram; L and G keys to the scratch copy's front and back
            const int sg = (int)std::max<size_t>(
                1, std::min<size_t>((n + SplShape<C>::STEP - 1) / SplShape<C>::STEP,
                                    (size_t)sms * 4));
            XSS_LAUNCH(PK_SEL_COLLECT, s,
                       (sel_split3_kernel<C, V><<<sg, SPL_BLOCK, 0, s>>>(a, lo, bits)));
        } else if (r == 1) {
            // one read of every key: candidates, their next-digit histogram,
            // and the lists and holes of the few misplaced L / G keys
            const int sg = (int)std::max<size_t>(
                1, std::min<size_t>((n + 8 * SplShape<C>::WSUB - 1) / (8 * SplShape<C>::WSUB),
                                    (size_t)sms * 8));
            XSS_LAUNCH(PK_SEL_COLLECT, s,
                       (sel_split_sparse_kernel<C, V><<<sg, 256, 0, s>>>(a, lo, bits)));
        } else {
            // round 0 reads every key (and, out of place, copies the keys and
            // a key-value select's values to the scratch copy the split pass
            // reads); later rounds read only the candidates
            const int g = r >= 2 ? std::max(1, grid / 4) : grid;
            const int copy = r == 0 && out_of_place && op != SOP_ARG;
            XSS_LAUNCH(PK_SEL_HIST, s,
                       sel_hist_kernel<C><<<g, 256, 0, s>>>(a, r, lo, bits, r == 0 ? 1 : 0,
                                                            copy, op == SOP_KV ? vbytes : 0));
        }
        XSS_CUDA_TRY(cudaGetLastError());
        XSS_LAUNCH(PK_SEL_FIND, s,
                   sel_find_kernel<C><<<1, 1024, 0, s>>>(a, r, lo, bits, r == rounds - 1, 0, kk));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    XSS_LAUNCH(PK_SEL_PLACE, s, (sel_bpart_kernel<C, V><<<grid, 256, 0, s>>>(a)));
    XSS_CUDA_TRY(cudaGetLastError());
    if (!out_of_place) {
        XSS_LAUNCH(PK_SEL_PLACE, s, (sel_place_kernel<C, V><<<grid, 256, 0, s>>>(a, 0)));
        XSS_CUDA_TRY(cudaGetLastError());
    }
    return XSS_OK;
}

template <typename C>
static int select_c(int op, KeyXform xf, void *keys, void *vals, int vbytes,
                    uint64_t *out_idx, size_t k, size_t n, void *ws, size_t ws_bytes,
                    cudaStream_t s)
{
    if (op == SOP_KV && vbytes == 2)
        return select_launch<C, uint16_t>(op, xf, keys, vals, out_idx, k, n, ws, ws_bytes, s);
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
    if (n <= SMALL_SORT_MAX || big_sort_needed(n)) {
        // a full sort satisfies the select contract (small inputs, and arrays
        // beyond one radix sort's size, which the chunked sort takes)
        return radix_sort(op, kbytes, xf, keys, vals, vbytes, out_idx, n, ws, ws_bytes, s);
    }
    // 16-bit keys only: a full sort by counting (two memory passes) satisfies
    // the select contract and costs less than the partition
    if (count16_wanted(op, kbytes, n)) return count16_sort(xf, keys, n, 0, ws, ws_bytes, s);
    switch (kbytes) {
    case 2: return select_c<uint16_t>(op, xf, keys, vals, vbytes, out_idx, k, n, ws, ws_bytes, s);
    case 4: return select_c<uint32_t>(op, xf, keys, vals, vbytes, out_idx, k, n, ws, ws_bytes, s);
    case 8: return select_c<uint64_t>(op, xf, keys, vals, vbytes, out_idx, k, n, ws, ws_bytes, s);
    default: return XSS_EINVAL;
    }
}

}  // namespace xss
