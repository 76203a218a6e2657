// xss_merge.cu -- sorts of arrays larger than one radix sort takes.
//
// The onesweep radix sort handles up to XSS_RADIX_MAX_N keys (its look-back
// words hold a 30-bit count and its tile arithmetic is 32-bit).  Larger
// arrays -- the reference takes any size_t length (lib/x86simdsort.h:16-18,
// src/xss-common-qsort.h:652-710) -- are cut into chunks of at most that many
// keys, each chunk is radix-sorted where it lies, and the sorted chunks are
// merged pairwise (merge path: every CTA finds where its slice of the output
// starts in both inputs by a binary search on the cross diagonal, then merges
// its slice in shared memory).  The merge compares order-preserving codes, so
// descending order and NaN placement follow the chunks' own sort; it is
// stable (the left run wins ties), so key-value and index outputs are the
// stable order of the whole array.  argsort sorts (key copy, 64-bit position)
// pairs and writes only the positions of the last merge.
#include <algorithm>
#include <cstdlib>
#include <type_traits>
#include "xss_internal.cuh"

namespace xss {

constexpr int MERGE_BLOCK = 256;
// Output elements per CTA: the slice's codes in and out plus a 16-bit source
// index each stay within 48 KiB of static shared memory.
template <typename C> constexpr int merge_ipt() { return sizeof(C) == 8 ? 8 : 16; }
template <typename C> constexpr int merge_tile() { return MERGE_BLOCK * merge_ipt<C>(); }

template <typename C> struct MergeArgs {
    const C *a, *b;          // sorted runs (original key bits)
    const void *av, *bv;     // their values (or null)
    C *out_k;                // merged keys (null: keys not written)
    void *out_v;             // merged values (or null)
    size_t na, nb;
    const size_t *split;     // co-rank in a of every tile boundary (tiles + 1)
    KeyXform xf;
    size_t tile0;            // first output tile of this launch (sliced merges)
};

// Smallest i in [max(0, k - nb), min(k, na)] such that the first k outputs of
// the stable merge are a[0, i) and b[0, k - i): a[i] goes before b[j - 1]
// exactly when code(a[i]) <= code(b[j - 1]).
template <typename C, typename GetA, typename GetB>
__device__ __forceinline__ size_t co_rank(size_t k, size_t na, size_t nb, GetA ga, GetB gb)
{
    size_t lo = k > nb ? k - nb : 0, hi = k < na ? k : na;
    while (lo < hi) {
        const size_t i = lo + (hi - lo) / 2, j = k - i;
        if (j > 0 && ga(i) <= gb(j - 1)) lo = i + 1;
        else hi = i;
    }
    return lo;
}

template <typename C>
__global__ void merge_split_kernel(MergeArgs<C> m, size_t *split, size_t tiles)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t > tiles) return;
    const size_t total = m.na + m.nb;
    const size_t k = std::min(t * (size_t)merge_tile<C>(), total);
    const KeyXform xf = m.xf;
    split[t] = co_rank<C>(k, m.na, m.nb,
                          [&](size_t i) { return to_code(m.a[i], xf); },
                          [&](size_t j) { return to_code(m.b[j], xf); });
}

template <typename C, typename V>
__global__ void __launch_bounds__(MERGE_BLOCK) merge_kernel(MergeArgs<C> m)
{
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    constexpr int TILE = merge_tile<C>(), IPT = merge_ipt<C>();
    __shared__ C s_in[TILE];      // a's slice, then b's slice (codes)
    __shared__ C s_out[TILE];     // merged codes
    __shared__ uint16_t s_src[TILE];
    const size_t total = m.na + m.nb;
    const size_t tile = m.tile0 + blockIdx.x;
    const size_t o0 = tile * TILE;
    const size_t o1 = std::min(o0 + (size_t)TILE, total);
    const size_t i0 = m.split[tile], i1 = m.split[tile + 1];
    const size_t j0 = o0 - i0, j1 = o1 - i1;
    const int la = (int)(i1 - i0), lb = (int)(j1 - j0), len = (int)(o1 - o0);
    const KeyXform xf = m.xf;
    for (int q = threadIdx.x; q < la; q += MERGE_BLOCK) s_in[q] = to_code(m.a[i0 + q], xf);
    for (int q = threadIdx.x; q < lb; q += MERGE_BLOCK) s_in[la + q] = to_code(m.b[j0 + q], xf);
    __syncthreads();

    // this thread's outputs [p0, p0 + MERGE_IPT) of the slice
    const int p0 = threadIdx.x * IPT;
    if (p0 < len) {
        const C *sa = s_in, *sb = s_in + la;
        int ia = (int)co_rank<C>((size_t)p0, (size_t)la, (size_t)lb,
                                 [&](size_t i) { return sa[i]; },
                                 [&](size_t j) { return sb[j]; });
        int ib = p0 - ia;
#pragma unroll 4
        for (int q = 0; q < IPT && p0 + q < len; ++q) {
            const bool take_a = ib >= lb || (ia < la && sa[ia] <= sb[ib]);
            if (take_a) {
                s_out[p0 + q] = sa[ia];
                s_src[p0 + q] = (uint16_t)ia;
                ++ia;
            } else {
                s_out[p0 + q] = sb[ib];
                s_src[p0 + q] = (uint16_t)(la + ib);
                ++ib;
            }
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < len; q += MERGE_BLOCK) {
        if (m.out_k) m.out_k[o0 + q] = from_code(s_out[q], xf);
        if constexpr (HAS_V) {
            const int src = s_src[q];
            const V v = src < la ? static_cast<const V *>(m.av)[i0 + src]
                                 : static_cast<const V *>(m.bv)[j0 + (src - la)];
            static_cast<V *>(m.out_v)[o0 + q] = v;
        }
    }
}

template <typename V>
__global__ void iota_kernel(V *out, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = (V)i;
}

// ---------------------------------------------------------------------------
// Host side.

// Chunk length: the radix limit rounded down to a multiple of 256 keys, so
// every chunk starts 16-byte aligned (the radix passes' bulk copies need it).
// XSS_MERGE_CHUNK=<keys> lowers it (rounded down to a multiple of 256, at
// least 8192), so the chunked path can be exercised on small arrays.
static size_t merge_chunk()
{
    static const size_t v = [] {
        size_t c = XSS_RADIX_MAX_N;
        if (const char *e = getenv("XSS_MERGE_CHUNK")) {
            const unsigned long long want = strtoull(e, nullptr, 10);
            if (want >= 8192 && want < c) c = (size_t)want;
        }
        return c / 256 * 256;
    }();
    return v;
}

bool big_sort_needed(size_t n) { return n > merge_chunk(); }

// Tiles of a merge's output (the smallest tile, 64-bit keys, bounds them all).
static size_t merge_tiles(size_t total)
{
    constexpr size_t t = (size_t)merge_tile<uint64_t>();
    return (total + t - 1) / t;
}
template <typename C> static size_t merge_tiles_c(size_t total)
{
    return (total + merge_tile<C>() - 1) / merge_tile<C>();
}

struct BigLayout {
    size_t chunk_ws, k0, k1, v1, split, total;
};

// Workspace of a chunked sort of n keys: the radix workspace of one chunk,
// the merge's partner buffers (keys k1, values v1), the tile split points;
// argsort also sorts a copy of the keys (k0) -- its positions start in the
// caller's index array, whose partner is v1.
static BigLayout big_layout(int op, int kbytes, int vbytes, size_t n)
{
    BigLayout L{};
    const int sop = op == SOP_ARG ? SOP_KV : op;
    const int vb = op == SOP_ARG ? 8 : (op == SOP_KV ? vbytes : 0);
    size_t off = 0;
    L.chunk_ws = off;
    off = align_up(off + radix_chunk_workspace_bytes(sop, kbytes, vb, merge_chunk()), 256);
    L.k0 = off;
    if (op == SOP_ARG) off = align_up(off + n * kbytes, 256);
    L.k1 = off;
    off = align_up(off + n * kbytes, 256);
    L.v1 = off;
    off = align_up(off + n * vb, 256);
    L.split = off;
    off = align_up(off + (merge_tiles(n) + 1) * sizeof(size_t), 256);
    L.total = off;
    return L;
}

size_t big_sort_workspace_bytes(int op, int kbytes, int vbytes, size_t n)
{
    return big_layout(op, kbytes, vbytes, n).total;
}

template <typename C, typename V>
static int merge_pass(const C *a, const C *b, const V *av, const V *bv, size_t na, size_t nb,
                      C *out_k, V *out_v, size_t *split, KeyXform xf, cudaStream_t s)
{
    MergeArgs<C> m{};
    m.a = a;
    m.b = b;
    m.av = av;
    m.bv = bv;
    m.out_k = out_k;
    m.out_v = out_v;
    m.na = na;
    m.nb = nb;
    m.split = split;
    m.xf = xf;
    m.tile0 = 0;
    const size_t tiles = merge_tiles_c<C>(na + nb);
    XSS_LAUNCH(PK_MERGE, s,
               (merge_split_kernel<C><<<(unsigned)((tiles + 1 + 255) / 256), 256, 0, s>>>(
                   m, split, tiles)));
    XSS_CUDA_TRY(cudaGetLastError());
    XSS_LAUNCH(PK_MERGE, s, (merge_kernel<C, V><<<(unsigned)tiles, MERGE_BLOCK, 0, s>>>(m)));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

// Merge sorted runs of `run` keys pairwise until one run remains.  src holds
// the runs; the result ends in src or dst: *in_dst tells which.  out_k null:
// the last pass writes values only (argsort's positions).
template <typename C, typename V>
static int merge_all(C *src_k, V *src_v, C *dst_k, V *dst_v, size_t n, size_t run,
                     size_t *split, KeyXform xf, cudaStream_t s, bool &in_dst)
{
    in_dst = false;
    for (; run < n; run *= 2) {
        for (size_t b = 0; b < n; b += 2 * run) {
            const size_t na = std::min(run, n - b);
            const size_t nb = std::min(run, n - b - na);
            if (nb == 0) {
                // an unpaired last run is copied across
                XSS_CUDA_TRY(cudaMemcpyAsync(dst_k + b, src_k + b, na * sizeof(C),
                                             cudaMemcpyDeviceToDevice, s));
                if constexpr (!std::is_same<V, NoVal>::value)
                    XSS_CUDA_TRY(cudaMemcpyAsync(dst_v + b, src_v + b, na * sizeof(V),
                                                 cudaMemcpyDeviceToDevice, s));
                continue;
            }
            const V *av = nullptr, *bv = nullptr;
            V *ov = nullptr;
            if constexpr (!std::is_same<V, NoVal>::value) {
                av = src_v + b;
                bv = src_v + b + na;
                ov = dst_v + b;
            }
            const int rc = merge_pass<C, V>(src_k + b, src_k + b + na, av, bv, na, nb,
                                            dst_k + b, ov, split, xf, s);
            if (rc) return rc;
        }
        std::swap(src_k, dst_k);
        std::swap(src_v, dst_v);
        in_dst = !in_dst;
    }
    return XSS_OK;
}

int radix_sort_chunk(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
                     uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s);

template <typename C>
static int big_sort_c(int op, KeyXform xf, void *keys, void *vals, int vbytes,
                      uint64_t *out_idx, size_t n, char *ws, const BigLayout &L,
                      cudaStream_t s)
{
    const int kb = sizeof(C);
    const size_t cws_bytes = radix_chunk_workspace_bytes(op == SOP_ARG ? SOP_KV : op, kb,
                                                   op == SOP_ARG ? 8 : vbytes, merge_chunk());
    void *cws = ws + L.chunk_ws;
    size_t *split = reinterpret_cast<size_t *>(ws + L.split);
    C *k = static_cast<C *>(keys);
    C *k1 = reinterpret_cast<C *>(ws + L.k1);
    bool in_dst = false;
    if (op == SOP_KEYS) {
        for (size_t b = 0; b < n; b += merge_chunk()) {
            const int rc = radix_sort_chunk(SOP_KEYS, kb, xf, k + b, nullptr, 0, nullptr,
                                            std::min(merge_chunk(), n - b), cws, cws_bytes, s);
            if (rc) return rc;
        }
        // canonical NaNs are already written by the chunk sorts
        const KeyXform mxf{xf.kind, xf.desc, 0};
        int rc = merge_all<C, NoVal>(k, nullptr, k1, nullptr, n, merge_chunk(), split, mxf, s,
                                     in_dst);
        if (rc) return rc;
        if (in_dst)
            XSS_CUDA_TRY(cudaMemcpyAsync(k, k1, n * sizeof(C), cudaMemcpyDeviceToDevice, s));
        return XSS_OK;
    }
    if (op == SOP_KV) {
        for (size_t b = 0; b < n; b += merge_chunk()) {
            const int rc = radix_sort_chunk(SOP_KV, kb, xf, k + b,
                                            static_cast<char *>(vals) + b * vbytes, vbytes,
                                            nullptr, std::min(merge_chunk(), n - b), cws,
                                            cws_bytes, s);
            if (rc) return rc;
        }
        int rc;
        if (vbytes == 2) {
            uint16_t *v = static_cast<uint16_t *>(vals), *v1 = reinterpret_cast<uint16_t *>(ws + L.v1);
            rc = merge_all<C, uint16_t>(k, v, k1, v1, n, merge_chunk(), split, xf, s, in_dst);
        } else if (vbytes == 4) {
            uint32_t *v = static_cast<uint32_t *>(vals), *v1 = reinterpret_cast<uint32_t *>(ws + L.v1);
            rc = merge_all<C, uint32_t>(k, v, k1, v1, n, merge_chunk(), split, xf, s, in_dst);
        } else {
            uint64_t *v = static_cast<uint64_t *>(vals), *v1 = reinterpret_cast<uint64_t *>(ws + L.v1);
            rc = merge_all<C, uint64_t>(k, v, k1, v1, n, merge_chunk(), split, xf, s, in_dst);
        }
        if (rc) return rc;
        if (in_dst) {
            XSS_CUDA_TRY(cudaMemcpyAsync(k, k1, n * sizeof(C), cudaMemcpyDeviceToDevice, s));
            XSS_CUDA_TRY(cudaMemcpyAsync(vals, ws + L.v1, n * (size_t)vbytes,
                                         cudaMemcpyDeviceToDevice, s));
        }
        return XSS_OK;
    }
    // SOP_ARG: sort (key copy, position) pairs; positions start in out_idx
    C *k0 = reinterpret_cast<C *>(ws + L.k0);
    uint64_t *v1 = reinterpret_cast<uint64_t *>(ws + L.v1);
    XSS_CUDA_TRY(cudaMemcpyAsync(k0, keys, n * sizeof(C), cudaMemcpyDeviceToDevice, s));
    XSS_LAUNCH(PK_MERGE, s, (iota_kernel<uint64_t><<<num_sms() * 4, 256, 0, s>>>(out_idx, n)));
    XSS_CUDA_TRY(cudaGetLastError());
    for (size_t b = 0; b < n; b += merge_chunk()) {
        const int rc = radix_sort_chunk(SOP_KV, kb, xf, k0 + b, out_idx + b, 8, nullptr,
                                        std::min(merge_chunk(), n - b), cws, cws_bytes, s);
        if (rc) return rc;
    }
    int rc = merge_all<C, uint64_t>(k0, out_idx, k1, v1, n, merge_chunk(), split, xf, s, in_dst);
    if (rc) return rc;
    if (in_dst)
        XSS_CUDA_TRY(cudaMemcpyAsync(out_idx, v1, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice,
                                     s));
    return XSS_OK;
}

int big_sort(int op, int kbytes, KeyXform xf, void *keys, void *vals, int vbytes,
             uint64_t *out_idx, size_t n, void *ws, size_t ws_bytes, cudaStream_t s)
{
    const BigLayout L = big_layout(op, kbytes, vbytes, n);
    if (ws == nullptr || ws_bytes < L.total) return XSS_ENOMEM;
    char *w = static_cast<char *>(ws);
    switch (kbytes) {
    case 2: return big_sort_c<uint16_t>(op, xf, keys, vals, vbytes, out_idx, n, w, L, s);
    case 4: return big_sort_c<uint32_t>(op, xf, keys, vals, vbytes, out_idx, n, w, L, s);
    case 8: return big_sort_c<uint64_t>(op, xf, keys, vals, vbytes, out_idx, n, w, L, s);
    default: return XSS_EINVAL;
    }
}

// ---------------------------------------------------------------------------
// Host-pointer sorts of large arrays, pipelined: the array is cut into
// chunks; each chunk's host-to-device copy runs on its own stream while the
// previous chunks are already being radix-sorted, the sorted runs are merged
// as soon as both halves of a merge are sorted, and the last merge runs in
// PIPE_SLICES output slices, each copied
// back to the host as soon as it is written.  The copies in and out (the host
// link) then bound the call instead of copy-in + sort + copy-out.  Chunk sorts
// and the merge are stable, so results equal the one-piece sort's.  Pinned
// host buffers make every copy asynchronous; pageable ones are staged by the
// driver chunk by chunk, which still overlaps the chunk sorts.
// Chunks: PIPE_CHUNKS_LARGE from PIPE_LARGE_N keys on, else PIPE_CHUNKS (the
// chunks of a smaller array stay long enough for the large-array pass lines).
// Measured on 2^28 int64 -> uint64 pairs from pinned buffers (median of 12
// calls, all variants in one process): 49.65 ms with every merge level after
// the last chunk sort, 48.52 with the levels between the chunk sorts, 48.24
// with 6 chunks, 47.73 with 8.
#ifndef XSS_PIPE_CHUNKS_LARGE
#define XSS_PIPE_CHUNKS_LARGE 8
#endif
constexpr int PIPE_CHUNKS = 4;
constexpr int PIPE_CHUNKS_LARGE = XSS_PIPE_CHUNKS_LARGE;
constexpr size_t PIPE_LARGE_N = size_t(1) << 27;
constexpr int PIPE_SLICES = 8;

struct PipeCtx {
    cudaStream_t s_in = nullptr, s_cmp = nullptr, s_out = nullptr;
    cudaEvent_t ev_in[64] = {}, ev_out[PIPE_SLICES] = {};
    void *buf = nullptr;
    size_t cap = 0;
};
static thread_local PipeCtx t_pipe[64];

static int pipe_ctx(PipeCtx *&c, size_t bytes)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return XSS_ECUDA;
    c = &t_pipe[dev];
    if (!c->s_in) {
        for (cudaStream_t *sp : {&c->s_in, &c->s_cmp, &c->s_out})
            XSS_CUDA_TRY(cudaStreamCreateWithFlags(sp, cudaStreamNonBlocking));
        for (auto &e : c->ev_in) XSS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (auto &e : c->ev_out) XSS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (c->cap < bytes) {
        if (c->buf) {
            cudaStreamSynchronize(c->s_out);
            cudaStreamSynchronize(c->s_cmp);
            cudaFree(c->buf);
            c->buf = nullptr;
            c->cap = 0;
        }
        if (cudaMalloc(&c->buf, bytes) != cudaSuccess) {
            cudaGetLastError();
            return XSS_ENOMEM;
        }
        c->cap = bytes;
    }
    return XSS_OK;
}

bool host_pipeline_wanted(size_t n) { return n >= PIPE_MIN_N; }

bool release_pipeline_buffer()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    PipeCtx &c = t_pipe[dev];
    const bool ok = c.buf == nullptr || cudaFree(c.buf) == cudaSuccess;
    c.buf = nullptr;
    c.cap = 0;
    return ok;
}

template <typename C, typename V>
static int pipelined_sort_c(int op, KeyXform xf, C *hk, V *hv, uint64_t *hidx, size_t n)
{
    constexpr bool HAS_V = !std::is_same<V, NoVal>::value;
    constexpr size_t VB = HAS_V ? sizeof(V) : 0;
    const int kb = sizeof(C);
    const int sop = op == SOP_ARG ? SOP_KV : op;         // argsort sorts (key, position)
    const size_t parts = n >= PIPE_LARGE_N ? PIPE_CHUNKS_LARGE : PIPE_CHUNKS;
    size_t chunk = align_up((n + parts - 1) / parts, 256);
    chunk = std::min(chunk, merge_chunk());
    const size_t nch = (n + chunk - 1) / chunk;
    if (nch > 64) return XSS_ETOOBIG;
    // device layout: keys, values, one chunk's radix workspace, the merge's
    // partner buffers and split points
    const size_t cws_bytes = radix_chunk_workspace_bytes(sop, kb, (int)VB, chunk);
    size_t off = 0;
    const size_t o_k = off;  off = align_up(off + n * kb, 256);
    const size_t o_v = off;  off = align_up(off + n * VB, 256);
    const size_t o_w = off;  off = align_up(off + cws_bytes, 256);
    const size_t o_k1 = off; off = align_up(off + n * kb, 256);
    const size_t o_v1 = off; off = align_up(off + n * VB, 256);
    const size_t o_sp = off; off = align_up(off + (merge_tiles(n) + 1) * sizeof(size_t), 256);
    PipeCtx *c;
    int rc = pipe_ctx(c, off);
    if (rc) return rc;
    char *base = static_cast<char *>(c->buf);
    C *dk = reinterpret_cast<C *>(base + o_k), *dk1 = reinterpret_cast<C *>(base + o_k1);
    V *dv = reinterpret_cast<V *>(base + o_v), *dv1 = reinterpret_cast<V *>(base + o_v1);
    size_t *split = reinterpret_cast<size_t *>(base + o_sp);

    // chunks in, each sorted once it has landed
    if (op == SOP_ARG) {
        if constexpr (std::is_same<V, uint64_t>::value) {
            XSS_LAUNCH(PK_MERGE, c->s_cmp,
                       (iota_kernel<uint64_t><<<num_sms() * 4, 256, 0, c->s_cmp>>>(dv, n)));
            XSS_CUDA_TRY(cudaGetLastError());
        }
    }
    // Merge levels: level l (1..L) merges pairs of level l-1 runs of chunk << (l-1)
    // keys; level l's runs live in buffer l % 2 (level 0: the sorted chunks, in
    // buffer 0).  Every level below L merges a block as soon as the chunks under
    // it are sorted, between the chunk sorts, so the merges overlap the copies
    // of later chunks; level L runs in slices, each copied out once written.
    const KeyXform mxf{xf.kind, xf.desc, 0};   // the chunk sorts wrote canonical NaNs
    int L = 0;
    while ((chunk << L) < n) ++L;
    C *const bk[2] = {dk, dk1};
    V *const bv[2] = {dv, dv1};
    auto merge_block = [&](int l, size_t j) -> int {
        const size_t run = chunk << (l - 1), b = j * 2 * run;
        if (b >= n) return XSS_OK;
        const size_t na = std::min(run, n - b), nb = std::min(run, n - b - na);
        C *const sk = bk[(l - 1) & 1], *const tk = bk[l & 1];
        V *const sv = bv[(l - 1) & 1], *const tv = bv[l & 1];
        if (nb == 0) {
            XSS_CUDA_TRY(cudaMemcpyAsync(tk + b, sk + b, na * kb, cudaMemcpyDeviceToDevice,
                                         c->s_cmp));
            if constexpr (HAS_V)
                XSS_CUDA_TRY(cudaMemcpyAsync(tv + b, sv + b, na * VB, cudaMemcpyDeviceToDevice,
                                             c->s_cmp));
            return XSS_OK;
        }
        return merge_pass<C, V>(sk + b, sk + b + na, HAS_V ? sv + b : nullptr,
                                HAS_V ? sv + b + na : nullptr, na, nb, tk + b,
                                HAS_V ? tv + b : nullptr, split, mxf, c->s_cmp);
    };
    for (size_t i = 0; i < nch; ++i) {
        const size_t b = i * chunk, len = std::min(chunk, n - b);
        touch_host_pages(hk + b, len * kb);
        XSS_CUDA_TRY(cudaMemcpyAsync(dk + b, hk + b, len * kb, cudaMemcpyHostToDevice, c->s_in));
        if constexpr (HAS_V)
            if (op == SOP_KV) {
                touch_host_pages(hv + b, len * VB);
                XSS_CUDA_TRY(cudaMemcpyAsync(dv + b, hv + b, len * VB, cudaMemcpyHostToDevice,
                                             c->s_in));
            }
        XSS_CUDA_TRY(cudaEventRecord(c->ev_in[i], c->s_in));
        XSS_CUDA_TRY(cudaStreamWaitEvent(c->s_cmp, c->ev_in[i], 0));
        rc = radix_sort_chunk(sop, kb, xf, dk + b, HAS_V ? (void *)(dv + b) : nullptr, (int)VB,
                              nullptr, len, base + o_w, cws_bytes, c->s_cmp);
        if (rc) return rc;
        // the level-l blocks this chunk completes (after the last chunk: every
        // remaining, possibly partial, block); a block's halves were written
        // by the lower levels just before it, on the same stream
        for (int l = 1; l < L; ++l) {
            const size_t per_block = size_t(1) << l;   // chunks under a level-l block
            if ((i + 1) % per_block == 0 || i == nch - 1) {
                rc = merge_block(l, i / per_block);
                if (rc) return rc;
            }
        }
    }
    // level L's input (with one chunk: the sorted chunk itself) and output
    const int li = L > 0 ? (L - 1) & 1 : 0;
    C *const sk = bk[li], *const tk = bk[L & 1];
    V *const sv = bv[li], *const tv = bv[L & 1];
    const size_t run = L > 0 ? chunk << (L - 1) : n;
    // the last level in slices, each copied out once written
    C *ok = sk;
    V *ov = sv;
    const size_t tiles = merge_tiles_c<C>(n);
    MergeArgs<C> m{};
    const bool merged = run < n;
    if (merged) {
        m.a = sk;
        m.b = sk + run;
        m.av = HAS_V ? (const void *)sv : nullptr;
        m.bv = HAS_V ? (const void *)(sv + run) : nullptr;
        m.out_k = op == SOP_ARG ? nullptr : tk;
        m.out_v = HAS_V ? (void *)tv : nullptr;
        m.na = run;
        m.nb = n - run;
        m.split = split;
        m.xf = mxf;
        XSS_LAUNCH(PK_MERGE, c->s_cmp,
                   (merge_split_kernel<C><<<(unsigned)((tiles + 1 + 255) / 256), 256, 0,
                                            c->s_cmp>>>(m, split, tiles)));
        XSS_CUDA_TRY(cudaGetLastError());
        ok = tk;
        ov = tv;
    }
    const size_t per = (tiles + PIPE_SLICES - 1) / PIPE_SLICES;
    for (int j = 0; j < PIPE_SLICES; ++j) {
        const size_t t0 = (size_t)j * per, t1 = std::min(tiles, t0 + per);
        if (t0 >= t1) break;
        if (merged) {
            m.tile0 = t0;
            XSS_LAUNCH(PK_MERGE, c->s_cmp,
                       (merge_kernel<C, V><<<(unsigned)(t1 - t0), MERGE_BLOCK, 0, c->s_cmp>>>(m)));
            XSS_CUDA_TRY(cudaGetLastError());
        }
        XSS_CUDA_TRY(cudaEventRecord(c->ev_out[j], c->s_cmp));
        XSS_CUDA_TRY(cudaStreamWaitEvent(c->s_out, c->ev_out[j], 0));
        const size_t e0 = t0 * merge_tile<C>(), e1 = std::min(n, t1 * (size_t)merge_tile<C>());
        if (op == SOP_ARG) {
            if constexpr (std::is_same<V, uint64_t>::value)
                XSS_CUDA_TRY(cudaMemcpyAsync(hidx + e0, ov + e0, (e1 - e0) * 8,
                                             cudaMemcpyDeviceToHost, c->s_out));
        } else {
            XSS_CUDA_TRY(cudaMemcpyAsync(hk + e0, ok + e0, (e1 - e0) * kb,
                                         cudaMemcpyDeviceToHost, c->s_out));
            if constexpr (HAS_V)
                XSS_CUDA_TRY(cudaMemcpyAsync(hv + e0, ov + e0, (e1 - e0) * VB,
                                             cudaMemcpyDeviceToHost, c->s_out));
        }
    }
    XSS_CUDA_TRY(cudaStreamSynchronize(c->s_out));
    XSS_CUDA_TRY(cudaStreamSynchronize(c->s_cmp));
    return XSS_OK;
}

template <typename C>
static int pipelined_sort_k(int op, KeyXform xf, void *hk, void *hv, int vbytes,
                            uint64_t *hidx, size_t n)
{
    C *k = static_cast<C *>(hk);
    if (op == SOP_KEYS) return pipelined_sort_c<C, NoVal>(op, xf, k, nullptr, nullptr, n);
    if (op == SOP_ARG) return pipelined_sort_c<C, uint64_t>(op, xf, k, nullptr, hidx, n);
    switch (vbytes) {
    case 2: return pipelined_sort_c<C, uint16_t>(op, xf, k, static_cast<uint16_t *>(hv), nullptr, n);
    case 4: return pipelined_sort_c<C, uint32_t>(op, xf, k, static_cast<uint32_t *>(hv), nullptr, n);
    case 8: return pipelined_sort_c<C, uint64_t>(op, xf, k, static_cast<uint64_t *>(hv), nullptr, n);
    default: return XSS_EINVAL;
    }
}

int host_pipelined_sort(int op, int kbytes, KeyXform xf, void *hk, void *hv, int vbytes,
                        uint64_t *hidx, size_t n)
{
    switch (kbytes) {
    case 2: return pipelined_sort_k<uint16_t>(op, xf, hk, hv, vbytes, hidx, n);
    case 4: return pipelined_sort_k<uint32_t>(op, xf, hk, hv, vbytes, hidx, n);
    case 8: return pipelined_sort_k<uint64_t>(op, xf, hk, hv, vbytes, hidx, n);
    default: return XSS_EINVAL;
    }
}

}  // namespace xss
