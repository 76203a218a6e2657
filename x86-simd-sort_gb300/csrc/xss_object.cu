// xss_object.cu -- device form of object_qsort (lib/x86simdsort.h:73-106)
// for records whose sort key is a member at a fixed byte offset.
//
// The reference extracts keys on the host with a key function, sorts
// (key, position) pairs with keyvalue_qsort and permutes the objects along
// the permutation's cycles.  Here every step runs on the device: one kernel
// reads the keys out of the records, the key-value radix sort orders
// (key, position) pairs, and one kernel gathers whole records into a
// scratch copy in sorted order, which is then copied back.  Records are
// moved with the widest word (16, 8, 4 or 1 bytes) that the record size and
// the array's alignment allow.
#include <algorithm>
#include <cstring>
#include "xss_internal.cuh"

namespace xss {

// Positions are 32-bit up to 2^32 - 1 records, 64-bit beyond (P).
template <typename K, typename P, bool ALIGNED>
__global__ void __launch_bounds__(256) obj_extract_kernel(const unsigned char *recs, size_t n,
                                                          size_t rec_bytes, size_t key_off,
                                                          K *keys, P *pos)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned char *p = recs + i * rec_bytes + key_off;
        K k;
        if constexpr (ALIGNED) {
            k = *reinterpret_cast<const K *>(p);
        } else {
            memcpy(&k, p, sizeof(K));
        }
        keys[i] = k;
        pos[i] = (P)i;
    }
}

// dst record i = src record pos[i]; W-byte words, wpr words per record.
template <typename W, typename P>
__global__ void __launch_bounds__(256) obj_gather_kernel(const W *src, W *dst, const P *pos,
                                                         size_t n, size_t wpr)
{
    const size_t total = n * wpr;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += stride) {
        const size_t i = w / wpr, j = w - i * wpr;
        const size_t from = pos[i];
        if (from < n) dst[w] = src[from * wpr + j];
    }
}

struct ObjLayout {
    size_t keys, pos, radix, recs, total;
};

static int pos_bytes(size_t n) { return n > 0xffffffffull ? 8 : 4; }

static ObjLayout obj_layout(size_t n, size_t rec_bytes, int kbytes)
{
    ObjLayout L{};
    const int pb = pos_bytes(n);
    size_t off = 0;
    L.keys = off;  off = align_up(off + n * kbytes, 256);
    L.pos = off;   off = align_up(off + n * pb, 256);
    L.radix = off; off = align_up(off + radix_workspace_bytes(SOP_KV, kbytes, pb, n), 256);
    L.recs = off;  off = align_up(off + n * rec_bytes, 256);
    L.total = off;
    return L;
}

static int key_kind(int dt, int &kbytes)
{
    switch (dt) {
    case XSS_DT_U32: kbytes = 4; return XK_UINT;
    case XSS_DT_I32: kbytes = 4; return XK_INT;
    case XSS_DT_F32: kbytes = 4; return XK_FLOAT;
    case XSS_DT_U64: kbytes = 8; return XK_UINT;
    case XSS_DT_I64: kbytes = 8; return XK_INT;
    case XSS_DT_F64: kbytes = 8; return XK_FLOAT;
    default: return -1;   // 32- and 64-bit keys only (lib/x86simdsort.h:80-81)
    }
}

template <typename W, typename P>
static int gather(const void *src, void *dst, const P *pos, size_t n, size_t rec_bytes,
                  cudaStream_t s)
{
    const size_t wpr = rec_bytes / sizeof(W);
    const size_t total = n * wpr;
    const int grid = (int)std::min<size_t>((total + 255) / 256, (size_t)num_sms() * 16);
    XSS_LAUNCH(PK_OBJECT, s,
               (obj_gather_kernel<W, P><<<grid, 256, 0, s>>>(static_cast<const W *>(src),
                                                           static_cast<W *>(dst), pos, n, wpr)));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

template <typename K, typename P>
static int extract(const unsigned char *recs, size_t n, size_t rec_bytes, size_t key_off,
                   void *keys, P *pos, cudaStream_t s)
{
    const bool aligned = (reinterpret_cast<uintptr_t>(recs) % sizeof(K)) == 0 &&
                         rec_bytes % sizeof(K) == 0 && key_off % sizeof(K) == 0;
    const int grid = (int)std::min<size_t>((n + 255) / 256, (size_t)num_sms() * 16);
    if (aligned)
        XSS_LAUNCH(PK_OBJECT, s, (obj_extract_kernel<K, P, true><<<grid, 256, 0, s>>>(
                                     recs, n, rec_bytes, key_off, static_cast<K *>(keys), pos)));
    else
        XSS_LAUNCH(PK_OBJECT, s, (obj_extract_kernel<K, P, false><<<grid, 256, 0, s>>>(
                                     recs, n, rec_bytes, key_off, static_cast<K *>(keys), pos)));
    XSS_CUDA_TRY(cudaGetLastError());
    return XSS_OK;
}

// Extract, key-value sort (key, position P), gather into the scratch copy.
template <typename P>
static int object_sort(void *d_recs, size_t n, size_t rec_bytes, size_t key_offset, int kb,
                       KeyXform xf, char *ws, const ObjLayout &L, cudaStream_t s)
{
    void *keys = ws + L.keys;
    P *pos = reinterpret_cast<P *>(ws + L.pos);
    void *tmp = ws + L.recs;
    const unsigned char *recs = static_cast<const unsigned char *>(d_recs);
    int rc = kb == 4 ? extract<uint32_t, P>(recs, n, rec_bytes, key_offset, keys, pos, s)
                     : extract<uint64_t, P>(recs, n, rec_bytes, key_offset, keys, pos, s);
    if (rc) return rc;
    rc = radix_sort(SOP_KV, kb, xf, keys, pos, sizeof(P), nullptr, n, ws + L.radix,
                    radix_workspace_bytes(SOP_KV, kb, sizeof(P), n), s);
    if (rc) return rc;
    const uintptr_t base = reinterpret_cast<uintptr_t>(d_recs);
    if (rec_bytes % 16 == 0 && base % 16 == 0)
        return gather<uint4, P>(d_recs, tmp, pos, n, rec_bytes, s);
    if (rec_bytes % 8 == 0 && base % 8 == 0)
        return gather<uint64_t, P>(d_recs, tmp, pos, n, rec_bytes, s);
    if (rec_bytes % 4 == 0 && base % 4 == 0)
        return gather<uint32_t, P>(d_recs, tmp, pos, n, rec_bytes, s);
    return gather<unsigned char, P>(d_recs, tmp, pos, n, rec_bytes, s);
}

}  // namespace xss

using namespace xss;

extern "C" size_t xss_gpu_object_workspace_size(size_t n, size_t rec_bytes, int key_dtype)
{
    int kb = 0;
    if (key_kind(key_dtype, kb) < 0 || n <= 1) return 0;
    return obj_layout(n, rec_bytes, kb).total;
}

extern "C" int xss_gpu_object_qsort(void *d_recs, size_t n, size_t rec_bytes, size_t key_offset,
                                    int key_dtype, int hasnan, int descending, void *d_ws,
                                    size_t ws_bytes, xss_stream_t stream)
{
    (void)hasnan;   // NaN keys order after +inf either way; records are never rewritten
    int kb = 0;
    const int kind = key_kind(key_dtype, kb);
    if (kind < 0) return XSS_EUNSUPPORTED;
    if (n > XSS_MAX_N) return XSS_ETOOBIG;
    if (n <= 1) return XSS_OK;
    if (d_recs == nullptr || rec_bytes == 0 || key_offset + (size_t)kb > rec_bytes)
        return XSS_EINVAL;
    if (rec_bytes > ((size_t)1 << 40) / n) return XSS_ETOOBIG;
    cudaStream_t s = (cudaStream_t)stream;
    const ObjLayout L = obj_layout(n, rec_bytes, kb);
    if (d_ws == nullptr) {
        const int rc = cached_workspace(s, L.total, &d_ws);
        if (rc) return rc;
    } else if (ws_bytes < L.total) {
        return XSS_ENOMEM;
    }
    char *ws = static_cast<char *>(d_ws);
    const KeyXform xf{kind, descending ? 1 : 0, 0};
    const int rc = pos_bytes(n) == 4
                       ? object_sort<uint32_t>(d_recs, n, rec_bytes, key_offset, kb, xf, ws, L, s)
                       : object_sort<uint64_t>(d_recs, n, rec_bytes, key_offset, kb, xf, ws, L, s);
    if (rc) return rc;
    XSS_CUDA_TRY(cudaMemcpyAsync(d_recs, ws + L.recs, n * rec_bytes, cudaMemcpyDeviceToDevice,
                                 s));
    return XSS_OK;
}
