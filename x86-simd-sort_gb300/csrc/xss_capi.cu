// xss_capi.cu -- the C ABI: argument checks, dtype mapping, workspace
// management, device-pointer and host-pointer entry points, and the
// reference's own eight extern "C" key-value symbols
// (lib/x86simdsort.cpp:298-339).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <unistd.h>
#include "xss_internal.cuh"

namespace xss {

struct DtypeInfo {
    int kbytes;
    int kind;
};

static bool dtype_info(int dt, DtypeInfo &o)
{
    switch (dt) {
    case XSS_DT_U16: o = {2, XK_UINT}; return true;
    case XSS_DT_I16: o = {2, XK_INT}; return true;
    case XSS_DT_F16: o = {2, XK_FLOAT}; return true;
    case XSS_DT_U32: o = {4, XK_UINT}; return true;
    case XSS_DT_I32: o = {4, XK_INT}; return true;
    case XSS_DT_F32: o = {4, XK_FLOAT}; return true;
    case XSS_DT_U64: o = {8, XK_UINT}; return true;
    case XSS_DT_I64: o = {8, XK_INT}; return true;
    case XSS_DT_F64: o = {8, XK_FLOAT}; return true;
    default: return false;
    }
}

// The reference has key-value sorts for 32/64-bit keys and values only
// (lib/x86simdsort.cpp:274-293, README.md:53-55); here every key type takes
// every value type, 16-bit keys (uint16, int16, _Float16) and 16-bit values
// included.  Values are moved as their bits.
static bool kv_key_ok(int dt) { return dt >= XSS_DT_U16 && dt <= XSS_DT_F64; }
static bool kv_type_ok(int dt) { return dt >= XSS_DT_U16 && dt <= XSS_DT_F64; }

constexpr int MAX_DEV = 64;
static std::mutex g_mu;
static unsigned *g_err[MAX_DEV];
static int g_sms[MAX_DEV];

static int cur_device()
{
    int d = 0;
    cudaGetDevice(&d);
    return (d >= 0 && d < MAX_DEV) ? d : 0;
}

unsigned *device_error_word()
{
    const int d = cur_device();
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_err[d]) {
        unsigned *p = nullptr;
        if (cudaMalloc(&p, 256) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, 256);
        g_err[d] = p;
    }
    return g_err[d];
}

int set_max_dyn_smem(const void *kernel, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> done;
    const int d = cur_device();
    std::lock_guard<std::mutex> lk(mu);
    size_t &have = done[std::make_pair(kernel, d)];
    if (have >= bytes) return XSS_OK;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess) {
        cudaGetLastError();
        return XSS_ECUDA;
    }
    have = bytes;
    return XSS_OK;
}

int num_sms()
{
    const int d = cur_device();
    if (!g_sms[d]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d);
        g_sms[d] = v > 0 ? v : 1;
    }
    return g_sms[d];
}

// Library-owned scratch, one growing buffer per (device, stream).  Growth
// synchronises the stream first so queued work never sees a freed buffer.
struct WsEntry {
    void *p = nullptr;
    size_t cap = 0;
};
static std::map<std::pair<int, cudaStream_t>, WsEntry> g_ws;

int cached_workspace(cudaStream_t s, size_t bytes, void **out)
{
    *out = nullptr;
    if (bytes == 0) return XSS_OK;
    const int d = cur_device();
    std::lock_guard<std::mutex> lk(g_mu);
    WsEntry &e = g_ws[{d, s}];
    if (e.cap < bytes) {
        if (e.p) {
            if (cudaStreamSynchronize(s) != cudaSuccess) return XSS_ECUDA;
            cudaFree(e.p);
            e.p = nullptr;
            e.cap = 0;
        }
        size_t want = bytes + bytes / 8;
        if (cudaMalloc(&e.p, want) != cudaSuccess) {
            cudaGetLastError();
            want = bytes;
            if (cudaMalloc(&e.p, want) != cudaSuccess) {
                cudaGetLastError();
                e.p = nullptr;
                return XSS_ENOMEM;
            }
        }
        e.cap = want;
    }
    *out = e.p;
    return XSS_OK;
}

static int resolve_ws(cudaStream_t s, size_t need, void *&ws, size_t &ws_bytes)
{
    if (need == 0) return XSS_OK;
    if (ws) return ws_bytes >= need ? XSS_OK : XSS_ENOMEM;
    ws_bytes = need;
    return cached_workspace(s, need, &ws);
}

static int check_n(const void *p, size_t n)
{
    if (n > XSS_MAX_N) return XSS_ETOOBIG;
    if (n > 1 && p == nullptr) return XSS_EINVAL;
    return XSS_OK;
}

static int value_bytes(int vdt) { return vdt >= XSS_DT_U64 ? 8 : (vdt >= XSS_DT_U32 ? 4 : 2); }

// ---- device entry points ---------------------------------------------------
static int gpu_qsort(int dt, void *d, size_t n, int hasnan, int desc, void *ws, size_t wsb,
                     cudaStream_t s)
{
    DtypeInfo di;
    if (!dtype_info(dt, di)) return XSS_EINVAL;
    int rc = check_n(d, n);
    if (rc || n <= 1) return rc;
    KeyXform xf{di.kind, desc ? 1 : 0, hasnan ? 1 : 0};
    rc = resolve_ws(s, radix_workspace_bytes(SOP_KEYS, di.kbytes, 0, n), ws, wsb);
    if (rc) return rc;
    return radix_sort(SOP_KEYS, di.kbytes, xf, d, nullptr, 0, nullptr, n, ws, wsb, s);
}

static int gpu_qselect(int dt, void *d, size_t k, size_t n, int hasnan, int desc, void *ws,
                       size_t wsb, cudaStream_t s)
{
    DtypeInfo di;
    if (!dtype_info(dt, di)) return XSS_EINVAL;
    int rc = check_n(d, n);
    if (rc || n <= 1) return rc;
    if (k >= n) return XSS_EINVAL;
    (void)hasnan;  // NaNs always order after +inf; payloads are kept
    KeyXform xf{di.kind, desc ? 1 : 0, 0};
    rc = resolve_ws(s, select_workspace_bytes(SOP_KEYS, di.kbytes, 0, n), ws, wsb);
    if (rc) return rc;
    return radix_select(SOP_KEYS, di.kbytes, xf, d, nullptr, 0, nullptr, k, n, ws, wsb, s);
}

static int gpu_partial_qsort(int dt, void *d, size_t k, size_t n, int hasnan, int desc,
                             void *ws, size_t wsb, cudaStream_t s)
{
    DtypeInfo di;
    if (!dtype_info(dt, di)) return XSS_EINVAL;
    int rc = check_n(d, n);
    if (rc || n <= 1 || k == 0) return rc;
    if (k > n) return XSS_EINVAL;
    // reference: qselect(k-1) then qsort of the first k-1 (src/xss-common-qsort.h:755-762)
    KeyXform sort_xf{di.kind, desc ? 1 : 0, hasnan ? 1 : 0};
    if (n <= SMALL_SORT_MAX || k == n)
        return gpu_qsort(dt, d, (k == n) ? n : n, hasnan, desc, ws, wsb, s);
    if (count16_wanted(SOP_KEYS, di.kbytes, n)) {
        // 16-bit keys: one full sort by counting; canonical NaNs only in the
        // sorted prefix, as select + prefix sort would leave them
        rc = resolve_ws(s, count16_workspace_bytes(n), ws, wsb);
        if (rc) return rc;
        return count16_sort(sort_xf, d, n, k, ws, wsb, s);
    }
    KeyXform sel_xf{di.kind, desc ? 1 : 0, 0};
    const size_t need = std::max(select_workspace_bytes(SOP_KEYS, di.kbytes, 0, n),
                                 radix_workspace_bytes(SOP_KEYS, di.kbytes, 0, k));
    rc = resolve_ws(s, need, ws, wsb);
    if (rc) return rc;
    rc = radix_select(SOP_KEYS, di.kbytes, sel_xf, d, nullptr, 0, nullptr, k - 1, n, ws, wsb, s);
    if (rc) return rc;
    return radix_sort(SOP_KEYS, di.kbytes, sort_xf, d, nullptr, 0, nullptr, k, ws, wsb, s);
}

static int gpu_argsort(int dt, const void *d, uint64_t *arg, size_t n, int hasnan, int desc,
                       void *ws, size_t wsb, cudaStream_t s)
{
    DtypeInfo di;
    if (!dtype_info(dt, di)) return XSS_EINVAL;
    int rc = check_n(d, n);
    if (rc) return rc;
    if (n >= 1 && arg == nullptr) return XSS_EINVAL;
    if (n == 0) return XSS_OK;
    (void)hasnan;
    KeyXform xf{di.kind, desc ? 1 : 0, 0};
    rc = resolve_ws(s, radix_workspace_bytes(SOP_ARG, di.kbytes, 4, n), ws, wsb);
    if (rc) return rc;
    return radix_sort(SOP_ARG, di.kbytes, xf, const_cast<void *>(d), nullptr, 4, arg, n, ws,
                      wsb, s);
}

static int gpu_argselect(int dt, const void *d, uint64_t *arg, size_t k, size_t n, int hasnan,
                         void *ws, size_t wsb, cudaStream_t s)
{
    DtypeInfo di;
    if (!dtype_info(dt, di)) return XSS_EINVAL;
    int rc = check_n(d, n);
    if (rc) return rc;
    if (n >= 1 && arg == nullptr) return XSS_EINVAL;
    if (n == 0) return XSS_OK;
    if (n == 1) return radix_sort(SOP_ARG, di.kbytes, KeyXform{di.kind, 0, 0},
                                  const_cast<void *>(d), nullptr, 4, arg, n, nullptr, 0, s);
    if (k >= n) return XSS_EINVAL;
    (void)hasnan;
    KeyXform xf{di.kind, 0, 0};
    rc = resolve_ws(s, select_workspace_bytes(SOP_ARG, di.kbytes, 4, n), ws, wsb);
    if (rc) return rc;
    return radix_select(SOP_ARG, di.kbytes, xf, const_cast<void *>(d), nullptr, 4, arg, k, n,
                        ws, wsb, s);
}

static int kv_check(int kdt, int vdt, DtypeInfo &di)
{
    if (!dtype_info(kdt, di)) return XSS_EINVAL;
    DtypeInfo vi;
    if (!dtype_info(vdt, vi)) return XSS_EINVAL;
    if (!kv_key_ok(kdt) || !kv_type_ok(vdt)) return XSS_EUNSUPPORTED;
    return XSS_OK;
}

static int gpu_kv_qsort(int kdt, int vdt, void *keys, void *vals, size_t n, int hasnan, int desc,
                        void *ws, size_t wsb, cudaStream_t s)
{
    DtypeInfo di;
    int rc = kv_check(kdt, vdt, di);
    if (rc) return rc;
    rc = check_n(keys, n);
    if (rc || n <= 1) return rc;
    if (vals == nullptr) return XSS_EINVAL;
    (void)hasnan;
    const int vb = value_bytes(vdt);
    KeyXform xf{di.kind, desc ? 1 : 0, 0};
    rc = resolve_ws(s, radix_workspace_bytes(SOP_KV, di.kbytes, vb, n), ws, wsb);
    if (rc) return rc;
    return radix_sort(SOP_KV, di.kbytes, xf, keys, vals, vb, nullptr, n, ws, wsb, s);
}

static int gpu_kv_select(int kdt, int vdt, void *keys, void *vals, size_t k, size_t n,
                         int hasnan, int desc, void *ws, size_t wsb, cudaStream_t s)
{
    DtypeInfo di;
    int rc = kv_check(kdt, vdt, di);
    if (rc) return rc;
    rc = check_n(keys, n);
    if (rc || n <= 1) return rc;
    if (vals == nullptr || k >= n) return XSS_EINVAL;
    (void)hasnan;
    const int vb = value_bytes(vdt);
    KeyXform xf{di.kind, desc ? 1 : 0, 0};
    rc = resolve_ws(s, select_workspace_bytes(SOP_KV, di.kbytes, vb, n), ws, wsb);
    if (rc) return rc;
    return radix_select(SOP_KV, di.kbytes, xf, keys, vals, vb, nullptr, k, n, ws, wsb, s);
}

static int gpu_kv_partial(int kdt, int vdt, void *keys, void *vals, size_t k, size_t n,
                          int hasnan, int desc, void *ws, size_t wsb, cudaStream_t s)
{
    DtypeInfo di;
    int rc = kv_check(kdt, vdt, di);
    if (rc) return rc;
    rc = check_n(keys, n);
    if (rc || n <= 1 || k == 0) return rc;
    if (vals == nullptr || k > n) return XSS_EINVAL;
    if (n <= SMALL_SORT_MAX || k == n) return gpu_kv_qsort(kdt, vdt, keys, vals, n, hasnan, desc, ws, wsb, s);
    const int vb = value_bytes(vdt);
    KeyXform xf{di.kind, desc ? 1 : 0, 0};
    const size_t need = std::max(select_workspace_bytes(SOP_KV, di.kbytes, vb, n),
                                 radix_workspace_bytes(SOP_KV, di.kbytes, vb, k));
    rc = resolve_ws(s, need, ws, wsb);
    if (rc) return rc;
    rc = radix_select(SOP_KV, di.kbytes, xf, keys, vals, vb, nullptr, k - 1, n, ws, wsb, s);
    if (rc) return rc;
    return radix_sort(SOP_KV, di.kbytes, xf, keys, vals, vb, nullptr, k, ws, wsb, s);
}

// Synchronise `s`, then read and clear the device error word.
int stream_status(cudaStream_t s)
{
    if (cudaStreamSynchronize(s) != cudaSuccess) return XSS_ECUDA;
    unsigned *d_err = device_error_word();
    if (!d_err) return XSS_ECUDA;
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, d_err, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return XSS_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return XSS_ECUDA;
    if (h) {
        cudaMemsetAsync(d_err, 0, sizeof(h), s);
        cudaStreamSynchronize(s);
        return XSS_ETIMEOUT;
    }
    return XSS_OK;
}

// ---- host-pointer staging ---------------------------------------------------
struct HostCtx {
    cudaStream_t s = nullptr;
    void *buf[3] = {nullptr, nullptr, nullptr};
    size_t cap[3] = {0, 0, 0};
};
static thread_local HostCtx t_ctx[MAX_DEV];

static int host_ctx(HostCtx *&c)
{
    c = &t_ctx[cur_device()];
    if (!c->s) {
        if (cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess) {
            c->s = nullptr;
            return XSS_ECUDA;
        }
    }
    return XSS_OK;
}

static int host_buf(HostCtx &c, int i, size_t bytes, void *&out)
{
    if (c.cap[i] < bytes) {
        if (c.buf[i]) {
            cudaStreamSynchronize(c.s);
            cudaFree(c.buf[i]);
            c.buf[i] = nullptr;
            c.cap[i] = 0;
        }
        if (cudaMalloc(&c.buf[i], bytes) != cudaSuccess) {
            cudaGetLastError();
            c.buf[i] = nullptr;
            return XSS_ENOMEM;
        }
        c.cap[i] = bytes;
    }
    out = c.buf[i];
    return XSS_OK;
}

// Read one byte of every page of a host range that a copy is about to read.
// Hosts that unmap idle pages now and then to place memory (NUMA balancing)
// leave the copy engine a slow fault path for every page unmapped since the
// caller wrote it; a CPU read maps the page back first for the cost of a
// minor fault.  On the GB300 host this took the 2^28-pair host-pointer
// key-value sort from 50-124 ms (median 74) to a steady 51 ms (with an
// occasional 123 ms), at about 1 ms per 2 GB of touching.
void touch_host_pages(const void *p, size_t bytes)
{
    static const size_t page = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? (size_t)v : (size_t)4096;
    }();
    if (p == nullptr || bytes == 0) return;
    const volatile unsigned char *b = static_cast<const volatile unsigned char *>(p);
    unsigned char acc = 0;
    for (size_t off = 0; off < bytes; off += page) acc ^= b[off];
    acc ^= b[bytes - 1];
    (void)acc;
}

static int h2d(HostCtx &c, void *d, const void *h, size_t bytes)
{
    touch_host_pages(h, bytes);
    return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c.s) == cudaSuccess ? XSS_OK
                                                                                     : XSS_ECUDA;
}
static int d2h(HostCtx &c, void *h, const void *d, size_t bytes)
{
    return cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c.s) == cudaSuccess ? XSS_OK
                                                                                     : XSS_ECUDA;
}

// Host-pointer sorts of at least PIPE_MIN_N keys take the pipelined path
// (chunk copies overlapped with chunk sorts, xss_merge.cu) unless the
// environment sets XSS_HOST_PIPELINE=0.
static bool use_pipeline(size_t n)
{
    static const bool on = [] {
        const char *e = getenv("XSS_HOST_PIPELINE");
        return !(e && strcmp(e, "0") == 0);
    }();
    return on && host_pipeline_wanted(n);
}

static size_t key_bytes(int dt)
{
    DtypeInfo di;
    return dtype_info(dt, di) ? (size_t)di.kbytes : 0;
}

}  // namespace xss

using namespace xss;

extern "C" {

const char *xss_strerror(int status)
{
    switch (status) {
    case XSS_OK: return "ok";
    case XSS_EINVAL: return "invalid argument";
    case XSS_ENOMEM: return "out of device memory or workspace too small";
    case XSS_ETIMEOUT: return "device-side bounded wait expired";
    case XSS_ECUDA: return "CUDA runtime error";
    case XSS_EUNSUPPORTED: return "unsupported type combination";
    case XSS_ETOOBIG: return "array larger than XSS_MAX_N";
    case XSS_EBUSY: return "server busy: request refused";
    case XSS_EAGAIN: return "request still pending";
    default: return "unknown status";
    }
}

const char *xss_version(void) { return "xss-gb300 0.1 (sm_103a)"; }

size_t xss_gpu_workspace_size(int op, int key_dtype, int val_dtype, size_t n, size_t k)
{
    DtypeInfo di;
    if (!dtype_info(key_dtype, di)) return 0;
    const int vb = (op >= XSS_OP_KV_QSORT) ? value_bytes(val_dtype) : 0;
    switch (op) {
    case XSS_OP_QSORT: return radix_workspace_bytes(SOP_KEYS, di.kbytes, 0, n);
    case XSS_OP_QSELECT: return select_workspace_bytes(SOP_KEYS, di.kbytes, 0, n);
    case XSS_OP_PARTIAL_QSORT:
        return std::max(select_workspace_bytes(SOP_KEYS, di.kbytes, 0, n),
                        radix_workspace_bytes(SOP_KEYS, di.kbytes, 0, n));
    case XSS_OP_ARGSORT: return radix_workspace_bytes(SOP_ARG, di.kbytes, 4, n);
    case XSS_OP_ARGSELECT: return select_workspace_bytes(SOP_ARG, di.kbytes, 4, n);
    case XSS_OP_KV_QSORT: return radix_workspace_bytes(SOP_KV, di.kbytes, vb, n);
    case XSS_OP_KV_SELECT: return select_workspace_bytes(SOP_KV, di.kbytes, vb, n);
    case XSS_OP_KV_PARTIAL_SORT:
        return std::max(select_workspace_bytes(SOP_KV, di.kbytes, vb, n),
                        radix_workspace_bytes(SOP_KV, di.kbytes, vb, n));
    default: return 0;
    }
    (void)k;
}

int xss_gpu_stream_status(xss_stream_t stream) { return stream_status((cudaStream_t)stream); }

int xss_release_cached(void)
{
    using namespace xss;
    // the cached buffers may be in use by work queued on any stream, including
    // streams the caller has destroyed since: wait for the whole device
    if (cudaDeviceSynchronize() != cudaSuccess) return XSS_ECUDA;
    const int d = cur_device();
    bool ok = true;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        for (auto it = g_ws.begin(); it != g_ws.end();) {
            if (it->first.first == d) {
                if (it->second.p && cudaFree(it->second.p) != cudaSuccess) ok = false;
                it = g_ws.erase(it);
            } else {
                ++it;
            }
        }
    }
    HostCtx &c = t_ctx[d];
    for (int i = 0; i < 3; ++i) {
        if (c.buf[i] && cudaFree(c.buf[i]) != cudaSuccess) ok = false;
        c.buf[i] = nullptr;
        c.cap[i] = 0;
    }
    if (!release_pipeline_buffer()) ok = false;
    return ok ? XSS_OK : XSS_ECUDA;
}

int xss_gpu_qsort(int dtype, void *d_arr, size_t n, int hasnan, int descending, void *d_ws,
                  size_t ws_bytes, xss_stream_t stream)
{
    return gpu_qsort(dtype, d_arr, n, hasnan, descending, d_ws, ws_bytes, (cudaStream_t)stream);
}
int xss_gpu_qselect(int dtype, void *d_arr, size_t k, size_t n, int hasnan, int descending,
                    void *d_ws, size_t ws_bytes, xss_stream_t stream)
{
    return gpu_qselect(dtype, d_arr, k, n, hasnan, descending, d_ws, ws_bytes,
                       (cudaStream_t)stream);
}
int xss_gpu_partial_qsort(int dtype, void *d_arr, size_t k, size_t n, int hasnan,
                          int descending, void *d_ws, size_t ws_bytes, xss_stream_t stream)
{
    return gpu_partial_qsort(dtype, d_arr, k, n, hasnan, descending, d_ws, ws_bytes,
                             (cudaStream_t)stream);
}
int xss_gpu_argsort(int dtype, const void *d_arr, uint64_t *d_arg, size_t n, int hasnan,
                    int descending, void *d_ws, size_t ws_bytes, xss_stream_t stream)
{
    return gpu_argsort(dtype, d_arr, d_arg, n, hasnan, descending, d_ws, ws_bytes,
                       (cudaStream_t)stream);
}
int xss_gpu_argselect(int dtype, const void *d_arr, uint64_t *d_arg, size_t k, size_t n,
                      int hasnan, void *d_ws, size_t ws_bytes, xss_stream_t stream)
{
    return gpu_argselect(dtype, d_arr, d_arg, k, n, hasnan, d_ws, ws_bytes,
                         (cudaStream_t)stream);
}
int xss_gpu_keyvalue_qsort(int key_dtype, int val_dtype, void *d_keys, void *d_vals, size_t n,
                           int hasnan, int descending, void *d_ws, size_t ws_bytes,
                           xss_stream_t stream)
{
    return gpu_kv_qsort(key_dtype, val_dtype, d_keys, d_vals, n, hasnan, descending, d_ws,
                        ws_bytes, (cudaStream_t)stream);
}
int xss_gpu_keyvalue_select(int key_dtype, int val_dtype, void *d_keys, void *d_vals, size_t k,
                            size_t n, int hasnan, int descending, void *d_ws, size_t ws_bytes,
                            xss_stream_t stream)
{
    return gpu_kv_select(key_dtype, val_dtype, d_keys, d_vals, k, n, hasnan, descending, d_ws,
                         ws_bytes, (cudaStream_t)stream);
}
int xss_gpu_keyvalue_partial_sort(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                                  size_t k, size_t n, int hasnan, int descending, void *d_ws,
                                  size_t ws_bytes, xss_stream_t stream)
{
    return gpu_kv_partial(key_dtype, val_dtype, d_keys, d_vals, k, n, hasnan, descending, d_ws,
                          ws_bytes, (cudaStream_t)stream);
}

// ---- host-pointer entry points ---------------------------------------------
#define XSS_HOST_TRY(expr)      \
    do {                        \
        int _rc = (expr);       \
        if (_rc) return _rc;    \
    } while (0)

int xss_qsort(int dtype, void *arr, size_t n, int hasnan, int descending)
{
    const size_t kb = key_bytes(dtype);
    if (!kb) return XSS_EINVAL;
    XSS_HOST_TRY(check_n(arr, n));
    if (n <= 1) return XSS_OK;
    if (use_pipeline(n)) {
        DtypeInfo di;
        dtype_info(dtype, di);
        XSS_HOST_TRY(host_pipelined_sort(SOP_KEYS, di.kbytes,
                                         KeyXform{di.kind, descending ? 1 : 0, hasnan ? 1 : 0},
                                         arr, nullptr, 0, nullptr, n));
        return stream_status(nullptr);
    }
    HostCtx *c;
    XSS_HOST_TRY(host_ctx(c));
    void *d;
    XSS_HOST_TRY(host_buf(*c, 0, n * kb, d));
    XSS_HOST_TRY(h2d(*c, d, arr, n * kb));
    XSS_HOST_TRY(gpu_qsort(dtype, d, n, hasnan, descending, nullptr, 0, c->s));
    XSS_HOST_TRY(d2h(*c, arr, d, n * kb));
    return stream_status(c->s);
}

int xss_qselect(int dtype, void *arr, size_t k, size_t n, int hasnan, int descending)
{
    const size_t kb = key_bytes(dtype);
    if (!kb) return XSS_EINVAL;
    XSS_HOST_TRY(check_n(arr, n));
    if (n <= 1) return XSS_OK;
    if (k >= n) return XSS_EINVAL;
    HostCtx *c;
    XSS_HOST_TRY(host_ctx(c));
    void *d;
    XSS_HOST_TRY(host_buf(*c, 0, n * kb, d));
    XSS_HOST_TRY(h2d(*c, d, arr, n * kb));
    XSS_HOST_TRY(gpu_qselect(dtype, d, k, n, hasnan, descending, nullptr, 0, c->s));
    XSS_HOST_TRY(d2h(*c, arr, d, n * kb));
    return stream_status(c->s);
}

int xss_partial_qsort(int dtype, void *arr, size_t k, size_t n, int hasnan, int descending)
{
    const size_t kb = key_bytes(dtype);
    if (!kb) return XSS_EINVAL;
    XSS_HOST_TRY(check_n(arr, n));
    if (n <= 1 || k == 0) return XSS_OK;
    if (k > n) return XSS_EINVAL;
    HostCtx *c;
    XSS_HOST_TRY(host_ctx(c));
    void *d;
    XSS_HOST_TRY(host_buf(*c, 0, n * kb, d));
    XSS_HOST_TRY(h2d(*c, d, arr, n * kb));
    XSS_HOST_TRY(gpu_partial_qsort(dtype, d, k, n, hasnan, descending, nullptr, 0, c->s));
    XSS_HOST_TRY(d2h(*c, arr, d, n * kb));
    return stream_status(c->s);
}

int xss_argsort(int dtype, const void *arr, uint64_t *arg, size_t n, int hasnan, int descending)
{
    const size_t kb = key_bytes(dtype);
    if (!kb) return XSS_EINVAL;
    XSS_HOST_TRY(check_n(arr, n));
    if (n == 0) return XSS_OK;
    if (!arg) return XSS_EINVAL;
    if (n == 1) {
        arg[0] = 0;
        return XSS_OK;
    }
    if (use_pipeline(n)) {
        DtypeInfo dt;
        dtype_info(dtype, dt);
        XSS_HOST_TRY(host_pipelined_sort(SOP_ARG, dt.kbytes,
                                         KeyXform{dt.kind, descending ? 1 : 0, 0},
                                         const_cast<void *>(arr), nullptr, 0, arg, n));
        return stream_status(nullptr);
    }
    HostCtx *c;
    XSS_HOST_TRY(host_ctx(c));
    void *d, *di;
    XSS_HOST_TRY(host_buf(*c, 0, n * kb, d));
    XSS_HOST_TRY(host_buf(*c, 2, n * 8, di));
    XSS_HOST_TRY(h2d(*c, d, arr, n * kb));
    XSS_HOST_TRY(gpu_argsort(dtype, d, (uint64_t *)di, n, hasnan, descending, nullptr, 0, c->s));
    XSS_HOST_TRY(d2h(*c, arg, di, n * 8));
    return stream_status(c->s);
}

int xss_argselect(int dtype, const void *arr, uint64_t *arg, size_t k, size_t n, int hasnan)
{
    const size_t kb = key_bytes(dtype);
    if (!kb) return XSS_EINVAL;
    XSS_HOST_TRY(check_n(arr, n));
    if (n == 0) return XSS_OK;
    if (!arg) return XSS_EINVAL;
    if (n == 1) {
        arg[0] = 0;
        return XSS_OK;
    }
    if (k >= n) return XSS_EINVAL;
    HostCtx *c;
    XSS_HOST_TRY(host_ctx(c));
    void *d, *di;
    XSS_HOST_TRY(host_buf(*c, 0, n * kb, d));
    XSS_HOST_TRY(host_buf(*c, 2, n * 8, di));
    XSS_HOST_TRY(h2d(*c, d, arr, n * kb));
    XSS_HOST_TRY(gpu_argselect(dtype, d, (uint64_t *)di, k, n, hasnan, nullptr, 0, c->s));
    XSS_HOST_TRY(d2h(*c, arg, di, n * 8));
    return stream_status(c->s);
}

static int host_kv(int which, int kdt, int vdt, void *keys, void *vals, size_t k, size_t n,
                   int hasnan, int desc)
{
    DtypeInfo di;
    XSS_HOST_TRY(kv_check(kdt, vdt, di));
    XSS_HOST_TRY(check_n(keys, n));
    if (n <= 1) return XSS_OK;
    if (!vals) return XSS_EINVAL;
    if (which == 1 && k >= n) return XSS_EINVAL;
    if (which == 2 && k == 0) return XSS_OK;
    if (which == 2 && k > n) return XSS_EINVAL;
    const size_t kb = di.kbytes, vb = value_bytes(vdt);
    if (which == 0 && use_pipeline(n)) {
        XSS_HOST_TRY(host_pipelined_sort(SOP_KV, (int)kb, KeyXform{di.kind, desc ? 1 : 0, 0},
                                         keys, vals, (int)vb, nullptr, n));
        return stream_status(nullptr);
    }
    HostCtx *c;
    XSS_HOST_TRY(host_ctx(c));
    void *dk, *dv;
    XSS_HOST_TRY(host_buf(*c, 0, n * kb, dk));
    XSS_HOST_TRY(host_buf(*c, 1, n * vb, dv));
    XSS_HOST_TRY(h2d(*c, dk, keys, n * kb));
    XSS_HOST_TRY(h2d(*c, dv, vals, n * vb));
    if (which == 0) XSS_HOST_TRY(gpu_kv_qsort(kdt, vdt, dk, dv, n, hasnan, desc, nullptr, 0, c->s));
    else if (which == 1) XSS_HOST_TRY(gpu_kv_select(kdt, vdt, dk, dv, k, n, hasnan, desc, nullptr, 0, c->s));
    else XSS_HOST_TRY(gpu_kv_partial(kdt, vdt, dk, dv, k, n, hasnan, desc, nullptr, 0, c->s));
    XSS_HOST_TRY(d2h(*c, keys, dk, n * kb));
    XSS_HOST_TRY(d2h(*c, vals, dv, n * vb));
    return stream_status(c->s);
}

int xss_keyvalue_qsort(int key_dtype, int val_dtype, void *keys, void *vals, size_t n, int hasnan,
                       int descending)
{
    return host_kv(0, key_dtype, val_dtype, keys, vals, 0, n, hasnan, descending);
}
int xss_keyvalue_select(int key_dtype, int val_dtype, void *keys, void *vals, size_t k, size_t n,
                        int hasnan, int descending)
{
    return host_kv(1, key_dtype, val_dtype, keys, vals, k, n, hasnan, descending);
}
int xss_keyvalue_partial_sort(int key_dtype, int val_dtype, void *keys, void *vals, size_t k,
                              size_t n, int hasnan, int descending)
{
    return host_kv(2, key_dtype, val_dtype, keys, vals, k, n, hasnan, descending);
}

// ---- the reference's C symbols (lib/x86simdsort.cpp:298-339) ---------------
static void ref_kv_or_die(int kdt, int vdt, void *k, void *v, size_t n, const char *name)
{
    const int rc = xss_keyvalue_qsort(kdt, vdt, k, v, n, 1, 0);
    if (rc != XSS_OK) {
        fprintf(stderr, "%s: %s\n", name, xss_strerror(rc));
        abort();
    }
}

#define XSS_REF_KV(KN, VN, KT, VT, KDT, VDT)                                   \
    void keyvalue_qsort_##KN##_##VN(KT *key, VT *val, size_t size)             \
    {                                                                          \
        ref_kv_or_die(KDT, VDT, key, val, size, "keyvalue_qsort_" #KN "_" #VN); \
    }

XSS_REF_KV(float, uint32, float, uint32_t, XSS_DT_F32, XSS_DT_U32)
XSS_REF_KV(float, uint64, float, uint64_t, XSS_DT_F32, XSS_DT_U64)
XSS_REF_KV(uint64, uint32, uint64_t, uint32_t, XSS_DT_U64, XSS_DT_U32)
XSS_REF_KV(uint64, uint64, uint64_t, uint64_t, XSS_DT_U64, XSS_DT_U64)
XSS_REF_KV(int32, uint32, int32_t, uint32_t, XSS_DT_I32, XSS_DT_U32)
XSS_REF_KV(int32, uint64, int32_t, uint64_t, XSS_DT_I32, XSS_DT_U64)
XSS_REF_KV(uint32, uint32, uint32_t, uint32_t, XSS_DT_U32, XSS_DT_U32)
XSS_REF_KV(uint32, uint64, uint32_t, uint64_t, XSS_DT_U32, XSS_DT_U64)

}  // extern "C"
