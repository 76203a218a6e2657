// xss_segmented.cu -- batched sort of many independent segments.
#include <algorithm>
#include <vector>
#include "xss_internal.cuh"

namespace xss {
int stream_status(cudaStream_t s);
}

using namespace xss;

static bool seg_dtype(int dt, int &kbytes, int &kind)
{
    switch (dt) {
    case XSS_DT_U16: kbytes = 2; kind = XK_UINT; return true;
    case XSS_DT_I16: kbytes = 2; kind = XK_INT; return true;
    case XSS_DT_F16: kbytes = 2; kind = XK_FLOAT; return true;
    case XSS_DT_U32: kbytes = 4; kind = XK_UINT; return true;
    case XSS_DT_I32: kbytes = 4; kind = XK_INT; return true;
    case XSS_DT_F32: kbytes = 4; kind = XK_FLOAT; return true;
    case XSS_DT_U64: kbytes = 8; kind = XK_UINT; return true;
    case XSS_DT_I64: kbytes = 8; kind = XK_INT; return true;
    case XSS_DT_F64: kbytes = 8; kind = XK_FLOAT; return true;
    default: return false;
    }
}

extern "C" {

size_t xss_gpu_segmented_workspace_size(int key_dtype, int val_dtype, const uint64_t *h_offsets,
                                        size_t num_segments)
{
    int kb, kind;
    if (!seg_dtype(key_dtype, kb, kind) || !h_offsets) return 0;
    const int vb = val_dtype < 0 ? 0 : (val_dtype >= XSS_DT_U64 ? 8 : 4);
    size_t biggest = 0;
    for (size_t i = 0; i < num_segments; ++i)
        biggest = std::max<size_t>(biggest, h_offsets[i + 1] - h_offsets[i]);
    return radix_workspace_bytes(vb ? SOP_KV : SOP_KEYS, kb, vb, biggest);
}

int xss_gpu_segmented_sort(int key_dtype, int val_dtype, void *d_keys, void *d_vals,
                           const uint64_t *d_offsets, const uint64_t *h_offsets,
                           size_t num_segments, int hasnan, int descending, void *d_ws,
                           size_t ws_bytes, xss_stream_t stream)
{
    int kb, kind;
    if (!seg_dtype(key_dtype, kb, kind)) return XSS_EINVAL;
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
    const int vb = d_vals ? (val_dtype >= XSS_DT_U64 ? 8 : 4) : 0;
    const int op = vb ? SOP_KV : SOP_KEYS;
    const size_t need = xss_gpu_segmented_workspace_size(key_dtype, vb ? val_dtype : -1,
                                                         h_offsets, num_segments);
    if (need && (!d_ws || ws_bytes < need)) return XSS_ENOMEM;
    KeyXform xf{kind, descending ? 1 : 0, (op == SOP_KEYS && hasnan) ? 1 : 0};
    for (size_t i = 0; i < num_segments; ++i) {
        const uint64_t b = h_offsets[i], e = h_offsets[i + 1];
        if (e < b) return XSS_EINVAL;
        const int rc = radix_sort(op, kb, xf, static_cast<char *>(d_keys) + b * kb,
                                  vb ? static_cast<char *>(d_vals) + b * vb : nullptr, vb,
                                  nullptr, e - b, d_ws, ws_bytes, s);
        if (rc) return rc;
    }
    return XSS_OK;
}

}  // extern "C"
