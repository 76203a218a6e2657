/*
 * x86simdsort.h -- C++ drop-in for intel/x86-simd-sort's public API
 * (lib/x86simdsort.h:13-108), backed by the GB300 kernels in libxss_gb300.so.
 *
 * The host-pointer templates keep the reference's names, argument order and
 * defaults; they copy the array to the GPU, sort/select there and copy the
 * result back.  Explicit specialisations exist for the reference's type set:
 * qsort / qselect / partial_qsort / argsort / argselect for uint16_t,
 * int16_t, _Float16 (when the compiler has it), float, double, uint32_t,
 * int32_t, uint64_t, int64_t; the keyvalue_* family for every pair of
 * {uint32_t, int32_t, float, uint64_t, int64_t, double}.
 *
 * Unlike the reference (which has no error channel), a failure -- no GPU,
 * out of memory, k out of range -- throws std::runtime_error.
 *
 * x86simdsort::gpu holds the device-pointer forms, which take a stream and
 * an optional caller-owned workspace and return without synchronising.
 */
#ifndef XSS_GB300_X86SIMDSORT_H
#define XSS_GB300_X86SIMDSORT_H

#include <stdint.h>
#include <cstddef>
#include <functional>
#include <numeric>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "xss_gpu.h"

#define XSS_EXPORT_SYMBOL __attribute__((visibility("default")))

namespace x86simdsort {

// quicksort (lib/x86simdsort.h:15-18)
template <typename T>
XSS_EXPORT_SYMBOL void
qsort(T *arr, size_t arrsize, bool hasnan = false, bool descending = false);

// quickselect (lib/x86simdsort.h:20-26)
template <typename T>
XSS_EXPORT_SYMBOL void qselect(T *arr, size_t k, size_t arrsize, bool hasnan = false,
                               bool descending = false);

// partial sort (lib/x86simdsort.h:28-34)
template <typename T>
XSS_EXPORT_SYMBOL void partial_qsort(T *arr, size_t k, size_t arrsize, bool hasnan = false,
                                     bool descending = false);

// argsort (lib/x86simdsort.h:36-39)
template <typename T>
XSS_EXPORT_SYMBOL std::vector<size_t>
argsort(T *arr, size_t arrsize, bool hasnan = false, bool descending = false);

// argselect (lib/x86simdsort.h:41-44)
template <typename T>
XSS_EXPORT_SYMBOL std::vector<size_t>
argselect(T *arr, size_t k, size_t arrsize, bool hasnan = false);

// keyvalue sort (lib/x86simdsort.h:46-52)
template <typename T1, typename T2>
XSS_EXPORT_SYMBOL void keyvalue_qsort(T1 *key, T2 *val, size_t arrsize, bool hasnan = false,
                                      bool descending = false);

// keyvalue select (lib/x86simdsort.h:54-61)
template <typename T1, typename T2>
XSS_EXPORT_SYMBOL void keyvalue_select(T1 *key, T2 *val, size_t k, size_t arrsize,
                                       bool hasnan = false, bool descending = false);

// keyvalue partial sort (lib/x86simdsort.h:63-70)
template <typename T1, typename T2>
XSS_EXPORT_SYMBOL void keyvalue_partial_sort(T1 *key, T2 *val, size_t k, size_t arrsize,
                                             bool hasnan = false, bool descending = false);

/*
 * object_qsort (lib/x86simdsort.h:73-106): sort objects by a 32- or 64-bit
 * key.  The keys are extracted on the host, sorted on the GPU together with
 * the objects' positions (keyvalue_qsort), and the objects are then moved
 * into place by following the permutation's cycles.
 */
template <typename T, typename U, typename Func>
XSS_EXPORT_SYMBOL void object_qsort(T *arr, U arrsize, Func key_func)
{
    static_assert(std::is_integral<U>::value, "arrsize must be an integral type");
    static_assert(sizeof(U) == 4 || sizeof(U) == 8, "arrsize must be 32 or 64 bits");
    using K = typename decltype(std::function{key_func})::result_type;
    static_assert(sizeof(K) == 4 || sizeof(K) == 8, "key_func must return a 32 or 64 bit key");
    if (arrsize <= 1) return;
    const size_t n = (size_t)arrsize;
    std::vector<K> keys(n);
    for (size_t i = 0; i < n; ++i) keys[i] = key_func(arr[i]);
    std::vector<U> src(n);
    std::iota(src.begin(), src.end(), (U)0);
    keyvalue_qsort(keys.data(), src.data(), n);
    // slot i must receive the object that was at src[i]
    std::vector<bool> placed(n, false);
    for (size_t start = 0; start < n; ++start) {
        if (placed[start]) continue;
        size_t hole = start;
        T carried = std::move(arr[start]);
        while (true) {
            placed[hole] = true;
            const size_t from = (size_t)src[hole];
            if (from == start) {
                arr[hole] = std::move(carried);
                break;
            }
            arr[hole] = std::move(arr[from]);
            hole = from;
        }
    }
}

// ---------------------------------------------------------------------------
// Device-pointer forms.
namespace gpu {

template <typename T> struct dtype_of;
template <> struct dtype_of<uint16_t> { static constexpr int value = XSS_DT_U16; };
template <> struct dtype_of<int16_t> { static constexpr int value = XSS_DT_I16; };
template <> struct dtype_of<uint32_t> { static constexpr int value = XSS_DT_U32; };
template <> struct dtype_of<int32_t> { static constexpr int value = XSS_DT_I32; };
template <> struct dtype_of<float> { static constexpr int value = XSS_DT_F32; };
template <> struct dtype_of<uint64_t> { static constexpr int value = XSS_DT_U64; };
template <> struct dtype_of<int64_t> { static constexpr int value = XSS_DT_I64; };
template <> struct dtype_of<double> { static constexpr int value = XSS_DT_F64; };
#ifdef __FLT16_MAX__
template <> struct dtype_of<_Float16> { static constexpr int value = XSS_DT_F16; };
#endif

inline void check(int rc)
{
    if (rc != XSS_OK) throw std::runtime_error(std::string("xss-gb300: ") + xss_strerror(rc));
}

template <typename T>
void qsort(T *d_arr, size_t n, bool hasnan = false, bool descending = false,
           xss_stream_t stream = nullptr, void *d_ws = nullptr, size_t ws_bytes = 0)
{
    check(xss_gpu_qsort(dtype_of<T>::value, d_arr, n, hasnan, descending, d_ws, ws_bytes, stream));
}
template <typename T>
void qselect(T *d_arr, size_t k, size_t n, bool hasnan = false, bool descending = false,
             xss_stream_t stream = nullptr, void *d_ws = nullptr, size_t ws_bytes = 0)
{
    check(xss_gpu_qselect(dtype_of<T>::value, d_arr, k, n, hasnan, descending, d_ws, ws_bytes,
                          stream));
}
template <typename T>
void partial_qsort(T *d_arr, size_t k, size_t n, bool hasnan = false, bool descending = false,
                   xss_stream_t stream = nullptr, void *d_ws = nullptr, size_t ws_bytes = 0)
{
    check(xss_gpu_partial_qsort(dtype_of<T>::value, d_arr, k, n, hasnan, descending, d_ws,
                                ws_bytes, stream));
}
// NumPy-style argsort into a caller array (src/x86simdsort-static-incl.h:31-37)
template <typename T>
void argsort(const T *d_arr, uint64_t *d_arg, size_t n, bool hasnan = false,
             bool descending = false, xss_stream_t stream = nullptr, void *d_ws = nullptr,
             size_t ws_bytes = 0)
{
    check(xss_gpu_argsort(dtype_of<T>::value, d_arr, d_arg, n, hasnan, descending, d_ws,
                          ws_bytes, stream));
}
// NumPy-style argselect into a caller array (src/x86simdsort-static-incl.h:42-46)
template <typename T>
void argselect(const T *d_arr, uint64_t *d_arg, size_t k, size_t n, bool hasnan = false,
               xss_stream_t stream = nullptr, void *d_ws = nullptr, size_t ws_bytes = 0)
{
    check(xss_gpu_argselect(dtype_of<T>::value, d_arr, d_arg, k, n, hasnan, d_ws, ws_bytes,
                            stream));
}
template <typename T1, typename T2>
void keyvalue_qsort(T1 *d_keys, T2 *d_vals, size_t n, bool hasnan = false,
                    bool descending = false, xss_stream_t stream = nullptr,
                    void *d_ws = nullptr, size_t ws_bytes = 0)
{
    check(xss_gpu_keyvalue_qsort(dtype_of<T1>::value, dtype_of<T2>::value, d_keys, d_vals, n,
                                 hasnan, descending, d_ws, ws_bytes, stream));
}
template <typename T1, typename T2>
void keyvalue_select(T1 *d_keys, T2 *d_vals, size_t k, size_t n, bool hasnan = false,
                     bool descending = false, xss_stream_t stream = nullptr,
                     void *d_ws = nullptr, size_t ws_bytes = 0)
{
    check(xss_gpu_keyvalue_select(dtype_of<T1>::value, dtype_of<T2>::value, d_keys, d_vals, k,
                                  n, hasnan, descending, d_ws, ws_bytes, stream));
}
template <typename T1, typename T2>
void keyvalue_partial_sort(T1 *d_keys, T2 *d_vals, size_t k, size_t n, bool hasnan = false,
                           bool descending = false, xss_stream_t stream = nullptr,
                           void *d_ws = nullptr, size_t ws_bytes = 0)
{
    check(xss_gpu_keyvalue_partial_sort(dtype_of<T1>::value, dtype_of<T2>::value, d_keys,
                                        d_vals, k, n, hasnan, descending, d_ws, ws_bytes,
                                        stream));
}
// Device form of object_qsort (lib/x86simdsort.h:73-106) for records whose key
// is a data member: sorts n records of type T in device memory by
// record.*key.  K must be a 32- or 64-bit key type, as in the host form.
// Equal keys keep their input order.
template <typename T, typename K>
void object_qsort(T *d_arr, size_t n, K T::*key, bool hasnan = false, bool descending = false,
                  xss_stream_t stream = nullptr, void *d_ws = nullptr, size_t ws_bytes = 0)
{
    static_assert(sizeof(K) == 4 || sizeof(K) == 8, "the key member must be 32 or 64 bits");
    static_assert(std::is_trivially_copyable<T>::value, "records are moved as bytes");
    // byte offset of the member, computed on suitably aligned raw storage
    alignas(T) unsigned char probe[sizeof(T)];
    const T *p = reinterpret_cast<const T *>(probe);
    const size_t off = (size_t)(reinterpret_cast<const unsigned char *>(&(p->*key)) - probe);
    check(xss_gpu_object_qsort(d_arr, n, sizeof(T), off, dtype_of<K>::value, hasnan, descending,
                               d_ws, ws_bytes, stream));
}

// Wait for `stream` and report a device-side error latched by earlier calls.
inline void synchronize(xss_stream_t stream = nullptr) { check(xss_gpu_stream_status(stream)); }

// Free the device memory the library caches between calls on the current
// device (every stream's workspace, this thread's host-pointer buffers).
inline void release_cached() { check(xss_release_cached()); }

}  // namespace gpu
}  // namespace x86simdsort

#endif  // XSS_GB300_X86SIMDSORT_H
