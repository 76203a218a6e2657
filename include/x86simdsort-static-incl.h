// x86simdsort-static-incl.h -- the reference's header-only "static" API
// (src/x86simdsort-static-incl.h:8-71, namespace x86simdsortStatic, the form
// NumPy builds against), served by the GB300 library: every function is an
// inline forwarder to the host-pointer C ABI in xss_gpu.h, so a caller that
// includes this header links libxss_gb300.so instead of compiling the SIMD
// templates.  Same names, argument order and defaults; errors throw
// std::runtime_error (the reference has no error channel).
#ifndef XSS_GB300_STATIC_INCL_H
#define XSS_GB300_STATIC_INCL_H

#include <stdint.h>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "xss_gpu.h"

namespace x86simdsortStatic {
namespace detail {

template <typename T> struct dt;
template <> struct dt<uint16_t> { static constexpr int v = XSS_DT_U16; };
template <> struct dt<int16_t> { static constexpr int v = XSS_DT_I16; };
template <> struct dt<uint32_t> { static constexpr int v = XSS_DT_U32; };
template <> struct dt<int32_t> { static constexpr int v = XSS_DT_I32; };
template <> struct dt<float> { static constexpr int v = XSS_DT_F32; };
template <> struct dt<uint64_t> { static constexpr int v = XSS_DT_U64; };
template <> struct dt<int64_t> { static constexpr int v = XSS_DT_I64; };
template <> struct dt<double> { static constexpr int v = XSS_DT_F64; };
#ifdef __FLT16_MAX__
template <> struct dt<_Float16> { static constexpr int v = XSS_DT_F16; };
#endif

inline void check(int rc)
{
    if (rc != XSS_OK) throw std::runtime_error(std::string("x86simdsortStatic: ") + xss_strerror(rc));
}

template <typename T> constexpr int key_dt()
{
    using U = typename std::remove_cv<T>::type;
    return dt<U>::v;
}

}  // namespace detail

template <typename T>
inline void qsort(T *arr, size_t size, bool hasnan = false, bool descending = false)
{
    detail::check(xss_qsort(detail::key_dt<T>(), arr, size, hasnan, descending));
}

template <typename T>
inline void qselect(T *arr, size_t k, size_t size, bool hasnan = false, bool descending = false)
{
    detail::check(xss_qselect(detail::key_dt<T>(), arr, k, size, hasnan, descending));
}

template <typename T>
inline void partial_qsort(T *arr, size_t k, size_t size, bool hasnan = false,
                          bool descending = false)
{
    detail::check(xss_partial_qsort(detail::key_dt<T>(), arr, k, size, hasnan, descending));
}

// argsort API required by NumPy: indices into a caller array
template <typename T>
inline void argsort(T *arr, size_t *arg, size_t size, bool hasnan = false, bool descending = false)
{
    static_assert(sizeof(size_t) == sizeof(uint64_t), "64-bit size_t");
    detail::check(xss_argsort(detail::key_dt<T>(), arr, reinterpret_cast<uint64_t *>(arg), size,
                              hasnan, descending));
}

template <typename T>
inline std::vector<size_t> argsort(T *arr, size_t size, bool hasnan = false,
                                   bool descending = false)
{
    std::vector<size_t> arg(size);
    if (size) argsort(arr, arg.data(), size, hasnan, descending);
    return arg;
}

// argselect API required by NumPy
template <typename T>
inline void argselect(T *arr, size_t *arg, size_t k, size_t size, bool hasnan = false)
{
    static_assert(sizeof(size_t) == sizeof(uint64_t), "64-bit size_t");
    detail::check(xss_argselect(detail::key_dt<T>(), arr, reinterpret_cast<uint64_t *>(arg), k,
                                size, hasnan));
}

template <typename T>
inline std::vector<size_t> argselect(T *arr, size_t k, size_t size, bool hasnan = false)
{
    std::vector<size_t> arg(size);
    if (size) argselect(arr, arg.data(), k, size, hasnan);
    return arg;
}

template <typename T1, typename T2>
inline void keyvalue_qsort(T1 *key, T2 *val, size_t size, bool hasnan = false,
                           bool descending = false)
{
    detail::check(xss_keyvalue_qsort(detail::key_dt<T1>(), detail::key_dt<T2>(), key, val, size,
                                     hasnan, descending));
}

template <typename T1, typename T2>
inline void keyvalue_select(T1 *key, T2 *val, size_t k, size_t size, bool hasnan = false,
                            bool descending = false)
{
    detail::check(xss_keyvalue_select(detail::key_dt<T1>(), detail::key_dt<T2>(), key, val, k,
                                      size, hasnan, descending));
}

template <typename T1, typename T2>
inline void keyvalue_partial_sort(T1 *key, T2 *val, size_t k, size_t size, bool hasnan = false,
                                  bool descending = false)
{
    detail::check(xss_keyvalue_partial_sort(detail::key_dt<T1>(), detail::key_dt<T2>(), key, val,
                                            k, size, hasnan, descending));
}

}  // namespace x86simdsortStatic

#endif
