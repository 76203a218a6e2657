// xss_cxx.cpp -- explicit specialisations of the x86simdsort:: templates
// (include/x86simdsort.h) over the host-pointer C ABI.  The type set is the
// reference's (lib/x86simdsort.cpp:167-293).
#include "../../include/x86simdsort.h"

static_assert(sizeof(size_t) == sizeof(uint64_t), "argsort indices are 64-bit");

namespace x86simdsort {

namespace {
inline void ok(int rc) { gpu::check(rc); }
}  // namespace

#define XSS_DEFINE_ARRAY_FUNCS(T)                                                            \
    template <>                                                                              \
    void qsort<T>(T * arr, size_t arrsize, bool hasnan, bool descending)                     \
    {                                                                                        \
        ok(xss_qsort(gpu::dtype_of<T>::value, arr, arrsize, hasnan, descending));            \
    }                                                                                        \
    template <>                                                                              \
    void qselect<T>(T * arr, size_t k, size_t arrsize, bool hasnan, bool descending)        \
    {                                                                                        \
        ok(xss_qselect(gpu::dtype_of<T>::value, arr, k, arrsize, hasnan, descending));       \
    }                                                                                        \
    template <>                                                                              \
    void partial_qsort<T>(T * arr, size_t k, size_t arrsize, bool hasnan, bool descending)  \
    {                                                                                        \
        ok(xss_partial_qsort(gpu::dtype_of<T>::value, arr, k, arrsize, hasnan, descending)); \
    }                                                                                        \
    template <>                                                                              \
    std::vector<size_t> argsort<T>(T * arr, size_t arrsize, bool hasnan, bool descending)   \
    {                                                                                        \
        std::vector<size_t> arg(arrsize);                                                    \
        ok(xss_argsort(gpu::dtype_of<T>::value, arr, reinterpret_cast<uint64_t *>(arg.data()), \
                       arrsize, hasnan, descending));                                        \
        return arg;                                                                          \
    }                                                                                        \
    template <>                                                                              \
    std::vector<size_t> argselect<T>(T * arr, size_t k, size_t arrsize, bool hasnan)        \
    {                                                                                        \
        std::vector<size_t> arg(arrsize);                                                    \
        ok(xss_argselect(gpu::dtype_of<T>::value, arr,                                       \
                         reinterpret_cast<uint64_t *>(arg.data()), k, arrsize, hasnan));     \
        return arg;                                                                          \
    }

XSS_DEFINE_ARRAY_FUNCS(uint16_t)
XSS_DEFINE_ARRAY_FUNCS(int16_t)
XSS_DEFINE_ARRAY_FUNCS(uint32_t)
XSS_DEFINE_ARRAY_FUNCS(int32_t)
XSS_DEFINE_ARRAY_FUNCS(float)
XSS_DEFINE_ARRAY_FUNCS(uint64_t)
XSS_DEFINE_ARRAY_FUNCS(int64_t)
XSS_DEFINE_ARRAY_FUNCS(double)
#ifdef __FLT16_MAX__
XSS_DEFINE_ARRAY_FUNCS(_Float16)
#endif

#define XSS_DEFINE_KV_FUNCS(T1, T2)                                                          \
    template <>                                                                              \
    void keyvalue_qsort<T1, T2>(T1 * key, T2 * val, size_t arrsize, bool hasnan,             \
                                bool descending)                                             \
    {                                                                                        \
        ok(xss_keyvalue_qsort(gpu::dtype_of<T1>::value, gpu::dtype_of<T2>::value, key, val,  \
                              arrsize, hasnan, descending));                                 \
    }                                                                                        \
    template <>                                                                              \
    void keyvalue_select<T1, T2>(T1 * key, T2 * val, size_t k, size_t arrsize, bool hasnan,  \
                                 bool descending)                                            \
    {                                                                                        \
        ok(xss_keyvalue_select(gpu::dtype_of<T1>::value, gpu::dtype_of<T2>::value, key, val, \
                               k, arrsize, hasnan, descending));                             \
    }                                                                                        \
    template <>                                                                              \
    void keyvalue_partial_sort<T1, T2>(T1 * key, T2 * val, size_t k, size_t arrsize,         \
                                       bool hasnan, bool descending)                         \
    {                                                                                        \
        ok(xss_keyvalue_partial_sort(gpu::dtype_of<T1>::value, gpu::dtype_of<T2>::value,     \
                                     key, val, k, arrsize, hasnan, descending));             \
    }

#define XSS_DEFINE_KV_FOR_KEY(T1)      \
    XSS_DEFINE_KV_FUNCS(T1, uint32_t)  \
    XSS_DEFINE_KV_FUNCS(T1, int32_t)   \
    XSS_DEFINE_KV_FUNCS(T1, float)     \
    XSS_DEFINE_KV_FUNCS(T1, uint64_t)  \
    XSS_DEFINE_KV_FUNCS(T1, int64_t)   \
    XSS_DEFINE_KV_FUNCS(T1, double)

XSS_DEFINE_KV_FOR_KEY(uint32_t)
XSS_DEFINE_KV_FOR_KEY(int32_t)
XSS_DEFINE_KV_FOR_KEY(float)
XSS_DEFINE_KV_FOR_KEY(uint64_t)
XSS_DEFINE_KV_FOR_KEY(int64_t)
XSS_DEFINE_KV_FOR_KEY(double)

}  // namespace x86simdsort
