// refshim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// extern "C" wrappers around the reference library itself (intel/x86-simd-sort,
// lib/x86simdsort.h), compiled from the reference's own sources by
// oracle/Makefile into oracle/_ref/.  Used to generate golden fixtures and to
// pin the CPU oracle against the real reference on hosts where it builds
// (x86-64 with AVX2/AVX-512).  Same signatures as the oracle's xo_* functions.
#include <cstdint>
#include <cstring>
#include <vector>
#include "x86simdsort.h"
#include "../include/xss_gpu.h"

namespace {
template <typename F> int with_key(int dt, F &&f)
{
    switch (dt) {
    case XSS_DT_U16: f((uint16_t *)nullptr); return 0;
    case XSS_DT_I16: f((int16_t *)nullptr); return 0;
#ifdef __FLT16_MAX__
    case XSS_DT_F16: f((_Float16 *)nullptr); return 0;
#endif
    case XSS_DT_U32: f((uint32_t *)nullptr); return 0;
    case XSS_DT_I32: f((int32_t *)nullptr); return 0;
    case XSS_DT_F32: f((float *)nullptr); return 0;
    case XSS_DT_U64: f((uint64_t *)nullptr); return 0;
    case XSS_DT_I64: f((int64_t *)nullptr); return 0;
    case XSS_DT_F64: f((double *)nullptr); return 0;
    default: return XSS_EINVAL;
    }
}
template <typename F> int with_val(int dt, F &&f)
{
    switch (dt) {
    case XSS_DT_U32: f((uint32_t *)nullptr); return 0;
    case XSS_DT_I32: f((int32_t *)nullptr); return 0;
    case XSS_DT_F32: f((float *)nullptr); return 0;
    case XSS_DT_U64: f((uint64_t *)nullptr); return 0;
    case XSS_DT_I64: f((int64_t *)nullptr); return 0;
    case XSS_DT_F64: f((double *)nullptr); return 0;
    default: return XSS_EINVAL;
    }
}
template <typename F> int with_kv(int kdt, int vdt, F &&f)
{
    int rc = 0;
    const int r1 = with_key(kdt, [&](auto *kt) {
        if constexpr (sizeof(*kt) >= 4) rc = with_val(vdt, [&](auto *vt) { f(kt, vt); });
        else rc = XSS_EUNSUPPORTED;
    });
    return r1 ? r1 : rc;
}
}  // namespace

extern "C" {

int xr_qsort(int dt, void *a, size_t n, int hasnan, int desc)
{
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        x86simdsort::qsort((T *)a, n, hasnan, desc);
    });
}
int xr_qselect(int dt, void *a, size_t k, size_t n, int hasnan, int desc)
{
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        x86simdsort::qselect((T *)a, k, n, hasnan, desc);
    });
}
int xr_partial_qsort(int dt, void *a, size_t k, size_t n, int hasnan, int desc)
{
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        x86simdsort::partial_qsort((T *)a, k, n, hasnan, desc);
    });
}
int xr_argsort(int dt, const void *a, uint64_t *arg, size_t n, int hasnan, int desc)
{
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        std::vector<size_t> r = x86simdsort::argsort((T *)a, n, hasnan, desc);
        std::memcpy(arg, r.data(), n * sizeof(uint64_t));
    });
}
int xr_argselect(int dt, const void *a, uint64_t *arg, size_t k, size_t n, int hasnan)
{
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        std::vector<size_t> r = x86simdsort::argselect((T *)a, k, n, hasnan);
        std::memcpy(arg, r.data(), n * sizeof(uint64_t));
    });
}
int xr_keyvalue_qsort(int kdt, int vdt, void *k, void *v, size_t n, int hasnan, int desc)
{
    return with_kv(kdt, vdt, [&](auto *kt, auto *vt) {
        using K = std::remove_pointer_t<decltype(kt)>;
        using V = std::remove_pointer_t<decltype(vt)>;
        x86simdsort::keyvalue_qsort((K *)k, (V *)v, n, hasnan, desc);
    });
}
int xr_keyvalue_select(int kdt, int vdt, void *k, void *v, size_t kk, size_t n, int hasnan,
                       int desc)
{
    return with_kv(kdt, vdt, [&](auto *kt, auto *vt) {
        using K = std::remove_pointer_t<decltype(kt)>;
        using V = std::remove_pointer_t<decltype(vt)>;
        x86simdsort::keyvalue_select((K *)k, (V *)v, kk, n, hasnan, desc);
    });
}
int xr_keyvalue_partial_sort(int kdt, int vdt, void *k, void *v, size_t kk, size_t n,
                             int hasnan, int desc)
{
    return with_kv(kdt, vdt, [&](auto *kt, auto *vt) {
        using K = std::remove_pointer_t<decltype(kt)>;
        using V = std::remove_pointer_t<decltype(vt)>;
        x86simdsort::keyvalue_partial_sort((K *)k, (V *)v, kk, n, hasnan, desc);
    });
}

}  // extern "C"
