// xss_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of intel/x86-simd-sort's portable scalar path, used as the
// parity checker for the GPU library and as the timed CPU baseline.  It is
// never linked into, loaded by or called from the product library.
//
// What it restates:
//   * ordering rule of utils/custom-compare.h:11-34: NaN compares above every
//     number (including +inf), all NaNs compare equal, otherwise the usual
//     IEEE order (so -0.0 == +0.0);
//   * xss::scalar::{qsort, qselect, partial_qsort, argsort, argselect,
//     keyvalue_qsort, keyvalue_select, keyvalue_partial_sort}
//     (lib/x86simdsort-scalar.h:45-134): std::sort / std::nth_element /
//     std::partial_sort with that rule; keyvalue = argsort of the keys then
//     the permutation applied to both arrays; keyvalue select/partial = full
//     keyvalue sort;
//   * the OpenMP task-parallel quicksort structure of the vectorised path
//     (src/xss-common-qsort.h:529-605, 670-697: recursion branches become
//     tasks above max(1e5, n/100) elements for qsort, max(1e4, n/100) for
//     key-value and arg sorts, at most 16 threads, iteration cap
//     2*log2(n) then std::sort) with a scalar three-way partition in place of
//     the AVX-512 compress-store partition -- the *_mt entry points, which
//     serve as the CPU baseline on hosts without AVX-512.
//
// One deliberate difference: the reference's scalar qsort uses the plain
// std::less when hasnan is false; with NaNs present that is undefined
// behaviour for std::sort.  The oracle always uses the NaN-aware rule, which
// agrees with std::less whenever the input has no NaN.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <numeric>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/xss_gpu.h"

namespace {

template <typename T>
constexpr bool is_fp_v = std::is_floating_point<T>::value
#ifdef __FLT16_MAX__
                         || std::is_same<T, _Float16>::value
#endif
    ;

template <typename T> inline bool is_nan(T x)
{
    if constexpr (is_fp_v<T>) return x != x;
    else return false;
}

// Three-way order with NaN above everything and all NaNs equal.
template <typename T> inline int order(T a, T b)
{
    if constexpr (is_fp_v<T>) {
        const bool na = is_nan(a), nb = is_nan(b);
        if (na || nb) return na == nb ? 0 : (na ? 1 : -1);
    }
    return a < b ? -1 : (b < a ? 1 : 0);
}

template <typename T> struct Less {
    bool operator()(const T &a, const T &b) const { return order(a, b) < 0; }
};
template <typename T> struct Greater {
    bool operator()(const T &a, const T &b) const { return order(a, b) > 0; }
};

template <typename T, typename Cmp> struct ByKey {
    const T *keys;
    Cmp cmp;
    bool operator()(uint64_t a, uint64_t b) const { return cmp(keys[a], keys[b]); }
};

// ---- scalar path ----------------------------------------------------------
template <typename T> void s_qsort(T *a, size_t n, bool desc)
{
    if (desc) std::sort(a, a + n, Greater<T>());
    else std::sort(a, a + n, Less<T>());
}
template <typename T> void s_qselect(T *a, size_t k, size_t n, bool desc)
{
    if (desc) std::nth_element(a, a + k, a + n, Greater<T>());
    else std::nth_element(a, a + k, a + n, Less<T>());
}
template <typename T> void s_partial(T *a, size_t k, size_t n, bool desc)
{
    if (desc) std::partial_sort(a, a + k, a + n, Greater<T>());
    else std::partial_sort(a, a + k, a + n, Less<T>());
}
template <typename T> void s_argsort(const T *a, uint64_t *arg, size_t n, bool desc)
{
    std::iota(arg, arg + n, (uint64_t)0);
    if (desc) std::sort(arg, arg + n, ByKey<T, Greater<T>>{a, {}});
    else std::sort(arg, arg + n, ByKey<T, Less<T>>{a, {}});
}
template <typename T> void s_argselect(const T *a, uint64_t *arg, size_t k, size_t n)
{
    std::iota(arg, arg + n, (uint64_t)0);
    std::nth_element(arg, arg + k, arg + n, ByKey<T, Less<T>>{a, {}});
}
// out[i] = in[perm[i]] for both arrays
template <typename K, typename V> void s_kvsort(K *k, V *v, size_t n, bool desc)
{
    std::vector<uint64_t> p(n);
    s_argsort(k, p.data(), n, desc);
    std::vector<K> kk(n);
    std::vector<V> vv(n);
    for (size_t i = 0; i < n; ++i) {
        kk[i] = k[p[i]];
        vv[i] = v[p[i]];
    }
    std::copy(kk.begin(), kk.end(), k);
    std::copy(vv.begin(), vv.end(), v);
}

// ---- task-parallel quicksort (CPU baseline) ---------------------------------
template <typename It, typename Cmp>
void par_qsort(It lo, It hi, Cmp cmp, std::ptrdiff_t task_min, int iters)
{
    while (hi - lo > 512) {
        if (iters-- <= 0) {
            std::sort(lo, hi, cmp);
            return;
        }
        const auto x = *lo, y = *(lo + (hi - lo) / 2), z = *(hi - 1);
        const auto pivot = cmp(x, y) ? (cmp(y, z) ? y : (cmp(x, z) ? z : x))
                                     : (cmp(x, z) ? x : (cmp(y, z) ? z : y));
        It m1 = std::partition(lo, hi, [&](const auto &e) { return cmp(e, pivot); });
        It m2 = std::partition(m1, hi, [&](const auto &e) { return !cmp(pivot, e); });
        if (m1 - lo > task_min) {
#pragma omp task default(none) firstprivate(lo, m1, cmp, task_min, iters)
            par_qsort(lo, m1, cmp, task_min, iters);
        } else {
            par_qsort(lo, m1, cmp, task_min, iters);
        }
        lo = m2;
    }
    std::sort(lo, hi, cmp);
}

inline int clamp_threads(int t)
{
#ifdef _OPENMP
    if (t <= 0) t = omp_get_max_threads();
#else
    t = 1;
#endif
    return std::max(1, std::min(16, t));
}

template <typename It, typename Cmp>
void par_sort(It lo, It hi, Cmp cmp, size_t min_task, int threads)
{
    const size_t n = hi - lo;
    const std::ptrdiff_t task_min = (std::ptrdiff_t)std::max(min_task, n / 100);
    const int iters = 2 * (int)std::log2((double)std::max<size_t>(n, 2));
#ifdef _OPENMP
#pragma omp parallel num_threads(threads)
#pragma omp single
#else
    (void)threads;
#endif
    par_qsort(lo, hi, cmp, task_min, iters);
}

template <typename T> void m_qsort(T *a, size_t n, bool desc, int threads)
{
    if (desc) par_sort(a, a + n, Greater<T>(), 100000, threads);
    else par_sort(a, a + n, Less<T>(), 100000, threads);
}
template <typename T> void m_argsort(const T *a, uint64_t *arg, size_t n, bool desc, int threads)
{
    std::iota(arg, arg + n, (uint64_t)0);
    if (desc) par_sort(arg, arg + n, ByKey<T, Greater<T>>{a, {}}, 10000, threads);
    else par_sort(arg, arg + n, ByKey<T, Less<T>>{a, {}}, 10000, threads);
}
template <typename K, typename V> struct Pair {
    K k;
    V v;
};
template <typename K, typename V> void m_kvsort(K *k, V *v, size_t n, bool desc, int threads)
{
    std::vector<Pair<K, V>> p(n);
    for (size_t i = 0; i < n; ++i) p[i] = {k[i], v[i]};
    auto lt = [](const Pair<K, V> &a, const Pair<K, V> &b) { return order(a.k, b.k) < 0; };
    auto gt = [](const Pair<K, V> &a, const Pair<K, V> &b) { return order(a.k, b.k) > 0; };
    if (desc) par_sort(p.begin(), p.end(), gt, 10000, threads);
    else par_sort(p.begin(), p.end(), lt, 10000, threads);
    for (size_t i = 0; i < n; ++i) {
        k[i] = p[i].k;
        v[i] = p[i].v;
    }
}

// ---- dtype dispatch -----------------------------------------------------------
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
    // 16-bit payloads (beyond the reference's 32/64-bit values): values only
    // move with their keys, so _Float16 values travel as their bits
    case XSS_DT_U16: f((uint16_t *)nullptr); return 0;
    case XSS_DT_I16: f((int16_t *)nullptr); return 0;
    case XSS_DT_F16: f((uint16_t *)nullptr); return 0;
    case XSS_DT_U32: f((uint32_t *)nullptr); return 0;
    case XSS_DT_I32: f((int32_t *)nullptr); return 0;
    case XSS_DT_F32: f((float *)nullptr); return 0;
    case XSS_DT_U64: f((uint64_t *)nullptr); return 0;
    case XSS_DT_I64: f((int64_t *)nullptr); return 0;
    case XSS_DT_F64: f((double *)nullptr); return 0;
    default: return XSS_EINVAL;
    }
}

}  // namespace

extern "C" {

int xo_qsort(int dt, void *a, size_t n, int hasnan, int desc)
{
    (void)hasnan;
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        if (n > 1) s_qsort((T *)a, n, desc);
    });
}
int xo_qselect(int dt, void *a, size_t k, size_t n, int hasnan, int desc)
{
    (void)hasnan;
    if (n > 1 && k >= n) return XSS_EINVAL;
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        if (n > 1) s_qselect((T *)a, k, n, desc);
    });
}
int xo_partial_qsort(int dt, void *a, size_t k, size_t n, int hasnan, int desc)
{
    (void)hasnan;
    if (k > n) return XSS_EINVAL;
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        if (n > 1 && k > 0) s_partial((T *)a, k, n, desc);
    });
}
int xo_argsort(int dt, const void *a, uint64_t *arg, size_t n, int hasnan, int desc)
{
    (void)hasnan;
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        s_argsort((const T *)a, arg, n, desc);
    });
}
int xo_argselect(int dt, const void *a, uint64_t *arg, size_t k, size_t n, int hasnan)
{
    (void)hasnan;
    if (n > 1 && k >= n) return XSS_EINVAL;
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        if (n == 0) return;
        if (n == 1) arg[0] = 0;
        else s_argselect((const T *)a, arg, k, n);
    });
}
int xo_keyvalue_qsort(int kdt, int vdt, void *k, void *v, size_t n, int hasnan, int desc)
{
    (void)hasnan;
    int rc = 0;
    const int r1 = with_key(kdt, [&](auto *kt) {
        using K = std::remove_pointer_t<decltype(kt)>;
        rc = with_val(vdt, [&](auto *vt) {
            using V = std::remove_pointer_t<decltype(vt)>;
            if (n > 1) s_kvsort((K *)k, (V *)v, n, desc);
        });
    });
    return r1 ? r1 : rc;
}
int xo_keyvalue_select(int kdt, int vdt, void *k, void *v, size_t kk, size_t n, int hasnan,
                       int desc)
{
    if (n > 1 && kk >= n) return XSS_EINVAL;
    return xo_keyvalue_qsort(kdt, vdt, k, v, n, hasnan, desc);
}
int xo_keyvalue_partial_sort(int kdt, int vdt, void *k, void *v, size_t kk, size_t n,
                             int hasnan, int desc)
{
    if (kk > n) return XSS_EINVAL;
    return xo_keyvalue_qsort(kdt, vdt, k, v, n, hasnan, desc);
}

// Comparator known-answer hook: op 0 <, 1 <=, 2 >, 3 >=, 4 ==.
int xo_compare(int dt, int op, const void *a, const void *b)
{
    int res = -1;
    with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        T x, y;
        std::memcpy(&x, a, sizeof(T));
        std::memcpy(&y, b, sizeof(T));
        const int o = order(x, y);
        switch (op) {
        case 0: res = o < 0; break;
        case 1: res = o <= 0; break;
        case 2: res = o > 0; break;
        case 3: res = o >= 0; break;
        case 4: res = o == 0; break;
        }
    });
    return res;
}

// ---- task-parallel CPU baseline ------------------------------------------------
int xo_max_threads(void) { return clamp_threads(0); }

int xo_qsort_mt(int dt, void *a, size_t n, int hasnan, int desc, int threads)
{
    (void)hasnan;
    const int th = clamp_threads(threads);
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        if (n > 1) m_qsort((T *)a, n, desc, th);
    });
}
int xo_argsort_mt(int dt, const void *a, uint64_t *arg, size_t n, int hasnan, int desc,
                  int threads)
{
    (void)hasnan;
    const int th = clamp_threads(threads);
    return with_key(dt, [&](auto *t) {
        using T = std::remove_pointer_t<decltype(t)>;
        m_argsort((const T *)a, arg, n, desc, th);
    });
}
int xo_keyvalue_qsort_mt(int kdt, int vdt, void *k, void *v, size_t n, int hasnan, int desc,
                         int threads)
{
    (void)hasnan;
    const int th = clamp_threads(threads);
    int rc = 0;
    const int r1 = with_key(kdt, [&](auto *kt) {
        using K = std::remove_pointer_t<decltype(kt)>;
        rc = with_val(vdt, [&](auto *vt) {
            using V = std::remove_pointer_t<decltype(vt)>;
            if (n > 1) m_kvsort((K *)k, (V *)v, n, desc, th);
        });
    });
    return r1 ? r1 : rc;
}

}  // extern "C"
