// xss_keys.cuh -- order-preserving key codes for the nine reference key types.
//
// Every kernel in this library sorts unsigned "codes" of the key width
// (16, 32 or 64 bits).  The code is a bijection of the key's bit pattern whose
// unsigned order equals the reference comparator's order:
//
//   * unsigned ints: identity;  signed ints: flip the sign bit;
//   * floats (_Float16, float, double): the usual sign-magnitude flip
//     (negative: all bits inverted; positive: sign bit set), then rotated down
//     by the number of negative-NaN patterns so that every NaN -- positive or
//     negative payload -- lands above +inf.  This is the reference's
//     "NaN is larger than +inf" rule (utils/custom-compare.h:11-34,
//     src/xss-common-qsort.h:54-79) without losing payload bits, which the
//     key-value and arg paths keep (src/xss-common-keyvaluesort.hpp:14-73);
//   * descending: bitwise NOT of the ascending code, so NaNs come first, as
//     the reference's reverse-after-ascending-sort gives
//     (src/xss-common-keyvaluesort.hpp:643-646, src/xss-common-argsort.h:662).
//
// -0.0 and +0.0 get distinct, adjacent codes (-0 first); the reference treats
// them as equal (_CMP_GE_OQ, src/avx512-32bit-qsort.hpp:388-446) so any
// relative order of the two is a valid reference result.
#pragma once
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#define XSS_HD __host__ __device__ __forceinline__

enum XssKind : int { XK_UINT = 0, XK_INT = 1, XK_FLOAT = 2 };

template <typename C> struct CodeTraits;
template <> struct CodeTraits<uint16_t> {
    static constexpr uint16_t sign = 0x8000u;
    static constexpr uint16_t exp_mask = 0x7c00u;
    static constexpr uint16_t neg_nans = 0x03ffu;       // NaN patterns per sign
    static constexpr uint16_t canon_nan = 0x7c01u;      // src/xss-custom-float.h:81-85
    static constexpr int bits = 16;
};
template <> struct CodeTraits<uint32_t> {
    static constexpr uint32_t sign = 0x80000000u;
    static constexpr uint32_t exp_mask = 0x7f800000u;
    static constexpr uint32_t neg_nans = 0x007fffffu;
    static constexpr uint32_t canon_nan = 0x7fc00000u;  // std::numeric_limits<float>::quiet_NaN
    static constexpr int bits = 32;
};
template <> struct CodeTraits<uint64_t> {
    static constexpr uint64_t sign = 0x8000000000000000ull;
    static constexpr uint64_t exp_mask = 0x7ff0000000000000ull;
    static constexpr uint64_t neg_nans = 0x000fffffffffffffull;
    static constexpr uint64_t canon_nan = 0x7ff8000000000000ull;
    static constexpr int bits = 64;
};

// Runtime description of the key transform; uniform across a launch.
struct KeyXform {
    int kind;    // XssKind
    int desc;    // descending order
    int canon;   // rewrite every NaN to the canonical quiet NaN (qsort with hasnan)
};

template <typename C> XSS_HD bool bits_isnan(C b)
{
    return C(b & C(~CodeTraits<C>::sign)) > CodeTraits<C>::exp_mask;
}

template <typename C> XSS_HD C to_code(C b, const KeyXform &x)
{
    using T = CodeTraits<C>;
    C c;
    if (x.kind == XK_FLOAT) {
        if (x.canon && bits_isnan(b)) b = T::canon_nan;
        c = (b & T::sign) ? C(~b) : C(b | T::sign);
        c = C(c - T::neg_nans);
    } else if (x.kind == XK_INT) {
        c = C(b ^ T::sign);
    } else {
        c = b;
    }
    return x.desc ? C(~c) : c;
}

template <typename C> XSS_HD C from_code(C c, const KeyXform &x)
{
    using T = CodeTraits<C>;
    if (x.desc) c = C(~c);
    if (x.kind == XK_FLOAT) {
        c = C(c + T::neg_nans);
        return (c & T::sign) ? C(c ^ T::sign) : C(~c);
    } else if (x.kind == XK_INT) {
        return C(c ^ T::sign);
    }
    return c;
}

// The same bijection in branch-free form, for the radix passes: masks built
// once per launch from the KeyXform, then per key a shift, two logic ops and
// a subtraction each way.  With s = the key's sign bit spread over the word:
//   code = ((b ^ ((s & fm) | sm)) - sub) ^ dm
// fm = all ones for floats (negative floats invert), sm = the sign bit for
// signed and float keys, sub = the negative-NaN count for floats (rotation),
// dm = all ones for descending.  from_canon additionally writes the canonical
// quiet NaN for every NaN code when the sort canonicalises (qsort with hasnan):
// NaN codes are exactly the ascending codes above the code of +inf.
template <typename C> struct Codec {
    using T = CodeTraits<C>;
    using S = typename std::conditional<sizeof(C) == 2, int16_t,
              typename std::conditional<sizeof(C) == 4, int32_t, int64_t>::type>::type;
    C fm, sm, sub, dm, thr;

    XSS_HD explicit Codec(const KeyXform &x)
    {
        const bool fl = x.kind == XK_FLOAT;
        fm = fl ? C(~C(0)) : C(0);
        sm = x.kind != XK_UINT ? T::sign : C(0);
        sub = fl ? T::neg_nans : C(0);
        dm = x.desc ? C(~C(0)) : C(0);
        thr = (fl && x.canon) ? C(C(T::exp_mask | T::sign) - T::neg_nans) : C(~C(0));
    }
    XSS_HD static C spread_sign(C v) { return C(S(v) >> (T::bits - 1)); }
    XSS_HD C to(C b) const
    {
        return C(C(C(b ^ C(C(spread_sign(b) & fm) | sm)) - sub) ^ dm);
    }
    XSS_HD C from(C c) const
    {
        const C u = C(C(c ^ dm) + sub);
        return C(u ^ C(C(C(~spread_sign(u)) & fm) | sm));
    }
    XSS_HD C from_canon(C c) const
    {
        return C(c ^ dm) > thr ? T::canon_nan : from(c);
    }
};

// Canonicalise a raw key in place of a full round trip (used when no radix
// pass runs because every code is equal).
template <typename C> XSS_HD C canon_bits(C b, const KeyXform &x)
{
    if (x.kind == XK_FLOAT && x.canon && bits_isnan(b)) return CodeTraits<C>::canon_nan;
    return b;
}

// Status word bits a kernel may raise in the workspace error word.
enum : unsigned {
    XSS_DEVERR_TIMEOUT = 1u,   // decoupled look-back spin exceeded its limit
    XSS_DEVERR_BOUNDS = 2u     // an index check failed (debug checks)
};

// Spin limit for every device-side wait (look-back).  At well under a
// microsecond per probe this bounds a wait to about a second.
#ifndef XSS_SPIN_LIMIT
#define XSS_SPIN_LIMIT (1u << 20)
#endif

__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t *p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// N consecutive status words (N = 1, 2, 4; p aligned to 4N bytes).  Each
// 32-bit element is read / written as one relaxed access of its own.
template <int N> __device__ __forceinline__ void ld_relaxed_vec(const uint32_t *p, uint32_t (&v)[N])
{
    static_assert(N == 1 || N == 2 || N == 4, "1, 2 or 4 words");
    if constexpr (N == 1) {
        v[0] = ld_relaxed_u32(p);
    } else if constexpr (N == 2) {
        asm volatile("ld.relaxed.gpu.global.v2.u32 {%0, %1}, [%2];"
                     : "=r"(v[0]), "=r"(v[1]) : "l"(p) : "memory");
    } else {
        asm volatile("ld.relaxed.gpu.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]) : "l"(p) : "memory");
    }
}
template <int N> __device__ __forceinline__ void st_relaxed_vec(uint32_t *p, const uint32_t (&v)[N])
{
    static_assert(N == 1 || N == 2 || N == 4, "1, 2 or 4 words");
    if constexpr (N == 1) {
        st_relaxed_u32(p, v[0]);
    } else if constexpr (N == 2) {
        asm volatile("st.relaxed.gpu.global.v2.u32 [%0], {%1, %2};"
                     ::"l"(p), "r"(v[0]), "r"(v[1]) : "memory");
    } else {
        asm volatile("st.relaxed.gpu.global.v4.u32 [%0], {%1, %2, %3, %4};"
                     ::"l"(p), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]) : "memory");
    }
}
