// Host-only wrappers of the library's key transform (xss_keys.cuh), compiled
// by the CPU tests to check the transform exhaustively without a GPU.
#include "../x86-simd-sort_gb300/csrc/xss_keys.cuh"

template <typename C>
static void fwd(const C *in, C *out, size_t n, int kind, int desc, int canon)
{
    const KeyXform x{kind, desc, canon};
    for (size_t i = 0; i < n; ++i) out[i] = to_code(in[i], x);
}
template <typename C>
static void inv(const C *in, C *out, size_t n, int kind, int desc)
{
    const KeyXform x{kind, desc, 0};
    for (size_t i = 0; i < n; ++i) out[i] = from_code(in[i], x);
}

// The radix passes' branch-free form (Codec): returns the number of keys whose
// to / from / from_canon disagree with to_code / from_code (+ canonical NaN).
template <typename C>
static size_t codec_mismatches(const C *in, size_t n, int kind, int desc, int canon)
{
    const KeyXform x{kind, desc, canon}, xn{kind, desc, 0};
    const Codec<C> cd(x);
    size_t bad = 0;
    for (size_t i = 0; i < n; ++i) {
        const C b = in[i], c = cd.to(b);
        const C want = (kind == XK_FLOAT && canon && bits_isnan(b)) ? CodeTraits<C>::canon_nan : b;
        bad += (c != to_code(b, xn)) + (cd.from(c) != b) + (cd.from_canon(c) != want);
    }
    return bad;
}

extern "C" {
void kh_to_code16(const uint16_t *i, uint16_t *o, size_t n, int k, int d, int c) { fwd(i, o, n, k, d, c); }
void kh_to_code32(const uint32_t *i, uint32_t *o, size_t n, int k, int d, int c) { fwd(i, o, n, k, d, c); }
void kh_to_code64(const uint64_t *i, uint64_t *o, size_t n, int k, int d, int c) { fwd(i, o, n, k, d, c); }
void kh_from_code16(const uint16_t *i, uint16_t *o, size_t n, int k, int d) { inv(i, o, n, k, d); }
void kh_from_code32(const uint32_t *i, uint32_t *o, size_t n, int k, int d) { inv(i, o, n, k, d); }
void kh_from_code64(const uint64_t *i, uint64_t *o, size_t n, int k, int d) { inv(i, o, n, k, d); }
size_t kh_codec16(const uint16_t *i, size_t n, int k, int d, int c) { return codec_mismatches(i, n, k, d, c); }
size_t kh_codec32(const uint32_t *i, size_t n, int k, int d, int c) { return codec_mismatches(i, n, k, d, c); }
size_t kh_codec64(const uint64_t *i, size_t n, int k, int d, int c) { return codec_mismatches(i, n, k, d, c); }
}
