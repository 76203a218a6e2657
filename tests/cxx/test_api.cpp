// C++ drop-in check: code written against the reference's x86simdsort.h
// (lib/x86simdsort.h) compiles unchanged against include/x86simdsort.h and
// gives std::sort's results, now computed on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <stdexcept>
#include <vector>

#include "x86simdsort.h"
#include "x86simdsort-static-incl.h"

#define CHECK(c)                                                             \
    do {                                                                     \
        if (!(c)) {                                                          \
            std::fprintf(stderr, "FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
            return 1;                                                        \
        }                                                                    \
    } while (0)

struct Point {
    double x, y;
};

// the record shape of the reference's example.c (object sort by a member)
struct Rec {
    int x;
    int y;
    float distance;
    uint64_t metric;
};

int main()
{
    std::mt19937 gen(0);
    std::uniform_real_distribution<float> uni(-1.0f, 1.0f);

    // qsort<float>, ascending, 2^20 keys -- checked against std::sort
    std::vector<float> a(1 << 20);
    for (auto &v : a) v = uni(gen);
    std::vector<float> b = a;
    x86simdsort::qsort(a.data(), a.size());
    std::sort(b.begin(), b.end());
    CHECK(std::memcmp(a.data(), b.data(), a.size() * sizeof(float)) == 0);

    // descending with NaN: the quiet NaN comes first
    std::vector<double> d(100000);
    std::normal_distribution<double> nd;
    for (auto &v : d) v = nd(gen);
    d[17] = std::nan("");
    d[99] = std::nan("");
    x86simdsort::qsort(d.data(), d.size(), true, true);
    CHECK(std::isnan(d[0]) && std::isnan(d[1]) && !std::isnan(d[2]));
    for (size_t i = 3; i < d.size(); ++i) CHECK(d[i - 1] >= d[i]);

    // argsort<double>: a permutation whose gathered keys are sorted
    std::vector<double> e(50000);
    for (auto &v : e) v = nd(gen);
    std::vector<size_t> arg = x86simdsort::argsort(e.data(), e.size());
    std::vector<size_t> chk = arg;
    std::sort(chk.begin(), chk.end());
    for (size_t i = 0; i < chk.size(); ++i) CHECK(chk[i] == i);
    for (size_t i = 1; i < arg.size(); ++i) CHECK(e[arg[i - 1]] <= e[arg[i]]);

    // keyvalue_qsort<int64_t, uint64_t>
    std::vector<int64_t> k(300000);
    std::vector<uint64_t> v(k.size());
    for (size_t i = 0; i < k.size(); ++i) {
        k[i] = (int64_t)(gen() % 1000) - 500;
        v[i] = i;
    }
    std::vector<int64_t> k0 = k;
    x86simdsort::keyvalue_qsort(k.data(), v.data(), k.size());
    for (size_t i = 1; i < k.size(); ++i) CHECK(k[i - 1] <= k[i]);
    for (size_t i = 0; i < k.size(); ++i) CHECK(k0[v[i]] == k[i]);

    // qselect / partial_qsort
    std::vector<float> s = b;
    std::shuffle(s.begin(), s.end(), gen);
    std::vector<float> p = s;
    x86simdsort::qselect(s.data(), 1000, s.size());
    CHECK(s[1000] == b[1000]);
    for (size_t i = 0; i < 1000; ++i) CHECK(s[i] <= s[1000]);
    x86simdsort::partial_qsort(p.data(), 1000, p.size());
    CHECK(std::memcmp(p.data(), b.data(), 1000 * sizeof(float)) == 0);

    // object_qsort by member
    std::vector<Point> objs(100000);
    for (auto &o : objs) o = {nd(gen), nd(gen)};
    std::vector<Point> ref = objs;
    x86simdsort::object_qsort(objs.data(), objs.size(), [](Point q) { return q.x; });
    std::sort(ref.begin(), ref.end(), [](const Point &l, const Point &r) { return l.x < r.x; });
    for (size_t i = 0; i < objs.size(); ++i) CHECK(objs[i].x == ref[i].x && objs[i].y == ref[i].y);

    // device-pointer overloads
    float *d_arr = nullptr;
    CHECK(cudaMalloc(&d_arr, a.size() * sizeof(float)) == cudaSuccess);
    std::vector<float> c(a.size());
    for (auto &x : c) x = uni(gen);
    std::vector<float> cs = c;
    std::sort(cs.begin(), cs.end(), std::greater<float>());
    CHECK(cudaMemcpy(d_arr, c.data(), c.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess);
    x86simdsort::gpu::qsort(d_arr, c.size(), false, true);
    x86simdsort::gpu::synchronize();
    CHECK(cudaMemcpy(c.data(), d_arr, c.size() * 4, cudaMemcpyDeviceToHost) == cudaSuccess);
    CHECK(c == cs);
    cudaFree(d_arr);

    // device record sort by a member key; equal keys keep their input order
    std::vector<Rec> recs(200000);
    for (size_t i = 0; i < recs.size(); ++i)
        recs[i] = {(int)i, (int)(gen() % 7), uni(gen), (uint64_t)(gen() % 5000)};
    Rec *d_recs = nullptr;
    CHECK(cudaMalloc(&d_recs, recs.size() * sizeof(Rec)) == cudaSuccess);
    for (int by = 0; by < 2; ++by) {
        CHECK(cudaMemcpy(d_recs, recs.data(), recs.size() * sizeof(Rec), cudaMemcpyHostToDevice) ==
              cudaSuccess);
        std::vector<Rec> want = recs;
        if (by == 0) {
            x86simdsort::gpu::object_qsort(d_recs, recs.size(), &Rec::metric);
            std::stable_sort(want.begin(), want.end(),
                             [](const Rec &l, const Rec &r) { return l.metric < r.metric; });
        } else {
            x86simdsort::gpu::object_qsort(d_recs, recs.size(), &Rec::distance, false, true);
            std::stable_sort(want.begin(), want.end(),
                             [](const Rec &l, const Rec &r) { return l.distance > r.distance; });
        }
        x86simdsort::gpu::synchronize();
        std::vector<Rec> got(recs.size());
        CHECK(cudaMemcpy(got.data(), d_recs, got.size() * sizeof(Rec), cudaMemcpyDeviceToHost) ==
              cudaSuccess);
        for (size_t i = 0; i < got.size(); ++i)   // member-wise: padding bytes are unspecified
            CHECK(got[i].x == want[i].x && got[i].y == want[i].y &&
                  got[i].distance == want[i].distance && got[i].metric == want[i].metric);
    }
    cudaFree(d_recs);

    // the header-only static API (namespace x86simdsortStatic), NumPy's argsort form
    {
        std::vector<double> sv(70000);
        for (auto &x : sv) x = nd(gen);
        std::vector<double> sref = sv;
        std::vector<size_t> sarg(sv.size());
        x86simdsortStatic::argsort(sv.data(), sarg.data(), sv.size());
        std::sort(sref.begin(), sref.end());
        for (size_t i = 0; i < sv.size(); ++i) CHECK(sv[sarg[i]] == sref[i]);
        x86simdsortStatic::qsort(sv.data(), sv.size());
        CHECK(sv == sref);
        std::vector<uint32_t> kk(5000), vv(5000);
        for (size_t i = 0; i < kk.size(); ++i) { kk[i] = (uint32_t)(gen() % 97); vv[i] = (uint32_t)i; }
        std::vector<uint32_t> k0 = kk;
        x86simdsortStatic::keyvalue_qsort(kk.data(), vv.data(), kk.size());
        for (size_t i = 0; i < kk.size(); ++i) CHECK(k0[vv[i]] == kk[i] && (i == 0 || kk[i - 1] <= kk[i]));
    }

    // errors surface as exceptions (the reference has no error channel)
    bool threw = false;
    try {
        x86simdsort::qselect(a.data(), a.size(), a.size());
    } catch (const std::runtime_error &) {
        threw = true;
    }
    CHECK(threw);

    std::puts("cxx api ok");
    return 0;
}
