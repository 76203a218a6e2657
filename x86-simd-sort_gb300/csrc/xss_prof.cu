// xss_prof.cu -- per-kernel launch counters and optional CUDA-event timing.
//
// Every kernel launch site brackets its launch with prof_begin / prof_end.
// Launch counts are always kept.  When timing is enabled (xss_prof_enable),
// an event pair is recorded on the launching stream around each launch and
// xss_prof_read turns them into per-kernel-kind totals.
#include <atomic>
#include <mutex>
#include <vector>
#include "xss_internal.cuh"
#include "xss_prof.cuh"

namespace xss {

static std::atomic<bool> g_prof_on{false};
static std::atomic<unsigned long long> g_launches[PK_COUNT];
static std::mutex g_prof_mu;
struct Pending {
    int kind;
    cudaEvent_t a, b;
};
static std::vector<Pending> g_pending;
static std::vector<cudaEvent_t> g_free;
static double g_ms[PK_COUNT];
static unsigned long long g_timed[PK_COUNT];
static thread_local cudaEvent_t t_open[PK_COUNT];

static cudaEvent_t take_event()
{
    if (!g_free.empty()) {
        cudaEvent_t e = g_free.back();
        g_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void prof_begin(cudaStream_t s, int kind)
{
    if (!g_prof_on.load(std::memory_order_relaxed)) return;
    // launches being captured into a graph are counted, not timed
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return;
    }
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEvent_t e = take_event();
    cudaEventRecord(e, s);
    t_open[kind] = e;
}

void prof_snapshot(unsigned long long *out)
{
    for (int k = 0; k < PK_COUNT; ++k) out[k] = g_launches[k].load();
}

void prof_add(const unsigned long long *counts)
{
    for (int k = 0; k < PK_COUNT; ++k)
        if (counts[k]) g_launches[k].fetch_add(counts[k], std::memory_order_relaxed);
}

void prof_sub(const unsigned long long *counts)
{
    for (int k = 0; k < PK_COUNT; ++k)
        if (counts[k]) g_launches[k].fetch_sub(counts[k], std::memory_order_relaxed);
}

void prof_end(cudaStream_t s, int kind)
{
    g_launches[kind].fetch_add(1, std::memory_order_relaxed);
    if (!g_prof_on.load(std::memory_order_relaxed) || !t_open[kind]) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEvent_t e = take_event();
    cudaEventRecord(e, s);
    g_pending.push_back({kind, t_open[kind], e});
    t_open[kind] = nullptr;
}

static void drain()
{
    for (auto &p : g_pending) {
        cudaEventSynchronize(p.b);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            g_ms[p.kind] += ms;
            g_timed[p.kind] += 1;
        }
        g_free.push_back(p.a);
        g_free.push_back(p.b);
    }
    g_pending.clear();
}

}  // namespace xss

using namespace xss;

extern "C" {

// Enable (1) or disable (0) event timing of every kernel launch.
void xss_prof_enable(int on) { g_prof_on.store(on != 0); }

// Zero the timing totals (launch counters keep running).
void xss_prof_reset(void)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    drain();
    for (int k = 0; k < PK_COUNT; ++k) {
        g_ms[k] = 0.0;
        g_timed[k] = 0;
    }
}

// Total event-timed milliseconds and timed launches of `kind` since the last
// reset (waits for outstanding events).  Returns -1 for an unknown kind.
int xss_prof_read(int kind, double *total_ms, unsigned long long *timed_launches)
{
    if (kind < 0 || kind >= PK_COUNT) return -1;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    drain();
    if (total_ms) *total_ms = g_ms[kind];
    if (timed_launches) *timed_launches = g_timed[kind];
    return 0;
}

// Launches of `kind` since the library was loaded (always counted).
unsigned long long xss_prof_launches(int kind)
{
    if (kind < 0 || kind >= PK_COUNT) return 0;
    return g_launches[kind].load();
}

const char *xss_prof_kind_name(int kind)
{
    static const char *names[PK_COUNT] = {"hist", "onesweep", "fixup", "small_sort",
                                          "sel_hist", "sel_find", "sel_collect", "sel_place",
                                          "seg_small", "seg_block", "seg_misc", "object",
                                          "merge", "count16"};
    return (kind >= 0 && kind < PK_COUNT) ? names[kind] : "unknown";
}

}  // extern "C"
