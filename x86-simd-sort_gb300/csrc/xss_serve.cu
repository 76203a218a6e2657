// xss_serve.cu -- a request-serving loop over the sort/select entry points.
//
// Clients submit sort / select / argsort / key-value requests on host buffers;
// one scheduler thread per server:
//   * admits queued requests whenever the device pool (one allocation made at
//     start-up) has room for the request's data *and* its scratch, so requests
//     that arrive while others run are admitted as memory frees up
//     (continuous batching, not a queue drained in rounds);
//   * coalesces small keys-only and key-value requests of one kind into a
//     single batched segmented sort (xss_segmented.cu) -- a full sort also
//     satisfies select and partial-sort requests;
//   * gives each large request its own stream from a pool, so copies in,
//     kernels and copies out of different requests overlap on the device;
//   * records arrival -> completion latency per request (p50 / p99).
// Requests beyond the queue limit are refused at submission (shed).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>
#include "xss_internal.cuh"

namespace xss {

using Clock = std::chrono::steady_clock;

// First-fit allocator over one device allocation (256-byte granules).
class DevicePool {
public:
    int init(size_t bytes)
    {
        bytes = bytes / 256 * 256;
        if (cudaMalloc(&base_, bytes) != cudaSuccess) {
            cudaGetLastError();
            base_ = nullptr;
            return XSS_ENOMEM;
        }
        size_ = bytes;
        free_[0] = bytes;
        return XSS_OK;
    }
    ~DevicePool()
    {
        if (base_) cudaFree(base_);
    }
    void *alloc(size_t bytes)
    {
        bytes = align_up(std::max<size_t>(bytes, 1), 256);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                const size_t off = it->first, len = it->second;
                free_.erase(it);
                if (len > bytes) free_[off + bytes] = len - bytes;
                used_[off] = bytes;
                in_use_ += bytes;
                return static_cast<char *>(base_) + off;
            }
        }
        return nullptr;
    }
    void release(void *p)
    {
        if (!p) return;
        const size_t off = static_cast<char *>(p) - static_cast<char *>(base_);
        auto u = used_.find(off);
        if (u == used_.end()) return;
        size_t start = off, len = u->second;
        used_.erase(u);
        in_use_ -= len;
        auto nx = free_.lower_bound(start);
        if (nx != free_.end() && start + len == nx->first) {
            len += nx->second;
            nx = free_.erase(nx);
        }
        if (nx != free_.begin()) {
            auto pv = std::prev(nx);
            if (pv->first + pv->second == start) {
                start = pv->first;
                len += pv->second;
                free_.erase(pv);
            }
        }
        free_[start] = len;
    }
    size_t capacity() const { return size_; }
    size_t in_use() const { return in_use_; }

private:
    void *base_ = nullptr;
    size_t size_ = 0, in_use_ = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    std::map<size_t, size_t> used_;
};

static bool is_kv(int op) { return op >= XSS_OP_KV_QSORT; }
static bool is_arg(int op) { return op == XSS_OP_ARGSORT || op == XSS_OP_ARGSELECT; }
static size_t dt_bytes(int dt) { return dt <= XSS_DT_F16 ? 2 : (dt <= XSS_DT_F32 ? 4 : 8); }

struct Job {
    uint64_t ticket;
    xss_serve_request r;
    Clock::time_point arrival;
    int status = XSS_OK;
};

struct Inflight {
    std::vector<uint64_t> tickets;   // one for a single request, many for a batch
    std::vector<void *> blocks;      // pool blocks to release
    cudaEvent_t done = nullptr;
    size_t keys = 0;
};

}  // namespace xss

using namespace xss;

struct xss_server_s {
    xss_server_config cfg{};
    int device = 0;
    DevicePool pool;
    std::vector<cudaStream_t> streams;
    size_t next_stream = 0;
    cudaStream_t batch_stream = nullptr;

    std::mutex mu;                        // inbox, results, stats
    std::condition_variable cv_work, cv_done;
    std::deque<Job> inbox;
    std::unordered_map<uint64_t, int> finished;   // ticket -> status
    uint64_t next_ticket = 1;
    bool stopping = false, draining = false;

    // scheduler-thread state (queued_ is read by submitters)
    std::deque<Job> pending;
    std::atomic<size_t> queued_{0};
    std::vector<Inflight> inflight;
    std::unordered_map<uint64_t, Job> running;
    std::vector<cudaEvent_t> free_events;
    std::thread worker;

    // statistics (under mu)
    std::vector<double> lat_us;
    uint64_t submitted = 0, shed = 0, completed = 0, failed = 0, batches = 0, batched_reqs = 0;
    double keys_done = 0;
    Clock::time_point t0;

    cudaEvent_t take_event()
    {
        if (!free_events.empty()) {
            cudaEvent_t e = free_events.back();
            free_events.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        return e;
    }

    size_t request_bytes(const xss_serve_request &r) const
    {
        size_t b = align_up(r.n * dt_bytes(r.key_dtype), 256);
        if (is_kv(r.op)) b += align_up(r.n * dt_bytes(r.val_dtype), 256);
        if (is_arg(r.op)) b += align_up(r.n * 8, 256);
        return b;
    }

    size_t request_ws(const xss_serve_request &r) const
    {
        return align_up(xss_gpu_workspace_size(r.op, r.key_dtype, r.val_dtype, r.n, r.k), 256);
    }

    bool coalescible(const xss_serve_request &r) const
    {
        if (r.n > cfg.small_max) return false;
        return r.op == XSS_OP_QSORT || r.op == XSS_OP_QSELECT || r.op == XSS_OP_PARTIAL_QSORT ||
               r.op == XSS_OP_KV_QSORT || r.op == XSS_OP_KV_SELECT ||
               r.op == XSS_OP_KV_PARTIAL_SORT;
    }

    void finish(const std::vector<uint64_t> &tickets, int status, Clock::time_point now)
    {
        std::lock_guard<std::mutex> lk(mu);
        for (uint64_t t : tickets) {
            auto it = running.find(t);
            if (it == running.end()) continue;
            const double us =
                std::chrono::duration<double, std::micro>(now - it->second.arrival).count();
            lat_us.push_back(us);
            keys_done += (double)it->second.r.n;
            finished[t] = status;
            if (status == XSS_OK) ++completed;
            else ++failed;
            running.erase(it);
        }
        cv_done.notify_all();
    }

    // -- single request on its own stream -----------------------------------
    int launch_single(Job &j)
    {
        const xss_serve_request &r = j.r;
        const size_t kb = dt_bytes(r.key_dtype), n = r.n;
        const size_t ws_b = request_ws(r);
        void *data = pool.alloc(request_bytes(r));
        if (!data) return XSS_ENOMEM;
        void *ws = nullptr;
        if (ws_b) {
            ws = pool.alloc(ws_b);
            if (!ws) {
                pool.release(data);
                return XSS_ENOMEM;
            }
        }
        cudaStream_t s = streams[next_stream++ % streams.size()];
        char *dk = static_cast<char *>(data);
        char *dv = dk + align_up(n * kb, 256);
        uint64_t *da = reinterpret_cast<uint64_t *>(dv);
        int rc = XSS_OK;
        if (cudaMemcpyAsync(dk, r.keys_in, n * kb, cudaMemcpyHostToDevice, s) != cudaSuccess)
            rc = XSS_ECUDA;
        if (!rc && is_kv(r.op) &&
            cudaMemcpyAsync(dv, r.vals_in, n * dt_bytes(r.val_dtype), cudaMemcpyHostToDevice, s) !=
                cudaSuccess)
            rc = XSS_ECUDA;
        xss_stream_t xs = (xss_stream_t)s;
        if (!rc) {
            switch (r.op) {
            case XSS_OP_QSORT: rc = xss_gpu_qsort(r.key_dtype, dk, n, r.hasnan, r.descending, ws, ws_b, xs); break;
            case XSS_OP_QSELECT: rc = xss_gpu_qselect(r.key_dtype, dk, r.k, n, r.hasnan, r.descending, ws, ws_b, xs); break;
            case XSS_OP_PARTIAL_QSORT: rc = xss_gpu_partial_qsort(r.key_dtype, dk, r.k, n, r.hasnan, r.descending, ws, ws_b, xs); break;
            case XSS_OP_ARGSORT: rc = xss_gpu_argsort(r.key_dtype, dk, da, n, r.hasnan, r.descending, ws, ws_b, xs); break;
            case XSS_OP_ARGSELECT: rc = xss_gpu_argselect(r.key_dtype, dk, da, r.k, n, r.hasnan, ws, ws_b, xs); break;
            case XSS_OP_KV_QSORT: rc = xss_gpu_keyvalue_qsort(r.key_dtype, r.val_dtype, dk, dv, n, r.hasnan, r.descending, ws, ws_b, xs); break;
            case XSS_OP_KV_SELECT: rc = xss_gpu_keyvalue_select(r.key_dtype, r.val_dtype, dk, dv, r.k, n, r.hasnan, r.descending, ws, ws_b, xs); break;
            case XSS_OP_KV_PARTIAL_SORT: rc = xss_gpu_keyvalue_partial_sort(r.key_dtype, r.val_dtype, dk, dv, r.k, n, r.hasnan, r.descending, ws, ws_b, xs); break;
            default: rc = XSS_EINVAL;
            }
        }
        if (!rc) {
            if (is_arg(r.op)) {
                if (cudaMemcpyAsync(r.arg_out, da, n * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess)
                    rc = XSS_ECUDA;
            } else {
                if (cudaMemcpyAsync(r.keys_out, dk, n * kb, cudaMemcpyDeviceToHost, s) !=
                    cudaSuccess)
                    rc = XSS_ECUDA;
                if (!rc && is_kv(r.op) &&
                    cudaMemcpyAsync(r.vals_out, dv, n * dt_bytes(r.val_dtype),
                                    cudaMemcpyDeviceToHost, s) != cudaSuccess)
                    rc = XSS_ECUDA;
            }
        }
        Inflight f;
        f.tickets.push_back(j.ticket);
        f.blocks = {data, ws};
        f.keys = n;
        f.done = take_event();
        cudaEventRecord(f.done, s);
        {
            std::lock_guard<std::mutex> lk(mu);
            running.emplace(j.ticket, j);
        }
        if (rc) {
            // the request failed to enqueue: wait for what was queued, report it
            cudaStreamSynchronize(s);
            pool.release(data);
            pool.release(ws);
            free_events.push_back(f.done);
            finish(f.tickets, rc, Clock::now());
            return XSS_OK;
        }
        inflight.push_back(std::move(f));
        return XSS_OK;
    }

    // -- many small requests of one kind: one segmented sort -------------------
    int launch_batch(std::vector<Job> &jobs)
    {
        const xss_serve_request &r0 = jobs[0].r;
        const bool kv = is_kv(r0.op);
        const size_t kb = dt_bytes(r0.key_dtype), vb = kv ? dt_bytes(r0.val_dtype) : 0;
        std::vector<uint64_t> off(jobs.size() + 1, 0);
        for (size_t i = 0; i < jobs.size(); ++i) off[i + 1] = off[i] + jobs[i].r.n;
        const size_t n = off.back();
        const size_t ws_b = align_up(
            xss_gpu_segmented_workspace_size(r0.key_dtype, kv ? r0.val_dtype : -1, off.data(),
                                             jobs.size()),
            256);
        const size_t data_b = align_up(n * kb, 256) + align_up(n * vb, 256) +
                              align_up(off.size() * 8, 256);
        void *data = pool.alloc(data_b);
        if (!data) return XSS_ENOMEM;
        void *ws = pool.alloc(ws_b);
        if (!ws) {
            pool.release(data);
            return XSS_ENOMEM;
        }
        char *dk = static_cast<char *>(data);
        char *dv = dk + align_up(n * kb, 256);
        uint64_t *doff = reinterpret_cast<uint64_t *>(dv + align_up(n * vb, 256));
        cudaStream_t s = batch_stream;
        int rc = XSS_OK;
        for (size_t i = 0; i < jobs.size() && !rc; ++i) {
            const xss_serve_request &r = jobs[i].r;
            if (cudaMemcpyAsync(dk + off[i] * kb, r.keys_in, r.n * kb, cudaMemcpyHostToDevice, s) !=
                cudaSuccess)
                rc = XSS_ECUDA;
            if (!rc && kv &&
                cudaMemcpyAsync(dv + off[i] * vb, r.vals_in, r.n * vb, cudaMemcpyHostToDevice, s) !=
                    cudaSuccess)
                rc = XSS_ECUDA;
        }
        // the offsets come from a host vector: copy them before it goes away
        // (a pageable copy: it returns once the offsets are staged)
        if (!rc && cudaMemcpyAsync(doff, off.data(), off.size() * 8, cudaMemcpyHostToDevice, s) !=
                       cudaSuccess)
            rc = XSS_ECUDA;
        if (!rc)
            rc = xss_gpu_segmented_sort(r0.key_dtype, kv ? r0.val_dtype : -1, dk, kv ? dv : nullptr,
                                        doff, off.data(), jobs.size(), r0.hasnan, r0.descending, ws,
                                        ws_b, (xss_stream_t)s);
        for (size_t i = 0; i < jobs.size() && !rc; ++i) {
            const xss_serve_request &r = jobs[i].r;
            if (cudaMemcpyAsync(r.keys_out, dk + off[i] * kb, r.n * kb, cudaMemcpyDeviceToHost, s) !=
                cudaSuccess)
                rc = XSS_ECUDA;
            if (!rc && kv &&
                cudaMemcpyAsync(r.vals_out, dv + off[i] * vb, r.n * vb, cudaMemcpyDeviceToHost, s) !=
                    cudaSuccess)
                rc = XSS_ECUDA;
        }
        Inflight f;
        for (auto &j : jobs) f.tickets.push_back(j.ticket);
        f.blocks = {data, ws};
        f.keys = n;
        f.done = take_event();
        cudaEventRecord(f.done, s);
        {
            std::lock_guard<std::mutex> lk(mu);
            for (auto &j : jobs) running.emplace(j.ticket, j);
            ++batches;
            batched_reqs += jobs.size();
        }
        if (rc) {
            cudaStreamSynchronize(s);
            pool.release(data);
            pool.release(ws);
            free_events.push_back(f.done);
            finish(f.tickets, rc, Clock::now());
            return XSS_OK;
        }
        inflight.push_back(std::move(f));
        return XSS_OK;
    }

    void reap()
    {
        for (size_t i = 0; i < inflight.size();) {
            Inflight &f = inflight[i];
            const cudaError_t q = cudaEventQuery(f.done);
            if (q == cudaErrorNotReady) {
                ++i;
                continue;
            }
            int rc = q == cudaSuccess ? XSS_OK : XSS_ECUDA;
            if (q != cudaSuccess) cudaGetLastError();
            for (void *b : f.blocks) pool.release(b);
            free_events.push_back(f.done);
            finish(f.tickets, rc, Clock::now());
            inflight[i] = std::move(inflight.back());
            inflight.pop_back();
        }
    }

    void admit()
    {
        // small requests: gather same-kind ones into batches
        std::vector<Job> batch;
        for (size_t i = 0; i < pending.size();) {
            Job &j = pending[i];
            if (!coalescible(j.r)) {
                ++i;
                continue;
            }
            if (batch.empty() ||
                (batch[0].r.op >= XSS_OP_KV_QSORT) == (j.r.op >= XSS_OP_KV_QSORT) &&
                    batch[0].r.key_dtype == j.r.key_dtype &&
                    (!is_kv(j.r.op) || batch[0].r.val_dtype == j.r.val_dtype) &&
                    batch[0].r.hasnan == j.r.hasnan && batch[0].r.descending == j.r.descending) {
                batch.push_back(j);
                pending.erase(pending.begin() + i);
                if (batch.size() >= cfg.max_batch) {
                    if (launch_batch(batch) == XSS_ENOMEM) {
                        for (auto &b : batch) pending.push_front(b);
                        return;  // pool full: wait for completions
                    }
                    batch.clear();
                }
                continue;
            }
            ++i;
        }
        if (!batch.empty() && launch_batch(batch) == XSS_ENOMEM) {
            for (auto &b : batch) pending.push_front(b);
            return;
        }
        // large requests in arrival order; one that does not fit yet waits,
        // smaller ones behind it may pass (bounded look-ahead)
        size_t looked = 0;
        for (size_t i = 0; i < pending.size() && looked < 8;) {
            if (coalescible(pending[i].r)) {
                ++i;
                continue;
            }
            ++looked;
            const size_t need = request_bytes(pending[i].r) + request_ws(pending[i].r);
            if (need > pool.capacity()) {
                Job j = pending[i];
                pending.erase(pending.begin() + i);
                {
                    std::lock_guard<std::mutex> lk(mu);
                    running.emplace(j.ticket, j);
                }
                finish({j.ticket}, XSS_ENOMEM, Clock::now());
                continue;
            }
            if (launch_single(pending[i]) == XSS_ENOMEM) {
                ++i;
                continue;
            }
            pending.erase(pending.begin() + i);
        }
    }

    void run()
    {
        cudaSetDevice(device);
        set_prefer_shared_sm(true);   // requests on several streams share the SMs
        while (true) {
            {
                std::unique_lock<std::mutex> lk(mu);
                if (inbox.empty() && pending.empty() && inflight.empty()) {
                    if (stopping) break;
                    cv_work.wait_for(lk, std::chrono::microseconds(200));
                }
                while (!inbox.empty()) {
                    pending.push_back(inbox.front());
                    inbox.pop_front();
                }
                if (stopping && !draining) {
                    // refuse what has not started
                    for (auto &j : pending) finished[j.ticket] = XSS_EBUSY;
                    pending.clear();
                    cv_done.notify_all();
                }
            }
            reap();
            if (!pending.empty()) admit();
            queued_.store(pending.size());
            if (!inflight.empty() && pending.empty()) std::this_thread::yield();
        }
    }
};

extern "C" {

int xss_server_create(xss_server *out, const xss_server_config *cfg)
{
    if (!out || !cfg) return XSS_EINVAL;
    *out = nullptr;
    auto *s = new (std::nothrow) xss_server_s();
    if (!s) return XSS_ENOMEM;
    s->cfg = *cfg;
    if (s->cfg.streams <= 0) s->cfg.streams = 4;
    if (s->cfg.small_max == 0) s->cfg.small_max = 1 << 16;
    if (s->cfg.max_batch == 0) s->cfg.max_batch = 4096;
    if (s->cfg.max_queue == 0) s->cfg.max_queue = 1024;
    s->device = cfg->device;
    if (cudaSetDevice(s->device) != cudaSuccess) {
        delete s;
        return XSS_ECUDA;
    }
    size_t freeb = 0, total = 0;
    cudaMemGetInfo(&freeb, &total);
    size_t budget = cfg->hbm_budget_bytes ? cfg->hbm_budget_bytes : freeb / 2;
    if (budget > freeb) budget = freeb;
    if (s->pool.init(budget)) {
        delete s;
        return XSS_ENOMEM;
    }
    for (int i = 0; i < s->cfg.streams; ++i) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            delete s;
            return XSS_ECUDA;
        }
        s->streams.push_back(st);
    }
    cudaStreamCreateWithFlags(&s->batch_stream, cudaStreamNonBlocking);
    device_error_word();  // allocated before the scheduler runs
    s->t0 = Clock::now();
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return XSS_OK;
}

int xss_server_submit(xss_server s, const xss_serve_request *r, uint64_t *ticket)
{
    if (!s || !r || !ticket) return XSS_EINVAL;
    if (r->key_dtype < 0 || r->key_dtype > XSS_DT_F64 || r->op < 0 || r->op > XSS_OP_KV_PARTIAL_SORT)
        return XSS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return XSS_EBUSY;
    ++s->submitted;
    if (s->inbox.size() + s->queued_.load() >= s->cfg.max_queue) {
        ++s->shed;
        return XSS_EBUSY;
    }
    Job j;
    j.ticket = s->next_ticket++;
    j.r = *r;
    j.arrival = Clock::now();
    *ticket = j.ticket;
    s->inbox.push_back(j);
    s->cv_work.notify_one();
    return XSS_OK;
}

int xss_server_wait(xss_server s, uint64_t ticket, int *status)
{
    if (!s) return XSS_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->finished.count(ticket) != 0; });
    if (status) *status = s->finished[ticket];
    s->finished.erase(ticket);
    return XSS_OK;
}

int xss_server_poll(xss_server s, uint64_t ticket, int *status)
{
    if (!s) return XSS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->finished.find(ticket);
    if (it == s->finished.end()) return XSS_EAGAIN;
    if (status) *status = it->second;
    s->finished.erase(it);
    return XSS_OK;
}

int xss_server_get_stats(xss_server s, xss_server_stats *out)
{
    if (!s || !out) return XSS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->shed = s->shed;
    out->completed = s->completed;
    out->failed = s->failed;
    out->batches = s->batches;
    out->batched_requests = s->batched_reqs;
    out->keys = s->keys_done;
    out->wall_s = std::chrono::duration<double>(Clock::now() - s->t0).count();
    out->pool_bytes = s->pool.capacity();
    if (!s->lat_us.empty()) {
        std::vector<double> v = s->lat_us;
        auto q = [&](double f) {
            const size_t i = std::min(v.size() - 1, (size_t)(f * (double)(v.size() - 1) + 0.5));
            std::nth_element(v.begin(), v.begin() + i, v.end());
            return v[i];
        };
        out->p50_us = q(0.50);
        out->p99_us = q(0.99);
        out->max_us = *std::max_element(v.begin(), v.end());
    }
    return XSS_OK;
}

int xss_server_reset_stats(xss_server s)
{
    if (!s) return XSS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat_us.clear();
    s->submitted = s->shed = s->completed = s->failed = s->batches = s->batched_reqs = 0;
    s->keys_done = 0;
    s->t0 = Clock::now();
    return XSS_OK;
}

void xss_server_destroy(xss_server s, int drain)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->draining = drain != 0;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    for (cudaStream_t st : s->streams) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    if (s->batch_stream) {
        cudaStreamSynchronize(s->batch_stream);
        cudaStreamDestroy(s->batch_stream);
    }
    for (cudaEvent_t e : s->free_events) cudaEventDestroy(e);
    delete s;
}

}  // extern "C"
