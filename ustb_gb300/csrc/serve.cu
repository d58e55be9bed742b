// Continuous-batching server over resident plans.
//
// Requests are queued by ustb_serve_submit (any thread).  A request with more
// pixel x channel x wave x frame units than large_units goes to the large queue,
// every other one to the small queue.  A scheduler thread takes small requests in
// arrival order into batches whose interpolation entries fit the workspace budget
// (at most max_batch requests) and launches each batch with ustb_das_fast_batch_ex,
// alternating between two small-request streams, each with its own workspace and
// queue counters, so one batch's entries pass overlaps the tail of the previous
// batch's beamforming.  Large requests launch one per batch on a third stream, at
// most two queued there, with at most SMs - reserve_sms persistent CTAs: small
// batches never queue behind a large launch on the same stream, and with
// reserve_sms > 0 they keep SMs of their own while it runs.  Each batch copies its
// flag word to pinned host memory and records an event.  One completion thread per
// class (small, large) waits for its batches in launch order and marks their
// tickets done, so a small batch is reported as soon as it ends, not after a large
// launch issued before it.  On one stream, a batch's entries pass only starts once
// the previous batch there is done, so each workspace is reused safely.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "common.cuh"

namespace ustb {
void plan_request(ustb_plan plan, const void* ch, const ustb_das_outputs* out, ustb_das_request* r);
}

namespace {

constexpr int kMaxBatchRequests = 40;  // the persistent kernel's request table
constexpr int kFlagSlots = 64;         // pinned flag words (batches in flight at most)
constexpr int kSmallStreams = 2;       // small batches alternate between these
constexpr int kLargeStream = kSmallStreams;
constexpr int kStreams = kSmallStreams + 1;
constexpr int kLargeInFlight = 2;  // large launches queued back to back on their stream
constexpr int kSmall = 0, kLarge = 1;  // batch classes, one completion thread each

struct Job {
    uint64_t ticket;
    ustb_plan plan;
    const void* ch;
    ustb_das_outputs out;
};

struct Done {
    int status;  // USTB_OK or an error code
    uint32_t flags;
    std::string message;
};

struct Batch {
    std::vector<uint64_t> tickets;
    cudaEvent_t ev = nullptr;
    int slot = -1;   // pinned flag word
    int status = USTB_OK;
    std::string message;
};

}  // namespace

struct ustb_server_s {
    std::mutex m;
    std::condition_variable cv_queue, cv_flight, cv_done;
    std::deque<Job> queue;        // small requests, arrival order
    std::deque<Job> large_queue;  // large requests, arrival order
    std::deque<Batch> flight[2];  // launched batches per class, launch order
    std::unordered_map<uint64_t, Done> done;
    std::unordered_set<uint64_t> live;  // submitted and not yet released by a wait
    uint64_t next_ticket = 1;
    bool stop = false;           // destroy requested: finish the queues, then exit
    bool sched_exited = false;   // the scheduler has launched everything it will
    int64_t budget = 0;
    int64_t large_units = 0;  // requests above this many units go to the large stream
    int large_ctas = 0;       // persistent CTAs of a large launch (0: one per SM)
    int large_flight = 0;     // large launches not yet completed
    int max_batch = 1;
    int device = 0;
    cudaStream_t stream[kStreams] = {};
    void* workspace[kStreams] = {};
    int64_t ws_bytes[kStreams] = {};
    uint64_t* scratch[kStreams] = {};  // device: flag word + queue counters
    int next = 0;                      // small stream of the next small batch
    uint64_t* host_flags = nullptr;  // pinned [kFlagSlots]
    std::vector<int> free_slots;
    std::thread scheduler, completer[2];

    bool is_large(const Job& j) const;
    void schedule();
    void complete(int cls);
    int launch(const std::vector<Job>& jobs, int i, int max_ctas, Batch& b);
    // CUDA resources (also after a failed create); the threads are joined first
    ~ustb_server_s() {
        for (int i = 0; i < kStreams; ++i) {
            if (stream[i]) cudaStreamDestroy(stream[i]);
            if (workspace[i]) cudaFree(workspace[i]);
            if (scratch[i]) cudaFree(scratch[i]);
        }
        if (host_flags) cudaFreeHost(host_flags);
    }
};

bool ustb_server_s::is_large(const Job& j) const {
    ustb_das_request r;
    ustb::plan_request(j.plan, j.ch, &j.out, &r);
    return r.L > 0 && (double)r.geometry->n_pixels * r.N * r.W * r.F > (double)large_units;
}

// Launch a batch on stream i (max_ctas 0: one persistent CTA per SM).
int ustb_server_s::launch(const std::vector<Job>& jobs, int i, int max_ctas, Batch& b) {
    std::vector<ustb_das_request> reqs(jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k) ustb::plan_request(jobs[k].plan, jobs[k].ch, &jobs[k].out, &reqs[k]);
    const int64_t need = ustb_das_fast_workspace_bytes(reqs.data(), (int32_t)reqs.size());
    if (need < 0) return (int)-need;
    if (need > ws_bytes[i]) {  // grow: the stream must be idle before the old block goes
        USTB_CUDA(cudaStreamSynchronize(stream[i]));
        if (workspace[i]) USTB_CUDA(cudaFree(workspace[i]));
        workspace[i] = nullptr;
        ws_bytes[i] = 0;
        USTB_CUDA(cudaMalloc(&workspace[i], (size_t)need));
        ws_bytes[i] = need;
    }
    const int rc = ustb_das_fast_batch_ex(reqs.data(), (int32_t)reqs.size(), scratch[i], workspace[i], ws_bytes[i],
                                          max_ctas, stream[i]);
    if (rc != USTB_OK) return rc;
    USTB_CUDA(cudaMemcpyAsync(host_flags + b.slot, scratch[i], sizeof(uint64_t), cudaMemcpyDeviceToHost, stream[i]));
    USTB_CUDA(cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming | cudaEventBlockingSync));
    USTB_CUDA(cudaEventRecord(b.ev, stream[i]));
    return USTB_OK;
}

void ustb_server_s::schedule() {
    cudaSetDevice(device);
    for (;;) {
        std::vector<Job> jobs;
        int slot = -1, cls = kSmall, i = 0;
        {
            std::unique_lock<std::mutex> lk(m);
            const auto large_ready = [&] { return !large_queue.empty() && large_flight < kLargeInFlight; };
            cv_queue.wait(lk, [&] {
                return !queue.empty() || large_ready() || (stop && large_queue.empty());
            });
            if (queue.empty() && large_queue.empty()) break;  // stop requested and nothing left
            cv_flight.wait(lk, [&] { return !free_slots.empty(); });
            slot = free_slots.back();
            free_slots.pop_back();
            // only this thread takes from the queues and only completions lower
            // large_flight, so what was ready above is still ready
            if (large_ready()) {
                cls = kLarge;
                i = kLargeStream;
                ++large_flight;
                jobs.push_back(large_queue.front());
                large_queue.pop_front();
            } else {
                i = next;
                next = (next + 1) % kSmallStreams;
                // arrival order; add requests while their entries fit the budget
                int64_t bytes = 0;
                while (!queue.empty() && (int)jobs.size() < max_batch) {
                    ustb_das_request r;
                    ustb::plan_request(queue.front().plan, queue.front().ch, &queue.front().out, &r);
                    const int64_t b = ustb_das_fast_workspace_bytes(&r, 1);
                    if (!jobs.empty() && bytes + b > budget) break;
                    bytes += b;
                    jobs.push_back(queue.front());
                    queue.pop_front();
                }
            }
        }
        Batch b;
        b.slot = slot;
        for (const Job& j : jobs) b.tickets.push_back(j.ticket);
        b.status = launch(jobs, i, cls == kLarge ? large_ctas : 0, b);
        if (b.status != USTB_OK) b.message = ustb_last_error();
        {
            std::lock_guard<std::mutex> lk(m);
            flight[cls].push_back(std::move(b));
        }
        cv_flight.notify_all();
    }
    {
        std::lock_guard<std::mutex> lk(m);
        sched_exited = true;
    }
    cv_flight.notify_all();
}

void ustb_server_s::complete(int cls) {
    cudaSetDevice(device);
    for (;;) {
        Batch b;
        {
            std::unique_lock<std::mutex> lk(m);
            cv_flight.wait(lk, [&] { return !flight[cls].empty() || sched_exited; });
            if (flight[cls].empty()) break;
            b = std::move(flight[cls].front());
            flight[cls].pop_front();
        }
        uint32_t flags = 0;
        if (b.status == USTB_OK) {
            const cudaError_t e = cudaEventSynchronize(b.ev);
            if (e != cudaSuccess) {
                b.status = USTB_E_CUDA;
                b.message = std::string("batch failed on the device: ") + cudaGetErrorString(e);
            } else {
                flags = (uint32_t)(host_flags[b.slot] & 0xffffffffu);
            }
        }
        if (b.ev) cudaEventDestroy(b.ev);
        {
            std::lock_guard<std::mutex> lk(m);
            for (uint64_t t : b.tickets) done[t] = Done{b.status, flags, b.message};
            free_slots.push_back(b.slot);
            if (cls == kLarge) --large_flight;
        }
        cv_done.notify_all();
        cv_flight.notify_all();
        if (cls == kLarge) cv_queue.notify_all();  // the large stream has room again
    }
}

extern "C" int ustb_serve_create_ex(int64_t workspace_budget, int32_t max_batch, int64_t large_units,
                                    int32_t reserve_sms, ustb_server* out) {
    ustb::clear_error();
    USTB_REQUIRE(out, USTB_E_ARG, "NULL pointer");
    *out = nullptr;
    USTB_REQUIRE(workspace_budget > 0, USTB_E_ARG, "workspace budget must be > 0");
    USTB_REQUIRE(max_batch >= 1 && max_batch <= kMaxBatchRequests, USTB_E_ARG, "max_batch must be in [1, %d]",
                 kMaxBatchRequests);
    USTB_REQUIRE(reserve_sms >= 0, USTB_E_ARG, "reserve_sms must be >= 0");
    std::unique_ptr<ustb_server_s> s(new ustb_server_s());
    s->budget = workspace_budget;
    s->max_batch = max_batch;
    s->large_units = large_units > 0 ? large_units : (int64_t)2000000000;
    USTB_CUDA(cudaGetDevice(&s->device));
    int sms = 0;
    USTB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
    USTB_REQUIRE(reserve_sms < sms, USTB_E_ARG, "reserve_sms must be below the %d SMs of the device", sms);
    s->large_ctas = reserve_sms > 0 ? sms - reserve_sms : 0;
    for (int i = 0; i < kStreams; ++i) {
        USTB_CUDA(cudaStreamCreateWithFlags(&s->stream[i], cudaStreamNonBlocking));
        USTB_CUDA(cudaMalloc(&s->scratch[i], sizeof(uint64_t) * (kMaxBatchRequests + 1)));
    }
    USTB_CUDA(cudaHostAlloc(&s->host_flags, sizeof(uint64_t) * kFlagSlots, cudaHostAllocDefault));
    for (int i = kFlagSlots - 1; i >= 0; --i) s->free_slots.push_back(i);
    ustb_server_s* raw = s.get();
    raw->scheduler = std::thread([raw] { raw->schedule(); });
    for (int c = 0; c < 2; ++c) raw->completer[c] = std::thread([raw, c] { raw->complete(c); });
    *out = s.release();
    return USTB_OK;
}

extern "C" int ustb_serve_create(int64_t workspace_budget, int32_t max_batch, int64_t large_units,
                                 ustb_server* out) {
    return ustb_serve_create_ex(workspace_budget, max_batch, large_units, 0, out);
}

extern "C" int ustb_serve_submit(ustb_server s, ustb_plan plan, const void* ch, const ustb_das_outputs* out,
                                 uint64_t* ticket) {
    ustb::clear_error();
    USTB_REQUIRE(s && plan && ch && out && ticket, USTB_E_ARG, "NULL pointer");
    ustb_das_request r;
    ustb::plan_request(plan, ch, out, &r);
    const int64_t need = ustb_das_fast_workspace_bytes(&r, 1);
    USTB_REQUIRE(need >= 0, (int)-need, "%s", ustb_last_error());
    {
        std::lock_guard<std::mutex> lk(s->m);
        USTB_REQUIRE(!s->stop, USTB_E_BUSY, "the server is shutting down");
        *ticket = s->next_ticket++;
        s->live.insert(*ticket);
        const Job j{*ticket, plan, ch, *out};
        (s->is_large(j) ? s->large_queue : s->queue).push_back(j);
    }
    s->cv_queue.notify_one();
    return USTB_OK;
}

extern "C" int ustb_serve_wait(ustb_server s, uint64_t ticket, int32_t timeout_ms, uint32_t* flags) {
    ustb::clear_error();
    USTB_REQUIRE(s, USTB_E_ARG, "NULL server");
    std::unique_lock<std::mutex> lk(s->m);
    USTB_REQUIRE(s->live.count(ticket), USTB_E_ARG, "unknown or released ticket %llu", (unsigned long long)ticket);
    // done, or released meanwhile by another waiter
    auto ready = [&] { return s->done.count(ticket) != 0 || !s->live.count(ticket); };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, ready);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        ustb::set_error("ticket %llu not done after %d ms", (unsigned long long)ticket, (int)timeout_ms);
        return USTB_E_TIMEOUT;
    }
    USTB_REQUIRE(s->live.count(ticket), USTB_E_ARG, "ticket %llu was released by another waiter",
                 (unsigned long long)ticket);
    const Done d = s->done[ticket];
    s->done.erase(ticket);
    s->live.erase(ticket);
    if (flags) *flags = d.flags;
    if (d.status != USTB_OK) ustb::set_error("%s", d.message.c_str());
    return d.status;
}

extern "C" int ustb_serve_destroy(ustb_server s) {
    ustb::clear_error();
    USTB_REQUIRE(s, USTB_E_ARG, "NULL server");
    {
        std::lock_guard<std::mutex> lk(s->m);
        s->stop = true;
    }
    s->cv_queue.notify_all();
    s->scheduler.join();
    for (std::thread& t : s->completer) t.join();
    int rc = USTB_OK;
    for (int i = 0; i < kStreams; ++i) {
        if (!s->stream[i]) continue;
        const cudaError_t e = cudaStreamSynchronize(s->stream[i]);
        if (e != cudaSuccess && rc == USTB_OK) rc = ustb::cuda_fail(e, "cudaStreamSynchronize", __FILE__, __LINE__);
    }
    delete s;  // frees the streams, workspaces and pinned flags
    return rc;
}
