// server.cpp -- a request server for whole scans: continuous batching over
// library contexts.
//
// The reference reconstructs one scan per process run (src/main.cu).  Here a
// server owns n worker threads, each with its own ctbb_context (work buffers,
// streams).  Requests queue first-in first-out; a free worker takes the head
// request as soon as the device memory it needs fits the budget next to what
// the other workers hold, so a request that arrives while others run starts
// as soon as a slot and memory free up, and its copies and kernels overlap
// theirs on the GPU.  A request that does not fit yet lets the queued requests
// behind it that do fit start first, until it has waited an age bound (2 s by
// default); from then on it is served next.  Each worker keeps its buffers between requests (no
// allocation, so no device-wide synchronisation, in the steady state); when a
// request does not fit, the worker first drops its own buffers, and idle
// workers are asked to drop theirs.  A request needing more than the whole
// budget is refused at submission.  Results do not depend on which worker ran
// a request or on what ran beside it: the same kernels on the same data.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "ctbb_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Job {
    uint64_t ticket = 0;
    struct recon_metadata *mr = nullptr;
    const float *h_scan = nullptr;
    float *h_final = nullptr;
    float mu_water = 0.0f;
    size_t need = 0;
    Clock::time_point submitted, started, finished;
    int status = CTBB_OK;
    int worker = -1;
    bool done = false;
    bool waited = false;  // a ctbb_server_wait call owns it
    std::string error;
};

struct Worker {
    ctbb_context ctx = nullptr;
    std::thread thread;
    size_t held = 0;      // device bytes its context holds while idle
    size_t reserved = 0;  // the running request's need while busy
    bool busy = false;
    bool release_asked = false;
};

}  // namespace

struct ctbb_server_s {
    std::mutex mu;
    std::condition_variable work_cv;  // queue, memory or shutdown changed
    std::condition_variable done_cv;  // a request finished
    std::deque<Job *> queue;
    std::map<uint64_t, Job *> jobs;   // submitted, not yet collected by ctbb_server_wait
    uint64_t next_ticket = 1;
    size_t budget = 0;
    int device = 0;
    Clock::time_point created = Clock::now();
    bool stopping = false;
    int waiters = 0;  // ctbb_server_wait calls in progress
    double age_bound_ms = 2000.0;  // after this a waiting head request is passed no more
    uint64_t passed = 0;           // requests started ahead of an older one
    std::vector<Worker> workers;
};

namespace {

size_t others_bytes(const ctbb_server_s &s, size_t w)
{
    size_t n = 0;
    for (size_t v = 0; v < s.workers.size(); ++v)
        if (v != w) n += s.workers[v].busy ? std::max(s.workers[v].held, s.workers[v].reserved) : s.workers[v].held;
    return n;
}

void worker_main(ctbb_server_s *s, size_t w)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        Worker &me = s->workers[w];
        if (me.release_asked && !me.busy) {
            lk.unlock();
            ctbb_context_release_workspace(me.ctx);
            lk.lock();
            me.held = 0;
            me.release_asked = false;
            s->work_cv.notify_all();
        }
        if (s->queue.empty()) {
            if (s->stopping) return;
            s->work_cv.wait(lk);
            continue;
        }
        // The head request, or -- while the head has waited less than the
        // age bound -- the first queued request that fits beside what the
        // other workers hold: a large request waiting for memory does not
        // hold up the small ones behind it, and after the age bound nothing
        // passes it any more.
        const size_t others = others_bytes(*s, w);
        size_t pick = 0;
        const bool head_aged = ms_between(s->queue.front()->submitted, Clock::now()) > s->age_bound_ms;
        if (!head_aged) {
            for (size_t q = 0; q < s->queue.size(); ++q)
                if (others + s->queue[q]->need <= s->budget) {
                    pick = q;
                    break;
                }
        }
        Job *j = s->queue[pick];
        bool release_first = false;
        if (others + std::max(me.held, j->need) > s->budget) {
            if (others + j->need <= s->budget) {
                release_first = true;  // this worker's own buffers give way
            } else {
                bool asked = false;
                for (size_t v = 0; v < s->workers.size(); ++v) {
                    Worker &o = s->workers[v];
                    if (v != w && !o.busy && o.held > 0 && !o.release_asked) {
                        o.release_asked = true;
                        asked = true;
                    }
                }
                if (asked) s->work_cv.notify_all();
                s->work_cv.wait(lk);  // a request finishes or a worker releases
                continue;
            }
        }
        s->queue.erase(s->queue.begin() + (long)pick);
        if (pick) ++s->passed;
        me.busy = true;
        me.reserved = j->need;
        j->started = Clock::now();
        j->worker = (int)w;
        lk.unlock();
        if (release_first) ctbb_context_release_workspace(me.ctx);
        int st = ctbb_context_reconstruct_scan_host(me.ctx, j->mr, j->h_scan, j->h_final, j->mu_water);
        std::string err = st != CTBB_OK ? std::string(ctbb_last_error()) : std::string();
        size_t held = ctbb_context_device_bytes(me.ctx);
        lk.lock();
        me.busy = false;
        me.held = held;
        me.reserved = 0;
        j->status = st;
        j->error = err;
        j->finished = Clock::now();
        j->done = true;
        s->done_cv.notify_all();
        s->work_cv.notify_all();
    }
}

}  // namespace

using namespace ctbb;

extern "C" int ctbb_server_create(int n_workers, size_t device_budget_bytes, ctbb_server *out)
{
    clear_error();
    if (!out || n_workers < 1 || n_workers > 64 || device_budget_bytes == 0) {
        set_error("ctbb_server_create: bad argument (1..64 workers, a non-zero budget)");
        return CTBB_ERR_ARGUMENT;
    }
    *out = nullptr;
    ctbb_server s = new (std::nothrow) ctbb_server_s;
    if (!s) {
        set_error("ctbb_server_create: out of host memory");
        return CTBB_ERR_ALLOC;
    }
    s->budget = device_budget_bytes;
    if (cudaGetDevice(&s->device) != cudaSuccess) s->device = 0;
    s->workers.resize((size_t)n_workers);
    for (Worker &w : s->workers) {
        int st = ctbb_context_create(&w.ctx);
        if (st != CTBB_OK) {
            std::string err = ctbb_last_error();
            for (Worker &x : s->workers) ctbb_context_destroy(x.ctx);
            delete s;
            set_error("%s", err.c_str());
            return st;
        }
    }
    for (size_t w = 0; w < s->workers.size(); ++w) s->workers[w].thread = std::thread(worker_main, s, w);
    *out = s;
    return CTBB_OK;
}

extern "C" int ctbb_server_configure(ctbb_server s, int storage, double age_bound_ms)
{
    clear_error();
    if (!s || !(age_bound_ms >= 0.0)) {
        set_error("ctbb_server_configure: bad argument");
        return CTBB_ERR_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    for (Worker &w : s->workers) {
        int st = ctbb_context_set_storage(w.ctx, storage);
        if (st != CTBB_OK) return st;
    }
    s->age_bound_ms = age_bound_ms;
    return CTBB_OK;
}

extern "C" uint64_t ctbb_server_passed_count(ctbb_server s)
{
    if (!s) return 0;
    std::lock_guard<std::mutex> lk(s->mu);
    return s->passed;
}

extern "C" int ctbb_server_submit(ctbb_server s, struct recon_metadata *mr, const float *h_scan, float *h_final,
                                  float mu_water, uint64_t *ticket)
{
    clear_error();
    if (!s || !mr || !h_scan || !h_final || !ticket) {
        set_error("ctbb_server_submit: null argument");
        return CTBB_ERR_ARGUMENT;
    }
    size_t need = ctbb_scan_workspace_bytes(mr);
    if (need == 0) {
        set_error("ctbb_server_submit: the plan is not usable for a whole-scan reconstruction");
        return CTBB_ERR_STATE;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (need > s->budget) {
        set_error("ctbb_server_submit: the scan needs %zu device bytes, more than the budget of %zu", need,
                  s->budget);
        return CTBB_ERR_ALLOC;
    }
    if (s->stopping) {
        set_error("ctbb_server_submit: the server is shutting down");
        return CTBB_ERR_STATE;
    }
    Job *j = new (std::nothrow) Job;
    if (!j) {
        set_error("ctbb_server_submit: out of host memory");
        return CTBB_ERR_ALLOC;
    }
    j->ticket = s->next_ticket++;
    j->mr = mr;
    j->h_scan = h_scan;
    j->h_final = h_final;
    j->mu_water = mu_water;
    j->need = need;
    j->submitted = Clock::now();
    s->jobs[j->ticket] = j;
    s->queue.push_back(j);
    *ticket = j->ticket;
    s->work_cv.notify_all();
    return CTBB_OK;
}

extern "C" int ctbb_server_wait(ctbb_server s, uint64_t ticket, struct ctbb_request_result *out)
{
    clear_error();
    if (!s) {
        set_error("ctbb_server_wait: null server");
        return CTBB_ERR_ARGUMENT;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) {
        set_error("ctbb_server_wait: unknown ticket %llu", (unsigned long long)ticket);
        return CTBB_ERR_ARGUMENT;
    }
    Job *j = it->second;
    if (j->waited) {
        set_error("ctbb_server_wait: ticket %llu is already being waited for", (unsigned long long)ticket);
        return CTBB_ERR_STATE;
    }
    j->waited = true;
    ++s->waiters;
    s->done_cv.wait(lk, [j] { return j->done; });
    s->jobs.erase(ticket);
    --s->waiters;
    s->done_cv.notify_all();  // a destroy may be waiting for the last waiter
    int st = j->status;
    if (out) {
        memset(out, 0, sizeof(*out));
        out->status = st;
        out->worker = j->worker;
        out->device_bytes = j->need;
        out->queue_ms = ms_between(j->submitted, j->started);
        out->run_ms = ms_between(j->started, j->finished);
        out->latency_ms = ms_between(j->submitted, j->finished);
        out->start_ms = ms_between(s->created, j->started);
        out->end_ms = ms_between(s->created, j->finished);
        snprintf(out->error, sizeof(out->error), "%s", j->error.c_str());
    }
    if (st != CTBB_OK) set_error("%s", j->error.c_str());
    delete j;
    return st;
}

extern "C" int ctbb_server_destroy(ctbb_server s)
{
    clear_error();
    if (!s) return CTBB_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->work_cv.notify_all();
    }
    for (Worker &w : s->workers)
        if (w.thread.joinable()) w.thread.join();
    {
        // every queued request has finished; let the waiters take their results
        std::unique_lock<std::mutex> lk(s->mu);
        s->done_cv.wait(lk, [s] { return s->waiters == 0; });
    }
    for (Worker &w : s->workers) ctbb_context_destroy(w.ctx);
    for (auto &kv : s->jobs) delete kv.second;
    delete s;
    return CTBB_OK;
}
