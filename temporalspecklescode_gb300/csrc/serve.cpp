// serve.cpp -- request loop over the C-ABI: continuous batching of renders.
//
// No counterpart in the reference, which renders one scene per MEX call
// (MatlabInterface.cu:1565-1825).  A server owns `slots` worker threads.
// A submitted request (scene, seed, host output buffers) waits in a FIFO
// queue; a free worker admits the first queued request whose device-memory
// reservation fits the budget next to the requests in flight (or any request
// when nothing is in flight, so an oversized one still runs alone), renders
// it on the scene's own stream with chunk buffers sized to the reservation,
// returns the buffers to the stream-ordered pool and marks the ticket done.
// Requests on different scenes therefore overlap on the device; requests on
// the same scene run one after another: a queued request whose scene is
// rendering is passed over (it would only wait for the scene's lock while
// holding a worker and a reservation), so requests on other scenes behind it
// are admitted first.  A render's
// result depends only on (scene, seed): the paths' random streams are keyed
// by path id and the chunking is invisible, so a request gives the same
// result alone and in the mix (up to the order of the FP64 accumulation).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sstmc_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct ServeRequest {
    uint64_t id = 0;
    sstmc_scene* scene = nullptr;
    uint64_t seed = 0;
    double* u = nullptr;
    double* iter = nullptr;
    size_t need = 0;
    int32_t status = SSTMC_NO_ERROR;
    bool done = false, cancelled = false;
    uint64_t contributions = 0;
    Clock::time_point t_submit, t_start, t_end;
};

}  // namespace

struct sstmc_server {
    int device = 0;
    size_t budget = 0, per_request = 0;
    uint32_t slots = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ServeRequest*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<ServeRequest>> reqs;
    size_t reserved = 0;
    uint32_t running = 0;
    std::unordered_map<const sstmc_scene*, uint32_t> busy;   // scenes with a request rendering
    bool stop = false;
    uint64_t next_id = 1;
    std::vector<std::thread> workers;
    // statistics of completed requests
    std::vector<double> latency_ms;
    uint64_t completed = 0, contributions = 0;
    bool any = false;
    Clock::time_point first_start, last_end;
};

namespace {

// First queued request whose scene is idle and whose reservation fits next to
// the requests in flight (cancelled ones are completed on the way).  Caller
// holds srv->mu.
ServeRequest* admit(sstmc_server* srv)
{
    for (auto it = srv->queue.begin(); it != srv->queue.end();) {
        ServeRequest* r = *it;
        if (r->cancelled) {
            r->done = true;
            r->status = SSTMC_CANCELLED;
            r->t_end = Clock::now();
            it = srv->queue.erase(it);
            srv->cv_done.notify_all();
            continue;
        }
        if (srv->busy.count(r->scene)) { ++it; continue; }
        if (srv->running == 0 || srv->reserved + r->need <= srv->budget) {
            srv->queue.erase(it);
            return r;
        }
        ++it;
    }
    return nullptr;
}

void worker(sstmc_server* srv)
{
    cudaSetDevice(srv->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    for (;;) {
        ServeRequest* r = nullptr;
        srv->cv_work.wait(lk, [&] { return srv->stop || (r = admit(srv)) != nullptr; });
        if (!r) return;   // stopping with nothing admissible
        srv->reserved += r->need;
        srv->running++;
        srv->busy[r->scene]++;
        r->t_start = Clock::now();
        if (!srv->any) { srv->any = true; srv->first_start = r->t_start; }
        lk.unlock();
        uint64_t contrib = 0;
        const int32_t st = sstmc::render_scene(r->scene, r->seed, r->u, r->iter, srv->per_request, true, &contrib);
        lk.lock();
        srv->reserved -= r->need;
        srv->running--;
        if (--srv->busy[r->scene] == 0) srv->busy.erase(r->scene);
        r->status = st;
        r->contributions = contrib;
        r->t_end = Clock::now();
        r->done = true;
        srv->last_end = r->t_end;
        srv->completed++;
        srv->contributions += contrib;
        srv->latency_ms.push_back(std::chrono::duration<double, std::milli>(r->t_end - r->t_submit).count());
        srv->cv_done.notify_all();
        srv->cv_work.notify_all();
    }
}

double percentile(std::vector<double> v, double p)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const size_t k = std::min(v.size() - 1, (size_t)(p * (double)(v.size() - 1) + 0.5));
    return v[k];
}

}  // namespace

extern "C" {

int32_t sstmc_server_create(int32_t device, uint64_t hbm_budget_bytes, uint32_t slots, sstmc_server** out)
{
    if (!out) return SSTMC_INVALID_HANDLE;
    *out = nullptr;
    if (slots == 0 || slots > 64) return SSTMC_INVALID_CONFIG;
    if (cudaSetDevice(device) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return SSTMC_DEVICE_ERROR;
    // freed request buffers stay in the stream-ordered pool for the next request
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = 0;
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        keep = std::max<uint64_t>(keep, hbm_budget_bytes ? hbm_budget_bytes : fr / 2);
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    sstmc_server* srv = new (std::nothrow) sstmc_server();
    if (!srv) return SSTMC_ALLOCATION_ERROR;
    srv->device = device;
    srv->budget = hbm_budget_bytes ? (size_t)hbm_budget_bytes : fr / 2;
    srv->slots = slots;
    srv->per_request = std::max<size_t>((size_t)64 << 20, srv->budget / slots);
    try {
        for (uint32_t i = 0; i < slots; ++i) srv->workers.emplace_back(worker, srv);
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->stop = true;
        }
        srv->cv_work.notify_all();
        for (auto& t : srv->workers) t.join();
        delete srv;
        return SSTMC_MISC_ERROR;
    }
    *out = srv;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_server_destroy(sstmc_server* srv)
{
    if (!srv) return SSTMC_INVALID_HANDLE;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        for (ServeRequest* r : srv->queue) { r->done = true; r->status = SSTMC_CANCELLED; }
        srv->queue.clear();
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    srv->cv_done.notify_all();
    for (auto& t : srv->workers) t.join();
    delete srv;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_submit(sstmc_server* srv, sstmc_scene* scene, uint64_t seed, double* u_out, double* iter_out, uint64_t* ticket)
{
    if (!srv || !scene || !ticket) return SSTMC_INVALID_HANDLE;
    if (sstmc::scene_device(scene) != srv->device) return SSTMC_DEVICE_ERROR;
    auto r = std::unique_ptr<ServeRequest>(new (std::nothrow) ServeRequest());
    if (!r) return SSTMC_ALLOCATION_ERROR;
    r->scene = scene;
    r->seed = seed;
    r->u = u_out;
    r->iter = iter_out;
    r->need = sstmc::scene_request_bytes(scene, srv->per_request);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return SSTMC_CANCELLED;
        r->id = srv->next_id++;
        *ticket = r->id;
        srv->queue.push_back(r.get());
        srv->reqs.emplace(r->id, std::move(r));
    }
    srv->cv_work.notify_one();
    return SSTMC_NO_ERROR;
}

int32_t sstmc_poll(sstmc_server* srv, uint64_t ticket, int32_t* done, int32_t* status)
{
    if (!srv) return SSTMC_INVALID_HANDLE;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return SSTMC_INVALID_HANDLE;
    if (done) *done = it->second->done ? 1 : 0;
    if (status) *status = it->second->done ? it->second->status : SSTMC_NO_ERROR;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_wait(sstmc_server* srv, uint64_t ticket, double timeout_s, int32_t* status)
{
    if (!srv) return SSTMC_INVALID_HANDLE;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return SSTMC_INVALID_HANDLE;
    ServeRequest* r = it->second.get();
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(std::max(0.0, timeout_s)));
    if (!srv->cv_done.wait_until(lk, until, [&] { return r->done; })) return SSTMC_TIMEOUT;
    if (status) *status = r->status;
    return SSTMC_NO_ERROR;
}

int32_t sstmc_cancel(sstmc_server* srv, uint64_t ticket)
{
    if (!srv) return SSTMC_INVALID_HANDLE;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return SSTMC_INVALID_HANDLE;
    it->second->cancelled = true;   // a queued request completes as cancelled; a running one finishes
    srv->cv_work.notify_all();
    return SSTMC_NO_ERROR;
}

int32_t sstmc_server_stats(sstmc_server* srv, double* p50_ms, double* p99_ms, double* contributions_per_s, uint64_t* completed)
{
    if (!srv) return SSTMC_INVALID_HANDLE;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (p50_ms) *p50_ms = percentile(srv->latency_ms, 0.50);
    if (p99_ms) *p99_ms = percentile(srv->latency_ms, 0.99);
    if (contributions_per_s) {
        const double s = srv->any ? std::chrono::duration<double>(srv->last_end - srv->first_start).count() : 0.0;
        *contributions_per_s = s > 0.0 ? (double)srv->contributions / s : 0.0;
    }
    if (completed) *completed = srv->completed;
    return SSTMC_NO_ERROR;
}

}  // extern "C"
