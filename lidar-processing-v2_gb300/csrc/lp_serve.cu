// lp_serve.cu — serving loop with continuous batching (lp_server_*, lidar_gb300_batch.h).
//
// Sensors submit scans as they arrive; one worker thread turns the pending queue into batches.
// Each batch runs in a slot: its own CUDA stream and a device region reserved up front, so
// several batches are on the GPU at once (upload of one, kernels of another, download of a
// third) and slots never allocate or free while others run. Admission is by memory: a batch is
// formed from the oldest pending scans while its planned layout fits the slot's region (the
// regions together are the server's device-memory budget); scans that arrive while the slots
// are busy wait and are admitted as soon as a slot frees up. A host callback on the slot's
// stream wakes the worker when a batch finishes; the worker then copies results into the
// caller's buffers and records the latency from submission to results in host memory.
// Every scan's results are the same whatever batch it lands in (kernels keep scans apart).
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "lidar_gb300.h"
#include "lidar_gb300_batch.h"
#include "lp_runtime.hpp"

namespace
{
double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request
{
    uint64_t tag;
    lp_scan_input in;
    lp_scan_output* out;
    double t_arrival;
};

struct Slot
{
    lp_context* ctx = nullptr;
    lp_batch batch;
    std::vector<Request> reqs;
    std::vector<lp_scan_output> outs;
    bool busy = false;
    std::atomic<bool> done{false};
    double t_start = 0.0;
    lp_server* server = nullptr;
};
} // namespace

struct lp_server
{
    int device = 0;
    lp_pipeline_config cfg{};
    lp_server_config scfg{};
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex m;
    std::condition_variable cv;
    std::deque<Request> pending;
    std::vector<lp_server_done> finished;
    std::thread worker;
    bool stop = false;
    lp_server_stats stats{};
    std::string error;
};

namespace
{
void CUDART_CB on_batch_done(void* p)
{
    Slot* s = static_cast<Slot*>(p);
    s->done.store(true, std::memory_order_release);
    std::lock_guard<std::mutex> lk(s->server->m);
    s->server->cv.notify_all();
}

// Builds the batch of the given requests into the slot; returns false when it does not fit.
lp_status plan_fits(Slot& slot, const lp_pipeline_config& cfg, const std::vector<Request>& reqs, size_t cap, bool& fits)
{
    std::vector<lp_scan_input> ins;
    ins.reserve(reqs.size());
    for (const Request& r : reqs)
        ins.push_back(r.in);
    lp_status st = lprt::fill_pipeline(slot.ctx, slot.batch, &cfg, ins.data(), static_cast<uint32_t>(ins.size()));
    if (st != LP_OK)
        return st;
    st = lprt::plan(slot.ctx, slot.batch);
    if (st != LP_OK)
        return st;
    fits = lprt::measure(slot.batch) <= cap;
    return LP_OK;
}

void finish_request(lp_server* sv, const Request& r, lp_status st, double t_start, uint32_t batch_size)
{
    const double t = now_s();
    lp_server_done d{};
    d.tag = r.tag;
    d.status = st;
    d.batch_scans = batch_size;
    d.latency_ms = (t - r.t_arrival) * 1e3;
    d.queue_ms = (t_start - r.t_arrival) * 1e3;
    std::lock_guard<std::mutex> lk(sv->m);
    sv->finished.push_back(d);
    sv->stats.completed += 1;
    if (st != LP_OK)
        sv->stats.failed += 1;
}

void harvest(lp_server* sv, Slot& slot)
{
    lp_status st = lprt::fetch_state(slot.ctx, slot.batch);
    if (st == LP_OK || st == LP_ERR_CAPACITY)
    {
        const lp_status dl = lprt::download(slot.ctx, slot.batch, slot.outs.data());
        if (st == LP_OK)
            st = dl;
    }
    for (size_t i = 0; i < slot.reqs.size(); ++i)
    {
        *slot.reqs[i].out = slot.outs[i];
        finish_request(sv, slot.reqs[i], st != LP_OK ? st : slot.outs[i].status, slot.t_start,
                       static_cast<uint32_t>(slot.reqs.size()));
    }
    slot.reqs.clear();
    slot.outs.clear();
    slot.busy = false;
    slot.done.store(false);
}

// Takes the oldest pending scans that fit into the slot and starts them. Called with the lock held.
void admit(lp_server* sv, Slot& slot, std::unique_lock<std::mutex>& lk)
{
    const size_t cap = slot.batch.cap;
    std::vector<Request> take;
    const size_t maxb = std::max<uint32_t>(1u, sv->scfg.max_batch_scans);
    while (!sv->pending.empty() && take.size() < maxb)
    {
        take.push_back(sv->pending.front());
        sv->pending.pop_front();
    }
    lk.unlock();
    // shrink the batch until its planned layout fits the slot's region
    bool fits = false;
    lp_status st = LP_OK;
    std::vector<Request> back;
    while (!take.empty())
    {
        st = plan_fits(slot, sv->cfg, take, cap, fits);
        if (st != LP_OK || fits || take.size() == 1)
            break;
        back.insert(back.begin(), take.back());
        take.pop_back();
    }
    if (!take.empty() && (st != LP_OK || !fits))
    {
        // a single scan larger than a slot (or malformed): fail it, keep the rest pending
        finish_request(sv, take.front(), st != LP_OK ? st : LP_ERR_CAPACITY, now_s(), 1);
        back.insert(back.begin(), take.begin() + 1, take.end());
        take.clear();
    }
    if (!take.empty())
    {
        slot.reqs = take;
        slot.outs.clear();
        for (const Request& r : take)
            slot.outs.push_back(*r.out);
        slot.t_start = now_s();
        slot.done.store(false);
        st = lprt::build(slot.ctx, slot.batch);
        if (st == LP_OK)
            st = lprt::upload(slot.ctx, slot.batch);
        if (st == LP_OK)
            st = lprt::execute(slot.ctx, slot.batch);
        if (st == LP_OK && cudaLaunchHostFunc(slot.ctx->stream, on_batch_done, &slot) != cudaSuccess)
            st = LP_ERR_CUDA;
        if (st != LP_OK)
        {
            cudaStreamSynchronize(slot.ctx->stream);
            for (const Request& r : take)
                finish_request(sv, r, st, slot.t_start, static_cast<uint32_t>(take.size()));
            slot.reqs.clear();
        }
        else
        {
            slot.busy = true;
        }
    }
    lk.lock();
    if (!take.empty() && slot.busy)
    {
        sv->stats.batches += 1;
        sv->stats.scans_in_batches += take.size();
        sv->stats.max_batch_seen = std::max<uint64_t>(sv->stats.max_batch_seen, take.size());
    }
    for (auto it = back.rbegin(); it != back.rend(); ++it)
        sv->pending.push_front(*it);
}

void worker_loop(lp_server* sv)
{
    cudaSetDevice(sv->device);
    std::unique_lock<std::mutex> lk(sv->m);
    for (;;)
    {
        bool any_done = false, any_busy = false;
        for (auto& s : sv->slots)
        {
            any_done |= s->busy && s->done.load(std::memory_order_acquire);
            any_busy |= s->busy;
        }
        if (sv->stop && sv->pending.empty() && !any_busy)
            break;
        bool idle_slot = false;
        for (auto& s : sv->slots)
            idle_slot |= !s->busy;
        if (!any_done && (sv->pending.empty() || !idle_slot))
        {
            sv->cv.wait_for(lk, std::chrono::microseconds(500));
            continue;
        }
        for (auto& s : sv->slots)
            if (s->busy && s->done.load(std::memory_order_acquire))
            {
                lk.unlock();
                harvest(sv, *s);
                lk.lock();
            }
        for (auto& s : sv->slots)
            if (!s->busy && !sv->pending.empty())
                admit(sv, *s, lk);
    }
}
} // namespace

extern "C" {

void lp_server_config_default(lp_server_config* c)
{
    c->memory_budget_bytes = 20ull << 30; // the serving workload's 20 GB admission budget
    c->max_batch_scans = 16;
    c->slots = 3;
}

lp_status lp_server_create(int32_t device, const lp_pipeline_config* cfg, const lp_server_config* scfg, lp_server** out)
{
    if (!cfg || !scfg || !out || scfg->slots == 0 || scfg->memory_budget_bytes == 0)
        return LP_ERR_BAD_ARG;
    *out = nullptr;
    auto sv = std::make_unique<lp_server>();
    sv->device = device;
    sv->cfg = *cfg;
    sv->scfg = *scfg;
    const size_t per_slot = static_cast<size_t>(scfg->memory_budget_bytes / scfg->slots);
    for (uint32_t i = 0; i < scfg->slots; ++i)
    {
        auto s = std::make_unique<Slot>();
        s->server = sv.get();
        lp_status st = lp_context_create(device, &s->ctx);
        if (st != LP_OK)
            return st;
        // the slot's region is reserved once; batches are admitted only when they fit it
        if (cudaMalloc(reinterpret_cast<void**>(&s->batch.mem), per_slot) != cudaSuccess)
        {
            cudaGetLastError();
            lp_context_destroy(s->ctx);
            for (auto& o : sv->slots)
            {
                cudaFree(o->batch.mem);
                o->batch.mem = nullptr;
                lp_context_destroy(o->ctx);
            }
            return LP_ERR_CAPACITY;
        }
        s->batch.cap = per_slot;
        sv->slots.push_back(std::move(s));
    }
    sv->stats.device_bytes = static_cast<uint64_t>(per_slot) * scfg->slots;
    lp_server* raw = sv.release();
    raw->worker = std::thread(worker_loop, raw);
    *out = raw;
    return LP_OK;
}

lp_status lp_server_submit(lp_server* sv, const lp_scan_input* scan, lp_scan_output* out, uint64_t tag)
{
    if (!sv || !scan || !out || (scan->n && !scan->xyzi))
        return LP_ERR_BAD_ARG;
    Request r{tag, *scan, out, now_s()};
    {
        std::lock_guard<std::mutex> lk(sv->m);
        if (sv->stop)
            return LP_ERR_BAD_ARG;
        sv->pending.push_back(r);
        sv->stats.submitted += 1;
    }
    sv->cv.notify_all();
    return LP_OK;
}

lp_status lp_server_poll(lp_server* sv, lp_server_done* done, uint32_t capacity, uint32_t* n_done, uint32_t wait_us)
{
    if (!sv || !n_done || (capacity && !done))
        return LP_ERR_BAD_ARG;
    std::unique_lock<std::mutex> lk(sv->m);
    if (sv->finished.empty() && wait_us)
        sv->cv.wait_for(lk, std::chrono::microseconds(wait_us), [&] { return !sv->finished.empty(); });
    const uint32_t k = static_cast<uint32_t>(std::min<size_t>(capacity, sv->finished.size()));
    for (uint32_t i = 0; i < k; ++i)
        done[i] = sv->finished[i];
    sv->finished.erase(sv->finished.begin(), sv->finished.begin() + k);
    *n_done = k;
    return LP_OK;
}

lp_status lp_server_stats_get(lp_server* sv, lp_server_stats* out)
{
    if (!sv || !out)
        return LP_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(sv->m);
    *out = sv->stats;
    out->pending = sv->pending.size();
    return LP_OK;
}

void lp_server_destroy(lp_server* sv)
{
    if (!sv)
        return;
    {
        std::lock_guard<std::mutex> lk(sv->m);
        sv->stop = true;
    }
    sv->cv.notify_all();
    if (sv->worker.joinable())
        sv->worker.join();
    for (auto& s : sv->slots)
    {
        cudaStreamSynchronize(s->ctx->stream);
        if (s->batch.graph)
            cudaGraphExecDestroy(s->batch.graph);
        cudaFree(s->batch.mem);
        s->batch.mem = nullptr;
        lp_context_destroy(s->ctx);
    }
    delete sv;
}

} // extern "C"
