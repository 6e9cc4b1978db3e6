// lp_serve.cu — serving loop with continuous batching (lp_server_*, lidar_gb300_batch.h).
//
// Sensors submit scans as they arrive; one worker thread turns the pending queue into batches.
// Each batch runs in a slot (its own CUDA stream and context), so several batches are on the GPU
// at once (upload of one, kernels of another, download of a third). Device memory is one pool of
// the server's budget, reserved once at creation: nothing allocates or frees device memory while
// batches run. Admission is by the memory free in the pool right now: a batch is formed from the
// oldest pending scans, shrunk until its planned layout fits the largest free region, and takes
// exactly that many bytes; its region returns to the pool (merged with free neighbours) when the
// batch is harvested. A scan that fits the budget but not the memory free now waits at the head
// of the queue (first in, first out) until running batches return theirs; only a scan larger
// than the whole budget is refused (LP_ERR_CAPACITY). A host callback on the slot's stream wakes
// the worker when a batch finishes; the worker then copies results into the caller's buffers and
// records the latency from submission to results in host memory. Every scan's results are the
// same whatever batch it lands in (kernels keep scans apart).
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
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
    lp_batch batch; // mem / cap: the slot's region of the pool while a batch runs
    size_t region = 0; // offset of that region in the pool
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
    // the device-memory pool and its free regions (offset -> bytes), 256-byte granules
    char* pool = nullptr;
    size_t pool_bytes = 0;
    std::map<size_t, size_t> free_regions;
    bool blocked = false; // the queue's head waits for memory: retry after a harvest
    bool held = false;    // lp_server_hold: scans queue, no batch is admitted
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

constexpr size_t kGranule = 256;

size_t round_up(size_t v)
{
    return (v + kGranule - 1) & ~(kGranule - 1);
}

// Largest free region of the pool (0 when none).
size_t largest_free(const lp_server* sv)
{
    size_t best = 0;
    for (const auto& r : sv->free_regions)
        best = std::max(best, r.second);
    return best;
}

// First free region of at least `bytes`; returns its offset (SIZE_MAX when none).
size_t pool_take(lp_server* sv, size_t bytes)
{
    for (auto it = sv->free_regions.begin(); it != sv->free_regions.end(); ++it)
        if (it->second >= bytes)
        {
            const size_t off = it->first, len = it->second;
            sv->free_regions.erase(it);
            if (len > bytes)
                sv->free_regions.emplace(off + bytes, len - bytes);
            return off;
        }
    return SIZE_MAX;
}

// Returns a region to the pool, merged with adjacent free regions.
void pool_give(lp_server* sv, size_t off, size_t bytes)
{
    auto next = sv->free_regions.lower_bound(off);
    if (next != sv->free_regions.end() && off + bytes == next->first)
    {
        bytes += next->second;
        next = sv->free_regions.erase(next);
    }
    if (next != sv->free_regions.begin())
    {
        auto prev = std::prev(next);
        if (prev->first + prev->second == off)
        {
            prev->second += bytes;
            return;
        }
    }
    sv->free_regions.emplace(off, bytes);
}

// Plans the batch of the given requests in the slot; `bytes` receives its device footprint.
lp_status plan_bytes(Slot& slot, const lp_pipeline_config& cfg, const std::vector<Request>& reqs, size_t& bytes)
{
    std::vector<lp_scan_input> ins;
    ins.reserve(reqs.size());
    for (const Request& r : reqs)
        ins.push_back(r.in);
    lp_status st = lprt::fill_pipeline(slot.ctx, slot.batch, &cfg, ins.data(), static_cast<uint32_t>(ins.size()));
    if (st != LP_OK)
        return st;
    slot.batch.tune = lprt::tuning_for(slot.ctx, ins.data(), static_cast<uint32_t>(ins.size())); // launch shapes
    st = lprt::plan(slot.ctx, slot.batch);
    if (st != LP_OK)
        return st;
    bytes = round_up(lprt::measure(slot.batch));
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
    std::lock_guard<std::mutex> lk(sv->m);
    pool_give(sv, slot.region, slot.batch.cap);
    slot.batch.mem = nullptr;
    slot.batch.cap = 0;
    slot.busy = false;
    slot.done.store(false);
    sv->blocked = false; // memory came back: the queue's head may fit now
}

// Takes the oldest pending scans whose batch fits the largest free region of the pool and starts
// them in the slot. The head scan waits (stays first in the queue) when even alone it does not
// fit the memory free now; it is refused only when it exceeds the whole pool. Called with the
// lock held.
void admit(lp_server* sv, Slot& slot, std::unique_lock<std::mutex>& lk)
{
    std::vector<Request> take;
    const size_t maxb = std::max<uint32_t>(1u, sv->scfg.max_batch_scans);
    while (!sv->pending.empty() && take.size() < maxb)
    {
        take.push_back(sv->pending.front());
        sv->pending.pop_front();
    }
    const size_t avail = largest_free(sv);
    lk.unlock();
    // shrink the batch until its planned layout fits the largest free region
    size_t bytes = 0;
    lp_status st = LP_OK;
    std::vector<Request> back;
    while (!take.empty())
    {
        st = plan_bytes(slot, sv->cfg, take, bytes);
        if (st != LP_OK || bytes <= avail || take.size() == 1)
            break;
        back.insert(back.begin(), take.back());
        take.pop_back();
    }
    bool wait = false;
    if (!take.empty() && st != LP_OK)
    {
        // malformed: fail it, keep the rest pending
        finish_request(sv, take.front(), st, now_s(), 1);
        back.insert(back.begin(), take.begin() + 1, take.end());
        take.clear();
    }
    else if (!take.empty() && bytes > avail)
    {
        if (bytes > sv->pool_bytes)
        {
            // larger than the whole budget: it can never run
            finish_request(sv, take.front(), LP_ERR_CAPACITY, now_s(), 1);
            back.insert(back.begin(), take.begin() + 1, take.end());
        }
        else
        {
            back.insert(back.begin(), take.begin(), take.end()); // wait for memory, first in line
            wait = true;
        }
        take.clear();
    }
    if (!take.empty())
    {
        lk.lock();
        const size_t off = pool_take(sv, bytes);
        lk.unlock();
        slot.region = off;
        slot.batch.mem = sv->pool + off;
        slot.batch.cap = bytes;
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
            lk.lock();
            pool_give(sv, slot.region, slot.batch.cap);
            lk.unlock();
            slot.batch.mem = nullptr;
            slot.batch.cap = 0;
        }
        else
        {
            slot.busy = true;
        }
    }
    lk.lock();
    if (wait)
    {
        sv->blocked = true;
        sv->stats.memory_waits += 1;
    }
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
        if (!any_done && (sv->pending.empty() || !idle_slot || sv->blocked || sv->held))
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
            if (!s->busy && !sv->pending.empty() && !sv->blocked && !sv->held)
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
    // one pool of the whole budget, reserved once; batches take regions of it as they are admitted
    const size_t pool = static_cast<size_t>(scfg->memory_budget_bytes) & ~(kGranule - 1);
    if (pool == 0)
        return LP_ERR_BAD_ARG;
    if (cudaSetDevice(device) != cudaSuccess || cudaMalloc(reinterpret_cast<void**>(&sv->pool), pool) != cudaSuccess)
    {
        cudaGetLastError();
        return LP_ERR_CAPACITY;
    }
    sv->pool_bytes = pool;
    sv->free_regions.emplace(0, pool);
    for (uint32_t i = 0; i < scfg->slots; ++i)
    {
        auto s = std::make_unique<Slot>();
        s->server = sv.get();
        lp_status st = lp_context_create(device, &s->ctx);
        if (st != LP_OK)
        {
            for (auto& o : sv->slots)
                lp_context_destroy(o->ctx);
            cudaFree(sv->pool);
            return st;
        }
        sv->slots.push_back(std::move(s));
    }
    sv->stats.device_bytes = static_cast<uint64_t>(pool);
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

lp_status lp_server_hold(lp_server* sv, int32_t hold)
{
    if (!sv)
        return LP_ERR_BAD_ARG;
    {
        std::lock_guard<std::mutex> lk(sv->m);
        sv->held = hold != 0;
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
        s->batch.mem = nullptr; // a region of the pool, not its own allocation
        s->batch.cap = 0;
        lp_context_destroy(s->ctx);
    }
    cudaFree(sv->pool);
    delete sv;
}

} // extern "C"
