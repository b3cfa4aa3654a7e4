// The serving loop: triangulation requests of mixed sizes admitted under an
// HBM budget onto resident GPU engines.
//
// * Large requests (at least small_threshold points) go to a FIFO served by
//   large_workers host threads; each thread owns an Engine -- its own CUDA
//   stream and its own device workspace, which stays allocated between
//   requests (a resident pool) and grows to the largest request it served.
// * Small requests go to a second FIFO served by one batching thread that owns
//   a many-set engine (qdtg_batch): whenever it is free it takes every small
//   request that has arrived (up to batch_max_points / batch_max_sets) and
//   triangulates them together in one pipeline. Requests that arrive while a
//   batch runs form the next batch (continuous batching).
// * The engines run on separate streams, so the work of different requests
//   overlaps on the device.
// * Admission: the device bytes of all pools (the batching pool is reserved
//   when the server starts) stay within hbm_budget_bytes. A worker whose pool
//   must grow for its next request waits until the growth fits; pools of idle
//   workers are released to make room. A request that cannot fit even alone,
//   or that finds max_queue requests waiting, is rejected with
//   QDT_ERR_OUT_OF_MEMORY. A request that finds no free worker of its kind is
//   counted as queued.
// Every result is the one qdt_execute() gives for the request alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "context.hpp"
#include "engine.hpp"
#include "host_copy.hpp"
#include "qdt.h"
#include "qdt_gpu.h"

namespace qdtg {

using Clock = std::chrono::steady_clock;

struct ServeRequest
{
    uint64_t              id = 0;
    const double*         xy = nullptr;
    size_t                n = 0;
    int                   state = 0;   // 0 waiting, 1 running, 2 done
    qdt_status            status = QDT_OK;
    std::vector<uint32_t> tris, rep;
    size_t                ntri = 0, unique = 0;
    Clock::time_point     t_submit, t_start, t_done;
    int                   path = 0;    // 0 engine, 1 coalesced batch
    bool                  queued = false;
};

struct ServeWorker
{
    Engine*             eng = nullptr;
    size_t              pool = 0;      // device bytes held (or reserved) by the engine
    bool                busy = false;
    PinnedVec<double>   pts;
    PinnedVec<uint32_t> tris, rep;
};

struct Server
{
    qdtg_server_config cfg{};
    int                device = 0;
    std::mutex         mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ServeRequest*> large_q, small_q;
    std::unordered_map<uint64_t, std::unique_ptr<ServeRequest>> reqs;
    uint64_t           next_id = 1;
    bool               stop = false;
    bool               batch_busy = false;
    std::vector<std::unique_ptr<ServeWorker>> workers;
    std::vector<std::thread> threads;
    qdtg_batch*        batch = nullptr;
    size_t             batch_pool = 0;
    PinnedVec<double>  bpts;
    qdtg_server_stats  st{};
    int                started = 0;    // worker threads that finished their set-up
    int                failed = 0;

    size_t resident() const
    {
        size_t r = batch_pool;
        for (auto& w : workers) r += w->pool;
        return r;
    }
    void note_resident()
    {
        st.resident_bytes = resident();
        st.peak_resident_bytes = std::max(st.peak_resident_bytes, st.resident_bytes);
    }

    void finish(ServeRequest* r, qdt_status s)
    {
        r->status = s;
        r->state = 2;
        r->t_done = Clock::now();
        ++st.completed;
    }

    void large_loop(ServeWorker* w);
    void batch_loop();
};

void Server::large_loop(ServeWorker* w)
{
    cudaSetDevice(device);
    int err = 0;
    w->eng = Engine::create(&err);
    {
        std::lock_guard<std::mutex> lk(mu);
        ++started;
        if (!w->eng) ++failed;
    }
    cv_done.notify_all();
    if (!w->eng) return;
    w->eng->set_cell_points(cfg.cell_points);
    // the server's engines share the GPU: the build's prefetch in line
    w->eng->set_side_prefetch(false);
    for (;;)
    {
        ServeRequest* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;)
            {
                if (!large_q.empty())
                {
                    ServeRequest* head = large_q.front();
                    size_t        need = w->eng->bytes_after(head->n);
                    if (need > w->pool && resident() - w->pool + need > cfg.hbm_budget_bytes)
                    {
                        // a pool that must grow is reallocated at the exact size
                        // (growth by a quarter may not fit), and the pools of
                        // idle workers are released
                        w->eng->release_workspace();
                        w->pool = 0;
                        need = Engine::workspace_bytes(head->n);
                        for (auto& o : workers)
                            if (o.get() != w && !o->busy && o->pool && o->eng)
                            {
                                o->eng->release_workspace();
                                o->pool = 0;
                                ++st.pool_releases;
                            }
                        note_resident();
                    }
                    const size_t grow = need > w->pool ? need - w->pool : 0;
                    if (resident() + grow <= cfg.hbm_budget_bytes)
                    {
                        large_q.pop_front();
                        r = head;
                        w->pool = std::max(w->pool, need);
                        w->busy = true;
                        note_resident();
                        break;
                    }
                }
                else if (stop)
                    return;
                cv_work.wait(lk);
            }
            r->state = 1;
            r->t_start = Clock::now();
        }
        size_t    ntri = 0, uniq = 0;
        const int s = w->eng->run_host(r->xy, r->n, w->pts, w->tris, &ntri, w->rep, &uniq);
        if (s == QDT_OK)
        {
            r->tris.assign(w->tris.begin(), w->tris.begin() + 3 * ntri);
            r->rep.assign(w->rep.begin(), w->rep.begin() + r->n);
            r->ntri = ntri;
            r->unique = uniq;
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            w->pool = w->eng->workspace_bytes();
            w->busy = false;
            note_resident();
            finish(r, (qdt_status)s);
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

void Server::batch_loop()
{
    cudaSetDevice(device);
    std::vector<ServeRequest*> take;
    std::vector<size_t>        off;
    std::vector<CopyItem>      gather;
    for (;;)
    {
        take.clear();
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stop || !small_q.empty(); });
            if (small_q.empty() && stop) return;
            size_t pts = 0;
            while (!small_q.empty() && take.size() < cfg.batch_max_sets)
            {
                ServeRequest* r = small_q.front();
                if (!take.empty() && pts + r->n > cfg.batch_max_points) break;
                small_q.pop_front();
                take.push_back(r);
                pts += r->n;
                r->state = 1;
                r->t_start = Clock::now();
            }
            batch_busy = true;
            ++st.batches;
            st.batched_requests += take.size();
        }
        off.assign(take.size() + 1, 0);
        for (size_t i = 0; i < take.size(); ++i) off[i + 1] = off[i] + take[i]->n;
        qdt_status s = QDT_OK;
        try
        {
            bpts.resize(2 * off.back());
        }
        catch (...)
        {
            s = QDT_ERR_OUT_OF_MEMORY;
        }
        if (s == QDT_OK)
        {
            gather.resize(take.size());
            for (size_t i = 0; i < take.size(); ++i)
                gather[i] = CopyItem{ bpts.data() + 2 * off[i], take[i]->xy, take[i]->n * 2 * sizeof(double) };
            parallel_copy_many(gather.data(), gather.size());
            s = qdtg_batch_execute(batch, reinterpret_cast<const qdt_vec2d*>(bpts.data()), off.data(), take.size());
        }
        for (size_t i = 0; i < take.size(); ++i)
        {
            ServeRequest* r = take[i];
            r->path = 1;
            if (s != QDT_OK)
            {
                r->status = s;
                continue;
            }
            r->status = qdtg_batch_set_status(batch, i);
            if (r->status != QDT_OK) continue;
            const uint32_t* t = nullptr;
            r->ntri = qdtg_batch_triangles(batch, i, &t);
            if (r->ntri) r->tris.assign(t, t + 3 * r->ntri);
            const uint32_t* rp = qdtg_batch_rep(batch, i);
            if (rp && r->n) r->rep.assign(rp, rp + r->n);
            r->unique = qdtg_batch_unique_points(batch, i);
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            for (ServeRequest* r : take) finish(r, r->status);
            batch_busy = false;
        }
        cv_done.notify_all();
    }
}

}  // namespace qdtg

struct qdtg_server
{
    qdtg::Server s;
};

namespace {

qdtg::ServeRequest* find_req(qdtg_server* srv, uint64_t ticket)
{
    auto it = srv->s.reqs.find(ticket);
    return it == srv->s.reqs.end() ? nullptr : it->second.get();
}

}  // namespace

extern "C" {

QDT_API void qdtg_server_default_config(qdtg_server_config* c)
{
    if (!c) return;
    c->hbm_budget_bytes = (size_t)150 << 30;
    c->large_workers = qdtg::tuning().server_large_workers;
    c->small_threshold = 65536;
    c->batch_max_points = (size_t)8 << 20;
    c->batch_max_sets = 4096;
    c->max_queue = 4096;
    c->cell_points = qdtg::tuning().cell_points;
    c->batch_cell_points = qdtg::tuning().batch_cell_points;
}

QDT_API qdtg_server* qdtg_server_create(const qdtg_server_config* config)
{
    qdtg_server_config c;
    qdtg_server_default_config(&c);
    if (config) c = *config;
    if (c.large_workers < 1 || c.large_workers > 64 || c.batch_max_sets < 1 || c.batch_max_points < 1 ||
        c.small_threshold > c.batch_max_points || c.batch_max_points > qdtg::kMaxPoints)
        return nullptr;
    qdtg_server* srv = new (std::nothrow) qdtg_server();
    if (!srv) return nullptr;
    qdtg::Server& s = srv->s;
    s.cfg = c;
    if (cudaGetDevice(&s.device) != cudaSuccess)
    {
        cudaGetLastError();
        delete srv;
        return nullptr;
    }
    // the batching pool: reserved for the largest batch up front
    s.batch = qdtg_batch_create();
    if (!s.batch)
    {
        delete srv;
        return nullptr;
    }
    qdtg_batch_set_options(s.batch, 0, 0, /*graphs: every batch has its own shape*/ 0, 0);
    qdtg_batch_set_cell_points(s.batch, c.batch_cell_points);
    if (c.small_threshold > 0)
    {
        if (qdtg::bcarve_bytes(std::max<size_t>(c.batch_max_points, 4096), std::max<size_t>(c.batch_max_sets, 64)) >
                c.hbm_budget_bytes ||
            qdtg_batch_reserve(s.batch, c.batch_max_points, c.batch_max_sets) != QDT_OK)
        {
            qdtg_batch_destroy(s.batch);
            delete srv;
            return nullptr;
        }
        s.batch_pool = qdtg_batch_workspace_bytes(s.batch);
    }
    s.st.hbm_budget_bytes = c.hbm_budget_bytes;
    s.note_resident();
    try
    {
        for (int i = 0; i < c.large_workers; ++i) s.workers.emplace_back(new qdtg::ServeWorker());
        for (auto& w : s.workers) s.threads.emplace_back(&qdtg::Server::large_loop, &s, w.get());
        s.threads.emplace_back(&qdtg::Server::batch_loop, &s);
    }
    catch (...)
    {
        {
            std::lock_guard<std::mutex> lk(s.mu);
            s.stop = true;
        }
        s.cv_work.notify_all();
        for (auto& t : s.threads) t.join();
        for (auto& w : s.workers) delete w->eng;
        qdtg_batch_destroy(s.batch);
        delete srv;
        return nullptr;
    }
    // wait until every worker has its engine
    {
        std::unique_lock<std::mutex> lk(s.mu);
        s.cv_done.wait(lk, [&] { return s.started == c.large_workers; });
    }
    if (s.failed)
    {
        qdtg_server_destroy(srv);
        return nullptr;
    }
    return srv;
}

QDT_API void qdtg_server_destroy(qdtg_server* srv)
{
    if (!srv) return;
    qdtg::Server& s = srv->s;
    {
        std::lock_guard<std::mutex> lk(s.mu);
        s.stop = true;
    }
    s.cv_work.notify_all();
    for (auto& t : s.threads) t.join();
    for (auto& w : s.workers) delete w->eng;
    if (s.batch) qdtg_batch_destroy(s.batch);
    delete srv;
}

QDT_API qdt_status qdtg_server_submit(qdtg_server* srv, const qdt_vec2d* pts, size_t n, uint64_t* ticket)
{
    if (!srv) return QDT_ERR_NULL_CONTEXT;
    if (!ticket) return QDT_ERR_NULL_ARGUMENT;
    *ticket = 0;
    if (n > qdtg::kMaxPoints) return QDT_ERR_TOO_MANY_POINTS;
    if (n > 0 && !pts) return QDT_ERR_NULL_ARGUMENT;
    qdtg::Server& s = srv->s;
    std::unique_ptr<qdtg::ServeRequest> r;
    try
    {
        r.reset(new qdtg::ServeRequest());
    }
    catch (...)
    {
        return QDT_ERR_OUT_OF_MEMORY;
    }
    r->xy = reinterpret_cast<const double*>(pts);
    r->n = n;
    r->t_submit = qdtg::Clock::now();
    const bool small = n < s.cfg.small_threshold;
    qdt_status ret = QDT_OK;
    {
        std::lock_guard<std::mutex> lk(s.mu);
        if (s.stop) return QDT_ERR_INTERNAL;
        qdtg::ServeRequest* p = r.get();
        p->id = s.next_id++;
        *ticket = p->id;
        ++s.st.submitted;
        try
        {
            s.reqs.emplace(p->id, std::move(r));
        }
        catch (...)
        {
            --s.st.submitted;
            *ticket = 0;
            return QDT_ERR_OUT_OF_MEMORY;
        }
        if (n == 0)
        {
            p->t_start = p->t_submit;
            s.finish(p, QDT_OK);
        }
        else if ((!small && qdtg::Engine::workspace_bytes(n) + s.batch_pool > s.cfg.hbm_budget_bytes) ||
                 s.large_q.size() + s.small_q.size() >= s.cfg.max_queue)
        {
            ++s.st.rejected;
            p->t_start = p->t_submit;
            s.finish(p, QDT_ERR_OUT_OF_MEMORY);
            ret = QDT_ERR_OUT_OF_MEMORY;
        }
        else if (small)
        {
            p->queued = s.batch_busy || !s.small_q.empty();
            s.small_q.push_back(p);
        }
        else
        {
            size_t idle = 0;
            for (auto& w : s.workers) idle += w->busy ? 0 : 1;
            p->queued = idle <= s.large_q.size();
            s.large_q.push_back(p);
        }
        if (p->queued) ++s.st.queued;
    }
    if (ret == QDT_OK && n > 0) s.cv_work.notify_all();
    else s.cv_done.notify_all();
    return ret;
}

QDT_API int qdtg_server_wait(qdtg_server* srv, uint64_t ticket, double timeout_s)
{
    if (!srv) return -1;
    qdtg::Server&                s = srv->s;
    std::unique_lock<std::mutex> lk(s.mu);
    qdtg::ServeRequest*          r = find_req(srv, ticket);
    if (!r) return -1;
    if (timeout_s < 0)
        s.cv_done.wait(lk, [&] { return r->state == 2; });
    else
        s.cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return r->state == 2; });
    return r->state == 2 ? 1 : 0;
}

QDT_API qdt_status qdtg_server_result(qdtg_server* srv, uint64_t ticket, const uint32_t** tris, size_t* ntri,
    const uint32_t** rep, size_t* unique_points)
{
    if (!srv) return QDT_ERR_NULL_CONTEXT;
    std::lock_guard<std::mutex> lk(srv->s.mu);
    qdtg::ServeRequest*         r = find_req(srv, ticket);
    if (!r) return QDT_ERR_INVALID_INDEX;
    if (r->state != 2) return QDT_ERR_NO_TRIANGLES;
    if (tris) *tris = r->tris.empty() ? nullptr : r->tris.data();
    if (ntri) *ntri = r->ntri;
    if (rep) *rep = r->rep.empty() ? nullptr : r->rep.data();
    if (unique_points) *unique_points = r->unique;
    return r->status;
}

QDT_API int qdtg_server_timing(qdtg_server* srv, uint64_t ticket, double* queue_ms, double* run_ms,
    double* total_ms, int* path)
{
    if (!srv) return 0;
    std::lock_guard<std::mutex> lk(srv->s.mu);
    qdtg::ServeRequest*         r = find_req(srv, ticket);
    if (!r || r->state != 2) return 0;
    using ms = std::chrono::duration<double, std::milli>;
    if (queue_ms) *queue_ms = ms(r->t_start - r->t_submit).count();
    if (run_ms) *run_ms = ms(r->t_done - r->t_start).count();
    if (total_ms) *total_ms = ms(r->t_done - r->t_submit).count();
    if (path) *path = r->path;
    return 1;
}

QDT_API int qdtg_server_release(qdtg_server* srv, uint64_t ticket)
{
    if (!srv) return 0;
    std::lock_guard<std::mutex> lk(srv->s.mu);
    auto                        it = srv->s.reqs.find(ticket);
    if (it == srv->s.reqs.end() || it->second->state != 2) return 0;
    srv->s.reqs.erase(it);
    return 1;
}

QDT_API void qdtg_server_get_stats(qdtg_server* srv, qdtg_server_stats* out)
{
    if (!srv || !out) return;
    std::lock_guard<std::mutex> lk(srv->s.mu);
    *out = srv->s.st;
    out->waiting = srv->s.large_q.size() + srv->s.small_q.size();
}

}  // extern "C"
