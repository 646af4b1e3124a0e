// gmle_server.cu - the serving loop of libgaussmle_sm100a.so (gmle_server_* and
// gmle_submit / gmle_poll / gmle_wait in include/gaussmle_gb300.h).
//
// One scheduler thread per context:
//   submit  -> pending (FIFO)          gmle_submit, any thread
//   admit   -> arena allocation (device memory budget), ROIs and corners copied
//              in on the input stream                        (admission by HBM)
//   step    -> every admitted request whose copy has landed joins the next
//              step: one persistent table launch per (camera family, model,
//              box) present; up to max_inflight_steps steps run concurrently
//              on their own streams, each kind's launch a replay of a CUDA
//              graph captured once per (slot, kind)        (continuous batching)
//   drain   -> results copied out on the output stream, memory released,
//              waiters woken; the latency submit -> results-on-host recorded.
// The scheduler never waits on the GPU: it polls events and sleeps briefly when
// nothing progressed, and no kernel waits on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gmle_internal.h"

namespace gmle_rt {

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxSlots = 8;
constexpr int kServerTableCap = 4096;  // groups (requests) per step and kind

enum ReqState { PENDING, STAGED, RUNNING, DRAINING, DONE, FAILED };

int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

struct Request {
    uint64_t ticket = 0;
    gmle_group host{};   // caller's descriptor and host pointers
    gmle_group dev{};    // the same with device pointers into the arena
    int64_t off = -1, bytes = 0;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    Clock::time_point t_submit, t_done;
    ReqState state = PENDING;
    gmle_status status = GMLE_OK;
};

// First-fit allocator over one device buffer.
struct Arena {
    char *base = nullptr;
    int64_t size = 0, in_use = 0, peak = 0;
    std::map<int64_t, int64_t> free_;  // offset -> length

    int64_t alloc(int64_t n)
    {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                const int64_t off = it->first, len = it->second;
                free_.erase(it);
                if (len > n) free_[off + n] = len - n;
                in_use += n;
                peak = std::max(peak, in_use);
                return off;
            }
        }
        return -1;
    }
    void release(int64_t off, int64_t n)
    {
        in_use -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct Step {
    int slot = -1;
    cudaEvent_t done = nullptr;
    std::vector<Request *> reqs;
};

}  // namespace

struct Server {
    gmle_ctx *ctx = nullptr;
    gmle_server_config cfg{};
    std::thread th;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stopping = false;
    uint64_t next_ticket = 1;
    std::deque<Request *> pending;
    std::vector<Request *> staged;
    std::vector<Step> inflight;
    std::vector<Request *> draining;
    std::unordered_map<uint64_t, Request *> table;
    std::vector<cudaEvent_t> event_pool;
    Arena arena;
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaStream_t s_step[kMaxSlots] = {};
    cudaEvent_t step_done[kMaxSlots] = {};
    bool slot_busy[kMaxSlots] = {};
    MixedSet sets[kMaxSlots];
    // per slot and kind: the captured counter reset + table launch, and the
    // shape and table it was captured for
    struct KindGraph {
        std::vector<int64_t> key;
        cudaGraphExec_t exec = nullptr;
    };
    KindGraph graphs[kMaxSlots][kKinds];
    // statistics
    int64_t submitted = 0, completed = 0, rejected = 0, failed = 0, rois_done = 0, steps = 0;
    std::vector<float> lat_ms;
    Clock::time_point first_submit, last_done;
    bool have_first = false;

    cudaEvent_t get_event()
    {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        return e;
    }
    void put_event(cudaEvent_t e)
    {
        if (e) event_pool.push_back(e);
    }

    int64_t footprint(const gmle_group &g) const
    {
        const int64_t n = g.n, b2 = (int64_t)g.desc.box * g.desc.box;
        const int P = nparams(g.desc.model);
        int64_t b = align256(4 * n * b2) + 2 * align256(4 * n * P) + align256(4 * n) + align256(n);
        if (g.desc.camera != GMLE_CAMERA_POISSON) b += 2 * align256(4 * n);
        return b;
    }

    void place(Request *r)
    {
        char *p = arena.base + r->off;
        const int64_t n = r->host.n, b2 = (int64_t)r->host.desc.box * r->host.desc.box;
        const int P = nparams(r->host.desc.model);
        r->dev = r->host;
        r->dev.data = reinterpret_cast<float *>(p);
        p += align256(4 * n * b2);
        r->dev.params = reinterpret_cast<float *>(p);
        p += align256(4 * n * P);
        r->dev.crlb = reinterpret_cast<float *>(p);
        p += align256(4 * n * P);
        r->dev.llr = reinterpret_cast<float *>(p);
        p += align256(4 * n);
        r->dev.flags = reinterpret_cast<uint8_t *>(p);
        p += align256(n);
        if (r->host.desc.camera != GMLE_CAMERA_POISSON) {
            r->dev.x_corners = reinterpret_cast<int32_t *>(p);
            p += align256(4 * n);
            r->dev.y_corners = reinterpret_cast<int32_t *>(p);
        } else {
            r->dev.x_corners = r->dev.y_corners = nullptr;
        }
    }

    void fail_request(Request *r, gmle_status st)
    {
        r->state = FAILED;
        r->status = st;
        failed++;
        if (r->off >= 0) arena.release(r->off, r->bytes);
        r->off = -1;
        cv_done.notify_all();
    }

    // Copy a request's inputs in (scheduler thread, lock not held).
    cudaError_t issue_in(Request *r)
    {
        const int64_t n = r->host.n, b2 = (int64_t)r->host.desc.box * r->host.desc.box;
        cudaError_t e = cudaMemcpyAsync((void *)r->dev.data, r->host.data, 4 * n * b2,
                                        cudaMemcpyHostToDevice, s_in);
        if (e == cudaSuccess && r->host.desc.camera != GMLE_CAMERA_POISSON) {
            e = cudaMemcpyAsync((void *)r->dev.x_corners, r->host.x_corners, 4 * n,
                                cudaMemcpyHostToDevice, s_in);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync((void *)r->dev.y_corners, r->host.y_corners, 4 * n,
                                    cudaMemcpyHostToDevice, s_in);
        }
        if (e == cudaSuccess) e = cudaEventRecord(r->ev_in, s_in);
        return e;
    }

    cudaError_t issue_out(Request *r)
    {
        const int64_t n = r->host.n;
        const int P = nparams(r->host.desc.model);
        cudaError_t e = cudaMemcpyAsync(r->host.params, r->dev.params, 4 * n * P,
                                        cudaMemcpyDeviceToHost, s_out);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(r->host.crlb, r->dev.crlb, 4 * n * P, cudaMemcpyDeviceToHost, s_out);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(r->host.llr, r->dev.llr, 4 * n, cudaMemcpyDeviceToHost, s_out);
        if (e == cudaSuccess && r->host.flags)
            e = cudaMemcpyAsync(r->host.flags, r->dev.flags, n, cudaMemcpyDeviceToHost, s_out);
        if (e == cudaSuccess) e = cudaEventRecord(r->ev_out, s_out);
        return e;
    }

    // One step: the tables of every kind in the slot's pinned buffers (read
    // in place by the kernels), then per kind present a replay of the slot's
    // graph for that kind (captured on first use, or again after its shape or
    // table changed), the kinds concurrently on the slot's fork streams.
    // Shapes come from the tuning for a full step and grids are full, so each
    // (slot, kind) is captured once: no capture stalls the loop once every
    // kind has been seen.
    gmle_status launch_step(int slot, const std::vector<Request *> &reqs)
    {
        std::vector<gmle_group> groups;
        groups.reserve(reqs.size());
        for (Request *r : reqs) groups.push_back(r->dev);
        MixedSet &m = sets[slot];
        MixedPlan plan;
        cudaStream_t s = s_step[slot];
        {
            std::lock_guard<std::mutex> lk(ctx->mu);
            PlanOptions opt;
            opt.allow_plain = false;
            opt.shape_rois = cfg.max_step_rois;
            opt.full_grid = true;
            opt.reserve_groups = kServerTableCap;
            opt.reserve_rois = cfg.max_step_rois;
            gmle_status st = plan_mixed(ctx, groups.data(), (int32_t)groups.size(), m, plan, opt);
            if (st != GMLE_OK) return st;
            if (!cfg.use_graphs) {
                st = enqueue_plan(ctx, m, plan, s);
                if (st != GMLE_OK) return st;
            } else {
                for (const TableLaunch &L : plan.launches) {
                    const TableBufs &b = m.tables[L.kind];
                    const std::vector<int64_t> key = {L.shape.tpr, L.shape.rois_per_block,
                                                      L.shape.grid, (int64_t)(uintptr_t)b.h_base,
                                                      b.cap_groups};
                    KindGraph &kg = graphs[slot][L.kind];
                    if (kg.exec && kg.key == key) continue;
                    if (kg.exec) cudaGraphExecDestroy(kg.exec);
                    kg.exec = nullptr;
                    cudaGraph_t g = nullptr;
                    GMLE_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                            "cudaStreamBeginCapture");
                    st = enqueue_table_launch(ctx, m, L, s);
                    ctx->launches--;  // counted when the graph is launched
                    const cudaError_t e = cudaStreamEndCapture(s, &g);
                    if (st != GMLE_OK) {
                        if (g) cudaGraphDestroy(g);
                        return st;
                    }
                    GMLE_CK(e, "cudaStreamEndCapture");
                    const cudaError_t e2 = cudaGraphInstantiate(&kg.exec, g, 0);
                    cudaGraphDestroy(g);
                    GMLE_CK(e2, "cudaGraphInstantiate");
                    kg.key = key;
                }
                const int nl = (int)plan.launches.size();
                const int nf = std::min(nl, kForks);
                if (nl > 1) {
                    GMLE_CK(cudaEventRecord(m.ev_fork, s), "cudaEventRecord");
                    for (int f = 0; f < nf; f++)
                        GMLE_CK(cudaStreamWaitEvent(m.fork[f], m.ev_fork, 0), "cudaStreamWaitEvent");
                }
                for (int l = 0; l < nl; l++) {
                    const TableLaunch &L = plan.launches[l];
                    const int f = plan_stream(l, holds_tmem(L.scmos, L.shape.tpr), nf);
                    GMLE_CK(cudaGraphLaunch(graphs[slot][L.kind].exec, nl > 1 ? m.fork[f] : s),
                            "cudaGraphLaunch");
                    ctx->launches++;
                }
                for (int f = 0; nl > 1 && f < nf; f++) {
                    GMLE_CK(cudaEventRecord(m.ev_join[f], m.fork[f]), "cudaEventRecord");
                    GMLE_CK(cudaStreamWaitEvent(s, m.ev_join[f], 0), "cudaStreamWaitEvent");
                }
            }
        }
        GMLE_CK(cudaEventRecord(step_done[slot], s), "cudaEventRecord");
        return GMLE_OK;
    }

    void loop()
    {
        cudaSetDevice(ctx->device);
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            bool progress = false;
            // 1. admission: FIFO into the arena, inputs copied in
            while (!pending.empty()) {
                Request *r = pending.front();
                const int64_t off = arena.alloc(r->bytes);
                if (off < 0) break;
                pending.pop_front();
                r->off = off;
                place(r);
                r->state = STAGED;
                lk.unlock();
                const cudaError_t e = issue_in(r);
                lk.lock();
                if (e != cudaSuccess) {
                    cuda_fail(nullptr, e, "input copy");
                    fail_request(r, GMLE_CUDA_ERROR);
                } else {
                    staged.push_back(r);
                }
                progress = true;
            }
            // 2. continuous batching: every request whose data has landed joins
            //    the next launch while a slot is free
            int slot = -1;
            for (int k = 0; k < cfg.max_inflight_steps; k++)
                if (!slot_busy[k]) { slot = k; break; }
            if (slot >= 0 && !staged.empty()) {
                std::vector<Request *> step;
                int64_t rois = 0;
                int ngroups = 0;
                for (auto it = staged.begin(); it != staged.end();) {
                    if (rois >= cfg.max_step_rois || ngroups >= kServerTableCap) break;
                    if (cudaEventQuery((*it)->ev_in) == cudaSuccess) {
                        rois += (*it)->host.n;
                        ngroups++;
                        (*it)->state = RUNNING;
                        step.push_back(*it);
                        it = staged.erase(it);
                    } else {
                        ++it;
                    }
                }
                if (!step.empty()) {
                    slot_busy[slot] = true;
                    lk.unlock();
                    const gmle_status st = launch_step(slot, step);
                    lk.lock();
                    if (st != GMLE_OK) {
                        for (Request *r : step) fail_request(r, st);
                        slot_busy[slot] = false;
                    } else {
                        steps++;
                        Step s;
                        s.slot = slot;
                        s.done = step_done[slot];
                        s.reqs = std::move(step);
                        inflight.push_back(std::move(s));
                    }
                    progress = true;
                }
            }
            // 3. finished launches: copy results out
            for (auto it = inflight.begin(); it != inflight.end();) {
                if (cudaEventQuery(it->done) != cudaSuccess) {
                    ++it;
                    continue;
                }
                std::vector<Request *> reqs = std::move(it->reqs);
                slot_busy[it->slot] = false;
                it = inflight.erase(it);
                lk.unlock();
                std::vector<cudaError_t> errs;
                for (Request *r : reqs) errs.push_back(issue_out(r));
                lk.lock();
                for (size_t q = 0; q < reqs.size(); q++) {
                    if (errs[q] != cudaSuccess) {
                        fail_request(reqs[q], GMLE_CUDA_ERROR);
                    } else {
                        reqs[q]->state = DRAINING;
                        draining.push_back(reqs[q]);
                    }
                }
                progress = true;
            }
            // 4. results on the host: release memory, wake waiters
            for (auto it = draining.begin(); it != draining.end();) {
                Request *r = *it;
                if (cudaEventQuery(r->ev_out) != cudaSuccess) {
                    ++it;
                    continue;
                }
                it = draining.erase(it);
                r->t_done = Clock::now();
                r->state = DONE;
                arena.release(r->off, r->bytes);
                r->off = -1;
                completed++;
                rois_done += r->host.n;
                last_done = r->t_done;
                if (lat_ms.size() < (1u << 22))
                    lat_ms.push_back(
                        std::chrono::duration<float, std::milli>(r->t_done - r->t_submit).count());
                cv_done.notify_all();
                progress = true;
            }
            const bool busy = !pending.empty() || !staged.empty() || !inflight.empty() ||
                              !draining.empty();
            if (stopping && !busy) break;
            if (!progress) {
                if (!busy) {
                    cv_work.wait(lk);
                } else {
                    lk.unlock();
                    std::this_thread::sleep_for(std::chrono::microseconds(20));
                    lk.lock();
                }
            }
        }
    }
};

void server_destroy(gmle_ctx *ctx)
{
    Server *S = ctx->server;
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stopping = true;
    }
    S->cv_work.notify_all();
    if (S->th.joinable()) S->th.join();
    cudaSetDevice(ctx->device);
    for (int k = 0; k < kMaxSlots; k++) {
        if (S->s_step[k]) cudaStreamSynchronize(S->s_step[k]);
        for (auto &g : S->graphs[k])
            if (g.exec) cudaGraphExecDestroy(g.exec);
        free_mixed_set(S->sets[k]);
        if (S->s_step[k]) cudaStreamDestroy(S->s_step[k]);
        if (S->step_done[k]) cudaEventDestroy(S->step_done[k]);
    }
    if (S->s_in) cudaStreamDestroy(S->s_in);
    if (S->s_out) cudaStreamDestroy(S->s_out);
    for (auto &kv : S->table) {
        if (kv.second->ev_in) cudaEventDestroy(kv.second->ev_in);
        if (kv.second->ev_out) cudaEventDestroy(kv.second->ev_out);
        delete kv.second;
    }
    for (cudaEvent_t e : S->event_pool) cudaEventDestroy(e);
    cudaFree(S->arena.base);
    delete S;
    ctx->server = nullptr;
}

}  // namespace gmle_rt

using namespace gmle_rt;

extern "C" {

gmle_status gmle_server_start(gmle_ctx *ctx, const gmle_server_config *config)
{
    if (!ctx) return GMLE_INVALID_ARG;
    if (ctx->server) return fail(ctx, GMLE_INVALID_ARG, "server already running");
    cudaSetDevice(ctx->device);
    Server *S = new Server();
    S->ctx = ctx;
    if (config) {
        S->cfg = *config;
    } else {
        S->cfg.use_graphs = 1;
    }
    if (S->cfg.max_inflight_steps <= 0) S->cfg.max_inflight_steps = 4;
    S->cfg.max_inflight_steps = std::min(S->cfg.max_inflight_steps, kMaxSlots);
    if (S->cfg.max_step_rois <= 0) S->cfg.max_step_rois = 1ll << 21;
    if (S->cfg.max_pending <= 0) S->cfg.max_pending = 1 << 16;
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) {
        delete S;
        return cuda_fail(ctx, e, "cudaMemGetInfo");
    }
    int64_t budget = S->cfg.hbm_budget_bytes > 0 ? S->cfg.hbm_budget_bytes : (int64_t)(free_b / 2);
    budget = std::min<int64_t>(budget, (int64_t)(free_b - std::min<size_t>(free_b, 1ull << 30)));
    budget &= ~int64_t(255);
    if (budget <= 0) {
        delete S;
        return fail(ctx, GMLE_OUT_OF_MEMORY, "no device memory for the serving arena");
    }
    S->cfg.hbm_budget_bytes = budget;
    e = cudaMalloc(&S->arena.base, budget);
    if (e != cudaSuccess) {
        delete S;
        return cuda_fail(ctx, e, "cudaMalloc(serving arena)");
    }
    S->arena.size = budget;
    S->arena.free_[0] = budget;
    bool ok = cudaStreamCreateWithFlags(&S->s_in, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&S->s_out, cudaStreamNonBlocking) == cudaSuccess;
    for (int k = 0; ok && k < S->cfg.max_inflight_steps; k++) {
        ok = cudaStreamCreateWithFlags(&S->s_step[k], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&S->step_done[k], cudaEventDisableTiming) == cudaSuccess;
        ok = ok && init_mixed_set(ctx, S->sets[k]) == GMLE_OK;
        S->sets[k].zero_copy = true;
    }
    ctx->server = S;
    if (!ok) {
        server_destroy(ctx);
        return fail(ctx, GMLE_CUDA_ERROR, "cannot create the serving streams and buffers");
    }
    S->th = std::thread([S] { S->loop(); });
    return GMLE_OK;
}

gmle_status gmle_server_stop(gmle_ctx *ctx)
{
    if (!ctx) return GMLE_INVALID_ARG;
    server_destroy(ctx);
    return GMLE_OK;
}

gmle_status gmle_submit(gmle_ctx *ctx, const gmle_group *request, uint64_t *ticket)
{
    if (!ctx || !request || !ticket) return GMLE_INVALID_ARG;
    Server *S = ctx->server;
    if (!S) return fail(ctx, GMLE_INVALID_ARG, "server not started");
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        gmle_status st = validate_groups(ctx, request, 1);
        if (st != GMLE_OK) return st;
        if (request->n <= 0) return fail(ctx, GMLE_INVALID_ARG, "request without ROIs");
        if (request->desc.camera != GMLE_CAMERA_POISSON) {
            const int64_t box = request->desc.box;
            for (int64_t k = 0; k < request->n; k++) {
                const int64_t x = request->x_corners[k], y = request->y_corners[k];
                if (x < 1 || y < 1 || x + box - 1 > ctx->nx || y + box - 1 > ctx->ny)
                    return fail(ctx, GMLE_INVALID_ARG,
                                "ROI %lld: corner outside the calibration map", (long long)k);
            }
        }
    }
    Request *r = new Request();
    r->host = *request;
    r->bytes = S->footprint(*request);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (r->bytes > S->arena.size || (int64_t)S->pending.size() >= S->cfg.max_pending) {
            S->rejected++;
            delete r;
            std::lock_guard<std::mutex> lk2(ctx->mu);
            return fail(ctx, GMLE_ADMISSION_REJECTED,
                        "request of %lld ROIs needs %lld bytes; arena %lld, queue %zu",
                        (long long)request->n, (long long)S->footprint(*request),
                        (long long)S->arena.size, S->pending.size());
        }
        r->ev_in = S->get_event();
        r->ev_out = S->get_event();
        r->ticket = S->next_ticket++;
        S->table[r->ticket] = r;
        S->pending.push_back(r);
        S->submitted++;
        if (!S->have_first) {
            S->first_submit = r->t_submit;
            S->have_first = true;
        }
        *ticket = r->ticket;
    }
    S->cv_work.notify_one();
    return GMLE_OK;
}

static gmle_status finish_locked(Server *S, Request *r)
{
    const gmle_status st = r->state == DONE ? GMLE_OK : r->status;
    S->table.erase(r->ticket);
    S->put_event(r->ev_in);
    S->put_event(r->ev_out);
    delete r;
    return st;
}

gmle_status gmle_poll(gmle_ctx *ctx, uint64_t ticket)
{
    if (!ctx || !ctx->server) return GMLE_INVALID_ARG;
    Server *S = ctx->server;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->table.find(ticket);
    if (it == S->table.end()) return GMLE_INVALID_ARG;
    Request *r = it->second;
    if (r->state != DONE && r->state != FAILED) return GMLE_NOT_READY;
    return finish_locked(S, r);
}

gmle_status gmle_wait(gmle_ctx *ctx, uint64_t ticket, int64_t timeout_ns)
{
    if (!ctx || !ctx->server) return GMLE_INVALID_ARG;
    Server *S = ctx->server;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->table.find(ticket);
    if (it == S->table.end()) return GMLE_INVALID_ARG;
    Request *r = it->second;
    auto ready = [r] { return r->state == DONE || r->state == FAILED; };
    if (timeout_ns < 0) {
        S->cv_done.wait(lk, ready);
    } else if (!S->cv_done.wait_for(lk, std::chrono::nanoseconds(timeout_ns), ready)) {
        return GMLE_TIMEOUT;
    }
    return finish_locked(S, r);
}

gmle_status gmle_server_stats_get(gmle_ctx *ctx, gmle_server_stats *out, int32_t reset)
{
    if (!ctx || !out || !ctx->server) return GMLE_INVALID_ARG;
    Server *S = ctx->server;
    std::lock_guard<std::mutex> lk(S->mu);
    std::memset(out, 0, sizeof *out);
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->rejected = S->rejected;
    out->failed = S->failed;
    out->rois_completed = S->rois_done;
    out->steps = S->steps;
    if (!S->lat_ms.empty()) {
        std::vector<float> v = S->lat_ms;
        std::sort(v.begin(), v.end());
        auto q = [&](double p) { return (double)v[std::min(v.size() - 1, (size_t)(p * v.size()))]; };
        out->p50_latency_ms = q(0.50);
        out->p99_latency_ms = q(0.99);
        out->max_latency_ms = v.back();
        double s = 0;
        for (float x : v) s += x;
        out->mean_latency_ms = s / v.size();
    }
    if (S->have_first && S->completed > 0) {
        const double secs = std::chrono::duration<double>(S->last_done - S->first_submit).count();
        out->fits_per_s = secs > 0 ? S->rois_done / secs : 0;
    }
    out->hbm_budget_bytes = S->arena.size;
    out->hbm_in_use_bytes = S->arena.in_use;
    out->hbm_peak_bytes = S->arena.peak;
    if (reset) {
        S->submitted = S->completed = S->rejected = S->failed = S->rois_done = S->steps = 0;
        S->lat_ms.clear();
        S->have_first = false;
        S->arena.peak = S->arena.in_use;
    }
    return GMLE_OK;
}

}  // extern "C"
