// gmle_server.cu - the serving loop of libgaussmle_sm100a.so (gmle_server_* and
// gmle_submit / gmle_poll / gmle_wait in include/gaussmle_gb300.h).
//
// One scheduler thread per context:
//   submit  -> pending (FIFO)          gmle_submit, any thread
//   admit   -> arena allocation (device memory budget); ROIs and corners
//              not in pinned memory copied in on the input stream; those in
//              pinned memory are read in place by the kernels, so such a
//              request is ready at once                      (admission by HBM)
//   step    -> every admitted request that is ready (read in place, or its
//              copy has landed) joins the next step: one table launch per (camera family, model, box)
//              present; up to max_inflight_steps steps run concurrently,
//              their launches spread over a few run streams: one block per
//              tile, or a replay of a CUDA graph of a persistent launch
//              captured once per (slot, kind)               (continuous batching)
//   drain   -> results copied out on the output stream, memory released,
//              waiters woken; the latency submit -> results-on-host recorded.
//              Outputs in pinned (page-locked) host memory are written by the
//              kernels themselves over the host link, so such a request is
//              done when its step is: no copy-out call and no output stream.
// The scheduler never waits on the GPU: it polls events and sleeps briefly when
// nothing progressed, and no kernel waits on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
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
// Streams that run the steps' launches.  With the input and output streams
// they are 8, the number of hardware work queues a CUDA context has by
// default (CUDA_DEVICE_MAX_CONNECTIONS): more streams would share queues, and
// a launch could then wait behind an unrelated one.
constexpr int kRunStreams = 6;
constexpr int kServerTableCap = 4096;  // groups (requests) per step and kind
constexpr size_t kLatencyRecord = 1 << 20;  // latencies kept for the percentiles

enum ReqState { PENDING, STAGED, RUNNING, DRAINING, DONE, FAILED };

int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

struct Request {
    uint64_t ticket = 0;
    gmle_group host{};   // caller's descriptor and host pointers
    gmle_group dev{};    // the same with device pointers into the arena
    // outputs written in place: device addresses of the caller's pinned
    // params, crlb, llr, flags (all pinned, or the request copies them out)
    bool direct_out = false;
    void *out_dev[4] = {};
    // corners read in place: device addresses of the caller's pinned corners
    // (sCMOS requests whose both corner arrays are pinned)
    bool direct_corners = false;
    const int32_t *corner_dev[2] = {};
    // pixels read in place: the device address of the caller's pinned ROI
    // data (no input copy; the request is ready when admitted)
    bool direct_in = false;
    const float *data_dev = nullptr;
    bool landed = false;  // nothing to copy in: ready when admitted
    int64_t off = -1, bytes = 0;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    Clock::time_point t_submit, t_done;
    // timeline (recorded when GMLE_SERVER_TRACE names a file): admitted (input
    // copy issued), joined a step (its copy had landed), step launched
    Clock::time_point t_admit, t_join, t_launch;
    int64_t step_id = -1;
    // GPU times (timed events, trace only): input copy start and end, and
    // the end of the request's step, in ms after the server's base event
    cudaEvent_t ev_in0 = nullptr;
    float g_copy0 = -1.f, g_copy1 = -1.f, g_step = -1.f;
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
    std::vector<cudaEvent_t> done;  // one per launch, recorded after it (the slot's)
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
    cudaStream_t s_run[kRunStreams] = {};
    cudaStream_t s_capture = nullptr;  // graph capture only: never runs work
    int next_run = 0;
    // per slot and kind: the event after that kind's launch (scheduler thread
    // only, created on first use; a slot's step has at most one launch per kind)
    cudaEvent_t launch_done[kMaxSlots][kKinds] = {};
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
    // request timeline, written to trace_path as CSV when the server stops
    std::string trace_path;
    struct TraceRow {
        uint64_t ticket;
        int64_t n, step;
        int kind;
        double submit, admit, join, launch, done;  // ms since the server started
        float copy0, copy1, gstep;                 // GPU ms after ev_base
    };
    std::vector<TraceRow> trace;
    Clock::time_point t_start;
    cudaEvent_t ev_base = nullptr;  // trace only: recorded on the input stream at start
    bool tracing() const { return !trace_path.empty(); }

    void trace_request(const Request *r)
    {
        if (trace_path.empty() || trace.size() >= (1u << 22)) return;
        auto ms = [&](Clock::time_point t) {
            return std::chrono::duration<double, std::milli>(t - t_start).count();
        };
        float c0 = -1.f, c1 = -1.f;
        if (!r->landed) {  // a request read in place made no copy
            if (r->ev_in0 && cudaEventElapsedTime(&c0, ev_base, r->ev_in0) != cudaSuccess) c0 = -1.f;
            if (cudaEventElapsedTime(&c1, ev_base, r->ev_in) != cudaSuccess) c1 = -1.f;
        }
        cudaGetLastError();
        trace.push_back({r->ticket, r->host.n, r->step_id, kind_of(r->host.desc), ms(r->t_submit),
                         ms(r->t_admit), ms(r->t_join), ms(r->t_launch), ms(r->t_done), c0, c1,
                         r->g_step});
    }
    void write_trace() const
    {
        if (trace_path.empty()) return;
        FILE *f = std::fopen(trace_path.c_str(), "w");
        if (!f) return;
        std::fprintf(f, "ticket,n,kind,step,submit_ms,admit_ms,join_ms,launch_ms,done_ms,"
                        "gpu_copy_start_ms,gpu_copy_end_ms,gpu_step_end_ms\n");
        for (const TraceRow &t : trace)
            std::fprintf(f, "%llu,%lld,%d,%lld,%.4f,%.4f,%.4f,%.4f,%.4f,%.4f,%.4f,%.4f\n",
                         (unsigned long long)t.ticket, (long long)t.n, t.kind, (long long)t.step,
                         t.submit, t.admit, t.join, t.launch, t.done, t.copy0, t.copy1, t.gstep);
        std::fclose(f);
    }

    cudaEvent_t get_event()
    {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreateWithFlags(&e, tracing() ? cudaEventDefault : cudaEventDisableTiming);
        return e;
    }
    void put_event(cudaEvent_t e)
    {
        if (e) event_pool.push_back(e);
    }

    static int64_t footprint(const gmle_group &g, bool direct_in, bool direct_out,
                             bool direct_corners)
    {
        const int64_t n = g.n, b2 = (int64_t)g.desc.box * g.desc.box;
        const int P = nparams(g.desc.model);
        int64_t b = direct_in ? 0 : align256(4 * n * b2);
        if (!direct_out) b += 2 * align256(4 * n * P) + align256(4 * n) + align256(n);
        if (g.desc.camera != GMLE_CAMERA_POISSON && !direct_corners) b += 2 * align256(4 * n);
        return b;
    }

    void place(Request *r)
    {
        char *p = arena.base + r->off;
        const int64_t n = r->host.n, b2 = (int64_t)r->host.desc.box * r->host.desc.box;
        const int P = nparams(r->host.desc.model);
        r->dev = r->host;
        if (r->direct_in) {
            r->dev.data = r->data_dev;
        } else {
            r->dev.data = reinterpret_cast<float *>(p);
            p += align256(4 * n * b2);
        }
        if (r->direct_out) {
            r->dev.params = static_cast<float *>(r->out_dev[0]);
            r->dev.crlb = static_cast<float *>(r->out_dev[1]);
            r->dev.llr = static_cast<float *>(r->out_dev[2]);
            r->dev.flags = static_cast<uint8_t *>(r->out_dev[3]);
        } else {
            r->dev.params = reinterpret_cast<float *>(p);
            p += align256(4 * n * P);
            r->dev.crlb = reinterpret_cast<float *>(p);
            p += align256(4 * n * P);
            r->dev.llr = reinterpret_cast<float *>(p);
            p += align256(4 * n);
            r->dev.flags = reinterpret_cast<uint8_t *>(p);
            p += align256(n);
        }
        if (r->host.desc.camera != GMLE_CAMERA_POISSON && r->direct_corners) {
            r->dev.x_corners = r->corner_dev[0];
            r->dev.y_corners = r->corner_dev[1];
        } else if (r->host.desc.camera != GMLE_CAMERA_POISSON) {
            r->dev.x_corners = reinterpret_cast<int32_t *>(p);
            p += align256(4 * n);
            r->dev.y_corners = reinterpret_cast<int32_t *>(p);
        } else {
            r->dev.x_corners = r->dev.y_corners = nullptr;
        }
    }

    // Results on the host: memory released, waiters woken (lock held).
    void complete(Request *r)
    {
        r->t_done = Clock::now();
        trace_request(r);
        r->state = DONE;
        arena.release(r->off, r->bytes);
        r->off = -1;
        completed++;
        rois_done += r->host.n;
        last_done = r->t_done;
        if (lat_ms.size() < kLatencyRecord)
            lat_ms.push_back(std::chrono::duration<float, std::milli>(r->t_done - r->t_submit).count());
        cv_done.notify_all();
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

    // Copy a request's inputs in (scheduler thread, lock not held).  A
    // request whose pixels and corners are all read in place has nothing to
    // copy and is ready at once.
    cudaError_t issue_in(Request *r)
    {
        const int64_t n = r->host.n, b2 = (int64_t)r->host.desc.box * r->host.desc.box;
        const bool copy_corners = r->host.desc.camera != GMLE_CAMERA_POISSON && !r->direct_corners;
        if (r->direct_in && !copy_corners) {
            r->landed = true;
            return cudaSuccess;
        }
        if (r->ev_in0) cudaEventRecord(r->ev_in0, s_in);  // trace only
        cudaError_t e = cudaSuccess;
        if (!r->direct_in)
            e = cudaMemcpyAsync((void *)r->dev.data, r->host.data, 4 * n * b2,
                                cudaMemcpyHostToDevice, s_in);
        if (e == cudaSuccess && r->host.desc.camera != GMLE_CAMERA_POISSON && !r->direct_corners) {
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
    // in place by the kernels), then one launch per kind present, spread over
    // the run streams, each followed by an event in `done`.  Direct launches
    // have one block per tile.  With graphs, each launch is a replay of the
    // slot's graph of a persistent launch for that kind (captured on first
    // use, or again after its shape or table changed); shapes come from the
    // tuning for a full step and grids are full, so each (slot, kind) is
    // captured once.  Persistent launches that hold tensor memory run in
    // sequence on the first run stream.
    gmle_status launch_step(int slot, const std::vector<Request *> &reqs,
                            std::vector<cudaEvent_t> &done)
    {
        std::vector<gmle_group> groups;
        groups.reserve(reqs.size());
        for (Request *r : reqs) groups.push_back(r->dev);
        MixedSet &m = sets[slot];
        MixedPlan plan;
        std::lock_guard<std::mutex> lk(ctx->mu);
        PlanOptions opt;
        opt.allow_plain = false;
        opt.shape_rois = cfg.max_step_rois;
        // a graph replays a fixed grid: persistent launches; direct launches
        // take one block per tile
        opt.persistent = cfg.use_graphs != 0;
        opt.full_grid = true;
        opt.reserve_groups = kServerTableCap;
        opt.reserve_rois = cfg.max_step_rois;
        gmle_status st = plan_mixed(ctx, groups.data(), (int32_t)groups.size(), m, plan, opt);
        if (st != GMLE_OK) return st;
        for (const TableLaunch &L : plan.launches) {
            cudaStream_t q;
            if (L.persistent && holds_tmem(L.scmos, L.shape.tpr))
                q = s_run[0];
            else if (L.persistent)
                q = s_run[1 + next_run++ % (kRunStreams - 1)];
            else
                q = s_run[next_run++ % kRunStreams];
            if (!cfg.use_graphs) {
                st = enqueue_table_launch(ctx, m, L, q);
                if (st != GMLE_OK) return st;
            } else {
                const TableBufs &b = m.tables[L.kind];
                const std::vector<int64_t> key = {L.shape.tpr, L.shape.rois_per_block,
                                                  L.shape.grid, (int64_t)(uintptr_t)b.h_base,
                                                  b.cap_groups};
                KindGraph &kg = graphs[slot][L.kind];
                if (!kg.exec || kg.key != key) {
                    if (kg.exec) cudaGraphExecDestroy(kg.exec);
                    kg.exec = nullptr;
                    cudaGraph_t g = nullptr;
                    GMLE_CK(cudaStreamBeginCapture(s_capture, cudaStreamCaptureModeThreadLocal),
                            "cudaStreamBeginCapture");
                    st = enqueue_table_launch(ctx, m, L, s_capture);
                    ctx->launches--;  // counted when the graph is launched
                    const cudaError_t e = cudaStreamEndCapture(s_capture, &g);
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
                GMLE_CK(cudaGraphLaunch(kg.exec, q), "cudaGraphLaunch");
                ctx->launches++;
            }
            cudaEvent_t &ev = launch_done[slot][L.kind];
            if (!ev)
                GMLE_CK(cudaEventCreateWithFlags(&ev, tracing() ? cudaEventDefault
                                                                : cudaEventDisableTiming),
                        "cudaEventCreate");
            GMLE_CK(cudaEventRecord(ev, q), "cudaEventRecord");
            done.push_back(ev);
        }
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
                r->t_admit = Clock::now();
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
                // every admitted request that is ready joins, in FIFO order:
                // those read in place at once, the others when their input
                // copy has landed.  The copies run in order on one stream, so
                // after the first one still in flight only in-place requests
                // can be ready; they do not wait behind it.
                bool copies_pending = false;
                size_t keep = 0;
                for (size_t q = 0; q < staged.size(); q++) {
                    Request *r = staged[q];
                    bool ready = false;
                    if (rois < cfg.max_step_rois && ngroups < kServerTableCap)
                        ready = r->landed ||
                                (!copies_pending && cudaEventQuery(r->ev_in) == cudaSuccess);
                    if (!ready) {
                        if (!r->landed) copies_pending = true;
                        staged[keep++] = r;
                        continue;
                    }
                    rois += r->host.n;
                    ngroups++;
                    r->state = RUNNING;
                    r->t_join = Clock::now();
                    r->step_id = steps;
                    step.push_back(r);
                }
                staged.resize(keep);
                if (!step.empty()) {
                    slot_busy[slot] = true;
                    std::vector<cudaEvent_t> done;
                    lk.unlock();
                    const gmle_status st = launch_step(slot, step, done);
                    const Clock::time_point tl = Clock::now();
                    for (Request *r : step) r->t_launch = tl;
                    lk.lock();
                    if (st != GMLE_OK) {
                        // launches already enqueued still read the slot's
                        // tables and the requests' memory: wait for them
                        for (cudaEvent_t e : done) cudaEventSynchronize(e);
                        for (Request *r : step) fail_request(r, st);
                        slot_busy[slot] = false;
                    } else {
                        steps++;
                        Step s;
                        s.slot = slot;
                        s.done = std::move(done);
                        s.reqs = std::move(step);
                        inflight.push_back(std::move(s));
                    }
                    progress = true;
                }
            }
            // 3. finished launches: copy results out
            for (auto it = inflight.begin(); it != inflight.end();) {
                bool finished = true;
                for (cudaEvent_t e : it->done)
                    if (cudaEventQuery(e) != cudaSuccess) { finished = false; break; }
                if (!finished) {
                    ++it;
                    continue;
                }
                std::vector<Request *> reqs = std::move(it->reqs);
                if (tracing()) {
                    float gs = -1.f;
                    for (cudaEvent_t e : it->done) {
                        float t = -1.f;
                        if (cudaEventElapsedTime(&t, ev_base, e) == cudaSuccess) gs = std::max(gs, t);
                    }
                    cudaGetLastError();
                    for (Request *r : reqs) r->g_step = gs;
                }
                slot_busy[it->slot] = false;
                it = inflight.erase(it);
                lk.unlock();
                std::vector<cudaError_t> errs;
                for (Request *r : reqs) errs.push_back(r->direct_out ? cudaSuccess : issue_out(r));
                lk.lock();
                for (size_t q = 0; q < reqs.size(); q++) {
                    if (errs[q] != cudaSuccess) {
                        fail_request(reqs[q], GMLE_CUDA_ERROR);
                    } else if (reqs[q]->direct_out) {
                        complete(reqs[q]);  // the kernels wrote the results in place
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
                complete(r);
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
    S->write_trace();
    cudaSetDevice(ctx->device);
    for (int k = 0; k < kRunStreams; k++)
        if (S->s_run[k]) cudaStreamSynchronize(S->s_run[k]);
    for (int k = 0; k < kMaxSlots; k++) {
        for (auto &g : S->graphs[k])
            if (g.exec) cudaGraphExecDestroy(g.exec);
        for (cudaEvent_t e : S->launch_done[k])
            if (e) cudaEventDestroy(e);
        free_mixed_set(S->sets[k]);
    }
    for (int k = 0; k < kRunStreams; k++)
        if (S->s_run[k]) cudaStreamDestroy(S->s_run[k]);
    if (S->s_capture) cudaStreamDestroy(S->s_capture);
    if (S->s_in) cudaStreamDestroy(S->s_in);
    if (S->s_out) cudaStreamDestroy(S->s_out);
    for (auto &kv : S->table) {
        if (kv.second->ev_in) cudaEventDestroy(kv.second->ev_in);
        if (kv.second->ev_out) cudaEventDestroy(kv.second->ev_out);
        if (kv.second->ev_in0) cudaEventDestroy(kv.second->ev_in0);
        delete kv.second;
    }
    for (cudaEvent_t e : S->event_pool) cudaEventDestroy(e);
    if (S->ev_base) cudaEventDestroy(S->ev_base);
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
    if (config) S->cfg = *config;
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
    // streams take the device's hardware queues round-robin in creation order
    // (8 by default): the eight that carry work are created back to back so
    // that each gets a queue of its own.  An input copy that shared a queue
    // with a run stream would wait behind the fits launched there.  The capture
    // stream never submits work, so it comes last and may share a queue.
    bool ok = cudaStreamCreateWithFlags(&S->s_in, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&S->s_out, cudaStreamNonBlocking) == cudaSuccess;
    for (int k = 0; ok && k < kRunStreams; k++)
        ok = cudaStreamCreateWithFlags(&S->s_run[k], cudaStreamNonBlocking) == cudaSuccess;
    if (ok && S->cfg.use_graphs)
        ok = cudaStreamCreateWithFlags(&S->s_capture, cudaStreamNonBlocking) == cudaSuccess;
    // a slot's tables are pinned host memory read in place by its launches.
    // Direct launches take them from one pinned pool per slot, allocated here
    // for a full step (up to kServerTableCap requests, tiles of >= 16 ROIs), so
    // that no step allocates: a first allocation would synchronise the device
    // mid-stream.  Graph replays keep a table per kind at a fixed address.
    const size_t pool_bytes =
        ((kTableHeader + 256) * kKinds + sizeof(gmle::KernelArgs) * (size_t)kServerTableCap +
         sizeof(int64_t) * (size_t)(S->cfg.max_step_rois / 16 + kServerTableCap + kKinds) + 4095) &
        ~size_t(4095);
    for (int k = 0; ok && k < S->cfg.max_inflight_steps; k++) {
        S->sets[k].zero_copy = true;
        if (!S->cfg.use_graphs) {
            ok = cudaMallocHost(&S->sets[k].pool, pool_bytes) == cudaSuccess;
            if (ok) S->sets[k].pool_bytes = pool_bytes;
        }
    }
    ctx->server = S;
    if (!ok) {
        server_destroy(ctx);
        return fail(ctx, GMLE_CUDA_ERROR, "cannot create the serving streams and buffers");
    }
    // a request timeline for diagnosis, written when the server stops
    if (const char *tp = std::getenv("GMLE_SERVER_TRACE")) {
        S->trace_path = tp;
        S->trace.reserve(1 << 16);
        if (cudaEventCreate(&S->ev_base) == cudaSuccess) cudaEventRecord(S->ev_base, S->s_in);
    }
    S->t_start = Clock::now();
    // what the loop would otherwise grow while it holds its lock: the latency
    // record, the ticket table and the request events
    S->lat_ms.reserve(kLatencyRecord);
    S->table.reserve(1 << 14);
    for (int k = 0; k < 512; k++) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, S->tracing() ? cudaEventDefault : cudaEventDisableTiming) ==
            cudaSuccess)
            S->event_pool.push_back(e);
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

// Whether every corner of n ROIs of edge `box` lies inside an nx x ny map
// (1-based): the smallest and largest corner along each axis, in a loop the
// compiler vectorises, then the first offending ROI only if one exists.
static int64_t first_bad_corner(const int32_t *xc, const int32_t *yc, int64_t n, int box,
                                int32_t nx, int32_t ny)
{
    int32_t mnx = INT32_MAX, mny = INT32_MAX, mxx = INT32_MIN, mxy = INT32_MIN;
    for (int64_t k = 0; k < n; k++) {
        mnx = std::min(mnx, xc[k]);
        mxx = std::max(mxx, xc[k]);
        mny = std::min(mny, yc[k]);
        mxy = std::max(mxy, yc[k]);
    }
    const auto bad = [&](int64_t x, int64_t y) {
        return x < 1 || y < 1 || x + box - 1 > nx || y + box - 1 > ny;
    };
    if (n <= 0 || !(bad(mnx, mny) || bad(mxx, mxy))) return -1;
    for (int64_t k = 0; k < n; k++)
        if (bad(xc[k], yc[k])) return k;
    return -1;
}

// gmle_submit without waking the scheduler (notify: whether to wake it).
static gmle_status submit_one(gmle_ctx *ctx, Server *S, const gmle_group *request,
                              uint64_t *ticket, bool notify)
{
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        gmle_status st = validate_groups(ctx, request, 1);
        if (st != GMLE_OK) return st;
        if (request->n <= 0) return fail(ctx, GMLE_INVALID_ARG, "request without ROIs");
        if (request->desc.camera != GMLE_CAMERA_POISSON) {
            const int64_t k = first_bad_corner(request->x_corners, request->y_corners,
                                               request->n, request->desc.box, ctx->nx, ctx->ny);
            if (k >= 0)
                return fail(ctx, GMLE_INVALID_ARG,
                            "ROI %lld: corner outside the calibration map", (long long)k);
        }
    }
    Request *r = new Request();
    r->host = *request;
    // outputs in pinned host memory are written in place by the kernels
    const void *outs[4] = {request->params, request->crlb, request->llr, request->flags};
    r->direct_out = true;
    for (int k = 0; k < 4 && r->direct_out; k++) {
        if (!outs[k]) continue;  // flags are optional
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, outs[k]) != cudaSuccess) {
            cudaGetLastError();
            r->direct_out = false;
        } else {
            // float outputs the kernels write must be 4-byte aligned
            r->direct_out = at.type == cudaMemoryTypeHost && at.devicePointer != nullptr &&
                            (k == 3 || (reinterpret_cast<uintptr_t>(outs[k]) & 3) == 0);
            r->out_dev[k] = at.devicePointer;
        }
    }
    // corners in pinned memory are read in place too: one copy per request
    // (the pixels) instead of three, which matters when many small requests
    // arrive at once and each copy's fixed cost adds up on the copy engine
    if (request->desc.camera != GMLE_CAMERA_POISSON && request->x_corners && request->y_corners) {
        r->direct_corners = true;
        const int32_t *cs[2] = {request->x_corners, request->y_corners};
        for (int k = 0; k < 2 && r->direct_corners; k++) {
            cudaPointerAttributes at;
            if (cudaPointerGetAttributes(&at, cs[k]) != cudaSuccess) {
                cudaGetLastError();
                r->direct_corners = false;
            } else {
                r->direct_corners = at.type == cudaMemoryTypeHost && at.devicePointer != nullptr &&
                                    (reinterpret_cast<uintptr_t>(cs[k]) & 3) == 0;
                r->corner_dev[k] = static_cast<const int32_t *>(at.devicePointer);
            }
        }
    }
    // pixels in pinned memory are read in place by the kernels' staging, so
    // that the request needs no input copy: the copy engine's queue (one
    // stream, in order) would otherwise make every later request wait behind
    // a large or slow copy
    {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, request->data) != cudaSuccess) {
            cudaGetLastError();
        } else if (at.type == cudaMemoryTypeHost && at.devicePointer != nullptr &&
                   (reinterpret_cast<uintptr_t>(request->data) & 3) == 0) {
            r->direct_in = true;
            r->data_dev = static_cast<const float *>(at.devicePointer);
        }
    }
    r->bytes = Server::footprint(*request, r->direct_in, r->direct_out, r->direct_corners);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (r->bytes > S->arena.size || (int64_t)S->pending.size() >= S->cfg.max_pending) {
            S->rejected++;
            const long long need = (long long)r->bytes;
            delete r;
            std::lock_guard<std::mutex> lk2(ctx->mu);
            return fail(ctx, GMLE_ADMISSION_REJECTED,
                        "request of %lld ROIs needs %lld bytes; arena %lld, queue %zu",
                        (long long)request->n, need, (long long)S->arena.size, S->pending.size());
        }
        r->ev_in = S->get_event();
        r->ev_out = S->get_event();
        if (S->tracing()) r->ev_in0 = S->get_event();
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
    if (notify) S->cv_work.notify_one();
    return GMLE_OK;
}

gmle_status gmle_submit(gmle_ctx *ctx, const gmle_group *request, uint64_t *ticket)
{
    if (!ctx || !request || !ticket) return GMLE_INVALID_ARG;
    Server *S = ctx->server;
    if (!S) return fail(ctx, GMLE_INVALID_ARG, "server not started");
    return submit_one(ctx, S, request, ticket, true);
}

gmle_status gmle_submit_many(gmle_ctx *ctx, const gmle_group *requests, int32_t n,
                             uint64_t *tickets, int32_t *submitted)
{
    if (submitted) *submitted = 0;
    if (!ctx || n < 0 || (n > 0 && (!requests || !tickets))) return GMLE_INVALID_ARG;
    Server *S = ctx->server;
    if (!S) return fail(ctx, GMLE_INVALID_ARG, "server not started");
    // the scheduler is woken after the first request and then every 16, so
    // that the first steps run while later requests are still being
    // validated (measured: one wake-up at the end left the GPU idle meanwhile,
    // 239 against 271 M fits/s for the same requests submitted one by one)
    gmle_status st = GMLE_OK;
    int32_t k = 0;
    for (; k < n; k++) {
        st = submit_one(ctx, S, &requests[k], &tickets[k], k == 0 || (k & 15) == 15);
        if (st != GMLE_OK) break;
    }
    if (submitted) *submitted = k;
    if (k > 0) S->cv_work.notify_one();
    return st;
}

static gmle_status finish_locked(Server *S, Request *r)
{
    const gmle_status st = r->state == DONE ? GMLE_OK : r->status;
    S->table.erase(r->ticket);
    S->put_event(r->ev_in);
    S->put_event(r->ev_out);
    S->put_event(r->ev_in0);
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
