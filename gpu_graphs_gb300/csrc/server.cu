// server.cu -- continuous-batching BFS serving loop over HBM-resident graphs.
//
// The reference answers one query per process run (1D Partition/main.cu:10-82).
// Here a server keeps graphs resident, admits them against an HBM budget and
// answers queries as they arrive:
//   * every query joins its graph's FIFO;
//   * `num_slots` slots, each a worker thread with SRV_SUB units (a CUDA
//     stream and a single-source workspace each) and a 64-lane multi-source
//     workspace, all sized for the largest admitted graph.  A slot's
//     launches together use at most 1/num_slots of the GPU's CTAs, so every
//     slot's launches fit on the GPU at once (each launch waits on all of
//     its own CTAs);
//   * whenever a unit is free, its worker serves the ready graphs in the
//     order of their oldest query:
//       - on a graph of small degree (meshes, grids, road networks) a
//         search is a long chain of latency-bound levels that the
//         label-correcting kernel runs at nearly the same speed on a
//         fraction of the GPU, while a multi-source launch is bound by its
//         lanes' combined frontiers: each free unit takes one query as a
//         single-source search capped to 1/SRV_SUB of the slot's CTAs (the
//         slot's whole share when it is the only query waiting).  Units
//         refill one by one as their searches end, so a long search holds
//         only its own unit;
//       - on other graphs a launch packs up to `max_lanes` queries into one
//         multi-source search on the whole slot.  Such a graph is ready
//         with a full batch or once its oldest query has waited
//         `batch_window_us`, or `window_pct` percent of the graph's recent
//         launch time if longer: a launch costs about the same for one
//         source as for 64, so slow graphs gather bigger batches.  A batch
//         of one query runs on one free unit (the whole slot if all its
//         units are free).  For a larger batch a partly busy slot stops
//         filling units until they are free (one slot per waiting batch
//         graph; the others keep filling behind it), so the batch is not
//         overtaken by later queries;
//   * a stream callback tells the worker when a launch's search, and then
//     its result copies, are done; results are in the caller's buffer
//     before the ticket completes (latency = submit -> result in place).
#include <algorithm>
#include <cstddef>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "graph.cuh"
#include "server_plan.h"

using namespace gbfs;
using Clock = std::chrono::steady_clock;

namespace {

struct SrvQuery {
    int64_t ticket = 0;
    int32_t gid = 0, source = 0;
    int32_t *out = nullptr;
    Clock::time_point t_submit, t_launch;
    bool done = false;
    int status = GBFS_OK;
    double latency_ms = 0, queue_ms = 0;
    int lanes = 0;
};

struct SrvGraph {
    gbfs_graph *g = nullptr;
    // the graph's device buffers as admitted (out-edges, pull pieces and, for
    // a directed graph, its transpose); none of them moves or is freed while
    // the graph is resident, so workers launch on this copy without g->mu
    DeviceCsr csr;
    int64_t bytes = 0;
    std::deque<std::shared_ptr<SrvQuery>> pending;
    int inflight = 0;
    double est_us = 0;     // recent launch time (moving average), 0 before the first
    bool singles = false;  // small degree: served as single-source searches
    int drainer = -1;      // the slot that stops filling units for this graph's next batch
};

// Units (concurrent single-source searches) per slot.  A 4000 x 4000 grid
// search takes 12.7 ms on the whole GPU and 18.8 ms capped to 19 CTAs; 16
// such searches at once finish in 21.5 ms each (677 queries/s against 76 one
// after another), given enough hardware work queues
// (CUDA_DEVICE_MAX_CONNECTIONS: with CUDA's default of 8, about four
// searches progress at a time).  On the 32-graph serving mix, with a slot's
// units refilled as a group: 6 slots of 4 units, capacity up to 3,358
// queries/s (4 slots 2,713, 8 slots 2,999; 8 units per slot 2,816);
// batching such a graph's queries into multi-source launches from 16
// pending on was slower.
#ifndef SRV_SUB_DEF
#define SRV_SUB_DEF 4
#endif
constexpr int SRV_SUB = SRV_SUB_DEF;

// 64-lane workspace + SRV_SUB single-source workspaces (level, 3 bitmaps +
// visited, 4 int lists, the row bounds beside the two queues, the control
// block)
int64_t slot_bytes(int64_t n)
{
    return n > 0 ? ms_work_bytes(n) + SRV_SUB * (4 * n * 5 + 16 * n + n / 2 + (int64_t)sizeof(BfsCtrl)) + (1 << 20)
                 : 0;
}

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// One launch on a slot: a single-source search on unit j's stream and
// workspace, or (the slot taken whole) a multi-source batch or a search with
// all of the slot's CTAs on unit 0.  busy and the queries are read and
// written under the server's mutex, signalled under the slot's signal mutex,
// phase only by the slot's worker.
struct SrvJob {
    gbfs_server *srv = nullptr;
    int slot = 0;
    bool busy = false;       // the unit holds a launch (planned or in flight)
    bool signalled = false;  // the stream passed the launch's callback
    int phase = 0;           // 1: search and status copy in flight, 2: result copies in flight
    bool batch = false;      // a multi-source launch on the slot's 64-lane workspace
    int cap = 0;             // CTA cap of a single-source search
    int32_t gid = 0;
    SrvGraph *sg = nullptr;  // stays valid: a graph with queries in flight is not removed
    std::vector<std::shared_ptr<SrvQuery>> qs;
    std::vector<int32_t> srcs;
    Clock::time_point t_launch;
};

}  // namespace

struct gbfs_server {
    gbfs_server_config cfg{};
    int device = 0;
    int max_ctas = 0;
    // held by gbfs_server_add_graph from its budget check to its commit, so
    // concurrent admissions see each other's bytes and never resize the slot
    // workspaces against a stale capacity (workers never take it)
    std::mutex admit_mu;
    std::mutex mu;
    std::condition_variable cv_done;
    std::map<int32_t, SrvGraph> graphs;
    int32_t next_gid = 1;
    std::unordered_map<int64_t, std::shared_ptr<SrvQuery>> queries;
    int64_t next_ticket = 1;
    int64_t n_cap = 0;            // slot workspaces cover graphs up to n_cap vertices
    int64_t resident = 0;         // graph bytes admitted
    int64_t peak = 0;
    int busy_jobs = 0;            // launches planned or in flight
    bool resizing = false;
    bool stop = false;
    // stats
    // latencies of completed queries since the last reset: the most recent
    // LAT_WINDOW of them (a ring), and the total count
    static constexpr size_t LAT_WINDOW = 1u << 17;
    std::vector<double> lat;
    size_t lat_next = 0;
    int64_t completed = 0;
    int64_t launches = 0, rejected = 0;
    double lanes_sum = 0;
    // slots
    struct Slot {
        cudaStream_t st[SRV_SUB] = {};  // unit j's stream; unit 0 also carries whole-slot launches
        MsWork w;                       // 64-lane workspace (multi-source batches)
        BfsWork bw[SRV_SUB];            // unit j's single-source workspace
        SrvJob job[SRV_SUB];            // unit j's launch
        // stream callbacks and wake-ups reach the worker through sig_mu alone,
        // never through the server's mutex (which admission holds across CUDA
        // calls that may wait for those callbacks)
        std::mutex sig_mu;
        std::condition_variable cv;     // the worker waits here, with sig_mu
        bool kick = false;              // queries to look at, admission or shutdown (under sig_mu)
        std::vector<std::pair<Clock::time_point, int32_t>> ready;  // plan's scratch (under mu)
        bool whole = false;             // job[0] holds every unit
        int32_t drain_for = 0;          // a batch graph taken once every unit is free
        int64_t cap = 0;
    };
    int bfs_ctas = 0;   // CTA cap of a single-source search holding a whole slot
    std::vector<std::unique_ptr<Slot>> slots;
    std::vector<std::thread> workers;

    int64_t slots_total(int64_t cap) const { return slot_bytes(cap) * (int64_t)slots.size(); }
    static void kick(Slot &sl)
    {
        std::lock_guard<std::mutex> lk(sl.sig_mu);
        sl.kick = true;
        sl.cv.notify_all();
    }
    void wake_all()
    {
        for (auto &sl : slots) kick(*sl);
    }
    // under mu: wake the slots other than idx that have a free unit
    void kick_others(int idx)
    {
        for (int o = 0; o < (int)slots.size(); o++) {
            Slot &sl = *slots[o];
            if (o == idx || sl.whole) continue;
            for (auto &jb : sl.job)
                if (!jb.busy) {
                    kick(sl);
                    break;
                }
        }
    }
    void worker(int idx);
    void plan(int idx, std::vector<int> &units, Clock::time_point &next_ready);
    void take(Slot &sl, int j, int32_t gid, SrvGraph &c, int k, int cap, int lanes, std::vector<int> &units);
    void launch(Slot &sl, int j);
    void advance(Slot &sl, int j);
    void finish(Slot &sl, int j, int status);
};

namespace {

// Stream callback after a launch's work: marks the job for its worker (no
// CUDA calls here).  The notification is made under the signal mutex, so the
// worker cannot see the mark, finish and leave before it.
void CUDART_CB job_signal(void *p)
{
    SrvJob *jb = static_cast<SrvJob *>(p);
    auto &sl = *jb->srv->slots[jb->slot];
    std::lock_guard<std::mutex> lk(sl.sig_mu);
    jb->signalled = true;
    sl.cv.notify_all();
}

}  // namespace

// Under mu: unit j of `sl` takes k of graph c's oldest queries.
void gbfs_server::take(Slot &sl, int j, int32_t gid, SrvGraph &c, int k, int cap, int lanes, std::vector<int> &units)
{
    SrvJob &jb = sl.job[j];
    const auto now = Clock::now();
    jb.busy = true;
    jb.batch = k > 1;
    jb.cap = cap;
    jb.gid = gid;
    jb.sg = &c;
    jb.t_launch = now;
    jb.qs.clear();
    jb.srcs.clear();
    for (int i = 0; i < k; i++) {
        auto q = c.pending.front();
        c.pending.pop_front();
        q->t_launch = now;
        q->lanes = lanes;
        jb.qs.push_back(q);
        jb.srcs.push_back(q->source);
    }
    c.inflight += k;
    ++busy_jobs;
    ++launches;
    lanes_sum += lanes;
    units.push_back(j);
}

// Under mu: the next launches of slot idx's free units (the rule is in
// server_plan.h).
void gbfs_server::plan(int idx, std::vector<int> &units, Clock::time_point &next_ready)
{
    plan_slot<SRV_SUB>(*this, idx, Clock::now(), units, next_ready);
}

// Outside mu: enqueue unit j's launch, its status read-back and its callback.
void gbfs_server::launch(Slot &sl, int j)
{
    SrvJob &jb = sl.job[j];
    gbfs_graph *g = jb.sg->g;
    const DeviceCsr &csr = jb.sg->csr;
    gbfs_params p = graph_params(g);
    p.timeout_ms = cfg.timeout_ms;
    if (!g->symmetric && !csr.trow) p.direction = GBFS_DIR_TOPDOWN;  // bottom-up needs in-edges
    cudaStream_t st = sl.st[j];
    cudaError_t e;
    if (jb.batch) {
        const int k = (int)jb.srcs.size();
        e = cudaMemcpyAsync(sl.w.src, jb.srcs.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = msbfs_enqueue(csr, p, g->symmetric, sl.w, sl.w.src, k, sl.w.out, st, max_ctas);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.w.h_ctrl, sl.w.ctrl, offsetof(MsCtrl, t_entry), cudaMemcpyDeviceToHost, st);
    } else {
        BfsWork &bw = sl.bw[j];
        e = bfs_enqueue(csr, p, bw, nullptr, 1, jb.srcs[0], bw.level, &bw.ctrl->out, st, g->symmetric, 0, 0, jb.cap);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&bw.h_ctrl->status, &bw.ctrl->status, sizeof(int), cudaMemcpyDeviceToHost, st);
    }
    // phase is set before the worker can next look at the signal
    jb.phase = 1;
    if (e == cudaSuccess) e = cudaLaunchHostFunc(st, job_signal, &jb);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(st);
        finish(sl, j, GBFS_ERR_CUDA);
    }
}

// Outside mu, after unit j's callback: check the search's status and copy
// the levels out (phase 1), or complete the queries (phase 2).
void gbfs_server::advance(Slot &sl, int j)
{
    SrvJob &jb = sl.job[j];
    if (jb.phase == 2) {
        finish(sl, j, GBFS_OK);
        return;
    }
    cudaStream_t st = sl.st[j];
    const int dev_status = jb.batch ? sl.w.h_ctrl->status : sl.bw[j].h_ctrl->status;
    if (dev_status != DEV_OK) {
        // a bounded wait ran out: clear the control block for the unit's
        // next launch (ordered before it on the same stream)
        if (jb.batch) cudaMemsetAsync(sl.w.ctrl, 0, sizeof(MsCtrl), st);
        else cudaMemsetAsync(sl.bw[j].ctrl, 0, sizeof(BfsCtrl), st);
        finish(sl, j, GBFS_ERR_TIMEOUT);
        return;
    }
    const size_t n = (size_t)jb.sg->csr.n;
    cudaError_t e = cudaSuccess;
    if (jb.batch) {
        for (size_t i = 0; i < jb.qs.size() && e == cudaSuccess; i++)
            e = cudaMemcpyAsync(jb.qs[i]->out, sl.w.out + n * i, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st);
    } else {
        e = cudaMemcpyAsync(jb.qs[0]->out, sl.bw[j].level, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st);
    }
    jb.phase = 2;
    if (e == cudaSuccess) e = cudaLaunchHostFunc(st, job_signal, &jb);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(st);
        finish(sl, j, GBFS_ERR_CUDA);
    }
}

// Complete unit j's queries with `status` and free the unit.
void gbfs_server::finish(Slot &sl, int j, int status)
{
    SrvJob &jb = sl.job[j];
    {
        std::lock_guard<std::mutex> lk(mu);
        const auto now = Clock::now();
        for (auto &q : jb.qs) {
            q->status = status;
            q->done = true;
            q->latency_ms = ms_between(q->t_submit, now);
            q->queue_ms = ms_between(q->t_submit, q->t_launch);
            if (status == GBFS_OK) {
                if (lat.size() < LAT_WINDOW) lat.push_back(q->latency_ms);
                else lat[lat_next] = q->latency_ms;
                lat_next = (lat_next + 1) % LAT_WINDOW;
                ++completed;
            }
        }
        SrvGraph &c = *jb.sg;
        c.inflight -= (int)jb.qs.size();
        const double us = std::chrono::duration<double, std::micro>(now - jb.t_launch).count();
        c.est_us = c.est_us > 0 ? 0.7 * c.est_us + 0.3 * us : us;
        // the graph's batch window moved with its launch time: slots timed
        // on the old one look again (this slot plans next anyway)
        if (!c.pending.empty()) kick_others(jb.slot);
        jb.qs.clear();
        jb.srcs.clear();
        jb.sg = nullptr;
        jb.phase = 0;
        jb.busy = false;
        if (j == 0) sl.whole = false;
        --busy_jobs;
    }
    cv_done.notify_all();
}

void gbfs_server::worker(int idx)
{
    cudaSetDevice(device);
    Slot &sl = *slots[idx];
    std::vector<int> start, done;
    Clock::time_point next_ready = Clock::time_point::max();
    for (;;) {
        // launches whose callbacks ran: the next phase
        done.clear();
        {
            std::lock_guard<std::mutex> lk(sl.sig_mu);
            sl.kick = false;
            for (int j = 0; j < SRV_SUB; j++)
                if (sl.job[j].signalled) {
                    sl.job[j].signalled = false;
                    done.push_back(j);
                }
        }
        for (int j : done) advance(sl, j);
        if (!done.empty()) continue;
        // free units: new launches
        start.clear();
        next_ready = Clock::time_point::max();
        {
            std::lock_guard<std::mutex> lk(mu);
            if (!resizing) plan(idx, start, next_ready);
            if (start.empty() && stop) {
                bool idle = true, pending = false;
                for (auto &jb : sl.job) idle = idle && !jb.busy;
                for (auto &kv : graphs)
                    pending = pending || (!kv.second.pending.empty() && kv.second.csr.n <= sl.cap);
                if (idle && !pending) return;
            }
        }
        for (int j : start) launch(sl, j);
        if (!start.empty()) continue;
        // nothing to do: wait for a callback, a wake-up or a batch window
        std::unique_lock<std::mutex> lk(sl.sig_mu);
        auto woken = [&] {
            if (sl.kick) return true;
            for (auto &jb : sl.job)
                if (jb.signalled) return true;
            return false;
        };
        if (next_ready != Clock::time_point::max()) sl.cv.wait_until(lk, next_ready, woken);
        else sl.cv.wait(lk, woken);
    }
}

extern "C" int gbfs_server_create(const gbfs_server_config *cfg, gbfs_server **out)
{
    if (!cfg || !out) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->num_slots < 1 || cfg->num_slots > 16 || cfg->max_lanes < 1 || cfg->max_lanes > MS_LANES ||
        cfg->mem_budget_bytes <= 0 || cfg->batch_window_us < 0 || cfg->timeout_ms < 1 || cfg->window_pct < 0 ||
        cfg->window_pct > 1000)
        return fail(GBFS_ERR_INVALID_ARG, "bad server configuration");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(GBFS_ERR_CUDA, "no CUDA device available");
    }
    gbfs_server *s = new (std::nothrow) gbfs_server();
    if (!s) return fail(GBFS_ERR_OOM, "host allocation failed");
    s->cfg = *cfg;
    cudaGetDevice(&s->device);
    const int total = ms_max_ctas();
    if (total <= 0) {
        delete s;
        return fail(GBFS_ERR_CUDA, "occupancy query failed");
    }
    s->max_ctas = std::max(1, total / cfg->num_slots);
    {
        gbfs_params dp;
        gbfs_default_params(&dp);
        const int tb = bfs_max_ctas(dp);
        if (tb <= 0) {
            delete s;
            return fail(GBFS_ERR_CUDA, "occupancy query failed");
        }
        s->bfs_ctas = std::max(1, tb / cfg->num_slots);
    }
    for (int i = 0; i < cfg->num_slots; i++) {
        s->slots.emplace_back(new (std::nothrow) gbfs_server::Slot());
        if (!s->slots.back()) {
            s->slots.pop_back();
            gbfs_server_destroy(s);
            return fail(GBFS_ERR_OOM, "host allocation failed");
        }
        for (int j = 0; j < SRV_SUB; j++) {
            s->slots.back()->job[j].srv = s;
            s->slots.back()->job[j].slot = i;
        }
    }
    for (auto &sl : s->slots)
        for (auto &st : sl->st)
            if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
                gbfs_server_destroy(s);
                return fail(GBFS_ERR_CUDA, "cudaStreamCreate");
            }
    try {
        s->workers.reserve(cfg->num_slots);
        for (int i = 0; i < cfg->num_slots; i++) s->workers.emplace_back(&gbfs_server::worker, s, i);
    } catch (const std::exception &) {
        // stops and joins the workers already started
        gbfs_server_destroy(s);
        return fail(GBFS_ERR_OOM, "cannot start the server's worker threads");
    }
    *out = s;
    return GBFS_OK;
}

extern "C" void gbfs_server_destroy(gbfs_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->wake_all();
    }
    for (auto &t : s->workers)
        if (t.joinable()) t.join();
    // the synchronisation also waits for the last callbacks to return
    for (auto &sl : s->slots) {
        for (auto st : sl->st)
            if (st) cudaStreamSynchronize(st);
        ms_work_free(sl->w);
        for (auto &bw : sl->bw) bfs_work_free(bw);
        for (auto st : sl->st)
            if (st) cudaStreamDestroy(st);
    }
    delete s;
}

extern "C" int gbfs_server_add_graph(gbfs_server *s, gbfs_graph *g, int32_t *graph_id)
{
    if (!s || !g || !graph_id) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    if (g->csr.wide) return fail(GBFS_ERR_TOO_LARGE, "the server's multi-source slots need 32-bit row offsets");
    std::lock_guard<std::mutex> admit(s->admit_mu);
    std::unique_lock<std::mutex> lk(s->mu);
    // a directed graph that may step bottom-up gets its transpose (in-edge
    // rows plus their heavy-row list) built here, inside the budget
    const bool want_t = !g->symmetric && graph_params(g).direction != GBFS_DIR_TOPDOWN;
    const bool has_t = want_t || g->csr.trow != nullptr;
    const int64_t tbytes =  // trow, tcol, theavy, tfirst still to build
        want_t && !g->csr.trow ? (int64_t)sizeof(int) * (3 * (int64_t)g->csr.n + 1 + g->csr.m) : 0;
    const int64_t gbytes = csr_device_bytes(g->csr) + tbytes + ms_prepare_bytes(g->csr, has_t);
    const int64_t new_cap = std::max<int64_t>(s->n_cap, g->csr.n);
    const int64_t need = s->resident + gbytes + s->slots_total(new_cap);
    if (need > s->cfg.mem_budget_bytes) {
        ++s->rejected;
        return fail(GBFS_ERR_BUDGET, "graph plus slot workspaces exceed the memory budget (" + std::to_string(need) +
                                         " > " + std::to_string(s->cfg.mem_budget_bytes) + " bytes)");
    }
    DeviceCsr csr_snapshot;
    if (new_cap > s->n_cap) {
        // grow every slot's workspace once the slots are idle
        s->resizing = true;
        s->cv_done.wait(lk, [&] { return s->busy_jobs == 0; });
        std::string err;
        int rc = GBFS_OK;
        auto slot_free = [](gbfs_server::Slot &sl) {
            ms_work_free(sl.w);
            for (auto &bw : sl.bw) bfs_work_free(bw);
            sl.cap = 0;
        };
        auto slot_alloc = [](gbfs_server::Slot &sl, int64_t cap, std::string &e) {
            int r = ms_work_alloc(sl.w, (int32_t)cap, e);
            for (auto &bw : sl.bw)
                if (!r) r = bfs_work_alloc(bw, (int32_t)cap, e);
            if (!r) sl.cap = cap;
            return r;
        };
        for (auto &sl : s->slots) {
            slot_free(*sl);
            rc = slot_alloc(*sl, new_cap, err);
            if (rc) break;
        }
        s->resizing = false;
        if (rc) {
            for (auto &sl : s->slots) slot_free(*sl);
            const int64_t old = s->n_cap;
            s->n_cap = 0;
            // restore the previous capacity if possible
            std::string err2;
            // (a slot left without a workspace takes no queries: its cap is 0)
            for (auto &sl : s->slots)
                if (old > 0 && slot_alloc(*sl, old, err2) != GBFS_OK) slot_free(*sl);
            s->n_cap = old;
            s->wake_all();
            return fail(rc, "slot workspace: " + err);
        }
        s->n_cap = new_cap;
        s->wake_all();
    }
    {
        std::lock_guard<std::mutex> glk(g->mu);
        std::string err;
        int rc = want_t ? csr_build_transpose(g->csr, g->stream, err) : GBFS_OK;
        if (!rc) rc = ms_prepare(g->csr, g->stream, err);
        if (rc) return fail(rc, err);
        csr_snapshot = g->csr;
    }
    const int32_t gid = s->next_gid++;
    SrvGraph sg;
    sg.g = g;
    sg.csr = csr_snapshot;
    sg.bytes = gbytes;
    sg.singles = bfs_relax_tail(csr_snapshot, graph_params(g));
    s->graphs.emplace(gid, std::move(sg));
    s->resident += gbytes;
    s->peak = std::max(s->peak, s->resident + s->slots_total(s->n_cap));
    *graph_id = gid;
    s->wake_all();
    return GBFS_OK;
}

extern "C" int gbfs_server_remove_graph(gbfs_server *s, int32_t graph_id)
{
    if (!s) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->graphs.find(graph_id);
    if (it == s->graphs.end()) return fail(GBFS_ERR_NOT_FOUND, "unknown graph id");
    if (!it->second.pending.empty() || it->second.inflight > 0)
        return fail(GBFS_ERR_INVALID_ARG, "graph has queries pending or in flight");
    s->resident -= it->second.bytes;
    s->graphs.erase(it);
    return GBFS_OK;
}

extern "C" int gbfs_server_submit(gbfs_server *s, int32_t graph_id, int32_t source, int32_t *levels_out,
                                  int64_t *ticket)
{
    if (!s || !levels_out || !ticket) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    std::shared_ptr<SrvQuery> q;
    try {
        q = std::make_shared<SrvQuery>();
    } catch (const std::bad_alloc &) {
        return fail(GBFS_ERR_OOM, "host allocation failed");
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return fail(GBFS_ERR_SHUTDOWN, "server is shutting down");
        auto it = s->graphs.find(graph_id);
        if (it == s->graphs.end()) return fail(GBFS_ERR_NOT_FOUND, "unknown graph id");
        if (source < 0 || source >= it->second.g->csr.n) return fail(GBFS_ERR_INVALID_ARG, "source outside [0, n)");
        q->ticket = s->next_ticket++;
        q->gid = graph_id;
        q->source = source;
        q->out = levels_out;
        q->t_submit = Clock::now();
        try {
            s->queries.emplace(q->ticket, q);
            try {
                it->second.pending.push_back(q);
            } catch (...) {
                s->queries.erase(q->ticket);
                throw;
            }
        } catch (const std::bad_alloc &) {
            return fail(GBFS_ERR_OOM, "host allocation failed");
        }
        *ticket = q->ticket;
        // wake the slots with a free unit; the others plan again when one of
        // their launches ends
        for (auto &sl : s->slots) {
            bool free_unit = false;
            for (auto &jb : sl->job) free_unit = free_unit || !jb.busy;
            if (free_unit && !sl->whole) gbfs_server::kick(*sl);
        }
    }
    return GBFS_OK;
}

extern "C" int gbfs_server_wait(gbfs_server *s, int64_t ticket, int32_t timeout_ms, gbfs_query_info *info)
{
    if (!s) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->queries.find(ticket);
    if (it == s->queries.end()) return fail(GBFS_ERR_NOT_FOUND, "unknown ticket");
    auto q = it->second;  // keeps the query alive across the wait
    auto pred = [&] { return q->done; };
    if (timeout_ms < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
        return fail(GBFS_ERR_TIMEOUT, "query still pending");
    if (info) {
        info->latency_ms = q->latency_ms;
        info->queue_ms = q->queue_ms;
        info->batch_lanes = q->lanes;
        info->status = q->status;
    }
    // erase by key: another thread waiting on the same ticket may have
    // erased it while this one slept (the iterator would be stale)
    s->queries.erase(ticket);
    return q->status == GBFS_OK ? GBFS_OK : fail(q->status, "query failed on the device");
}

extern "C" int gbfs_server_get_stats(gbfs_server *s, gbfs_server_stats *st)
{
    if (!s || !st) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *st = gbfs_server_stats{};
    st->completed = s->completed;
    st->launches = s->launches;
    st->rejected = s->rejected;
    st->resident_bytes = s->resident;
    st->peak_bytes = s->peak;
    st->mean_batch_lanes = s->launches ? s->lanes_sum / (double)s->launches : 0;
    if (!s->lat.empty()) {
        std::vector<double> v = s->lat;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (double)(v.size() - 1) + 0.5))]; };
        st->p50_ms = pct(0.50);
        st->p99_ms = pct(0.99);
        st->max_ms = v.back();
        double sum = 0;
        for (double x : v) sum += x;
        st->mean_ms = sum / (double)v.size();
    }
    return GBFS_OK;
}

extern "C" void gbfs_server_reset_stats(gbfs_server *s)
{
    if (!s) return;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat.clear();
    s->lat_next = 0;
    s->completed = 0;
    s->launches = 0;
    s->lanes_sum = 0;
}
