// server.cu -- continuous-batching BFS serving loop over HBM-resident graphs.
//
// The reference answers one query per process run (1D Partition/main.cu:10-82).
// Here a server keeps graphs resident, admits them against an HBM budget and
// answers queries as they arrive:
//   * every query joins its graph's FIFO;
//   * `num_slots` worker threads, each owning CUDA streams, a 64-lane
//     multi-source workspace and SRV_SUB single-source workspaces sized for
//     the largest admitted graph, take the ready graph whose oldest query
//     has waited longest:
//       - on most graphs they pack up to `max_lanes` of its queries into one
//         multi-source launch.  Such a graph is ready with a full batch or
//         once its oldest query has waited `batch_window_us`, or
//         `window_pct` percent of the graph's recent launch time if longer:
//         a launch costs about the same for one source as for 64, so slow
//         graphs gather bigger batches, while other graphs' queries keep the
//         slots busy meanwhile;
//       - on a graph of small degree (meshes, grids, road networks) a
//         search is a long chain of latency-bound levels that the
//         label-correcting kernel runs at about the same speed on a quarter
//         of the GPU, while a multi-source launch is bound by its lanes'
//         combined frontiers; such a graph is ready as soon as it has a
//         query, and a slot runs up to SRV_SUB of its queries as that many
//         single-source searches at once, on its own streams, each capped
//         to its share of the slot's CTAs;
//   * slots run concurrently on their streams, each launch capped to
//     1/num_slots of the GPU's CTAs so all of them fit on the GPU together
//     (every launch waits on all of its own CTAs);
//   * results are copied to the caller's buffer before the ticket completes;
//     latency = submit -> result in place.
#include <algorithm>
#include <cstddef>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "graph.cuh"

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
    double est_us = 0;   // recent launch time (moving average), 0 before the first
    bool singles = false;  // small degree: served as concurrent single-source searches
};

// Single-source searches a slot runs at once on a graph of small degree.
// A 4000 x 4000 grid search takes 12.7 ms on the whole GPU and 18.8 ms
// capped to 19 CTAs; 16 such searches at once finish in 21.5 ms each (677
// queries/s against 76 one after another), given enough hardware work
// queues (CUDA_DEVICE_MAX_CONNECTIONS: with CUDA's default of 8, about four
// searches progress at a time).  On the 32-graph serving mix, 6 slots of 4
// searches: capacity 3,358 queries/s (4 slots 2,713, 8 slots 2,999; 8
// searches per slot 2,816); batching such a graph's queries into
// multi-source launches from 16 pending on was slower.
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
    std::condition_variable cv_work, cv_done;
    std::map<int32_t, SrvGraph> graphs;
    int32_t next_gid = 1;
    std::unordered_map<int64_t, std::shared_ptr<SrvQuery>> queries;
    int64_t next_ticket = 1;
    int64_t n_cap = 0;            // slot workspaces cover graphs up to n_cap vertices
    int64_t resident = 0;         // graph bytes admitted
    int64_t peak = 0;
    int busy_slots = 0;
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
        cudaStream_t st[SRV_SUB] = {};  // st[0]: multi-source batches and the first search of a group
        MsWork w;                       // 64-lane workspace (multi-source batches)
        BfsWork bw[SRV_SUB];            // single-source workspaces (one per concurrent search)
        int64_t cap = 0;
    };
    int bfs_ctas = 0;   // CTA cap of a single-source launch in a slot
    std::vector<Slot> slots;
    std::vector<std::thread> workers;

    int64_t slots_total(int64_t cap) const { return slot_bytes(cap) * (int64_t)slots.size(); }
    void worker(int idx);
};

void gbfs_server::worker(int idx)
{
    cudaSetDevice(device);
    Slot &slot = slots[idx];
    std::vector<std::shared_ptr<SrvQuery>> batch;
    std::vector<int32_t> srcs;
    for (;;) {
        SrvGraph *sg = nullptr;
        int32_t gid = 0;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                Clock::time_point next_ready = Clock::time_point::max();
                if (!resizing) {
                    // among the graphs that are ready (a full batch, or their
                    // oldest query has waited out the graph's window), the one
                    // whose oldest query has waited longest
                    const auto now = Clock::now();
                    Clock::time_point oldest = Clock::time_point::max();
                    for (auto &kv : graphs) {
                        SrvGraph &c = kv.second;
                        if (c.pending.empty()) continue;
                        const auto t0 = c.pending.front()->t_submit;
                        const double window_us =
                            std::min(1e6, std::max<double>(cfg.batch_window_us, 0.01 * cfg.window_pct * c.est_us));
                        const auto ready_at = t0 + std::chrono::microseconds((int64_t)window_us);
                        if (c.singles || (int)c.pending.size() >= cfg.max_lanes || now >= ready_at || stop) {
                            if (t0 < oldest) {
                                oldest = t0;
                                sg = &c;
                                gid = kv.first;
                            }
                        } else {
                            next_ready = std::min(next_ready, ready_at);
                        }
                    }
                    if (sg) break;
                }
                if (stop && next_ready == Clock::time_point::max()) return;
                if (next_ready != Clock::time_point::max()) cv_work.wait_until(lk, next_ready);
                else cv_work.wait(lk);
            }
            const int k = std::min<int>((int)sg->pending.size(), sg->singles ? SRV_SUB : cfg.max_lanes);
            batch.clear();
            srcs.clear();
            const auto now = Clock::now();
            for (int i = 0; i < k; i++) {
                auto q = sg->pending.front();
                sg->pending.pop_front();
                q->t_launch = now;
                q->lanes = k;
                batch.push_back(q);
                srcs.push_back(q->source);
            }
            sg->inflight += k;
            ++busy_slots;
            ++launches;
            lanes_sum += k;
        }
        gbfs_graph *g = sg->g;
        const int k = (int)batch.size();
        const auto t_launch = Clock::now();
        const DeviceCsr &csr = sg->csr;
        const size_t n = (size_t)csr.n;
        gbfs_params p = graph_params(g);
        p.timeout_ms = cfg.timeout_ms;
        if (!g->symmetric && !csr.trow) p.direction = GBFS_DIR_TOPDOWN;  // bottom-up needs in-edges
        // per query: 0, or a status
        int qstatus[MS_LANES];
        for (int i = 0; i < k; i++) qstatus[i] = GBFS_OK;
        if (k == 1 || (k <= SRV_SUB && bfs_relax_tail(csr, p))) {
            // one query, or up to SRV_SUB on a graph of small degree: that
            // many single-source searches at once, each on its own stream
            // and workspace, sharing the slot's CTAs
            const int cap = k == 1 ? bfs_ctas : std::max(1, bfs_ctas / k);
            cudaError_t es[SRV_SUB];
            for (int j = 0; j < k; j++) {
                BfsWork &bw = slot.bw[j];
                es[j] = bfs_enqueue(csr, p, bw, nullptr, 1, srcs[j], bw.level, &bw.ctrl->out, slot.st[j],
                                    g->symmetric, 0, 0, cap);
                if (es[j] == cudaSuccess)
                    es[j] = cudaMemcpyAsync(&bw.h_ctrl->status, &bw.ctrl->status, sizeof(int), cudaMemcpyDeviceToHost,
                                            slot.st[j]);
            }
            for (int j = 0; j < k; j++) {
                BfsWork &bw = slot.bw[j];
                if (es[j] == cudaSuccess) es[j] = cudaStreamSynchronize(slot.st[j]);
                const int dev_status = es[j] == cudaSuccess ? bw.h_ctrl->status : DEV_OK;
                if (es[j] == cudaSuccess && dev_status == DEV_OK)
                    es[j] = cudaMemcpyAsync(batch[j]->out, bw.level, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                            slot.st[j]);
                if (es[j] == cudaSuccess && dev_status != DEV_OK) {
                    cudaMemsetAsync(bw.ctrl, 0, sizeof(BfsCtrl), slot.st[j]);
                    qstatus[j] = GBFS_ERR_TIMEOUT;
                }
            }
            for (int j = 0; j < k; j++) {
                if (es[j] == cudaSuccess) es[j] = cudaStreamSynchronize(slot.st[j]);
                if (es[j] != cudaSuccess) qstatus[j] = GBFS_ERR_CUDA;
            }
        } else {
            cudaError_t e = cudaMemcpyAsync(slot.w.src, srcs.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice,
                                            slot.st[0]);
            int dev_status = DEV_OK;
            if (e == cudaSuccess)
                e = msbfs_enqueue(csr, p, g->symmetric, slot.w, slot.w.src, k, slot.w.out, slot.st[0], max_ctas);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(slot.w.h_ctrl, slot.w.ctrl, offsetof(MsCtrl, t_entry), cudaMemcpyDeviceToHost,
                                    slot.st[0]);
            if (e == cudaSuccess) e = cudaStreamSynchronize(slot.st[0]);
            if (e == cudaSuccess) dev_status = slot.w.h_ctrl->status;
            if (e == cudaSuccess && dev_status != DEV_OK) {
                cudaMemsetAsync(slot.w.ctrl, 0, sizeof(MsCtrl), slot.st[0]);
                cudaStreamSynchronize(slot.st[0]);
            } else if (e == cudaSuccess) {
                for (int i = 0; i < k && e == cudaSuccess; i++)
                    e = cudaMemcpyAsync(batch[i]->out, slot.w.out + n * i, sizeof(int32_t) * n,
                                        cudaMemcpyDeviceToHost, slot.st[0]);
                if (e == cudaSuccess) e = cudaStreamSynchronize(slot.st[0]);
            }
            const int status = e != cudaSuccess ? GBFS_ERR_CUDA : dev_status != DEV_OK ? GBFS_ERR_TIMEOUT : GBFS_OK;
            for (int i = 0; i < k; i++) qstatus[i] = status;
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            const auto now = Clock::now();
            for (int i = 0; i < k; i++) {
                auto &q = batch[i];
                const int status = qstatus[i];
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
            auto it = graphs.find(gid);
            if (it != graphs.end()) {
                SrvGraph &c = it->second;
                c.inflight -= k;
                const double us = std::chrono::duration<double, std::micro>(now - t_launch).count();
                c.est_us = c.est_us > 0 ? 0.7 * c.est_us + 0.3 * us : us;
            }
            --busy_slots;
        }
        cv_done.notify_all();
        cv_work.notify_all();
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
    s->slots.resize(cfg->num_slots);
    for (auto &sl : s->slots)
        for (auto &st : sl.st)
            if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
                gbfs_server_destroy(s);
                return fail(GBFS_ERR_CUDA, "cudaStreamCreate");
            }
    for (int i = 0; i < cfg->num_slots; i++) s->workers.emplace_back(&gbfs_server::worker, s, i);
    *out = s;
    return GBFS_OK;
}

extern "C" void gbfs_server_destroy(gbfs_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers)
        if (t.joinable()) t.join();
    for (auto &sl : s->slots) {
        for (auto st : sl.st)
            if (st) cudaStreamSynchronize(st);
        ms_work_free(sl.w);
        for (auto &bw : sl.bw) bfs_work_free(bw);
        for (auto st : sl.st)
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
        s->cv_done.wait(lk, [&] { return s->busy_slots == 0; });
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
            slot_free(sl);
            rc = slot_alloc(sl, new_cap, err);
            if (rc) break;
        }
        s->resizing = false;
        if (rc) {
            for (auto &sl : s->slots) slot_free(sl);
            const int64_t old = s->n_cap;
            s->n_cap = 0;
            // restore the previous capacity if possible
            std::string err2;
            for (auto &sl : s->slots)
                if (old > 0 && slot_alloc(sl, old, err2) != GBFS_OK) slot_free(sl);
            s->n_cap = old;
            s->cv_work.notify_all();
            return fail(rc, "slot workspace: " + err);
        }
        s->n_cap = new_cap;
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
    s->cv_work.notify_all();
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
    auto q = std::make_shared<SrvQuery>();
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
        it->second.pending.push_back(q);
        s->queries.emplace(q->ticket, q);
        *ticket = q->ticket;
    }
    s->cv_work.notify_one();
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
