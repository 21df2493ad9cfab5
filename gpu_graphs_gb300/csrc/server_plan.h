// server_plan.h -- the serving loop's scheduling rule: which queries the free
// units of a slot launch next.  Host code without CUDA, shared by server.cu
// and a CPU test that drives it with simulated launches and arrivals.
#pragma once

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <utility>
#include <vector>

namespace gbfs {

// Under the server's mutex: the next launches of slot idx's free units,
// oldest waiting query first, at time `now`.
//   * A graph served by single-source searches (`singles`) gives each free
//     unit one query (all of the slot's units when it is the only query
//     waiting); so does a batch graph with one query waiting.
//   * A larger batch needs the whole slot: when the slot is not free it
//     stops filling units until it is (`drain_for`; one slot per batch graph,
//     recorded as the graph's `drainer`), while the other slots keep filling
//     behind it.  A batch graph is ready with `max_lanes` queries or once its
//     oldest query has waited `batch_window_us`, or `window_pct` percent of
//     the graph's recent launch time if longer (`est_us`); next_ready gets
//     the earliest time a batch graph not yet ready becomes ready.
// The server type S provides graphs (a map from graph id to a graph with
// pending, singles, est_us, csr.n and drainer), slots (pointers to slots
// with job[SUB].busy, whole, drain_for, cap and a scratch vector `ready`),
// cfg (max_lanes, batch_window_us, window_pct), stop, bfs_ctas (the CTA cap
// of a search holding a whole slot), take(slot, unit, graph id, graph,
// queries, CTA cap, lanes, units), which moves the graph's oldest queries
// to the unit and appends the unit to `units`, and kick_others(idx), which
// wakes the other slots that have a free unit.
template <int SUB, typename S, typename Time>
void plan_slot_pass(S &s, int idx, Time now, std::vector<int> &units, Time &next_ready)
{
    auto &sl = *s.slots[idx];
    if (sl.whole) return;
    int nfree = 0;
    for (auto &jb : sl.job) nfree += !jb.busy;
    if (nfree == 0) return;
    auto first_free = [&] {
        int j = 0;
        while (sl.job[j].busy) ++j;
        return j;
    };
    const int unit_cap = std::max(1, s.bfs_ctas / SUB);
    if (sl.drain_for) {
        auto it = s.graphs.find(sl.drain_for);
        if (it == s.graphs.end() || it->second.pending.empty()) {
            if (it != s.graphs.end() && it->second.drainer == idx) it->second.drainer = -1;
            sl.drain_for = 0;
        } else if (nfree < SUB) {
            return;
        } else if (it->second.csr.n <= sl.cap) {
            auto &c = it->second;
            c.drainer = -1;
            sl.drain_for = 0;
            const int k = std::min<int>((int)c.pending.size(), c.singles ? 1 : s.cfg.max_lanes);
            sl.whole = true;
            s.take(sl, 0, it->first, c, k, s.bfs_ctas, k, units);
            return;
        }
    }
    auto &ready = sl.ready;
    ready.clear();
    size_t ready_queries = 0;
    for (auto &kv : s.graphs) {
        auto &c = kv.second;
        if (c.pending.empty() || c.csr.n > sl.cap) continue;
        const auto t0 = c.pending.front()->t_submit;
        if (!c.singles && !s.stop && (int)c.pending.size() < s.cfg.max_lanes) {
            const double window_us =
                std::min(1e6, std::max<double>(s.cfg.batch_window_us, 0.01 * s.cfg.window_pct * c.est_us));
            const auto ready_at = t0 + std::chrono::microseconds((int64_t)window_us);
            if (now < ready_at) {
                next_ready = std::min(next_ready, ready_at);
                continue;
            }
        }
        ready.emplace_back(t0, kv.first);
        ready_queries += c.pending.size();
    }
    std::sort(ready.begin(), ready.end());
    for (auto &r : ready) {
        auto &c = s.graphs.find(r.second)->second;
        if (c.singles) {
            if (nfree == SUB && ready_queries == 1) {
                // the only query waiting: one search with the slot's CTAs
                sl.whole = true;
                s.take(sl, 0, r.second, c, 1, s.bfs_ctas, 1, units);
                return;
            }
            while (nfree > 0 && !c.pending.empty()) {
                s.take(sl, first_free(), r.second, c, 1, unit_cap, SUB - nfree + 1, units);
                --nfree;
            }
            if (nfree == 0) return;
        } else if (nfree == SUB) {
            const int k = std::min<int>((int)c.pending.size(), s.cfg.max_lanes);
            sl.whole = true;
            s.take(sl, 0, r.second, c, k, s.bfs_ctas, k, units);
            return;
        } else if (c.pending.size() == 1) {
            // a batch of one: a single-source search on one unit, no drain
            s.take(sl, first_free(), r.second, c, 1, unit_cap, SUB - nfree + 1, units);
            if (--nfree == 0) return;
        } else if (c.drainer < 0) {
            c.drainer = idx;
            sl.drain_for = r.second;
            return;
        }
    }
}

// plan_slot_pass, then: when this slot took queries and some remain, the
// other slots with a free unit plan again.  A launch can leave work that
// only they may take (the rest of a full batch, now a batch of one or a
// batch no slot drains for) or whose batch window they have no timer for
// (a graph that was ready with a full batch is again waiting for its
// window); nothing else would wake them before their own next event.
template <int SUB, typename S, typename Time>
void plan_slot(S &s, int idx, Time now, std::vector<int> &units, Time &next_ready)
{
    const size_t before = units.size();
    plan_slot_pass<SUB>(s, idx, now, units, next_ready);
    if (units.size() == before) return;
    for (auto &kv : s.graphs)
        if (!kv.second.pending.empty()) {
            s.kick_others(idx);
            return;
        }
}

}  // namespace gbfs
