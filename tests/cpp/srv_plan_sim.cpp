// Drives the serving loop's scheduling rule (gpu_graphs_gb300/csrc/server_plan.h,
// the code server.cu runs) with simulated launches and arrivals on the CPU.
//
// A slot plans when the server would wake its worker: a submitted query wakes
// the slots with a free unit, a finished launch wakes its own slot (and the
// others with a free unit when its graph still has queries waiting), a
// launch that leaves queries behind wakes the others with a free unit, a
// batch window wakes the slots waiting on it; a woken worker plans until it
// starts nothing.  After every event the simulation checks:
//   * a unit never takes a second launch, a slot's launches never hold more
//     than its CTA share, a batch of two or more queries runs only on a whole
//     free slot;
//   * each graph's queries launch in the order they were submitted;
//   * no query of a single-source graph (or a batch of one) waits while some
//     slot with a free unit is neither running a whole-slot launch nor
//     draining for a batch;
//   * every query is served (no starvation), within a bound on its wait.
// Prints "ok <stats>" and exits 0, or prints the failed check and exits 1.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <map>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "server_plan.h"

namespace {

struct SimClock {
    using rep = int64_t;
    using period = std::micro;
    using duration = std::chrono::microseconds;
    using time_point = std::chrono::time_point<SimClock>;
    static constexpr bool is_steady = true;
};
using Time = SimClock::time_point;
using us = std::chrono::microseconds;

constexpr int SUB = 4;

[[noreturn]] void fail(const std::string &what)
{
    std::printf("FAIL %s\n", what.c_str());
    std::exit(1);
}
#define CHECK(cond, what)          \
    do {                           \
        if (!(cond)) fail(what);   \
    } while (0)

struct Query {
    int64_t id = 0;
    int gid = 0;
    Time t_submit{}, t_launch{};
    bool launched = false, done = false;
};
struct Csr {
    int64_t n = 0;
};
struct Graph {
    std::deque<Query *> pending;
    bool singles = false;
    double est_us = 0;
    Csr csr;
    int drainer = -1;
    double base_us = 1000;  // a search's duration on one unit
    int64_t last_launched = -1;
};
struct Job {
    bool busy = false;
};
struct Slot {
    Job job[SUB];
    bool whole = false;
    int32_t drain_for = 0;
    int64_t cap = 1 << 30;
    std::vector<std::pair<Time, int32_t>> ready;
};
struct Cfg {
    int max_lanes = 64;
    int batch_window_us = 500;
    int window_pct = 10;
};
struct Launch {
    int slot = 0, unit = 0, gid = 0, cap = 0;
    std::vector<Query *> qs;
    Time start{}, end{};
};

struct Sim {
    Cfg cfg;
    std::map<int32_t, Graph> graphs;
    std::vector<std::unique_ptr<Slot>> slots;
    bool stop = false;
    int bfs_ctas = 48;
    Time now{};
    std::mt19937_64 rng;
    std::vector<Launch> running;
    std::vector<Time> next_ready;
    int64_t launches = 0, batches = 0, wholes = 0, units_used = 0, drains = 0;
    double max_wait_us = 0;

    explicit Sim(uint64_t seed) : rng(seed) {}

    double uni(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }

    // the server's take(): move k oldest queries of graph c to unit j
    void take(Slot &sl, int j, int32_t gid, Graph &c, int k, int cap, int lanes, std::vector<int> &units)
    {
        const int idx = slot_index(sl);
        CHECK(j >= 0 && j < SUB, "unit index");
        CHECK(!sl.job[j].busy, "a unit took a second launch");
        CHECK(k >= 1 && k <= (int)c.pending.size() && k <= cfg.max_lanes, "batch size");
        CHECK(lanes >= 1, "lanes");
        if (k > 1 || cap == bfs_ctas) {
            CHECK(sl.whole && j == 0, "a whole-slot launch without the whole flag on unit 0");
            for (int u = 0; u < SUB; u++) CHECK(!sl.job[u].busy, "a whole-slot launch on a busy slot");
        } else {
            CHECK(cap == std::max(1, bfs_ctas / SUB), "a unit's CTA cap");
        }
        if (k > 1) CHECK(!c.singles, "a batch on a single-source graph");
        CHECK(c.csr.n <= sl.cap, "a slot took a graph larger than its workspace");
        sl.job[j].busy = true;
        Launch L;
        L.slot = idx;
        L.unit = j;
        L.gid = gid;
        L.cap = cap;
        L.start = now;
        for (int i = 0; i < k; i++) {
            Query *q = c.pending.front();
            c.pending.pop_front();
            CHECK(q->id > c.last_launched, "a graph's queries launched out of order");
            c.last_launched = q->id;
            q->launched = true;
            q->t_launch = now;
            max_wait_us = std::max(max_wait_us, (double)(now - q->t_submit).count());
            L.qs.push_back(q);
        }
        // duration: single-source searches are latency-bound (weakly
        // dependent on their CTAs), batches cost more per lane and scale
        // with their CTAs
        const double share = (double)cap / bfs_ctas;
        double d = k > 1 ? c.base_us * (1.0 + 0.05 * k) / share : c.base_us * std::pow(1.0 / share, 0.3);
        d *= uni(0.5, 1.5);
        L.end = now + us((int64_t)std::max(1.0, d));
        ++launches;
        batches += k > 1;
        wholes += cap == bfs_ctas;
        units_used += cap == bfs_ctas ? 0 : 1;
        running.push_back(L);
        units.push_back(j);
        // the slot's launches together stay within its CTA share
        int used = 0;
        for (auto &r : running)
            if (r.slot == idx) used += r.cap;
        CHECK(used <= bfs_ctas, "a slot's launches hold more than its CTA share");
    }

    int slot_index(const Slot &sl) const
    {
        for (int i = 0; i < (int)slots.size(); i++)
            if (slots[i].get() == &sl) return i;
        fail("unknown slot");
    }

    // the server's kick_others(): the other slots with a free unit plan
    // again (after the slot planning now, as the server's workers would)
    std::vector<int> kicked;
    void kick_others(int idx)
    {
        for (int o = 0; o < (int)slots.size(); o++)
            if (o != idx && !slots[o]->whole && nfree(o) > 0) kicked.push_back(o);
    }
    int64_t kicks = 0;

    // a woken worker, and the workers its launches wake in turn
    void wake(int idx)
    {
        plan_until_idle(idx);
        while (!kicked.empty()) {
            const int o = kicked.back();
            kicked.pop_back();
            ++kicks;
            plan_until_idle(o);
        }
    }

    // the worker of slot idx after a wake-up: plan until nothing starts
    void plan_until_idle(int idx)
    {
        for (;;) {
            std::vector<int> units;
            Time nr = Time::max();
            const bool had_drain = slots[idx]->drain_for != 0;
            gbfs::plan_slot<SUB>(*this, idx, now, units, nr);
            drains += !had_drain && slots[idx]->drain_for != 0;
            next_ready[idx] = nr;
            if (units.empty()) return;
        }
    }

    int nfree(int idx) const
    {
        int f = 0;
        for (auto &jb : slots[idx]->job) f += !jb.busy;
        return f;
    }

    void finish(size_t i)
    {
        Launch L = running[i];
        running.erase(running.begin() + (long)i);
        Slot &sl = *slots[L.slot];
        sl.job[L.unit].busy = false;
        if (L.unit == 0) sl.whole = false;
        Graph &c = graphs[L.gid];
        const double d = (double)(L.end - L.start).count();
        c.est_us = c.est_us > 0 ? 0.7 * c.est_us + 0.3 * d : d;
        // the server's finish(): the graph's batch window moved, so the other
        // slots with a free unit look again
        if (!c.pending.empty()) kick_others(L.slot);
        for (Query *q : L.qs) q->done = true;
    }

    // work conservation: no single-source query (and no batch of one) waits
    // while a slot with a free unit is neither whole nor draining
    void check_idle()
    {
        for (int idx = 0; idx < (int)slots.size(); idx++) {
            const Slot &sl = *slots[idx];
            if (sl.whole || nfree(idx) == 0 || sl.drain_for != 0) continue;
            for (auto &kv : graphs) {
                const Graph &c = kv.second;
                if (c.pending.empty() || c.csr.n > sl.cap) continue;
                if (c.singles) fail("slot " + std::to_string(idx) + " idles beside a waiting single-source query");
                const bool ready_batch = stop || (int)c.pending.size() >= cfg.max_lanes ||
                                         now >= c.pending.front()->t_submit + us((int64_t)std::min(
                                                    1e6, std::max<double>(cfg.batch_window_us,
                                                                          0.01 * cfg.window_pct * c.est_us)));
                if (!ready_batch) continue;
                if (c.pending.size() == 1) fail("slot " + std::to_string(idx) + " idles beside a ready batch of one");
                if (nfree(idx) == SUB) fail("free slot " + std::to_string(idx) + " idles beside a ready batch");
                if (c.drainer < 0) fail("a ready batch has no slot draining for it");
            }
        }
    }
};

struct Stats {
    int64_t queries = 0, launches = 0, batches = 0, wholes = 0, units = 0, drains = 0;
    double max_wait_us = 0;
};

// One run: `n_slots` slots, `n_single` single-source graphs and `n_batch`
// batch graphs, `n_queries` Poisson arrivals at `rate` queries per ms
// (rate 0: all at time 0, a closed loop).  mixed_caps: slot 0 holds every
// graph, the others only some (workspaces of two sizes, as after a failed
// resize); shutdown: the server stops once half the queries have arrived
// (the rest still arrive and every pending batch is ready at once).
Stats run(uint64_t seed, int n_slots, int n_single, int n_batch, int n_queries, double rate, int max_lanes,
          bool mixed_caps, bool shutdown)
{
    Sim s(seed);
    s.cfg.max_lanes = max_lanes;
    s.cfg.window_pct = (int)(seed % 3) * 50;
    for (int i = 0; i < n_slots; i++) {
        s.slots.push_back(std::make_unique<Slot>());
        if (mixed_caps && i > 0) s.slots.back()->cap = (s.rng() & 1) ? 2000 : 1000;
    }
    s.next_ready.assign(n_slots, Time::max());
    int gid = 1;
    for (int i = 0; i < n_single + n_batch; i++) {
        Graph g;
        g.singles = i < n_single;
        g.csr.n = mixed_caps && (s.rng() & 1) ? 1500 : 1000;
        g.base_us = g.singles ? s.uni(200, 20000) : s.uni(50, 3000);
        s.graphs[gid++] = g;
    }
    const int ngraphs = n_single + n_batch;
    std::vector<std::unique_ptr<Query>> qs;
    double t = 0;
    for (int i = 0; i < n_queries; i++) {
        auto q = std::make_unique<Query>();
        q->id = i;
        q->gid = 1 + (int)(s.rng() % (uint64_t)ngraphs);
        if (rate > 0) t += -std::log(1.0 - s.uni(0.0, 0.999999)) * 1000.0 / rate;
        q->t_submit = Time(us((int64_t)t));
        qs.push_back(std::move(q));
    }
    size_t next_arrival = 0;
    const int64_t limit = 1000000;  // events
    int64_t events = 0;
    while (true) {
        CHECK(++events < limit, "the simulation does not finish (livelock or starvation)");
        Time t_next = Time::max();
        if (next_arrival < qs.size()) t_next = std::min(t_next, qs[next_arrival]->t_submit);
        for (auto &r : s.running) t_next = std::min(t_next, r.end);
        for (auto nr : s.next_ready) t_next = std::min(t_next, nr);
        if (t_next == Time::max()) break;
        s.now = std::max(s.now, t_next);
        // finished launches wake their slots
        std::vector<int> woken;
        for (size_t i = 0; i < s.running.size();) {
            if (s.running[i].end <= s.now) {
                woken.push_back(s.running[i].slot);
                s.finish(i);
            } else {
                ++i;
            }
        }
        for (int idx : woken) s.wake(idx);
        // batch windows that ran out wake the slots waiting on them
        for (int idx = 0; idx < n_slots; idx++)
            if (s.next_ready[idx] <= s.now) s.wake(idx);
        // shutdown: every slot's worker wakes
        if (shutdown && !s.stop && next_arrival >= qs.size() / 2) {
            s.stop = true;
            for (int idx = 0; idx < n_slots; idx++) s.wake(idx);
        }
        // arrivals: each wakes the slots with a free unit (not whole)
        while (next_arrival < qs.size() && qs[next_arrival]->t_submit <= s.now) {
            Query *q = qs[next_arrival++].get();
            s.graphs[q->gid].pending.push_back(q);
            for (int idx = 0; idx < n_slots; idx++)
                if (s.nfree(idx) > 0 && !s.slots[idx]->whole) s.wake(idx);
        }
        s.check_idle();
    }
    for (auto &q : qs) CHECK(q->launched && q->done, "a query was never served");
    for (auto &sl : s.slots)
        for (auto &jb : sl->job) CHECK(!jb.busy, "a unit stayed busy");
    // no query waits longer than the whole run takes one query at a time on
    // one unit of the slowest graph per query ahead of it
    CHECK(s.max_wait_us <= (double)n_queries * 25000.0 * 2.0, "a query waited too long");
    Stats st;
    st.queries = n_queries;
    st.launches = s.launches;
    st.batches = s.batches;
    st.wholes = s.wholes;
    st.units = s.units_used;
    st.drains = s.drains;
    st.max_wait_us = s.max_wait_us;
    return st;
}

// Deterministic cases: the rule's individual decisions.
void cases()
{
    // one single-source query on an idle server: the whole slot
    {
        Sim s(1);
        s.slots.push_back(std::make_unique<Slot>());
        s.next_ready.assign(1, Time::max());
        Graph g;
        g.singles = true;
        g.csr.n = 10;
        s.graphs[1] = g;
        Query q;
        q.gid = 1;
        s.graphs[1].pending.push_back(&q);
        s.wake(0);
        CHECK(s.running.size() == 1 && s.running[0].cap == s.bfs_ctas && s.slots[0]->whole, "lone query: whole slot");
    }
    // five single-source queries, one slot: four units, the fifth waits,
    // then takes the first unit that frees
    {
        Sim s(2);
        s.slots.push_back(std::make_unique<Slot>());
        s.next_ready.assign(1, Time::max());
        Graph g;
        g.singles = true;
        g.csr.n = 10;
        s.graphs[1] = g;
        std::vector<Query> q(5);
        for (int i = 0; i < 5; i++) {
            q[i].id = i;
            q[i].gid = 1;
            s.graphs[1].pending.push_back(&q[i]);
        }
        s.wake(0);
        CHECK(s.running.size() == 4 && s.graphs[1].pending.size() == 1, "four units filled, one query waits");
        for (auto &r : s.running) CHECK(r.cap == s.bfs_ctas / SUB, "unit cap");
        s.now += us(1);
        s.finish(2);
        s.wake(0);
        CHECK(s.running.size() == 4 && s.graphs[1].pending.empty() && q[4].launched, "the freed unit refills");
    }
    // a ready batch of three at the head of a partly busy slot: the slot
    // drains (younger single-source queries wait for another slot), then
    // runs the batch on the whole slot; a batch of one takes one unit
    {
        Sim s(3);
        s.slots.push_back(std::make_unique<Slot>());
        s.next_ready.assign(1, Time::max());
        Graph a, b, c;
        a.singles = true;
        a.csr.n = b.csr.n = c.csr.n = 10;
        s.graphs[1] = a;  // single-source
        s.graphs[2] = b;  // batch graph
        s.graphs[3] = c;  // batch graph
        std::vector<Query> q(8);
        for (int i = 0; i < 8; i++) q[i].id = i;
        q[0].gid = 1;
        s.graphs[1].pending.push_back(&q[0]);
        q[1].gid = 1;
        s.graphs[1].pending.push_back(&q[1]);
        s.wake(0);
        CHECK(s.running.size() == 2, "two units busy");
        s.now += us(1000);
        for (int i = 2; i < 5; i++) {
            q[i].gid = 2;
            q[i].t_submit = s.now;
            s.graphs[2].pending.push_back(&q[i]);
        }
        s.now += us(600);  // the batch window (500 us) has passed
        q[5].gid = 1;
        q[5].t_submit = s.now;
        s.graphs[1].pending.push_back(&q[5]);
        s.wake(0);
        CHECK(s.slots[0]->drain_for == 2 && s.graphs[2].drainer == 0, "the slot drains for the batch");
        CHECK(!q[5].launched, "a younger query does not pass the waiting batch on the draining slot");
        s.now += us(1);
        s.finish(1);
        s.wake(0);
        CHECK(!q[5].launched && s.slots[0]->drain_for == 2, "still draining with one unit busy");
        s.finish(0);
        s.wake(0);
        CHECK(s.running.size() == 1 && s.running[0].qs.size() == 3 && s.slots[0]->whole, "the batch runs whole");
        CHECK(s.graphs[2].drainer == -1 && s.slots[0]->drain_for == 0, "drain released");
        s.now += us(1);
        s.finish(0);
        // two single-source queries take a unit each; a batch of one beside
        // them takes a third unit (no drain)
        q[7].gid = 1;
        q[7].t_submit = s.now;
        s.graphs[1].pending.push_back(&q[7]);
        s.wake(0);
        CHECK(q[5].launched && q[7].launched && !s.slots[0]->whole && s.running.size() == 2, "two units");
        q[6].gid = 3;
        q[6].t_submit = s.now;
        s.graphs[3].pending.push_back(&q[6]);
        s.wake(0);
        CHECK(!q[6].launched && s.next_ready[0] == s.now + us(500), "the batch graph waits out its window");
        s.now += us(600);
        s.wake(0);
        CHECK(q[6].launched && s.slots[0]->drain_for == 0 && s.running.size() == 3, "a batch of one takes one unit");
        for (auto &r : s.running) CHECK(r.cap == s.bfs_ctas / SUB, "batch of one on a unit's share");
    }
}

}  // namespace

int main()
{
    cases();
    Stats tot;
    int runs = 0;
    for (uint64_t seed = 1; seed <= 60; seed++) {
        const int n_slots = 1 + (int)(seed % 6);
        const int n_single = (int)(seed % 5);
        const int n_batch = 1 + (int)((seed / 5) % 4);
        const double rate = seed % 4 == 0 ? 0.0 : 0.05 * (double)(1 + seed % 7) * n_slots;
        const int max_lanes = seed % 3 == 0 ? 4 : 64;
        const Stats st = run(seed, n_slots, n_single, n_batch, 600, rate, max_lanes, seed % 5 == 1 && n_slots > 1,
                             seed % 7 == 3);
        tot.queries += st.queries;
        tot.launches += st.launches;
        tot.batches += st.batches;
        tot.wholes += st.wholes;
        tot.units += st.units;
        tot.drains += st.drains;
        tot.max_wait_us = std::max(tot.max_wait_us, st.max_wait_us);
        ++runs;
    }
    CHECK(tot.batches > 0 && tot.drains > 0 && tot.units > 0 && tot.wholes > 0, "every kind of decision was taken");
    std::printf("ok runs=%d queries=%lld launches=%lld batches=%lld whole=%lld unit=%lld drains=%lld max_wait_ms=%.1f\n",
                runs, (long long)tot.queries, (long long)tot.launches, (long long)tot.batches, (long long)tot.wholes,
                (long long)tot.units, (long long)tot.drains, tot.max_wait_us / 1000.0);
    return 0;
}
