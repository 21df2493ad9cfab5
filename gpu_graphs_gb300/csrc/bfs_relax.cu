// bfs_relax.cu -- the long tail of a single-source search on a graph of
// small degree, in label-correcting rounds (sm_103a).
//
// A high-diameter graph (a road network, a mesh, the perturbed grid) makes
// a search of thousands of levels whose frontiers hold a few thousand
// vertices.  Level by level, each such level costs a grid-wide barrier and
// a chain of dependent memory round trips (queue entry -> column index ->
// claim -> queue append) for a few edges per SM.  Once a search has run
// yield_level levels on such a graph, the grid kernel (bfs.cu) parks its
// level loop and this persistent kernel, queued right behind it, finishes
// the search in ROUNDS:
//   * a round splits the global frontier queue evenly over the CTAs
//     (contiguous pieces, so each CTA holds a connected piece of the
//     wavefront) and each CTA advances its piece up to RX_HOPS levels on its
//     own: hop by hop, with a CTA barrier between hops and the frontier in
//     shared memory, without any grid-wide synchronisation;
//   * an edge (u, v) is relaxed with atomicMin(level[v], level[u] + 1) on
//     the level array itself (unreached = -1 = the largest unsigned); a
//     vertex whose level drops joins the CTA's next hop, or the global
//     queue of the next round after the CTA's last hop, when its local
//     queue is full, or when a piece is too large to hop;
//   * a CTA may reach a vertex before the piece that holds its shortest
//     path does; the later, shorter relaxation lowers the level again and
//     queues the vertex again, so levels only fall and every fall is
//     propagated.  The search ends when a round leaves the global queue
//     empty: then level[v] <= level[u] + 1 for every edge from a reached u,
//     and every assigned level is the length of a real path, so each level
//     is the exact hop distance: the array the level-synchronous kernels
//     write, bit for bit;
//   * an expansion reads level[u] when it runs (a queued vertex may have
//     fallen since it was queued), and a vertex joins the global queue at
//     most once per round (a per-vertex round stamp, atomicMax), so the
//     queue never holds more than n entries.
// Levels are exact, and so are the counts: a vertex's first relaxation
// (from unreached) adds it and its out-degree to the reached totals; the
// level count is the largest level, read once at the end.
// Replaces, for such graphs, the per-level host loop of gpuBFS::gpuBFS
// (1D Partition/src/gpuBFS.cu:66-100) and its one-launch-per-level
// linear_bfs expansion (1D Partition/src/gpuBFS_kernels.cu:16-40).
#include <algorithm>
#include <type_traits>

#include "bfs.cuh"
#include "bfs_args.cuh"
#include "common.cuh"

namespace gbfs {

namespace {

constexpr int RX_BLOCK = 512;
constexpr int RX_NW = RX_BLOCK / 32;
constexpr int RX_CAP = 1024;                 // entries of a CTA's local frontier (two held)
// Edges per thread in flight: local frontiers of up to 64 entries (a few
// hundred edges per CTA), and larger ones (searches capped to a few CTAs,
// e.g. the server's concurrent searches: 64 queries on a 4000 x 4000 grid,
// 16 at once with 19 CTAs each, 248 -> 209 ms with 4 instead of 2; 6 is
// slower everywhere)
constexpr int RX_ILP = 2;
constexpr int RX_ILP_BIG = 4;
// Levels a CTA advances its piece per round.  7000 x 7000 grid, 7,194
// levels: 8 hops 21.9 ms, 16 hops 20.1, 32 hops 18.7, 64 hops 18.9 (and
// 1.3-3.5 % faster than 32 on smaller grids and a 200 k-vertex path).
constexpr int RX_HOPS = 64;
constexpr int RX_BPS = 2;  // CTAs per SM (one: 7000^2 grid 19.6 ms, thin-start expander +30 %)

template <typename RT>
__global__ void __launch_bounds__(RX_BLOCK, 2) k_bfs_relax(BfsArgs a)
{
    using Sel = RowSel<RT>;
    using B = BndT<RT>;
    const RT *const row = Sel::row(a);
    __shared__ int s_v[2][RX_CAP];
    __shared__ B s_b[2][RX_CAP];              // row bounds beside s_v
    __shared__ unsigned s_cnt[3];
    __shared__ unsigned long long s_cd;
    __shared__ unsigned long long s_red[2][RX_NW];
    __shared__ int s_max[RX_NW];

    BfsCtrl *ctrl = a.ctrl;
    // run only when the grid kernel parked its loop for this kernel
    const BfsResume rs = ctrl->rs;
    if (rs.done || rs.mode != RESUME_RELAX || ctrl->status != DEV_OK) return;

    const int n = a.n;
    const unsigned t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const long long gtid = (long long)blockIdx.x * RX_BLOCK + t;
    const long long gthreads = (long long)gridDim.x * RX_BLOCK;
    unsigned epoch = 0;
    unsigned *const lvl = reinterpret_cast<unsigned *>(a.level);  // -1 (unreached) is the largest unsigned
    int *const stamp = a.bigl;  // round stamps (rows are never deferred on graphs of small degree)

    // round stamps start at 0: round j marks the vertices it queues with j + 1
    if (((uintptr_t)stamp & 15) == 0) {
        int4 *s4 = reinterpret_cast<int4 *>(stamp);
        const long long n4 = n >> 2;
        for (long long i = gtid; i < n4; i += gthreads) s4[i] = make_int4(0, 0, 0, 0);
        for (long long i = (n4 << 2) + gtid; i < n; i += gthreads) stamp[i] = 0;
    } else {
        for (long long i = gtid; i < n; i += gthreads) stamp[i] = 0;
    }
    if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;

    const int L0 = rs.L;
    // frontier L0 (handed over, not yet in the reached totals); its counter
    // is reused two rounds on
    const unsigned long long cd0 = ld_relaxed_u64(&ctrl->cd[L0 % 3]);
    unsigned long long my_reached = 0, my_edges = 0;
    int rounds = 0;

    for (int j = 0;; ++j) {
        const int Lj = L0 + j;
        if (t == 0) s_cd = ld_relaxed_u64(&ctrl->cd[Lj % 3]);
        __syncthreads();
        const unsigned long long F = cd_count(s_cd);
        if (F == 0) {
            rounds = j;
            break;
        }
        // the count two rounds back (read by every CTA before the last barrier)
        if (gtid == 0) ctrl->cd[(Lj + 2) % 3] = 0;
        const int *qin = (Lj & 1) ? a.q1 : a.q0;
        const B *qbin = Sel::qb(a, Lj & 1);
        int *qout = (Lj & 1) ? a.q0 : a.q1;
        B *qbout = Sel::qb(a, (Lj + 1) & 1);
        unsigned long long *cnt_out = &ctrl->cd[(Lj + 1) % 3];
        const int mark = j + 1;

        // global push of v (with its row bounds) by the lanes with `go`,
        // at most once per vertex and round
        auto push_global = [&](bool go, int v, B vb) {
            if (go) go = atomicMax(stamp + v, mark) < mark;
            const unsigned m = __ballot_sync(FULL, go);
            if (!m) return;
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if ((int)lane == leader) base = cd_count(atomicAdd(cnt_out, (unsigned long long)__popc(m)));
            base = __shfl_sync(FULL, base, leader) + __popc(m & lanemask_lt());
            if (go) {
                qout[base] = v;
                qbout[base] = vb;
            }
        };

        // relax the edges (u, w[q]) (w[q] < 0: none) with level[u] + 1;
        // improvements join local frontier `nb` (its counter cnt_nb), or the
        // global queue if `last` or that frontier is full
        auto relax = [&](auto ilp, const int *w, const int *u, bool last, int nb, unsigned *cnt_nb) {
            constexpr int Q = decltype(ilp)::value;
            unsigned nd[Q];
#pragma unroll
            for (int q = 0; q < Q; q++) nd[q] = w[q] >= 0 ? __ldcg(lvl + u[q]) + 1u : 0u;  // 0: skip
            unsigned old[Q];
            B wb[Q];
#pragma unroll
            for (int q = 0; q < Q; q++) {
                old[q] = 0;
                wb[q] = Sel::mk(0, 0);
                if (nd[q] != 0) {
                    old[q] = atomicMin(lvl + w[q], nd[q]);
                    wb[q] = Sel::mk(__ldg(row + w[q]), __ldg(row + w[q] + 1));
                }
            }
#pragma unroll
            for (int q = 0; q < Q; q++) {
                const bool imp = nd[q] != 0 && nd[q] < old[q];
                if (imp) {
                    // the next hop (or round) reads this row: start its fetch into L2
                    if (wb[q].y > wb[q].x) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.col + wb[q].x));
                    if (old[q] == 0xffffffffu) {
                        ++my_reached;
                        my_edges += (unsigned long long)(wb[q].y - wb[q].x);
                    }
                }
                bool glob = imp && last;
                if (!last) {
                    const unsigned m = __ballot_sync(FULL, imp);
                    if (m) {
                        const int leader = __ffs(m) - 1;
                        unsigned pos = 0;
                        if ((int)lane == leader) pos = atomicAdd(cnt_nb, (unsigned)__popc(m));
                        pos = __shfl_sync(FULL, pos, leader) + __popc(m & lanemask_lt());
                        if (imp) {
                            if (pos < (unsigned)RX_CAP) {
                                s_v[nb][pos] = w[q];
                                s_b[nb][pos] = wb[q];
                            } else {
                                glob = true;  // the counter passes RX_CAP: the hop overflowed
                            }
                        }
                    }
                }
                push_global(glob, w[q], wb[q]);
            }
        };

        // expand local frontier `cur` (nc entries) one level
        auto expand = [&](int cur, int nc, bool last, unsigned *cnt_nb) {
            const int nb = cur ^ 1;
            if (nc <= 64) {
                // a small frontier: every warp scans its (at most 64) out-degrees
                // itself, two entries per lane, and finds an edge's entry with
                // shuffles (no CTA barrier)
                const int i0 = 2 * (int)lane, i1 = i0 + 1;
                const B b0 = i0 < nc ? s_b[cur][i0] : Sel::mk(0, 0);
                const B b1 = i1 < nc ? s_b[cur][i1] : Sel::mk(0, 0);
                const int d0 = (int)(b0.y - b0.x), d1 = (int)(b1.y - b1.x);
                const int incl = warp_incl_scan(d0 + d1);
                const int ex0 = incl - d0 - d1, ex1 = ex0 + d0;
                const int E = __shfl_sync(FULL, incl, 31);
                for (int e0 = 0; e0 < E; e0 += RX_BLOCK * RX_ILP) {
                    if (e0 + (int)(warp * 32) >= E) break;  // no edge left for this warp
                    int w[RX_ILP], u[RX_ILP];
#pragma unroll
                    for (int q = 0; q < RX_ILP; q++) {
                        const int e = e0 + q * RX_BLOCK + (int)t;
                        // the lane holding edge e: the last lane whose first
                        // entry starts at or before e
                        int l = 0;
#pragma unroll
                        for (int st = 16; st > 0; st >>= 1)
                            if (__shfl_sync(FULL, ex0, l + st) <= e) l += st;
                        const int x0 = __shfl_sync(FULL, ex0, l), x1 = __shfl_sync(FULL, ex1, l);
                        const RT bx0 = __shfl_sync(FULL, b0.x, l), bx1 = __shfl_sync(FULL, b1.x, l);
                        w[q] = -1;
                        u[q] = 0;
                        if (e < E) {
                            const bool second = e >= x1;
                            const int i = 2 * l + (second ? 1 : 0);
                            w[q] = __ldg(a.col + (second ? bx1 + (e - x1) : bx0 + (e - x0)));
                            u[q] = s_v[cur][i];
                        }
                    }
                    relax(std::integral_constant<int, RX_ILP>{}, w, u, last, nb, cnt_nb);
                }
                return;
            }
            {
                // a larger frontier: warp w expands its own slice of at most
                // 64 entries, [w C, (w + 1) C), two per lane, with a warp scan
                // and shuffles, RX_ILP_BIG edges per lane in flight (no CTA
                // barrier; grid-like rows have similar degrees).  Against one
                // CTA-wide scan of the whole frontier: a 4000 x 4000 grid
                // search capped to 12 CTAs 22.0 -> 19.3 ms, 16 concurrent
                // searches of 19 CTAs 662 -> 726 queries/s
                const int C = (nc + RX_NW - 1) / RX_NW;
                const int base = (int)warp * C;
                const int cnt = max(0, min(C, nc - base));
                const int j0 = 2 * (int)lane, j1 = j0 + 1;
                const B b0 = j0 < cnt ? s_b[cur][base + j0] : Sel::mk(0, 0);
                const B b1 = j1 < cnt ? s_b[cur][base + j1] : Sel::mk(0, 0);
                const int d0 = (int)(b0.y - b0.x), d1 = (int)(b1.y - b1.x);
                const int incl = warp_incl_scan(d0 + d1);
                const int ex0 = incl - d0 - d1, ex1 = ex0 + d0;
                const int Ew = __shfl_sync(FULL, incl, 31);
                for (int e0 = 0; e0 < Ew; e0 += 32 * RX_ILP_BIG) {
                    int w[RX_ILP_BIG], u[RX_ILP_BIG];
#pragma unroll
                    for (int q = 0; q < RX_ILP_BIG; q++) {
                        const int e = e0 + q * 32 + (int)lane;
                        int l = 0;
#pragma unroll
                        for (int st = 16; st > 0; st >>= 1)
                            if (__shfl_sync(FULL, ex0, l + st) <= e) l += st;
                        const int x0 = __shfl_sync(FULL, ex0, l), x1 = __shfl_sync(FULL, ex1, l);
                        const RT bx0 = __shfl_sync(FULL, b0.x, l), bx1 = __shfl_sync(FULL, b1.x, l);
                        w[q] = -1;
                        u[q] = 0;
                        if (e < Ew) {
                            const bool second = e >= x1;
                            w[q] = __ldg(a.col + (second ? bx1 + (e - x1) : bx0 + (e - x0)));
                            u[q] = s_v[cur][base + 2 * l + (second ? 1 : 0)];
                        }
                    }
                    relax(std::integral_constant<int, RX_ILP_BIG>{}, w, u, last, nb, cnt_nb);
                }
                return;
            }
        };

        const unsigned long long lo = F * blockIdx.x / gridDim.x, hi = F * (blockIdx.x + 1) / gridDim.x;
        const bool hops = hi - lo <= (unsigned long long)RX_CAP;
        for (unsigned long long s0 = lo; s0 < hi; s0 += RX_CAP) {
            const int ns = (int)min((unsigned long long)RX_CAP, hi - s0);
            for (int i = (int)t; i < ns; i += RX_BLOCK) {
                s_v[0][i] = __ldcg(qin + s0 + i);
                s_b[0][i] = __ldcg(qbin + s0 + i);
            }
            // hop h expands local frontier h & 1, counted by s_cnt[h % 3], into
            // frontier (h + 1) & 1, counted by s_cnt[(h + 1) % 3]; s_cnt[(h + 2) % 3]
            // (hop h - 1's, read before the barrier that ended it) is zeroed
            // during hop h, so a hop needs one CTA barrier
            if (t == 0) {
                s_cnt[0] = (unsigned)ns;
                s_cnt[1] = 0;
                s_cnt[2] = 0;
            }
            __syncthreads();
            int nc = ns;
            for (int h = 0;; ++h) {
                const bool last = !hops || h == RX_HOPS - 1;
                if (t == 0 && h > 0) s_cnt[(h + 2) % 3] = 0;
                unsigned *cnt_nb = &s_cnt[(h + 1) % 3];
                expand(h & 1, nc, last, cnt_nb);
                __syncthreads();
                if (last) break;
                const unsigned raw = *cnt_nb;
                const unsigned nn = min(raw, (unsigned)RX_CAP);
                if (raw > (unsigned)RX_CAP || nn == 0) {
                    // the hop overflowed the local frontier (or found nothing):
                    // what it holds joins the global queue
                    for (unsigned k0 = 0; k0 < nn; k0 += RX_BLOCK) {
                        const unsigned i = k0 + t;
                        int v = 0;
                        B vb = Sel::mk(0, 0);
                        if (i < nn) {
                            v = s_v[(h + 1) & 1][i];
                            vb = s_b[(h + 1) & 1][i];
                        }
                        push_global(i < nn, v, vb);
                    }
                    break;
                }
                nc = (int)nn;
            }
            __syncthreads();  // before the next piece overwrites the local queues
        }
        if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
        if (gtid == 0) {
            LevelTrace tr;
            tr.level = Lj;
            tr.dir = 4;
            tr.frontier = F;
            tr.edges = 0;
            tr.t_ns = globaltimer_ns();
            ctrl->trace[Lj < TRACE_CAP - 1 ? Lj : TRACE_CAP - 1] = tr;
        }
    }

    // complete: the largest level, and the totals of first relaxations
    int mx = -1;
    if (((uintptr_t)a.level & 15) == 0) {
        const int4 *l4 = reinterpret_cast<const int4 *>(a.level);
        const long long n4 = n >> 2;
        for (long long i = gtid; i < n4; i += gthreads) {
            const int4 x = __ldcg(l4 + i);
            mx = max(mx, max(max(x.x, x.y), max(x.z, x.w)));
        }
        for (long long i = (n4 << 2) + gtid; i < n; i += gthreads) mx = max(mx, __ldcg(a.level + i));
    } else {
        for (long long i = gtid; i < n; i += gthreads) mx = max(mx, __ldcg(a.level + i));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
    const unsigned long long rsum = warp_sum(my_reached), esum = warp_sum(my_edges);
    if (lane == 0) {
        s_max[warp] = mx;
        s_red[0][warp] = rsum;
        s_red[1][warp] = esum;
    }
    __syncthreads();
    if (warp == 0) {
        int m2 = lane < RX_NW ? s_max[lane] : -1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m2 = max(m2, __shfl_xor_sync(FULL, m2, o));
        const unsigned long long r2 = warp_sum(lane < RX_NW ? s_red[0][lane] : 0ull);
        const unsigned long long e2 = warp_sum(lane < RX_NW ? s_red[1][lane] : 0ull);
        if (lane == 0) {
            atomicMax(&ctrl->rx_max, m2);
            atomicAdd(&ctrl->rx_reached, r2);
            atomicAdd(&ctrl->rx_edges, e2);
        }
    }
    if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
    if (gtid == 0) {
        const int levels = ctrl->rx_max + 1;
        BfsOut o;
        o.levels = levels;
        o.td_levels = levels - rs.bu_levels;
        o.bu_levels = rs.bu_levels;
        o.roots = (int)rs.roots;
        o.reached = rs.reached + cd_count(cd0) + ctrl->rx_reached;
        o.edges_c = rs.edges_c + cd_degree(cd0) + ctrl->rx_edges;
        *a.out = o;
        ctrl->t_end = globaltimer_ns();
        const int tl = L0 + rounds;
        ctrl->trace_len = tl < TRACE_CAP ? tl : TRACE_CAP;
        ctrl->rx_max = 0;
        ctrl->rx_reached = 0;
        ctrl->rx_edges = 0;
        for (int i = 0; i < 3; i++) {
            ctrl->cd[i] = 0;
            ctrl->big[i] = 0;
        }
        ctrl->fill = 0;
        ctrl->rs.done = 1;
        ctrl->rs.mode = RESUME_LEVEL;
    }
    grid_exit(&ctrl->bar, &ctrl->t_exit);
}

}  // namespace

cudaError_t bfs_relax_launch(const BfsArgs &args, cudaStream_t st, int max_ctas)
{
    static LaunchSetup setup;
    int sms = 0, occ = 0;
    cudaError_t e = setup.get(sms, occ, [](int dev, int &s_out, int &o_out) {
        cudaError_t r = cudaDeviceGetAttribute(&s_out, cudaDevAttrMultiProcessorCount, dev);
        if (r == cudaSuccess) r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o_out, k_bfs_relax<int>, RX_BLOCK, 0);
        return r;
    });
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int grid = sms * std::max(1, std::min(RX_BPS, occ));
    if (max_ctas > 0) grid = std::max(1, std::min(grid, max_ctas));
    BfsArgs a = args;
    void *kargs[] = {&a};
    // the wide kernel holds twice the row-bound bytes in shared memory; its
    // CTAs still fit two per SM
    const void *fn = a.wide ? (const void *)k_bfs_relax<long long> : (const void *)k_bfs_relax<int>;
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(RX_BLOCK), kargs, 0, st);
}

}  // namespace gbfs
