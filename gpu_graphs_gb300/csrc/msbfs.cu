// msbfs.cu -- 64-lane multi-source BFS in one persistent launch (sm_103a).
//
// The reference answers one source per gpuBFS construction
// (1D Partition/src/gpuBFS.cu:13-116).  Here up to 64 searches on the same
// graph share every pass over it: per vertex, uint64 lane masks record which
// searches reached it (vis) and which have it in their frontier (F).  A
// lane's level at v is the step in which its bit first appears in vis[v],
// written straight into that lane's int32 level row.
//
// Work per level follows the frontier, not the graph:
//   * the active vertices of a level (F != 0) are kept in a queue;
//   * push step (sparse frontiers): the queue's rows are expanded with the
//     edges split evenly over warps (per-CTA degree prefix in shared
//     memory); each edge claims its lanes at the neighbour with one atomicOr
//     on vis, the claimed lanes go into the next frontier mask with a second
//     atomicOr, whose first writer appends the neighbour to the next queue;
//   * pull step (dense frontiers): every vertex with unreached lanes ORs F
//     over its in-edges (its own row on a symmetric graph, its row of the
//     transpose on a directed one) until those lanes are covered --
//     one thread per light row, a whole warp per row of degree > 64;
//   * frontier masks and queues rotate by level, and the masks of level L-1
//     are cleared through their queue during level L, so no pass touches all
//     n vertices after initialisation except pull steps.
// Levels are separated by the bounded grid barrier of common.cuh.
#include <algorithm>
#include <cstddef>
#include <vector>

#include "blockq.cuh"
#include "msbfs.cuh"

namespace gbfs {

namespace {

constexpr int MS_BLOCK = 512;
constexpr int MS_SEG = 2048;                 // queue entries per edge-balanced pass
constexpr int MS_PER = MS_SEG / MS_BLOCK;    // entries per thread in the prefix
constexpr int MS_BIG = 256;                  // push rows this long go to a grid-wide pass

struct MsArgs {
    int n, n_active, k;
    const int *row, *col;     // out-edges: push steps
    const int *prow, *pcol;   // in-edges: pull steps (row/col on a symmetric graph)
    const int *heavy;
    int nheavy;
    const int2 *pieces;
    int npieces;
    unsigned long long *hacc;
    unsigned *hcnt;
    unsigned long long *vis;
    int *bigl;
    unsigned long long *F[3];
    int *Q[4];
    int *out;
    unsigned char *lv8;
    const int *src;
    MsCtrl *ctrl;
    int pull_allowed, direction, pull_div;
    int has_big;              // some push row has MS_BIG edges or more (else none is deferred)
    unsigned long long timeout_ns;
};

// Levels are recorded as bytes (lv8, 64 x n) while the search runs: a row of
// 4 x n level ints written a few entries per level leaves partly written
// sectors to be evicted and merged in DRAM over and over, while the byte
// rows of a million-vertex graph stay in L2.  The closing pass expands them
// into out with whole 128-byte lines.  Levels from LV8_DEEP on go straight
// to out, their byte marked LV8_DEEP.
constexpr int LV8_DEEP = 255;

__device__ __forceinline__ void record_level(unsigned char *lv8, int *out, int n, long long u, int j, int nl)
{
    const size_t i = (size_t)j * n + u;
    if (nl < LV8_DEEP) {
        lv8[i] = (unsigned char)nl;
    } else {
        lv8[i] = (unsigned char)LV8_DEEP;
        out[i] = nl;
    }
}

__device__ __forceinline__ void write_levels(unsigned char *lv8, int *out, int n, int u, unsigned long long bits,
                                             int nl)
{
    while (bits) {
        const int j = __ffsll((long long)bits) - 1;
        record_level(lv8, out, n, u, j, nl);
        bits &= bits - 1ull;
    }
}

__device__ __forceinline__ unsigned long long warp_or64(unsigned long long x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x |= __shfl_xor_sync(FULL, x, o);
    return x;
}

// Warp-wide level writes for 32 consecutive vertices u = base + lane: the loop
// runs over the union of the lanes' masks, so each store instruction covers
// one byte row and coalesces.  All 32 threads call it.
__device__ __forceinline__ void write_levels_warp(unsigned char *lv8, int *out, int n, long long u,
                                                  unsigned long long bits, int nl)
{
    unsigned long long any = warp_or64(bits);
    while (any) {
        const int j = __ffsll((long long)any) - 1;
        if ((bits >> j) & 1ull) record_level(lv8, out, n, u, j, nl);
        any &= any - 1ull;
    }
}

// Push step over list[0, cnt): every edge offers its row's frontier lanes
// to the neighbour.  grid_wide: all warps of the grid split each MS_SEG-row
// segment's edges (segments one after another); otherwise CTA b takes
// segments b, b+G, ... of about cnt/G rows and its own warps split them.
// defer: rows of MS_BIG edges or more are appended to a.bigl (count in
// *bigcnt) instead.  Each edge claims its lanes at the neighbour with one
// atomicOr on vis (after a plain-load filter; vis only gains bits, and the
// atomic's old value settles which lanes this edge discovers, so every
// (lane, vertex) pair is claimed exactly once), and the claimed lanes go
// into the next frontier mask with a second atomicOr whose first writer
// queues the neighbour.  All threads of the CTA call it.
__device__ __forceinline__ void push_rows(const MsArgs &a, const int *list, long long cnt, bool grid_wide, bool defer,
                                          int nl, const unsigned long long *Fc, unsigned long long *Fn, WarpQ &q,
                                          unsigned long long *qcnt_next, int *Qn, unsigned long long &my_or,
                                          int *s_pre, int *s_beg, unsigned long long *s_f, int *s_warp,
                                          unsigned long long *bigcnt)
{
    const unsigned lane = lane_id();
    const long long gwarp = ((long long)blockIdx.x * MS_BLOCK + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * MS_BLOCK) >> 5;
    const long long cta_seg = min((long long)MS_SEG, max(32LL, (cnt + gridDim.x - 1) / gridDim.x));
    const long long seg_len = grid_wide ? MS_SEG : cta_seg;
    const long long seg0 = grid_wide ? 0 : (long long)blockIdx.x * seg_len;
    const long long seg_step = grid_wide ? MS_SEG : (long long)gridDim.x * seg_len;
    const long long wid = grid_wide ? gwarp : (long long)(threadIdx.x >> 5);
    const long long wcount = grid_wide ? nwarps : (long long)(MS_BLOCK / 32);
    const int n = a.n;
    for (long long seg = seg0; seg < cnt; seg += seg_step) {
        const int segn = (int)min(seg_len, cnt - seg);
        int d[MS_PER];
        int sum = 0;
#pragma unroll
        for (int t = 0; t < MS_PER; t++) {
            const int j = threadIdx.x * MS_PER + t;
            d[t] = 0;
            if (j < segn) {
                const int v = __ldcg(list + seg + j);
                const int b = __ldg(a.row + v);
                s_beg[j] = b;
                s_f[j] = __ldcg(Fc + v);
                d[t] = __ldg(a.row + v + 1) - b;
                if (defer && d[t] >= MS_BIG) {
                    a.bigl[atomicAdd(bigcnt, 1ull)] = v;
                    d[t] = 0;
                }
            }
            sum += d[t];
        }
        int total;
        int run = block_excl_scan_int(sum, s_warp, &total);
#pragma unroll
        for (int t = 0; t < MS_PER; t++) {
            const int j = threadIdx.x * MS_PER + t;
            if (j < segn) s_pre[j] = run;
            run += d[t];
        }
        __syncthreads();
        const long long lo = (long long)total * wid / wcount;
        const long long hi = (long long)total * (wid + 1) / wcount;
        for (long long e0 = lo; e0 < hi; e0 += 64) {
            int uu[2];
            bool tt[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const long long e = e0 + h * 32 + lane;
                uu[h] = -1;
                tt[h] = false;
                if (e < hi) {
                    int l = 0, r = segn - 1;  // max j with s_pre[j] <= e
                    while (l < r) {
                        const int mid = (l + r + 1) >> 1;
                        if (s_pre[mid] <= e) l = mid; else r = mid - 1;
                    }
                    const int u = __ldg(a.col + s_beg[l] + (int)(e - s_pre[l]));
                    unsigned long long nw = s_f[l] & ~a.vis[u];
                    if (nw) {
                        nw &= ~atomicOr(a.vis + u, nw);
                        if (nw) {
                            tt[h] = atomicOr(Fn + u, nw) == 0ull;
                            uu[h] = u;
                            my_or |= nw;
                            write_levels(a.lv8, a.out, n, u, nw, nl);
                        }
                    }
                }
            }
            wq_push(q, tt[0], uu[0], qcnt_next, Qn);
            wq_push(q, tt[1], uu[1], qcnt_next, Qn);
        }
        __syncthreads();
    }
}

// block_flush with an OR of lane masks in the same pass: every warp queue of the block is
// appended with one global atomic on cnt, and the block's lanes (x, one mask
// per thread) are ORed into *dst with one more, both issued by thread 0 after
// the same two barriers (all threads call).
__device__ __forceinline__ void block_flush_or(WarpQ &q, unsigned long long *cnt, int *out, unsigned long long x,
                                               unsigned long long *dst, int *s_wq, unsigned long long *s_or,
                                               unsigned long long *s_base)
{
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned lane = lane_id();
    x = warp_or64(x);
    __syncwarp();
    if (lane == 0) {
        s_wq[w] = q.n;
        s_or[w] = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int c = (int)lane < nw ? s_wq[lane] : 0;
        const unsigned long long o = (int)lane < nw ? s_or[lane] : 0ull;
        const int incl = warp_incl_scan(c);
        const int tot = __shfl_sync(FULL, incl, 31);
        const unsigned long long ot = warp_or64(o);
        if ((int)lane < nw) s_wq[lane] = incl - c;
        if (lane == 0) {
            *s_base = tot ? atomicAdd(cnt, (unsigned long long)tot) : 0ull;
            if (ot) atomicOr(dst, ot);
        }
    }
    __syncthreads();
    const unsigned long long base = *s_base + (unsigned long long)s_wq[w];
    for (int i = lane; i < q.n; i += 32) out[base + i] = q.buf[i];
    q.n = 0;
    __syncthreads();
}

__global__ void __launch_bounds__(MS_BLOCK, 2) k_msbfs(MsArgs a)
{
    extern __shared__ int ms_smem[];
    __shared__ unsigned long long s_red[32];
    __shared__ unsigned long long s_base;
    __shared__ unsigned long long s_ctl[3];  // this level's queue size, live lanes, last level's queue size
    __shared__ int s_warp[33];
    __shared__ int s_wq[33];
    constexpr int NW = MS_BLOCK / 32;
    int *s_q = ms_smem;                                                // NW * QCAP
    int *s_pre = s_q + NW * QCAP;                                      // MS_SEG
    int *s_beg = s_pre + MS_SEG;                                       // MS_SEG
    unsigned long long *s_f = (unsigned long long *)(s_beg + MS_SEG);  // MS_SEG

    const int n = a.n;
    const long long gtid = (long long)blockIdx.x * MS_BLOCK + threadIdx.x;
    const long long gthreads = (long long)gridDim.x * MS_BLOCK;
    const long long gwarp = gtid >> 5;
    const long long nwarps = gthreads >> 5;
    const unsigned lane = lane_id();
    const unsigned long long all = a.k >= 64 ? ~0ull : ((1ull << a.k) - 1ull);
    MsCtrl *ctrl = a.ctrl;
    unsigned epoch = 0;
    WarpQ q{s_q + (threadIdx.x >> 5) * QCAP, 0};
    if (gtid == 0) ctrl->t_entry = globaltimer_ns();

    // ---- init ----
    for (long long c = gtid; c < a.npieces; c += gthreads) {
        const int2 pc = a.pieces[c];
        if (pc.y == 0) {
            a.hacc[pc.x] = 0;
            a.hcnt[pc.x] = 0;
        }
    }
    for (long long v = gtid; v < n; v += gthreads) {
        a.vis[v] = 0;
        a.F[0][v] = 0;
        a.F[1][v] = 0;
        a.F[2][v] = 0;
    }
    // out is not pre-filled: every (lane, vertex) entry is written exactly
    // once, with its level when reached, or with -1 after the last level
    if (gtid == 0) {
        for (int i = 0; i < 4; i++) {
            ctrl->qcnt[i] = 0;
            ctrl->alive[i] = 0;
        }
        ctrl->alive[0] = all;
        ctrl->big[0] = ctrl->big[1] = 0;
        ctrl->reached = 0;
        ctrl->edges_c = 0;
    }
    if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
    if (blockIdx.x == 0 && threadIdx.x < (unsigned)a.k) {
        const int s = a.src[threadIdx.x];
        const unsigned long long bit = 1ull << threadIdx.x;
        atomicOr(&a.vis[s], bit);
        const unsigned long long old = atomicOr(&a.F[0][s], bit);
        a.lv8[(size_t)threadIdx.x * n + s] = 0;
        if (old == 0) a.Q[0][atomicAdd(&ctrl->qcnt[0], 1ull)] = s;
    }
    if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
    if (gtid == 0) ctrl->t_start = globaltimer_ns();

    int L = 0, push_levels = 0, pull_levels = 0;
    for (;;) {
        // the level's control words: one load each per CTA, shared
        if (threadIdx.x == 0) {
            s_ctl[0] = ld_relaxed_u64(&ctrl->qcnt[L % 4]);
            s_ctl[1] = ld_relaxed_u64(&ctrl->alive[L % 4]);
            s_ctl[2] = L >= 1 ? ld_relaxed_u64(&ctrl->qcnt[(L + 3) % 4]) : 0ull;
        }
        __syncthreads();
        const unsigned long long nq = s_ctl[0];
        if (nq == 0) break;
        // only lanes with a frontier at level L can reach anything at L+1
        const unsigned long long live = s_ctl[1] & all;
        unsigned long long my_or = 0;   // lanes this thread puts in the next frontier
        const unsigned long long nz = s_ctl[2];
        bool pull;
        if (!a.pull_allowed || a.direction == GBFS_DIR_TOPDOWN) pull = false;
        else if (a.direction == GBFS_DIR_BOTTOMUP) pull = true;
        else pull = (long long)nq * a.pull_div > a.n_active;
        const unsigned long long *Fc = a.F[L % 3];
        unsigned long long *Fn = a.F[(L + 1) % 3];
        unsigned long long *Fz = a.F[(L + 2) % 3];   // level L-1's masks, cleared now
        const int *Qc = a.Q[L % 4];
        int *Qn = a.Q[(L + 1) % 4];
        const int *Qz = a.Q[(L + 3) % 4];            // level L-1's queue
        unsigned long long *qcnt_next = &ctrl->qcnt[(L + 1) % 4];
        const int nl = L + 1;
        // Q[(L+2)%4] held level L-2; its count was last read during level L-1
        if (gtid == 0) {
            ctrl->qcnt[(L + 2) % 4] = 0;
            ctrl->alive[(L + 2) % 4] = 0;
            ctrl->big[(L + 1) & 1] = 0;  // last read during level L-1
        }
        for (long long i = gtid; i < (long long)nz; i += gthreads) Fz[__ldcg(Qz + i)] = 0;

        if (pull) {
            ++pull_levels;
            // light rows: one thread per vertex
            for (long long base = gwarp * 32; base < n; base += nwarps * 32) {
                const long long u = base + lane;
                unsigned long long nw = 0;
                if (u < n) {
                    const int b = __ldg(a.prow + u), e = __ldg(a.prow + u + 1);
                    if (e > b && e - b <= HEAVY_DEGREE) {
                        const unsigned long long vu = __ldcg(a.vis + u);
                        const unsigned long long need = ~vu & live;
                        if (need) {
                            unsigned long long acc = 0;
                            for (int i = b; i < e; i += 4) {
                                const int v0 = __ldg(a.pcol + i);
                                const int v1 = i + 1 < e ? __ldg(a.pcol + i + 1) : v0;
                                const int v2 = i + 2 < e ? __ldg(a.pcol + i + 2) : v0;
                                const int v3 = i + 3 < e ? __ldg(a.pcol + i + 3) : v0;
                                acc |= __ldcg(Fc + v0) | __ldcg(Fc + v1) | __ldcg(Fc + v2) | __ldcg(Fc + v3);
                                if ((acc & need) == need) break;
                            }
                            nw = acc & need;
                            if (nw) {
                                a.vis[u] = vu | nw;
                                Fn[u] = nw;
                                my_or |= nw;
                            }
                        }
                    }
                }
                // level writes: one store per discovered lane, coalesced over the
                // warp's 32 consecutive vertices
                write_levels_warp(a.lv8, a.out, n, u, nw, nl);
                wq_push(q, nw != 0, (int)u, qcnt_next, Qn);
            }
            // heavy rows up to MS_HUGE edges: a warp screens 32 of them at once
            // (one lane each, strided by the warp count so busy rows spread
            // evenly over warps) and walks those with lanes to find, one by one
            for (long long h0 = gwarp; h0 < a.nheavy; h0 += nwarps * 32) {
                const long long h = h0 + (long long)lane * nwarps;
                int u = 0, b = 0, e = 0;
                unsigned long long vu = 0, need = 0;
                if (h < a.nheavy) {
                    u = __ldg(a.heavy + h);
                    b = __ldg(a.prow + u);
                    e = __ldg(a.prow + u + 1);
                    if (e - b <= MS_HUGE) {  // longer rows: split into pieces below
                        vu = __ldcg(a.vis + u);
                        need = ~vu & live;
                    }
                }
                unsigned todo = __ballot_sync(FULL, need != 0);
                while (todo) {
                    const int sl = __ffs(todo) - 1;
                    todo &= todo - 1;
                    const int ru = __shfl_sync(FULL, u, sl);
                    const int rb = __shfl_sync(FULL, b, sl), re = __shfl_sync(FULL, e, sl);
                    const unsigned long long rneed = __shfl_sync(FULL, need, sl);
                    const unsigned long long rvu = __shfl_sync(FULL, vu, sl);
                    unsigned long long acc = 0;
                    for (int i0 = rb; i0 < re; i0 += 128) {
                        unsigned long long x = 0;
#pragma unroll
                        for (int t = 0; t < 4; t++) {
                            const int i = i0 + t * 32 + (int)lane;
                            if (i < re) x |= __ldcg(Fc + __ldg(a.pcol + i));
                        }
                        acc |= warp_or64(x);
                        if ((acc & rneed) == rneed) break;
                    }
                    const unsigned long long nw = acc & rneed;
                    if (nw) {
                        if (lane == 0) {
                            a.vis[ru] = rvu | nw;
                            Fn[ru] = nw;
                            my_or |= nw;
                        }
                        if ((nw >> lane) & 1ull) record_level(a.lv8, a.out, n, ru, lane, nl);
                        if ((nw >> (lane + 32)) & 1ull) record_level(a.lv8, a.out, n, ru, lane + 32, nl);
                    }
                    wq_push(q, lane == 0 && nw != 0, ru, qcnt_next, Qn);
                }
            }
            // huge rows: pieces of MS_PIECE edges spread over all warps, so a
            // hub that must be scanned to its end is not one warp's tail.  Each
            // piece ORs what it found into hacc[u] and counts itself in
            // hcnt[u]; the warp that counts a row's last piece settles the row.
            // vis[u] only changes when the row is settled, after all of its
            // pieces have counted, so every piece sees the same need: a row
            // with nothing to find is skipped by all of its pieces.
            for (long long c0 = gwarp; c0 < a.npieces; c0 += nwarps * 32) {
                const long long c = c0 + (long long)lane * nwarps;
                int2 pc = make_int2(0, 0);
                unsigned long long vu = 0, need = 0;
                if (c < a.npieces) {
                    pc = __ldg(a.pieces + c);
                    vu = __ldcg(a.vis + pc.x);
                    need = ~vu & live;
                }
                unsigned todo = __ballot_sync(FULL, need != 0);
                while (todo) {
                    const int sl = __ffs(todo) - 1;
                    todo &= todo - 1;
                    const int u = __shfl_sync(FULL, pc.x, sl), j = __shfl_sync(FULL, pc.y, sl);
                    const unsigned long long rvu = __shfl_sync(FULL, vu, sl);
                    const unsigned long long rneed = __shfl_sync(FULL, need, sl);
                    const int rb = __ldg(a.prow + u), re = __ldg(a.prow + u + 1);
                    const unsigned pn = (unsigned)((re - rb + MS_PIECE - 1) / MS_PIECE);
                    const int b = rb + j * MS_PIECE;
                    const int e = min(re, b + MS_PIECE);
                    unsigned long long acc = 0;
                    // skip a piece whose row the others have already covered (one
                    // read, broadcast: the loop below must be warp-uniform)
                    unsigned long long seen = lane == 0 ? ld_relaxed_u64(a.hacc + u) : 0ull;
                    seen = __shfl_sync(FULL, seen, 0);
                    if ((seen & rneed) != rneed) {
                        for (int i0 = b; i0 < e; i0 += 128) {
                            unsigned long long x = 0;
#pragma unroll
                            for (int t = 0; t < 4; t++) {
                                const int i = i0 + t * 32 + (int)lane;
                                if (i < e) x |= __ldcg(Fc + __ldg(a.pcol + i));
                            }
                            acc |= warp_or64(x);
                            if ((acc & rneed) == rneed) break;
                        }
                    }
                    unsigned long long tot = 0;
                    int last = 0;
                    if (lane == 0) {
                        if (acc & rneed) atomicOr(a.hacc + u, acc & rneed);
                        if (atom_add_acq_rel_gpu(a.hcnt + u, 1u) == pn - 1u) {
                            tot = atomicExch(a.hacc + u, 0ull);
                            a.hcnt[u] = 0;
                            last = 1;
                        }
                    }
                    last = __shfl_sync(FULL, last, 0);
                    if (!last) continue;
                    const unsigned long long nw = __shfl_sync(FULL, tot, 0) & rneed;
                    if (nw) {
                        if (lane == 0) {
                            a.vis[u] = rvu | nw;
                            Fn[u] = nw;
                            my_or |= nw;
                        }
                        if ((nw >> lane) & 1ull) record_level(a.lv8, a.out, n, u, lane, nl);
                        if ((nw >> (lane + 32)) & 1ull) record_level(a.lv8, a.out, n, u, lane + 32, nl);
                    }
                    wq_push(q, lane == 0 && nw != 0, u, qcnt_next, Qn);
                }
            }
            block_flush_or(q, qcnt_next, Qn, my_or, &ctrl->alive[(L + 1) % 4], s_wq, s_red, &s_base);
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
        } else {
            ++push_levels;
            // the queue's edges.  A queue of at most MS_SEG rows: every CTA
            // builds its degree prefix and the grid's warps split the edges
            // evenly.  Longer queues: CTA b takes segments b, b+G, ... sized so
            // every CTA gets about one and its own warps split them, with rows
            // of MS_BIG edges or more deferred to a second, grid-wide pass
            // (hub rows of power-law graphs would leave a few CTAs with most
            // of the edges).
            const bool grid_wide = nq <= (unsigned long long)MS_SEG;
            unsigned long long *bigcnt = &ctrl->big[L & 1];
            push_rows(a, Qc, (long long)nq, grid_wide, !grid_wide, nl, Fc, Fn, q, qcnt_next, Qn, my_or, s_pre,
                      s_beg, s_f, s_warp, bigcnt);
            block_flush_or(q, qcnt_next, Qn, my_or, &ctrl->alive[(L + 1) % 4], s_wq, s_red, &s_base);
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
            // rows deferred to the grid pass (segmented queues only, and only
            // when some row is that long): one load per CTA, shared
            unsigned long long nb = 0;
            if (!grid_wide && a.has_big) {
                if (threadIdx.x == 0) s_ctl[0] = ld_relaxed_u64(bigcnt);
                __syncthreads();
                nb = s_ctl[0];
            }
            if (nb) {
                my_or = 0;
                push_rows(a, a.bigl, (long long)nb, true, false, nl, Fc, Fn, q, qcnt_next, Qn, my_or, s_pre, s_beg,
                          s_f, s_warp, bigcnt);
                block_flush_or(q, qcnt_next, Qn, my_or, &ctrl->alive[(L + 1) % 4], s_wq, s_red, &s_base);
                if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
            }
        }
        if (gtid == 0) {
            LevelTrace t;
            t.level = L;
            t.dir = pull ? 1 : 0;
            t.frontier = nq;
            t.edges = 0;
            t.t_ns = globaltimer_ns();
            ctrl->trace[L < TRACE_CAP - 1 ? L : TRACE_CAP - 1] = t;
        }
        ++L;
    }
    if (gtid == 0) {
        ctrl->t_end = globaltimer_ns();
        ctrl->trace_len = L < TRACE_CAP ? L : TRACE_CAP;
    }

    // closing pass: level rows from the byte rows (-1 where a lane never
    // arrived), 32 consecutive vertices per warp so every store is a whole
    // line of one row; per-lane totals for GTEPS
    unsigned long long r = 0, ec = 0;
    const bool vec = ((n & 3) == 0) && (((uintptr_t)a.out & 15) == 0) && (((uintptr_t)a.lv8 & 3) == 0);
    if (vec) {
        // four consecutive vertices per thread: uchar4 byte loads, int4 stores
        // (a lane whose level went straight to out, LV8_DEEP, keeps it)
        const int nq4 = n >> 2;
        for (long long q4 = gtid; q4 < nq4; q4 += gthreads) {
            const long long u0 = q4 << 2;
            unsigned long long vu[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                vu[t] = __ldcg(a.vis + u0 + t) & all;
                const int c = __popcll(vu[t]);
                if (c) {
                    r += c;
                    ec += (unsigned long long)c * (unsigned long long)(__ldg(a.row + u0 + t + 1) - __ldg(a.row + u0 + t));
                }
            }
            for (int j0 = 0; j0 < a.k; j0 += 4) {
                uchar4 b[4];
#pragma unroll
                for (int t = 0; t < 4; t++)
                    if (j0 + t < a.k) b[t] = __ldcg(reinterpret_cast<const uchar4 *>(a.lv8 + (size_t)(j0 + t) * n + u0));
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int j = j0 + t;
                    if (j >= a.k) break;
                    const int bv[4] = {b[t].x, b[t].y, b[t].z, b[t].w};
                    int o[4];
                    bool deep = false;
#pragma unroll
                    for (int x = 0; x < 4; x++) {
                        const bool hit = (vu[x] >> j) & 1ull;
                        o[x] = hit ? bv[x] : -1;
                        deep |= hit && bv[x] == LV8_DEEP;
                    }
                    int *dst = a.out + (size_t)j * n + u0;
                    if (!deep) {
                        *reinterpret_cast<int4 *>(dst) = make_int4(o[0], o[1], o[2], o[3]);
                    } else {
#pragma unroll
                        for (int x = 0; x < 4; x++)
                            if (o[x] != LV8_DEEP) dst[x] = o[x];
                    }
                }
            }
        }
    }
    for (long long base = gwarp * 32; !vec && base < n; base += nwarps * 32) {
        const long long u = base + lane;
        if (u >= n) continue;  // no warp-wide operations below
        const unsigned long long vu = __ldcg(a.vis + u) & all;
        const int c = __popcll(vu);
        if (c) {
            r += c;
            ec += (unsigned long long)c * (unsigned long long)(__ldg(a.row + u + 1) - __ldg(a.row + u));
        }
        // 16 lanes' bytes are loaded before any of their stores, so the
        // loads are in flight together
        for (int j0 = 0; j0 < a.k; j0 += 16) {
            int v[16];
#pragma unroll
            for (int t = 0; t < 16; t++) {
                const int j = j0 + t;
                v[t] = -1;
                if (j < a.k && ((vu >> j) & 1ull)) v[t] = __ldcg(a.lv8 + (size_t)j * n + u);
            }
#pragma unroll
            for (int t = 0; t < 16; t++)
                if (j0 + t < a.k && v[t] != LV8_DEEP) a.out[(size_t)(j0 + t) * n + u] = v[t];
        }
    }
    const unsigned long long br = block_reduce_sum(r, s_red);
    const unsigned long long be = block_reduce_sum(ec, s_red);
    if (threadIdx.x == 0) {
        if (br) atomicAdd(&ctrl->reached, br);
        if (be) atomicAdd(&ctrl->edges_c, be);
    }
    if (gtid == 0) {
        ctrl->levels = L;
        ctrl->push_levels = push_levels;
        ctrl->pull_levels = pull_levels;
    }
    grid_exit(&ctrl->bar, &ctrl->t_exit);
}

__global__ void k_heavy_degrees(const int *__restrict__ row, const int *__restrict__ heavy, int nheavy, int *deg)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nheavy; i += gridDim.x * blockDim.x)
        deg[i] = row[heavy[i] + 1] - row[heavy[i]];
}

size_t ms_smem_bytes()
{
    return sizeof(int) * ((size_t)(MS_BLOCK / 32) * QCAP + 2 * (size_t)MS_SEG) +
           sizeof(unsigned long long) * (size_t)MS_SEG;
}

}  // namespace

int64_t ms_prepare_bytes(const DeviceCsr &g, bool transpose)
{
    // rows of degree d > 2 * MS_PIECE give ceil(d / MS_PIECE) < 1.5 d / MS_PIECE pieces
    const int64_t one = (int64_t)sizeof(int2) * (3 * g.m / (2 * MS_PIECE) + 1);
    return (g.pieces_built ? 0 : one) + (transpose && !g.tpieces_built ? one : 0);
}

namespace {

// The pull pieces of one adjacency (out-edge rows, or the transpose's
// in-edge rows): {vertex, j} for the j-th MS_PIECE edges of every heavy row
// longer than MS_HUGE.
int build_pieces(const int *row, const int *heavy, int nheavy, cudaStream_t st, int2 *&out, int32_t &count,
                 std::string &err)
{
    std::vector<int2> h_pieces;
    if (nheavy > 0) {
        int *deg = nullptr;
        std::vector<int> h_heavy(nheavy), h_deg(nheavy);
        cudaError_t e = cudaMalloc(&deg, sizeof(int) * (size_t)nheavy);
        if (e == cudaSuccess) {
            k_heavy_degrees<<<std::max(1, std::min(1216, (nheavy + 255) / 256)), 256, 0, st>>>(row, heavy, nheavy,
                                                                                             deg);
            e = cudaMemcpyAsync(h_deg.data(), deg, sizeof(int) * (size_t)nheavy, cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_heavy.data(), heavy, sizeof(int) * (size_t)nheavy, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(deg);
        if (e != cudaSuccess) {
            err = std::string("pull pieces: ") + cudaGetErrorString(e);
            return GBFS_ERR_CUDA;
        }
        for (int i = 0; i < nheavy; i++)
            if (h_deg[i] > MS_HUGE)
                for (int j = 0; j * MS_PIECE < h_deg[i]; j++) h_pieces.push_back(make_int2(h_heavy[i], j));
    }
    int2 *d = nullptr;
    if (!h_pieces.empty()) {
        cudaError_t e = cudaMalloc(&d, sizeof(int2) * h_pieces.size());
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d, h_pieces.data(), sizeof(int2) * h_pieces.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaFree(d);
            err = std::string("pull pieces: ") + cudaGetErrorString(e);
            return e == cudaErrorMemoryAllocation ? GBFS_ERR_OOM : GBFS_ERR_CUDA;
        }
    }
    out = d;
    count = (int32_t)h_pieces.size();
    return GBFS_OK;
}

}  // namespace

int ms_prepare(DeviceCsr &g, cudaStream_t st, std::string &err)
{
    if (!g.pieces_built) {
        const int nh = g.max_degree > MS_HUGE ? g.nheavy : 0;
        const int rc = build_pieces(g.row, g.heavy, nh, st, g.pieces, g.npieces, err);
        if (rc) return rc;
        g.pieces_built = true;
    }
    if (g.trow && !g.tpieces_built) {
        const int rc = build_pieces(g.trow, g.theavy, g.ntheavy, st, g.tpieces, g.ntpieces, err);
        if (rc) return rc;
        g.tpieces_built = true;
    }
    return GBFS_OK;
}

int ms_work_alloc(MsWork &w, int32_t n, std::string &err)
{
    if (w.ctrl && w.n == n) return GBFS_OK;
    ms_work_free(w);
    auto al = [&](void **p, size_t b) -> bool {
        cudaError_t e = cudaMalloc(p, std::max<size_t>(b, 16));
        if (e != cudaSuccess) {
            err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
            return false;
        }
        w.bytes += (int64_t)std::max<size_t>(b, 16);
        return true;
    };
    w.bytes = 0;
    const size_t b8 = sizeof(unsigned long long) * (size_t)n, b4 = sizeof(int) * (size_t)n;
    bool ok = al((void **)&w.vis, b8) && al((void **)&w.hacc, b8) && al((void **)&w.hcnt, b4) &&
              al((void **)&w.lv8, (size_t)n * MS_LANES) && al((void **)&w.bigl, b4) &&
              al((void **)&w.out, b4 * MS_LANES) && al((void **)&w.src, sizeof(int) * MS_LANES) &&
              al((void **)&w.ctrl, sizeof(MsCtrl));
    for (int i = 0; ok && i < 3; i++) ok = al((void **)&w.F[i], b8);
    for (int i = 0; ok && i < 4; i++) ok = al((void **)&w.Q[i], b4);
    if (!ok) {
        ms_work_free(w);
        return GBFS_ERR_OOM;
    }
    if (cudaMemset(w.ctrl, 0, sizeof(MsCtrl)) != cudaSuccess ||
        cudaMallocHost(&w.h_ctrl, sizeof(MsCtrl)) != cudaSuccess ||
        cudaEventCreate(&w.ev0) != cudaSuccess || cudaEventCreate(&w.ev1) != cudaSuccess) {
        err = "multi-source workspace setup failed";
        ms_work_free(w);
        return GBFS_ERR_CUDA;
    }
    w.n = n;
    return GBFS_OK;
}

void ms_work_free(MsWork &w)
{
    void *ps[] = {w.vis, w.hacc, w.hcnt, w.lv8, w.bigl, w.out, w.src, w.ctrl, w.F[0], w.F[1], w.F[2], w.Q[0], w.Q[1], w.Q[2], w.Q[3]};
    for (void *p : ps)
        if (p) cudaFree(p);
    if (w.h_ctrl) cudaFreeHost(w.h_ctrl);
    if (w.ev0) cudaEventDestroy(w.ev0);
    if (w.ev1) cudaEventDestroy(w.ev1);
    w = MsWork{};
}

int64_t ms_work_bytes(int64_t n)
{
    return n > 0 ? (int64_t)(8 * 5 + 4 * 6 + 5 * MS_LANES) * n + 4096 : 0;
}

cudaError_t msbfs_enqueue(const DeviceCsr &g, const gbfs_params &p, bool symmetric, MsWork &w,
                          const int *d_src, int k, int *d_out, cudaStream_t st, int max_ctas)
{
    MsArgs a;
    a.n = g.n;
    a.n_active = (int)std::max<int64_t>(1, g.nonisolated);
    a.k = k;
    a.row = g.row;
    a.col = g.col;
    if (!g.pieces_built || (g.trow && !g.tpieces_built)) return cudaErrorInvalidValue;  // ms_prepare not run
    // pull steps gather over in-edges: the rows themselves on a symmetric
    // graph, the transpose on a directed one (no pull steps without it)
    const bool pull_allowed = symmetric || g.trow != nullptr;
    const bool tr = !symmetric && g.trow != nullptr;
    a.prow = tr ? g.trow : g.row;
    a.pcol = tr ? g.tcol : g.col;
    a.heavy = tr ? g.theavy : g.heavy;
    a.nheavy = tr ? g.ntheavy : g.nheavy;
    a.pieces = tr ? g.tpieces : g.pieces;
    a.npieces = tr ? g.ntpieces : g.npieces;
    a.hacc = w.hacc;
    a.hcnt = w.hcnt;
    a.vis = w.vis;
    for (int i = 0; i < 3; i++) a.F[i] = w.F[i];
    for (int i = 0; i < 4; i++) a.Q[i] = w.Q[i];
    a.out = d_out;
    a.lv8 = w.lv8;
    a.bigl = w.bigl;
    a.src = d_src;
    a.ctrl = w.ctrl;
    a.pull_allowed = pull_allowed ? 1 : 0;
    a.direction = p.direction;
    a.pull_div = 16;
    a.has_big = g.max_degree >= MS_BIG ? 1 : 0;
    a.timeout_ns = (unsigned long long)std::max(1, p.timeout_ms) * 1000000ull;
    static LaunchSetup setup;
    const size_t smem = ms_smem_bytes();
    int sms = 0, occ = 0;
    cudaError_t e = setup.get(sms, occ, [&](int dev, int &s_out, int &o_out) {
        cudaError_t r = cudaFuncSetAttribute(k_msbfs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (r == cudaSuccess) r = cudaDeviceGetAttribute(&s_out, cudaDevAttrMultiProcessorCount, dev);
        if (r == cudaSuccess) r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o_out, k_msbfs, MS_BLOCK, smem);
        return r;
    });
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const int per = std::max(1, std::min(occ, std::max(1, p.blocks_per_sm)));
    int grid = sms * per;
    if (max_ctas > 0) grid = std::max(1, std::min(grid, max_ctas));
    void *kargs[] = {&a};
    return cudaLaunchCooperativeKernel((const void *)k_msbfs, dim3(grid), dim3(MS_BLOCK), kargs, smem, st);
}

int ms_max_ctas()
{
    int dev = 0, sms = 0, occ = 0;
    const size_t smem = ms_smem_bytes();
    if (cudaFuncSetAttribute(k_msbfs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_msbfs, MS_BLOCK, smem) != cudaSuccess) return 0;
    return sms * occ;
}

int msbfs_run(const DeviceCsr &g, const gbfs_params &p, bool symmetric, MsWork &w, const int *d_src, int k,
              int *d_out, cudaStream_t st, MsResult &res, std::string &err)
{
    cudaError_t e = cudaEventRecord(w.ev0, st);
    if (e == cudaSuccess) e = msbfs_enqueue(g, p, symmetric, w, d_src, k, d_out, st, 0);
    if (e == cudaSuccess) e = cudaEventRecord(w.ev1, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.h_ctrl, w.ctrl, offsetof(MsCtrl, t_entry), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        err = std::string("multi-source BFS launch: ") + cudaGetErrorString(e);
        return GBFS_ERR_CUDA;
    }
    if (w.h_ctrl->status != DEV_OK) {
        cudaMemsetAsync(w.ctrl, 0, sizeof(MsCtrl), st);
        cudaStreamSynchronize(st);
        err = "a device-side wait ran out (grid barrier)";
        return GBFS_ERR_TIMEOUT;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, w.ev0, w.ev1);
    res.ms = ms;
    res.levels = w.h_ctrl->levels;
    res.push_levels = w.h_ctrl->push_levels;
    res.pull_levels = w.h_ctrl->pull_levels;
    res.reached = (int64_t)w.h_ctrl->reached;
    res.edges_c = (int64_t)w.h_ctrl->edges_c;
    return GBFS_OK;
}

}  // namespace gbfs
