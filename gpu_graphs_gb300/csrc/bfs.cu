// bfs.cu -- persistent direction-optimising BFS for one GB300 (sm_103a).
//
// Reference path replaced: the per-level host loop of gpuBFS::gpuBFS
// (1D Partition/src/gpuBFS.cu:66-100: memset, launch linear_bfs, sync,
// two D2H copies and NVSHMEM barriers per level) and its kernel linear_bfs
// (1D Partition/src/gpuBFS_kernels.cu:16-80: one thread per queue entry,
// serial adjacency loop, one global atomic per edge, no visited filter).
//
// Here one cooperative launch runs the whole traversal.  Levels are
// separated by a bounded grid barrier and every CTA takes the same
// direction decision from the same counters:
//   top-down step   frontier queue -> next queue.  Small frontiers: every
//                   edge balanced over the whole grid (degree prefix in
//                   shared memory).  Large ones: each warp takes 32
//                   frontier vertices and walks their rows (below
//                   big_degree) as one concatenated edge range; rows of
//                   degree >= big_degree are deferred to a grid-wide pass.
//                   A vertex is claimed with an atomicOr on the visited
//                   bitmap (after a plain-load filter), its level written
//                   once, and it is appended through a per-warp
//                   shared-memory queue (one global atomic per flush).
//   bottom-up step  every unvisited vertex looks for a parent in the
//                   frontier bitmap, stopping at the first hit.  The first
//                   probe reads the row's first entry from a compact array
//                   (coalesced, beside the row offsets); on hub-first rows
//                   four vertices per lane take it and the rows left over
//                   are walked from a per-warp stack, on other rows two per
//                   lane probe in place.
//   switching       Beamer's rule: top-down -> bottom-up when the frontier's
//                   out-edges exceed (unexplored edges)/alpha, back when the
//                   frontier has fewer than (non-isolated vertices)/beta
//                   vertices and is shrinking.  A top-down step likely to
//                   hand over marks its finds in the next frontier bitmap;
//                   a small frontier handed back to top-down is read from
//                   its bitmap directly; otherwise a queue <-> bitmap
//                   conversion phase runs at the switch.
// Bottom-up probes in-edges: the graph itself when symmetric, else its
// transpose (built on demand); without either, every level is top-down.
#include <algorithm>
#include <cstddef>
#include <cstring>

#include "bfs.cuh"
#include "bfs_args.cuh"
#include "blockq.cuh"

namespace gbfs {

namespace {

constexpr int SEG = 2048;    // frontier rows expanded edge-balanced per pass
constexpr int ILP = 4;       // edges in flight per lane in top-down passes
constexpr int PROBE = 8;     // neighbours probed per step in bottom-up
constexpr int COOP_ROWS = 4; // bottom-up rows left in a warp below which the warp walks them together
// Per warp, an int2 area of QCAP entries: in top-down steps the row bounds
// of the warp queue's entries, in bottom-up steps the deferred rows' bounds
// (under 64 left plus a 128-vertex round)
constexpr int BU_DEF = QCAP;
constexpr unsigned long long BMTD_EDGES = 65536;  // top-down from the bitmap up to this many frontier edges
// Long searches on graphs whose largest out-degree is at most
// RELAX_MAX_DEGREE (meshes, grids, road networks: thousands of levels of
// small frontiers): from level RELAX_YIELD_LEVEL on, at a top-down frontier
// of at most RELAX_ENTER_F vertices, the grid kernel parks its loop and the
// label-correcting kernel (bfs_relax.cu) queued behind it finishes the
// search, advancing pieces of the frontier many levels per grid-wide
// barrier.  Measured on the 7000 x 7000 grid (7,194 levels): 18.9 ms,
// against 78 ms level by level in the grid kernel.
constexpr int RELAX_MAX_DEGREE = 16;
constexpr int RELAX_YIELD_LEVEL = 4;
constexpr int RELAX_ENTER_F = 4500;

// A warp's staging queue whose entries carry their row bounds (row[v],
// row[v + 1]), so the next level reads a frontier vertex's edge range with
// the vertex instead of a dependent load of its row offsets.  The frontier
// queues have a bounds array beside them (qb[0] beside q0, qb[1] beside q1).
template <typename RT>
struct WarpQB {
    int *buf;
    BndT<RT> *bb;
    int n;
};

// Append the warp's staged entries to out / outb with one global atomic on
// the packed counter (its low 32 bits give the position).
template <typename RT>
__device__ __forceinline__ void wqb_flush(WarpQB<RT> &q, unsigned long long *cnt, int *out, BndT<RT> *outb)
{
    __syncwarp();
    if (q.n == 0) return;
    unsigned long long base = 0;
    if (lane_id() == 0) base = atomicAdd(cnt, (unsigned long long)q.n) & 0xffffffffull;
    base = __shfl_sync(FULL, base, 0);
    for (int i = lane_id(); i < q.n; i += 32) {
        out[base + i] = q.buf[i];
        outb[base + i] = q.bb[i];
    }
    __syncwarp();
    q.n = 0;
}

// All 32 lanes call; lanes with `has` stage v and its row bounds.
template <typename RT>
__device__ __forceinline__ void wqb_push(WarpQB<RT> &q, bool has, int v, BndT<RT> be, unsigned long long *cnt, int *out,
                                         BndT<RT> *outb)
{
    const unsigned m = __ballot_sync(FULL, has);
    if (!m) return;
    const int c = __popc(m);
    if (q.n + c > QCAP) wqb_flush(q, cnt, out, outb);
    if (has) {
        const int slot = q.n + __popc(m & lanemask_lt());
        q.buf[slot] = v;
        q.bb[slot] = be;
    }
    q.n += c;
}

// Flush every warp queue of the block with one global atomic on the packed
// count | degree counter, adding the block's `hi` values (its vertices'
// out-degrees) to the high half in the same atomic (all threads call).
template <typename RT>
__device__ __forceinline__ void block_flush_bounds(WarpQB<RT> &q, unsigned long long *cnt, int *out, BndT<RT> *outb,
                                                   unsigned long long hi, int *s_wq, unsigned long long *s_hi,
                                                   unsigned long long *s_base)
{
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned lane = lane_id();
    const unsigned long long wh = warp_sum(hi);
    __syncwarp();
    if (lane == 0) {
        s_wq[w] = q.n;
        s_hi[w] = wh;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int c = (int)lane < nw ? s_wq[lane] : 0;
        const unsigned long long h = (int)lane < nw ? s_hi[lane] : 0ull;
        const int incl = warp_incl_scan(c);
        const int tot = __shfl_sync(FULL, incl, 31);
        const unsigned long long htot = warp_sum(h);
        if ((int)lane < nw) s_wq[lane] = incl - c;
        if (lane == 0)
            *s_base = (tot || htot) ? (atomicAdd(cnt, cd_pack((unsigned long long)tot, htot)) & 0xffffffffull) : 0ull;
    }
    __syncthreads();
    const unsigned long long base = *s_base + (unsigned long long)s_wq[w];
    for (int i = lane; i < q.n; i += 32) {
        out[base + i] = q.buf[i];
        outb[base + i] = q.bb[i];
    }
    q.n = 0;
    __syncthreads();
}

// Top-down claim of ILP neighbours per lane, all loads and atomics issued
// before any result is used.  w[j] < 0 means "no edge".  After a plain-load
// filter on the visited bitmap, a candidate's atomicOr claim and the loads
// of its row bounds are issued together (the bounds of a candidate that
// loses are not used).  A vertex is won by the atomicOr that sets its
// visited bit; the winner writes its level, adds its out-degree to my_deg,
// appends itself and its bounds to the warp queue and, with fnw given,
// marks itself in the next frontier's bitmap too.
template <typename RT>
__device__ __forceinline__ void claim_batch(const int (&w)[ILP], const BfsArgs &a, int nl, WarpQB<RT> &q,
                                            unsigned long long *cnt, int *qn, BndT<RT> *qbn,
                                            unsigned long long &my_deg, unsigned *fnw)
{
    using Sel = RowSel<RT>;
    const RT *row = Sel::row(a);
    unsigned word[ILP];
#pragma unroll
    for (int j = 0; j < ILP; j++) word[j] = w[j] >= 0 ? a.visited[w[j] >> 5] : FULL;
    unsigned old[ILP];
    BndT<RT> be[ILP];
#pragma unroll
    for (int j = 0; j < ILP; j++) {
        const unsigned bit = 1u << (w[j] & 31);
        old[j] = FULL;
        be[j] = Sel::mk(0, 0);
        if (!(word[j] & bit)) {
            old[j] = atomicOr(&a.visited[w[j] >> 5], bit);
            be[j] = Sel::mk(__ldg(row + w[j]), __ldg(row + w[j] + 1));
        }
    }
    bool won[ILP];
#pragma unroll
    for (int j = 0; j < ILP; j++) {
        won[j] = !((old[j] >> (w[j] & 31)) & 1u);
        if (won[j]) {
            a.level[w[j]] = nl;
            my_deg += (unsigned long long)(be[j].y - be[j].x);
        }
    }
#pragma unroll
    for (int j = 0; j < ILP; j++) wqb_push(q, won[j], w[j], be[j], cnt, qn, qbn);
    if (fnw) {  // one branch, taken on whole levels or not at all
#pragma unroll
        for (int j = 0; j < ILP; j++)
            if (won[j]) atomicOr(&fnw[w[j] >> 5], 1u << (w[j] & 31));
    }
}

// Expand the rows of list[0, cnt) with the edges split evenly: each CTA
// builds the degree prefix of a SEG-row segment in shared memory and warp g
// of W takes edges [E*g/W, E*(g+1)/W) of it -- all warps of the grid when
// the list is one segment or `heavy` (every row long, so each segment holds
// enough edges for the whole grid: segments are walked one after another),
// the CTA's own warps on its own segments otherwise.  lb: the rows' bounds
// beside the list (a frontier queue), or null (then the row offsets are
// loaded).
template <int BLOCK, typename RT>
__device__ void grid_expand_list(const int *list, const BndT<RT> *lb, int cnt, const BfsArgs &a, int nl,
                                 WarpQB<RT> &q, unsigned long long *cnt_next, int *qn, BndT<RT> *qbn,
                                 unsigned long long &my_deg, int *s_pre, RT *s_beg, int *s_warp, unsigned *fnw,
                                 bool heavy = false)
{
    using Sel = RowSel<RT>;
    const RT *row = Sel::row(a);
    constexpr int PER = SEG / BLOCK;
    const int lane = (int)lane_id();
    // One segment (or long rows): the grid's warps split each segment's
    // edges.  Otherwise CTA b takes segments b, b+G, ... and its own warps
    // split each one.
    const bool one_seg = cnt <= SEG || heavy;
    const long long gwarp = one_seg ? ((long long)blockIdx.x * BLOCK + threadIdx.x) >> 5 : (long long)(threadIdx.x >> 5);
    const long long nwarps = one_seg ? ((long long)gridDim.x * BLOCK) >> 5 : (long long)(BLOCK / 32);
    const int seg0 = one_seg ? 0 : (int)blockIdx.x * SEG;
    const int seg_step = one_seg ? SEG : (int)gridDim.x * SEG;
    for (int seg = seg0; seg < cnt; seg += seg_step) {
        const int segn = min(SEG, cnt - seg);
        int d[PER];
        int sum = 0;
#pragma unroll
        for (int t = 0; t < PER; t++) {
            const int j = threadIdx.x * PER + t;
            d[t] = 0;
            if (j < segn) {
                BndT<RT> be;
                if (lb) {
                    be = __ldcg(lb + seg + j);
                } else {
                    const int v = __ldcg(list + seg + j);
                    be = Sel::mk(__ldg(row + v), __ldg(row + v + 1));
                }
                s_beg[j] = be.x;
                d[t] = (int)(be.y - be.x);
            }
            sum += d[t];
        }
        int total;
        int run = block_excl_scan_int(sum, s_warp, &total);
#pragma unroll
        for (int t = 0; t < PER; t++) {
            const int j = threadIdx.x * PER + t;
            if (j < segn) s_pre[j] = run;
            run += d[t];
        }
        __syncthreads();
        const long long lo = (long long)total * gwarp / nwarps;
        const long long hi = (long long)total * (gwarp + 1) / nwarps;
        for (long long base = lo; base < hi; base += 32 * ILP) {
            int w[ILP];
#pragma unroll
            for (int j = 0; j < ILP; j++) {
                const long long e = base + j * 32 + lane;
                w[j] = -1;
                if (e < hi) {
                    int l = 0, h = segn - 1;  // max r with s_pre[r] <= e
                    while (l < h) {
                        const int mid = (l + h + 1) >> 1;
                        if (s_pre[mid] <= e) l = mid; else h = mid - 1;
                    }
                    w[j] = __ldg(a.col + s_beg[l] + (int)(e - s_pre[l]));
                }
            }
            claim_batch(w, a, nl, q, cnt_next, qn, qbn, my_deg, fnw);
        }
        __syncthreads();
    }
}

// Bits of a bitmap word set through a tile of BLOCK words per CTA pass:
// appends the vertices whose bit is set in (want ? bits : ~bits & valid)
// to out, one global atomic per CTA tile.
template <int BLOCK, typename RT>
__device__ void bitmap_to_list(const unsigned *bm, bool complement, int n, int W, int *out, BndT<RT> *outb,
                               const RT *row, unsigned long long *cnt, int *s_warp, unsigned long long *s_base)
{
    for (long long t0 = (long long)blockIdx.x * BLOCK; t0 < W; t0 += (long long)gridDim.x * BLOCK) {
        const long long w = t0 + threadIdx.x;
        unsigned bits = 0;
        if (w < W) {
            bits = __ldcg(bm + w);
            if (complement) {
                const unsigned valid = (w == W - 1 && (n & 31)) ? ((1u << (n & 31)) - 1u) : FULL;
                bits = ~bits & valid;
            }
        }
        int total;
        const int off = block_excl_scan_int(__popc(bits), s_warp, &total);
        if (threadIdx.x == 0) *s_base = total ? atomicAdd(cnt, (unsigned long long)total) : 0ull;
        __syncthreads();
        unsigned long long pos = *s_base + (unsigned long long)off;
        while (bits) {
            const int b = __ffs(bits) - 1;
            const int v = (int)(w * 32 + b);
            out[pos] = v;
            outb[pos] = RowSel<RT>::mk(__ldg(row + v), __ldg(row + v + 1));
            ++pos;
            bits &= bits - 1u;
        }
        __syncthreads();
    }
}

// Top-down expansion of one row per lane (d = 0: none) as one concatenated
// edge range over the warp, ILP edges per lane in flight; rows of
// big_degree or more go to bigl (counted in *bigcnt) for a grid-wide pass.
template <typename RT>
__device__ __forceinline__ void expand_lane_rows(int v, RT b, int d, const BfsArgs &a, int nl, WarpQB<RT> &q,
                                                 unsigned long long *cnt, int *qn, BndT<RT> *qbn,
                                                 unsigned long long &my_deg, unsigned *bigcnt, unsigned lane,
                                                 unsigned *fnw)
{
    const bool isbig = d >= a.big_degree;
    const unsigned bm = __ballot_sync(FULL, isbig);
    if (bm) {
        unsigned pos = 0;
        const int leader = __ffs(bm) - 1;
        if ((int)lane == leader) pos = atomicAdd(bigcnt, (unsigned)__popc(bm));
        pos = __shfl_sync(FULL, pos, leader);
        if (isbig) a.bigl[pos + __popc(bm & lanemask_lt())] = v;
        if (isbig) d = 0;
    }
    const int incl = warp_incl_scan(d);
    const int excl = incl - d;
    const int T = __shfl_sync(FULL, incl, 31);
    for (int e0 = 0; e0 < T; e0 += 32 * ILP) {
        int w[ILP];
#pragma unroll
        for (int j = 0; j < ILP; j++) {
            const int k = e0 + j * 32 + (int)lane;
            const int kk = min(k, T - 1);
            int lo = 0;
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) {
                const int c = lo + s;
                if (__shfl_sync(FULL, excl, c) <= kk) lo = c;
            }
            const RT ob = __shfl_sync(FULL, b, lo);
            const int oe = __shfl_sync(FULL, excl, lo);
            w[j] = k < T ? __ldg(a.col + ob + (kk - oe)) : -1;
        }
        claim_batch(w, a, nl, q, cnt, qn, qbn, my_deg, fnw);
    }
}

// Top-down step over a frontier given as a bitmap (few edges, right after
// bottom-up steps), with no bitmap -> queue pass: a warp takes cw words at a
// time, deals their frontier vertices one per lane, and expands those rows
// with expand_lane_rows.  cw aims a chunk at about 32 frontier vertices.
template <typename RT>
__device__ __forceinline__ void bitmap_expand(const unsigned *fb, int W, long long nf, const BfsArgs &a, int nl,
                                              WarpQB<RT> &q, unsigned long long *cnt, int *qn, BndT<RT> *qbn,
                                              unsigned long long &my_deg, unsigned *bigcnt, long long gwarp,
                                              long long nwarps, unsigned lane, unsigned *fnw)
{
    const int cw = (int)min(32LL, max(1LL, (32LL * W) / max(1LL, nf)));
    for (long long w0 = gwarp * cw; w0 < W; w0 += nwarps * cw) {
        const long long wl = w0 + lane;
        const unsigned bits = ((int)lane < cw && wl < W) ? __ldcg(fb + wl) : 0u;
        const int c = __popc(bits);
        const int incl = warp_incl_scan(c);
        const int excl = incl - c;
        const int U = __shfl_sync(FULL, incl, 31);
        for (int r0 = 0; r0 < U; r0 += 32) {
            const int slot = r0 + (int)lane;
            const int jj = min(slot, U - 1);
            int owner = 0;
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) {
                const int cand = owner + s;
                if (__shfl_sync(FULL, excl, cand) <= jj) owner = cand;
            }
            unsigned um = __shfl_sync(FULL, bits, owner);
            int k = jj - __shfl_sync(FULL, excl, owner);
            int pos = 0;  // position of the k-th set bit of um
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) {
                const int lowc = __popc(um & ((1u << s) - 1u));
                if (k >= lowc) {
                    k -= lowc;
                    um >>= s;
                    pos += s;
                }
            }
            int v = 0, d = 0;
            RT b = 0;
            if (slot < U) {
                const RT *row = RowSel<RT>::row(a);
                v = (int)((w0 + owner) * 32 + pos);
                b = __ldg(row + v);
                d = (int)(__ldg(row + v + 1) - b);
            }
            expand_lane_rows(v, b, d, a, nl, q, cnt, qn, qbn, my_deg, bigcnt, lane, fnw);
        }
    }
}

// Bottom-up probing of up to two rows per lane (a: [ia, ea), b: [ib, eb)),
// PROBE entries per lane and step, until each row finds a parent in the
// frontier bitmap fc (fa / fb) or runs out.  When at most COOP_ROWS rows
// with more than 2 * PROBE entries left remain in the warp, the warp walks
// those together, 32 entries a step, instead of leaving most lanes idle.
// All 32 lanes call it.
template <typename RT>
__device__ __forceinline__ void probe_rows(RT &ia, RT ea, bool &fa, RT &ib, RT eb, bool &fb, const int *bcol,
                                           const unsigned *fc, unsigned lane)
{
    for (;;) {
        const bool aa = ia < ea && !fa, ab = ib < eb && !fb;
        const unsigned ma = __ballot_sync(FULL, aa), mb = __ballot_sync(FULL, ab);
        if (!(ma | mb)) return;
        if (__popc(ma) + __popc(mb) <= COOP_ROWS) {
            int rem = (int)max(aa ? ea - ia : (RT)0, ab ? eb - ib : (RT)0);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) rem = max(rem, __shfl_xor_sync(FULL, rem, o));
            if (rem > 2 * PROBE) {
                unsigned ta = ma, tb = mb;
                while (ta | tb) {
                    const bool isb = ta == 0;
                    const int sl = __ffs(isb ? tb : ta) - 1;
                    if (isb) tb &= tb - 1; else ta &= ta - 1;
                    const RT ri = __shfl_sync(FULL, isb ? ib : ia, sl);
                    const RT re = __shfl_sync(FULL, isb ? eb : ea, sl);
                    bool found = false;
                    for (RT i0 = ri; i0 < re && !found; i0 += 32) {
                        const RT i = i0 + (RT)lane;
                        unsigned hit = 0;
                        if (i < re) {
                            const int u = __ldg(bcol + i);
                            hit = (__ldcg(fc + (u >> 5)) >> (u & 31)) & 1u;
                        }
                        found = __any_sync(FULL, hit != 0);
                    }
                    if ((int)lane == sl) {
                        if (isb) { fb = found; ib = eb; }
                        else { fa = found; ia = ea; }
                    }
                }
                return;
            }
        }
        int ua[PROBE], ub[PROBE];
#pragma unroll
        for (int t = 0; t < PROBE; t++) {
            ua[t] = (aa && ia + t < ea) ? __ldg(bcol + ia + t) : -1;
            ub[t] = (ab && ib + t < eb) ? __ldg(bcol + ib + t) : -1;
        }
        unsigned ga = 0, gb = 0;
#pragma unroll
        for (int t = 0; t < PROBE; t++) {
            if (ua[t] >= 0) ga |= __ldcg(fc + (ua[t] >> 5)) >> (ua[t] & 31);
            if (ub[t] >= 0) gb |= __ldcg(fc + (ub[t] >> 5)) >> (ub[t] & 31);
        }
        if (aa) { if (ga & 1u) fa = true; else ia += PROBE; }
        if (ab) { if (gb & 1u) fb = true; else ib += PROBE; }
    }
}

// MINB (CTAs per SM the register budget is sized for) only shapes register
// allocation; the launch decides the actual grid.
template <int BLOCK, int MINB, typename RT>
__global__ void __launch_bounds__(BLOCK, MINB) k_bfs(BfsArgs a)
{
    using Sel = RowSel<RT>;
    using B = BndT<RT>;
    const RT *const row = Sel::row(a);
    const RT *const brow = Sel::brow(a);
    extern __shared__ __align__(16) int smem[];
    __shared__ unsigned long long s_red[32];
    __shared__ unsigned long long s_base;
    __shared__ unsigned long long s_cd;
    __shared__ unsigned s_nb;
    __shared__ int s_warp[33];
    __shared__ int s_wq[33];
    constexpr int NW = BLOCK / 32;
    int *s_q = smem;                           // NW * QCAP warp queues
    int *s_pre = s_q + NW * QCAP;              // SEG degree prefix
    RT *s_beg = (RT *)(s_pre + SEG);           // SEG row begins
    B *s_def = (B *)(s_beg + SEG);             // NW * BU_DEF: queue row bounds (top-down), deferred rows (bottom-up)

    const int n = a.n;
    const int W = (n + 31) >> 5;
    const unsigned lane = lane_id();
    const long long gtid = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const long long gthreads = (long long)gridDim.x * BLOCK;
    const long long gwarp = gtid >> 5;
    const long long nwarps = gthreads >> 5;
    BfsCtrl *ctrl = a.ctrl;
    WarpQB<RT> q{s_q + (threadIdx.x >> 5) * QCAP, s_def + (threadIdx.x >> 5) * BU_DEF, 0};
    unsigned epoch = 0;
    if (a.resume) {
        // a continuation: nothing to do when the search has ended or failed,
        // or when it was handed to the label-correcting kernel
        const int done = ctrl->rs.done, mode = ctrl->rs.mode, status = ctrl->status;
        if (done || mode == RESUME_RELAX || status != DEV_OK) return;
    } else if (gtid == 0) {
        ctrl->t_entry = globaltimer_ns();
    }

    // ---- init ----------------------------------------------------------
    if (!a.resume) {
        const int root = a.single_root;
        if (((uintptr_t)a.level & 15) == 0) {
            int4 *l4 = (int4 *)a.level;
            const long long n4 = n >> 2;
            for (long long i = gtid; i < n4; i += gthreads) l4[i] = make_int4(-1, -1, -1, -1);
            for (long long i = (n4 << 2) + gtid; i < n; i += gthreads) a.level[i] = -1;
        } else {
            for (long long i = gtid; i < n; i += gthreads) a.level[i] = -1;
        }
        for (long long w = gtid; w < W; w += gthreads) {
            unsigned z = a.zmask ? a.zmask[w] : 0u;
            if (root >= 0 && w == (root >> 5)) z |= 1u << (root & 31);
            a.visited[w] = z;
            a.fb[0][w] = 0;
            a.fb[1][w] = 0;
            a.fb[2][w] = 0;
        }
        if (root >= 0 && gtid == 0) {
            a.q0[0] = root;
            Sel::qb(a, 0)[0] = Sel::mk(__ldg(row + root), __ldg(row + root + 1));
            ctrl->cd[0] = cd_pack(1, (unsigned long long)(__ldg(row + root + 1) - __ldg(row + root)));
        }
        if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
        if (root >= 0) {
            if (gtid == 0) a.level[root] = 0;
        } else {
            if (blockIdx.x == 0) {
                for (int i = threadIdx.x; i < a.nroots; i += BLOCK) {
                    const int r = a.roots[i];
                    if (atomicCAS(&a.level[r], -1, 0) == -1) {
                        atomicOr(&a.visited[r >> 5], 1u << (r & 31));
                        const B be = Sel::mk(__ldg(row + r), __ldg(row + r + 1));
                        const unsigned long long pos =
                            cd_count(atomicAdd(&ctrl->cd[0], cd_pack(1, (unsigned long long)(be.y - be.x))));
                        a.q0[pos] = r;
                        Sel::qb(a, 0)[pos] = be;
                    }
                }
            }
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
        }
    }
    if (gtid == 0 && !a.resume) ctrl->t_start = globaltimer_ns();

    // ---- level loop ------------------------------------------------------
    // Frontier L lives in queue q[L&1] after a top-down step and in bitmap
    // fb[L%3] after a bottom-up step; switches convert.
    long long m_u = a.m;                 // out-edges of not-yet-reached vertices
    unsigned long long prev_nf = 0, reached = 0, edges_c = 0, roots = 0;
    int L = 0, td_levels = 0, bu_levels = 0;
    bool td = true;
    bool fn_set = false;  // the last top-down step marked its finds in fn
    unsigned long long prev_mf = 0;  // the last level's frontier edges
    // Frontier bitmaps that may hold set bits (bit i: fb[i]); a bitmap is
    // cleared two levels before it is next written only if it is dirty, so
    // levels that never touch the bitmaps (top-down steps without marking)
    // write none of them.  All three are zero after initialisation.
    unsigned dirty = 0;
    if (a.resume) {
        const BfsResume r = ctrl->rs;
        m_u = r.m_u;
        prev_nf = r.prev_nf;
        reached = r.reached;
        edges_c = r.edges_c;
        roots = r.roots;
        L = r.L;
        td_levels = r.td_levels;
        bu_levels = r.bu_levels;
        td = r.td != 0;
        dirty = (unsigned)r.dirty;
        prev_mf = r.prev_mf;
    }
    // park the loop state at the top of level L for the launch that
    // continues it (mode: ResumeMode)
    auto park = [&](int mode) {
        if (gtid == 0) {
            BfsResume r;
            r.m_u = m_u;
            r.prev_nf = prev_nf;
            r.reached = reached;
            r.edges_c = edges_c;
            r.roots = roots;
            r.prev_mf = prev_mf;
            r.L = L;
            r.td_levels = td_levels;
            r.bu_levels = bu_levels;
            r.td = td ? 1 : 0;
            r.done = 0;
            r.dirty = (int)dirty;
            r.mode = mode;
            r.pad = 0;
            ctrl->rs = r;
        }
        grid_exit(&ctrl->bar, &ctrl->t_exit);
    };
    for (int steps = 0;; ++steps) {
        if (a.max_steps > 0 && steps == a.max_steps) {
            // per-level-launch mode: park the loop state for the next launch
            park(RESUME_LEVEL);
            return;
        }
        // the frontier's count and degree sum: one load per CTA, shared
        if (threadIdx.x == 0) s_cd = ld_relaxed_u64(&ctrl->cd[L % 3]);
        __syncthreads();
        const unsigned long long cdv = s_cd;
        const unsigned long long nf = cd_count(cdv);
        const unsigned long long mf = cd_degree(cdv);
        if (nf == 0) break;
        if (L == 0) roots = nf;
        reached += nf;
        edges_c += mf;
        m_u -= (long long)mf;
        bool bu;
        if (a.direction == GBFS_DIR_TOPDOWN || brow == nullptr) bu = false;
        else if (a.direction == GBFS_DIR_BOTTOMUP) bu = true;
        else if (td) bu = (long long)mf * a.alpha > m_u;
        else bu = !((long long)nf * a.beta < a.n_active && nf < prev_nf);
        // a long search of small top-down frontiers (a high-diameter
        // graph): hand the loop to the label-correcting kernel queued after
        // this launch, with frontier L still in its queue
        if (a.may_yield && td && !bu && L >= a.yield_level && nf <= (unsigned long long)a.yield_max_f) {
            reached -= nf;
            edges_c -= mf;
            m_u += (long long)mf;
            park(RESUME_RELAX);
            return;
        }
        prev_nf = nf;

        int *qc = (L & 1) ? a.q1 : a.q0;
        int *qn = (L & 1) ? a.q0 : a.q1;
        const B *qbc = Sel::qb(a, L & 1);   // row bounds beside qc
        B *qbn = Sel::qb(a, (L + 1) & 1);   // and beside qn
        unsigned *fc = a.fb[L % 3];
        unsigned *fn = a.fb[(L + 1) % 3];
        unsigned *fz = a.fb[(L + 2) % 3];   // zeroed now: the next level's fn
        unsigned long long *cnt_next = &ctrl->cd[(L + 1) % 3];  // count | degree sum of frontier L+1
        const int nl = L + 1;
        const unsigned bit_c = 1u << (L % 3), bit_n = 1u << ((L + 1) % 3), bit_z = 1u << ((L + 2) % 3);

        bool traced_big = false;
        if (gtid == 0) {
            ctrl->cd[(L + 2) % 3] = 0;
            ctrl->big[(L + 1) % 3] = 0;
        }

        if (bu && td && !fn_set) {
            // queue -> bitmap (fc is zero: fb[L%3] was cleared two levels
            // ago and top-down steps that did not mark it do not write it)
            for (long long i = gtid; i < (long long)nf; i += gthreads) {
                const int v = __ldcg(qc + i);
                atomicOr(&fc[v >> 5], 1u << (v & 31));
            }
            dirty |= bit_c;
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
        }
        // back to top-down with few frontier edges: expand the frontier
        // straight from its bitmap (no bitmap -> queue pass and barrier)
        const bool from_bitmap = !bu && !td && mf <= BMTD_EDGES;
        if (!bu && !td && !from_bitmap) {
            // bitmap -> queue
            bitmap_to_list<BLOCK, RT>(fc, false, n, W, qc, Sel::qb(a, L & 1), row, &ctrl->fill, s_warp, &s_base);
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
        }
        td = !bu;

        if (dirty & bit_z) {
            for (long long w = gtid; w < W; w += gthreads) fz[w] = 0;
            dirty &= ~bit_z;
        }
        if (td) {
            ++td_levels;
            if (gtid == 0) ctrl->fill = 0;
            unsigned long long my_deg = 0;
            // direction-optimising, with the next level likely bottom-up
            // (this frontier's edges times their growth from the last level
            // past the switching rule): also mark the next frontier in its
            // bitmap, so the switch needs no queue -> bitmap pass
            const float growth = fmaxf(1.f, (float)mf / (float)(prev_mf ? prev_mf : 1ull));
            const bool likely_bu = (float)mf * growth * (float)a.alpha > (float)m_u;
            unsigned *fnw = a.direction == GBFS_DIR_OPTIMIZING && brow && likely_bu ? fn : nullptr;
            if (from_bitmap) {
                bitmap_expand(fc, W, (long long)nf, a, nl, q, cnt_next, qn, qbn, my_deg, &ctrl->big[L % 3], gwarp, nwarps,
                              lane, fnw);
            } else if (nf <= (unsigned long long)SEG) {
                // small frontier: every edge of it balanced over the whole grid
                grid_expand_list<BLOCK, RT>(qc, qbc, (int)nf, a, nl, q, cnt_next, qn, qbn, my_deg, s_pre, s_beg,
                                            s_warp, fnw);
            } else {
                // large frontier: 32 rows per warp as one concatenated edge
                // range, rows of degree >= big_degree deferred to a grid pass
                for (long long base = gwarp * 32; base < (long long)nf; base += nwarps * 32) {
                    const long long i = base + lane;
                    int v = 0, d = 0;
                    RT b = 0;
                    if (i < (long long)nf) {
                        v = __ldcg(qc + i);
                        const B be = __ldcg(qbc + i);
                        b = be.x;
                        d = (int)(be.y - be.x);
                    }
                    expand_lane_rows(v, b, d, a, nl, q, cnt_next, qn, qbn, my_deg, &ctrl->big[L % 3], lane, fnw);
                }
            }
            block_flush_bounds(q, cnt_next, qn, qbn, my_deg, s_wq, s_red, &s_base);
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;

            // rows deferred to the grid pass (only large frontiers defer, and
            // only when some row is that long)
            int nb = 0;
            if (a.has_big && (nf > (unsigned long long)SEG || from_bitmap)) {
                if (threadIdx.x == 0) s_nb = __ldcg(&ctrl->big[L % 3]);
                __syncthreads();
                nb = (int)s_nb;
            }
            traced_big = nb > 0;
            if (nb > 0) {
                my_deg = 0;
                grid_expand_list<BLOCK, RT>(a.bigl, (const B *)nullptr, nb, a, nl, q, cnt_next, qn, qbn, my_deg, s_pre,
                                            s_beg, s_warp, fnw, true);
                block_flush_bounds(q, cnt_next, qn, qbn, my_deg, s_wq, s_red, &s_base);
                if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
            }
            fn_set = fnw != nullptr;
            if (fn_set) dirty |= bit_n;
        } else {
            fn_set = false;
            dirty |= bit_n;
            ++bu_levels;
            unsigned long long my_cnt = 0, my_deg = 0;
            // A warp takes chunks of cw bitmap words and probes the chunk's
            // unvisited vertices (the two branches below).  cw aims a chunk
            // at about 120 unvisited vertices when that still gives every
            // warp two chunks, else at about 56 (small graphs and dense
            // levels keep every warp busy), up to 32 words on sparse levels.
            long long unv_est = (long long)a.n_active - (long long)reached;
            if (unv_est < 1) unv_est = 1;
            long long cwl = (120LL * n) / (32LL * unv_est);
            if (cwl < 1 || (long long)W < 2 * nwarps * cwl) cwl = (56LL * n) / (32LL * unv_est);
            const int cw = (int)min(32LL, max(1LL, cwl));
            unsigned *my_found = (unsigned *)(s_beg) + (threadIdx.x >> 5) * 32;  // s_beg is free here
            int *def_v = q.buf;  // the warp's queue is idle in bottom-up steps
            B *def_b = s_def + (threadIdx.x >> 5) * BU_DEF;
            my_found[lane] = 0;
            __syncwarp();
            if (a.bsecond == nullptr) {
                // Hub-first rows (other rows probe in place, below).  Phase A,
                // 128 vertices a round (four per lane): each row's first
                // entry, its highest-degree neighbour, from the compact
                // first-entry array, read coalesced with the row offsets;
                // most vertices settle here.
                // Rows left with entries to probe go on the warp's deferred
                // stack (shared memory); phase B walks them 64 at a time, two
                // per lane, PROBE entries per step.  The stack empties after
                // the warp's last chunk is done; it carries over chunks, so its
                // finds and the chunk's own go to fn / visited by atomicOr
                // (the words are this warp's alone in this step).
                constexpr int skip = 1;  // entries the first probe covers
                int dn = 0;  // deferred rows on the stack
                auto phase_b = [&](int cntb) {
                    const int base = dn - cntb;
                    const int ka = base + (int)lane, kb = base + 32 + (int)lane;
                    int va = -1, vb = -1;
                    RT ia = 0, ea = 0, ib = 0, eb = 0;
                    if (ka < dn) { va = def_v[ka]; ia = def_b[ka].x; ea = def_b[ka].y; }
                    if (kb < dn) { vb = def_v[kb]; ib = def_b[kb].x; eb = def_b[kb].y; }
                    const int da = (int)(ea - ia) + skip, db = (int)(eb - ib) + skip;
                    bool fa = false, fb = false;
                    probe_rows(ia, ea, fa, ib, eb, fb, a.bcol, fc, lane);
                    if (fa) {
                        a.level[va] = nl;
                        atomicOr(fn + (va >> 5), 1u << (va & 31));
                        atomicOr(a.visited + (va >> 5), 1u << (va & 31));
                        ++my_cnt;
                        my_deg += (unsigned long long)(brow == row ? (RT)da : __ldg(row + va + 1) - __ldg(row + va));
                    }
                    if (fb) {
                        a.level[vb] = nl;
                        atomicOr(fn + (vb >> 5), 1u << (vb & 31));
                        atomicOr(a.visited + (vb >> 5), 1u << (vb & 31));
                        ++my_cnt;
                        my_deg += (unsigned long long)(brow == row ? (RT)db : __ldg(row + vb + 1) - __ldg(row + vb));
                    }
                    __syncwarp();
                    dn = base;
                };
                for (long long w0 = gwarp * cw; w0 < W; w0 += nwarps * cw) {
                    const long long wl = w0 + lane;
                    unsigned vis = FULL, valid = 0;
                    if ((int)lane < cw && wl < W) {
                        vis = __ldcg(a.visited + wl);
                        valid = (wl == W - 1 && (n & 31)) ? ((1u << (n & 31)) - 1u) : FULL;
                    }
                    const unsigned unv = ~vis & valid;
                    const int c = __popc(unv);
                    const int incl = warp_incl_scan(c);
                    const int excl = incl - c;
                    const int U = __shfl_sync(FULL, incl, 31);
                    for (int r0 = 0; r0 < U; r0 += 128) {
                        int vv[4];
                        const int hn = U - r0 > 64 ? 4 : 2;  // a round's upper half only when it has vertices
#pragma unroll
                        for (int h = 0; h < 4; h++) {
                            vv[h] = -1;
                            if (h >= hn) continue;
                            const int slot = r0 + (int)lane + 32 * h;
                            const int jj = min(slot, U - 1);
                            int owner = 0;
#pragma unroll
                            for (int s = 16; s > 0; s >>= 1) {
                                const int cand = owner + s;
                                if (__shfl_sync(FULL, excl, cand) <= jj) owner = cand;
                            }
                            unsigned um = __shfl_sync(FULL, unv, owner);
                            int k = jj - __shfl_sync(FULL, excl, owner);
                            int pos = 0;  // position of the k-th set bit of um
#pragma unroll
                            for (int s = 16; s > 0; s >>= 1) {
                                const int lowc = __popc(um & ((1u << s) - 1u));
                                if (k >= lowc) {
                                    k -= lowc;
                                    um >>= s;
                                    pos += s;
                                }
                            }
                            vv[h] = slot < U ? (int)((w0 + owner) * 32 + pos) : -1;
                        }
                        int pf[4];
                        RT rb[4], re[4];
#pragma unroll
                        for (int h = 0; h < 4; h++) {
                            pf[h] = -1;
                            rb[h] = re[h] = 0;
                            if (vv[h] >= 0) {
                                pf[h] = __ldg(a.bfirst + vv[h]);
                                rb[h] = __ldg(brow + vv[h]);
                                re[h] = __ldg(brow + vv[h] + 1);
                            }
                        }
                        unsigned hit[4];
#pragma unroll
                        for (int h = 0; h < 4; h++) {
                            hit[h] = 0;
                            if (pf[h] >= 0) hit[h] |= __ldcg(fc + (pf[h] >> 5)) >> (pf[h] & 31);
                        }
#pragma unroll
                        for (int h = 0; h < 4; h++) {
                            const int v = vv[h];
                            const bool f = hit[h] & 1u;
                            if (f) {
                                a.level[v] = nl;
                                atomicOr(&my_found[(v >> 5) - w0], 1u << (v & 31));
                                ++my_cnt;
                                my_deg += (unsigned long long)(brow == row ? re[h] - rb[h]
                                                                           : __ldg(row + v + 1) - __ldg(row + v));
                            }
                            const bool defer = v >= 0 && !f && rb[h] + skip < re[h];
                            const unsigned dm = __ballot_sync(FULL, defer);
                            if (defer) {
                                const int slotd = dn + __popc(dm & lanemask_lt());
                                def_v[slotd] = v;
                                def_b[slotd] = Sel::mk(rb[h] + skip, re[h]);
                            }
                            dn += __popc(dm);
                        }
                        __syncwarp();
                        while (dn >= 64) phase_b(64);
                    }
                    __syncwarp();
                    if ((int)lane < cw && wl < W) {
                        const unsigned fw = my_found[lane];
                        if (fw) {
                            atomicOr(fn + wl, fw);
                            atomicOr(a.visited + wl, fw);
                        }
                        my_found[lane] = 0;
                    }
                    __syncwarp();
                }
                while (dn > 0) phase_b(min(64, dn));
            } else {
                // Rows that are not hub-first: two vertices per lane (64 per
                // round), each probed in place until it settles; the warp
                // owns the chunk's words, so fn / visited words are written
                // without atomics.
                for (long long w0 = gwarp * cw; w0 < W; w0 += nwarps * cw) {
                    const long long wl = w0 + lane;
                    unsigned vis = FULL, valid = 0;
                    if ((int)lane < cw && wl < W) {
                        vis = __ldcg(a.visited + wl);
                        valid = (wl == W - 1 && (n & 31)) ? ((1u << (n & 31)) - 1u) : FULL;
                    }
                    const unsigned unv = ~vis & valid;
                    const int c = __popc(unv);
                    const int incl = warp_incl_scan(c);
                    const int excl = incl - c;
                    const int U = __shfl_sync(FULL, incl, 31);
                    for (int r0 = 0; r0 < U; r0 += 64) {
                        int vv[2];
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            const int slot = r0 + (int)lane + 32 * h;
                            const int jj = min(slot, U - 1);
                            int owner = 0;
#pragma unroll
                            for (int s = 16; s > 0; s >>= 1) {
                                const int cand = owner + s;
                                if (__shfl_sync(FULL, excl, cand) <= jj) owner = cand;
                            }
                            unsigned um = __shfl_sync(FULL, unv, owner);
                            int k = jj - __shfl_sync(FULL, excl, owner);
                            int pos = 0;  // position of the k-th set bit of um
#pragma unroll
                            for (int s = 16; s > 0; s >>= 1) {
                                const int lowc = __popc(um & ((1u << s) - 1u));
                                if (k >= lowc) {
                                    k -= lowc;
                                    um >>= s;
                                    pos += s;
                                }
                            }
                            vv[h] = slot < U ? (int)((w0 + owner) * 32 + pos) : -1;
                        }
                        const int va = vv[0], vb = vv[1];
                        const bool two = a.bsecond != nullptr;
                        RT ia = 0, ea = 0, ib = 0, eb = 0;
                        int pa = -1, pb = -1, qa = -1, qb = -1;
                        if (va >= 0) {
                            pa = __ldg(a.bfirst + va);
                            if (two) qa = __ldg(a.bsecond + va);
                            ia = __ldg(brow + va);
                            ea = __ldg(brow + va + 1);
                        }
                        if (vb >= 0) {
                            pb = __ldg(a.bfirst + vb);
                            if (two) qb = __ldg(a.bsecond + vb);
                            ib = __ldg(brow + vb);
                            eb = __ldg(brow + vb + 1);
                        }
                        const int da = (int)(ea - ia), db = (int)(eb - ib);
                        // First step: each row's first entry (hub-first rows: the
                        // highest-degree neighbour, where most vertices find their
                        // parent), with its second on other rows, from the compact
                        // first-entry arrays, read coalesced with the row offsets
                        // instead of one col_idx sector per row.  Later steps walk
                        // the rest of the row, PROBE wide.
                        unsigned ha = 0, hb = 0;  // the entries' bits loaded at once
                        if (pa >= 0) ha |= __ldcg(fc + (pa >> 5)) >> (pa & 31);
                        if (qa >= 0) ha |= __ldcg(fc + (qa >> 5)) >> (qa & 31);
                        if (pb >= 0) hb |= __ldcg(fc + (pb >> 5)) >> (pb & 31);
                        if (qb >= 0) hb |= __ldcg(fc + (qb >> 5)) >> (qb & 31);
                        bool fa = ha & 1u, fb = hb & 1u;
                        ia += two ? 2 : 1;
                        ib += two ? 2 : 1;
                        probe_rows(ia, ea, fa, ib, eb, fb, a.bcol, fc, lane);
                        // the next frontier's out-edges (for the direction rule): the
                        // probed in-degree when in-edges are the out-edges
                        if (fa) {
                            a.level[va] = nl;
                            atomicOr(&my_found[(va >> 5) - w0], 1u << (va & 31));
                            ++my_cnt;
                            my_deg += (unsigned long long)(brow == row ? (RT)da : __ldg(row + va + 1) - __ldg(row + va));
                        }
                        if (fb) {
                            a.level[vb] = nl;
                            atomicOr(&my_found[(vb >> 5) - w0], 1u << (vb & 31));
                            ++my_cnt;
                            my_deg += (unsigned long long)(brow == row ? (RT)db : __ldg(row + vb + 1) - __ldg(row + vb));
                        }
                    }
                    __syncwarp();
                    if ((int)lane < cw && wl < W) {
                        const unsigned fw = my_found[lane];
                        fn[wl] = fw;
                        if (fw) a.visited[wl] = vis | fw;
                        my_found[lane] = 0;
                    }
                    __syncwarp();
                }
            }
            // both sums below 2^32 per block, so they add packed
            const unsigned long long bcd = block_reduce_sum(cd_pack(my_cnt, my_deg), s_red);
            if (threadIdx.x == 0 && bcd) atomicAdd(cnt_next, bcd);
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
        }
        prev_mf = mf;
        if (gtid == 0) {
            LevelTrace t;
            t.level = L;
            t.dir = (td ? 0 : 1) + (td && traced_big ? 2 : 0);
            t.frontier = nf;
            t.edges = mf;
            t.t_ns = globaltimer_ns();
            ctrl->trace[L < TRACE_CAP - 1 ? L : TRACE_CAP - 1] = t;
        }
        ++L;
    }

    if (gtid == 0) {
        ctrl->t_end = globaltimer_ns();
        ctrl->trace_len = L < TRACE_CAP ? L : TRACE_CAP;
        BfsOut o;
        o.levels = L;
        o.td_levels = td_levels;
        o.bu_levels = bu_levels;
        o.roots = (int)roots;
        o.reached = reached;
        o.edges_c = edges_c;
        *a.out = o;
        ctrl->rs.done = 1;
        ctrl->rs.mode = RESUME_LEVEL;
        for (int i = 0; i < 3; i++) {
            ctrl->cd[i] = 0;
            ctrl->big[i] = 0;
        }
        ctrl->fill = 0;
    }
    grid_exit(&ctrl->bar, &ctrl->t_exit);
}

template <int BLOCK, typename RT = int>
size_t bfs_smem_bytes()
{
    return sizeof(int) * ((size_t)(BLOCK / 32) * QCAP + (size_t)SEG) + sizeof(RT) * (size_t)SEG +
           sizeof(BndT<RT>) * (size_t)(BLOCK / 32) * BU_DEF;
}

template <int BLOCK, int MINB, typename RT = int>
cudaError_t bfs_launch(BfsArgs &args, int blocks_per_sm, cudaStream_t st, int max_ctas)
{
    static LaunchSetup setup;  // per template instance
    const size_t smem = bfs_smem_bytes<BLOCK, RT>();
    int sms = 0, occ = 0;
    cudaError_t e = setup.get(sms, occ, [&](int dev, int &s_out, int &o_out) {
        cudaError_t r =
            cudaFuncSetAttribute(k_bfs<BLOCK, MINB, RT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (r == cudaSuccess) r = cudaDeviceGetAttribute(&s_out, cudaDevAttrMultiProcessorCount, dev);
        if (r == cudaSuccess)
            r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o_out, k_bfs<BLOCK, MINB, RT>, BLOCK, smem);
        return r;
    });
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const int per = std::max(1, std::min(blocks_per_sm, occ));
    int grid = sms * per;
    if (max_ctas > 0) grid = std::max(1, std::min(grid, max_ctas));
    void *kargs[] = {&args};
    return cudaLaunchCooperativeKernel((const void *)k_bfs<BLOCK, MINB, RT>, dim3(grid), dim3(BLOCK), kargs, smem,
                                       st);
}

cudaError_t bfs_launch_any(BfsArgs &a, int threads, int bps, cudaStream_t st, int max_ctas)
{
    // wide graphs: one launch shape (512 threads, up to 2 CTAs per SM)
    if (a.wide) return bfs_launch<512, 2, long long>(a, std::min(bps, 2), st, max_ctas);
    switch (threads) {
    case 256: return bps <= 4 ? bfs_launch<256, 4>(a, bps, st, max_ctas) : bfs_launch<256, 8>(a, bps, st, max_ctas);
    case 1024:
        return bps <= 1 ? bfs_launch<1024, 1>(a, bps, st, max_ctas) : bfs_launch<1024, 2>(a, bps, st, max_ctas);
    default:
        if (bps <= 2) return bfs_launch<512, 2>(a, bps, st, max_ctas);
        if (bps == 3) return bfs_launch<512, 3>(a, bps, st, max_ctas);
        return bfs_launch<512, 4>(a, bps, st, max_ctas);
    }
}

template <int BLOCK, int MINB>
int occupancy_ctas(int blocks_per_sm)
{
    int dev = 0, sms = 0, occ = 0;
    if (cudaFuncSetAttribute(k_bfs<BLOCK, MINB, int>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bfs_smem_bytes<BLOCK>()) != cudaSuccess)
        return 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bfs<BLOCK, MINB, int>, BLOCK, bfs_smem_bytes<BLOCK>()) !=
        cudaSuccess)
        return 0;
    return sms * std::max(1, std::min(blocks_per_sm, occ));
}

}  // namespace

int bfs_max_ctas(const gbfs_params &p)
{
    const int bps = p.blocks_per_sm;
    switch (p.threads_per_block) {
    case 256: return bps <= 4 ? occupancy_ctas<256, 4>(bps) : occupancy_ctas<256, 8>(bps);
    case 1024: return bps <= 1 ? occupancy_ctas<1024, 1>(bps) : occupancy_ctas<1024, 2>(bps);
    default:
        if (bps <= 2) return occupancy_ctas<512, 2>(bps);
        if (bps == 3) return occupancy_ctas<512, 3>(bps);
        return occupancy_ctas<512, 4>(bps);
    }
}

int bfs_work_alloc(BfsWork &w, int32_t n, std::string &err, bool wide)
{
    if (w.ctrl && w.n == n && w.wide == wide) return GBFS_OK;
    bfs_work_free(w);
    const size_t W = ((size_t)n + 31) / 32;
    const size_t bytes_int = sizeof(int) * (size_t)n;
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
    if (!al((void **)&w.level, bytes_int) || !al((void **)&w.visited, W * 4) ||
        !al((void **)&w.fb0, W * 4) || !al((void **)&w.fb1, W * 4) || !al((void **)&w.fb2, W * 4) ||
        !al((void **)&w.q0, bytes_int) || !al((void **)&w.q1, bytes_int) ||
        !al((void **)&w.qb0, (wide ? 4 : 2) * bytes_int) || !al((void **)&w.qb1, (wide ? 4 : 2) * bytes_int) ||
        !al((void **)&w.big, bytes_int) || !al((void **)&w.roots, bytes_int) ||
        !al((void **)&w.ctrl, sizeof(BfsCtrl))) {
        bfs_work_free(w);
        return GBFS_ERR_OOM;
    }
    if (cudaMemset(w.ctrl, 0, sizeof(BfsCtrl)) != cudaSuccess ||
        cudaMallocHost(&w.h_ctrl, sizeof(BfsCtrl)) != cudaSuccess ||
        cudaEventCreate(&w.ev0) != cudaSuccess || cudaEventCreate(&w.ev1) != cudaSuccess) {
        err = "workspace setup failed";
        bfs_work_free(w);
        return GBFS_ERR_CUDA;
    }
    w.n = n;
    w.wide = wide;
    return GBFS_OK;
}

void bfs_work_free(BfsWork &w)
{
    void *ps[] = {w.level, w.visited, w.fb0, w.fb1, w.fb2, w.q0, w.q1, w.qb0, w.qb1, w.big, w.roots, w.ctrl, w.d_outs};
    for (void *p : ps)
        if (p) cudaFree(p);
    if (w.h_outs) cudaFreeHost(w.h_outs);
    if (w.evs) {
        for (int i = 0; i < w.evs_cap; i++) cudaEventDestroy(w.evs[i]);
        delete[] w.evs;
    }
    if (w.h_ctrl) cudaFreeHost(w.h_ctrl);
    if (w.ev0) cudaEventDestroy(w.ev0);
    if (w.ev1) cudaEventDestroy(w.ev1);
    bfs_graph_free(w);
    if (w.level2) cudaFree(w.level2);
    if (w.copy_st) cudaStreamDestroy(w.copy_st);
    for (int i = 0; i < 2; i++) {
        if (w.ev_ready[i]) cudaEventDestroy(w.ev_ready[i]);
        if (w.ev_copied[i]) cudaEventDestroy(w.ev_copied[i]);
    }
    w = BfsWork{};
}

int bfs_work_reserve_overlap(BfsWork &w, std::string &err)
{
    if (w.level2) return GBFS_OK;
    cudaError_t e = cudaMalloc(&w.level2, sizeof(int) * (size_t)std::max(1, w.n));
    if (e != cudaSuccess) {
        w.level2 = nullptr;
        err = "second level buffer";
        return GBFS_ERR_OOM;
    }
    w.bytes += (int64_t)sizeof(int) * std::max(1, w.n);
    if (cudaStreamCreateWithFlags(&w.copy_st, cudaStreamNonBlocking) != cudaSuccess) {
        err = "copy stream";
        return GBFS_ERR_CUDA;
    }
    for (int i = 0; i < 2; i++)
        if (cudaEventCreateWithFlags(&w.ev_ready[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&w.ev_copied[i], cudaEventDisableTiming) != cudaSuccess) {
            err = "copy events";
            return GBFS_ERR_CUDA;
        }
    return GBFS_OK;
}

namespace {

BfsArgs make_args(const DeviceCsr &g, const gbfs_params &p, BfsWork &w, const int *d_roots, int k, int single_root,
                  int *d_level, BfsOut *slot, bool symmetric, int resume, int max_steps)
{
    BfsArgs a{};
    a.n = g.n;
    a.n_active = (int)std::max<int64_t>(1, g.nonisolated);
    a.m = g.m;
    a.wide = g.wide ? 1 : 0;
    a.row = g.row;
    a.row64 = g.row64;
    a.col = g.col;
    // in-edges for bottom-up steps; null when neither (then every level is
    // top-down); the transpose is read only when bottom-up may run (wide
    // graphs have none)
    const bool bu_possible = p.direction != GBFS_DIR_TOPDOWN;
    a.brow = symmetric ? g.row : bu_possible ? g.trow : nullptr;
    a.brow64 = symmetric ? g.row64 : nullptr;
    a.bcol = symmetric ? g.col : bu_possible ? g.tcol : nullptr;
    a.bfirst = symmetric ? g.first : bu_possible ? g.tfirst : nullptr;
    if (!a.bfirst) {
        a.brow = a.bcol = nullptr;
        a.brow64 = nullptr;
    }
    // hub-first rows (the transpose's always are): most vertices find their
    // parent at the first entry, and a second lookup per vertex costs more
    // than it saves; other rows probe their first two entries at once
    a.bsecond = symmetric && !g.hub_rows ? g.second : nullptr;
    a.zmask = symmetric ? g.zmask : nullptr;
    a.level = d_level;
    a.visited = w.visited;
    a.fb[0] = w.fb0;
    a.fb[1] = w.fb1;
    a.fb[2] = w.fb2;
    a.q0 = w.q0;
    a.q1 = w.q1;
    a.qb[0] = w.qb0;
    a.qb[1] = w.qb1;
    a.qb64[0] = reinterpret_cast<longlong2 *>(w.qb0);  // the workspace of a wide graph has 16-byte bounds
    a.qb64[1] = reinterpret_cast<longlong2 *>(w.qb1);
    a.bigl = w.big;
    a.ctrl = w.ctrl;
    a.out = slot;
    a.roots = d_roots;
    a.nroots = k;
    a.single_root = single_root;
    a.resume = resume;
    a.max_steps = max_steps;
    a.alpha = std::max(1, p.alpha);
    a.beta = std::max(1, p.beta);
    a.big_degree = std::max(32, p.big_degree);
    a.direction = p.direction;
    a.has_big = g.max_degree >= a.big_degree ? 1 : 0;
    a.max_degree = std::max(1, (int)g.max_degree);
    a.may_yield = 0;
    a.yield_level = RELAX_YIELD_LEVEL;
    a.yield_max_f = RELAX_ENTER_F;
    a.timeout_ns = (unsigned long long)std::max(1, p.timeout_ms) * 1000000ull;
    return a;
}

// Kernel, block, grid and shared memory of a launch with these parameters.
template <int BLOCK, int MINB>
cudaError_t bfs_shape(int blocks_per_sm, int max_ctas, const void **func, int *block, int *grid, size_t *smem)
{
    static LaunchSetup setup;  // per template instance
    const size_t sm = bfs_smem_bytes<BLOCK>();
    int sms = 0, occ = 0;
    cudaError_t e = setup.get(sms, occ, [&](int dev, int &s_out, int &o_out) {
        cudaError_t r = cudaFuncSetAttribute(k_bfs<BLOCK, MINB, int>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (r == cudaSuccess) r = cudaDeviceGetAttribute(&s_out, cudaDevAttrMultiProcessorCount, dev);
        if (r == cudaSuccess) r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o_out, k_bfs<BLOCK, MINB, int>, BLOCK, sm);
        return r;
    });
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int gr = sms * std::max(1, std::min(blocks_per_sm, occ));
    if (max_ctas > 0) gr = std::max(1, std::min(gr, max_ctas));
    *func = (const void *)k_bfs<BLOCK, MINB, int>;
    *block = BLOCK;
    *grid = gr;
    *smem = sm;
    return cudaSuccess;
}

cudaError_t bfs_shape_any(int threads, int bps, int max_ctas, const void **func, int *block, int *grid, size_t *smem)
{
    switch (threads) {
    case 256:
        return bps <= 4 ? bfs_shape<256, 4>(bps, max_ctas, func, block, grid, smem)
                        : bfs_shape<256, 8>(bps, max_ctas, func, block, grid, smem);
    case 1024:
        return bps <= 1 ? bfs_shape<1024, 1>(bps, max_ctas, func, block, grid, smem)
                        : bfs_shape<1024, 2>(bps, max_ctas, func, block, grid, smem);
    default:
        if (bps <= 2) return bfs_shape<512, 2>(bps, max_ctas, func, block, grid, smem);
        if (bps == 3) return bfs_shape<512, 3>(bps, max_ctas, func, block, grid, smem);
        return bfs_shape<512, 4>(bps, max_ctas, func, block, grid, smem);
    }
}

// The while-loop condition of a graph-captured search: run another level
// launch while the last one parked its state without a device error.
__global__ void k_set_loop(BfsCtrl *ctrl, cudaGraphConditionalHandle h)
{
    const int st = ld_relaxed_i32(&ctrl->status);
    const unsigned go = st == DEV_OK && !ctrl->rs.done ? 1u : 0u;
    cudaGraphSetConditional(h, go);
}

cudaError_t add_set_loop_node(cudaGraph_t g, const cudaGraphNode_t *dep, size_t ndep, BfsCtrl *ctrl,
                              cudaGraphConditionalHandle h, cudaGraphNode_t *node)
{
    void *kargs[] = {&ctrl, &h};
    cudaGraphNodeParams kp = {};
    kp.type = cudaGraphNodeTypeKernel;
    kp.kernel.func = (void *)k_set_loop;
    kp.kernel.gridDim = dim3(1);
    kp.kernel.blockDim = dim3(1);
    kp.kernel.kernelParams = kargs;
    return cudaGraphAddNode(node, g, dep, nullptr, ndep, &kp);
}

// One cooperative kernel node for args `a` in graph g (after `dep`, if any).
cudaError_t add_bfs_node(cudaGraph_t g, const cudaGraphNode_t *dep, size_t ndep, BfsArgs &a, const void *func,
                         int block, int grid, size_t smem, cudaGraphNode_t *node)
{
    void *kargs[] = {&a};
    cudaGraphNodeParams kp = {};
    kp.type = cudaGraphNodeTypeKernel;
    kp.kernel.func = const_cast<void *>(func);
    kp.kernel.gridDim = dim3(grid);
    kp.kernel.blockDim = dim3(block);
    kp.kernel.sharedMemBytes = (unsigned)smem;
    kp.kernel.kernelParams = kargs;
    cudaError_t e = cudaGraphAddNode(node, g, dep, nullptr, ndep, &kp);
    if (e != cudaSuccess) return e;
    cudaLaunchAttributeValue v = {};
    v.cooperative = 1;
    return cudaGraphKernelNodeSetAttribute(*node, cudaLaunchAttributeCooperative, &v);
}

}  // namespace

bool bfs_relax_tail(const DeviceCsr &g, const gbfs_params &p)
{
    return !p.per_level_launch && p.direction != GBFS_DIR_BOTTOMUP && g.max_degree <= RELAX_MAX_DEGREE;
}

int bfs_launches_per_search(const DeviceCsr &g, const gbfs_params &p) { return bfs_relax_tail(g, p) ? 2 : 1; }

cudaError_t bfs_enqueue(const DeviceCsr &g, const gbfs_params &p, BfsWork &w, const int *d_roots, int k,
                        int single_root, int *d_level, BfsOut *slot, cudaStream_t st, bool symmetric, int resume,
                        int max_steps, int max_ctas)
{
    BfsArgs a = make_args(g, p, w, d_roots, k, single_root, d_level, slot, symmetric, resume, max_steps);
    if (resume || max_steps || !bfs_relax_tail(g, p))
        return bfs_launch_any(a, p.threads_per_block, p.blocks_per_sm, st, max_ctas);
    // a graph of small degree: a search still running at level
    // RELAX_YIELD_LEVEL with a small frontier is finished by the
    // label-correcting kernel queued behind the grid launch (which returns
    // at once when the search ended in the grid launch)
    a.may_yield = 1;
    cudaError_t e = bfs_launch_any(a, p.threads_per_block, p.blocks_per_sm, st, max_ctas);
    if (e == cudaSuccess) e = bfs_relax_launch(a, st, max_ctas);
    return e;
}

void bfs_graph_free(BfsWork &w)
{
    if (w.gexec) cudaGraphExecDestroy(w.gexec);
    if (w.graph) cudaGraphDestroy(w.graph);
    w.gexec = nullptr;
    w.graph = nullptr;
}

// Graph-captured per-level launches: an init launch (initialisation and
// level 0), then a while-loop node whose body is one per-level launch and a
// one-thread node that keeps the loop going while the launch parked its
// state for another level (and stops it on a device error).  The roots are
// read from w.roots, so one instantiated graph serves every query with the
// same shape; it is rebuilt when the arguments change.
cudaError_t bfs_graph_launch(const DeviceCsr &g, const gbfs_params &p, BfsWork &w, int k, int *d_level,
                             cudaStream_t st, bool symmetric)
{
    BfsArgs a0 = make_args(g, p, w, w.roots, k, -1, d_level, &w.ctrl->out, symmetric, 0, 1);
    const void *func = nullptr;
    int block = 0, grid = 0;
    size_t smem = 0;
    cudaError_t e = bfs_shape_any(p.threads_per_block, p.blocks_per_sm, 0, &func, &block, &grid, &smem);
    if (e != cudaSuccess) return e;
    static_assert(sizeof(BfsArgs) <= sizeof(w.graph_key), "graph key holds the launch arguments");
    unsigned char key[sizeof(w.graph_key)] = {};
    memcpy(key, &a0, sizeof(BfsArgs));
    const int shape[3] = {block, grid, (int)smem};
    if (!w.gexec || memcmp(key, w.graph_key, sizeof(key)) != 0 || memcmp(shape, w.graph_shape, sizeof(shape)) != 0) {
        bfs_graph_free(w);
        cudaGraph_t gr = nullptr;
        e = cudaGraphCreate(&gr, 0);
        cudaGraphConditionalHandle h = 0;
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, gr, 0u, cudaGraphCondAssignDefault);
        BfsArgs ai = a0, al = a0;
        al.resume = 1;
        // init launch -> condition -> while (condition) { level launch -> condition }
        cudaGraphNode_t n0 = nullptr, n1 = nullptr, nc = nullptr, nb = nullptr, nb2 = nullptr;
        if (e == cudaSuccess) e = add_bfs_node(gr, nullptr, 0, ai, func, block, grid, smem, &n0);
        if (e == cudaSuccess) e = add_set_loop_node(gr, &n0, 1, w.ctrl, h, &n1);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        if (e == cudaSuccess) e = cudaGraphAddNode(&nc, gr, &n1, nullptr, 1, &cp);
        cudaGraph_t body = e == cudaSuccess ? cp.conditional.phGraph_out[0] : nullptr;
        if (e == cudaSuccess) e = add_bfs_node(body, nullptr, 0, al, func, block, grid, smem, &nb);
        if (e == cudaSuccess) e = add_set_loop_node(body, &nb, 1, w.ctrl, h, &nb2);
        cudaGraphExec_t ex = nullptr;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ex, gr, 0);
        if (e != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            return e;
        }
        w.graph = gr;
        w.gexec = ex;
        memcpy(w.graph_key, key, sizeof(key));
        memcpy(w.graph_shape, shape, sizeof(shape));
    }
    return cudaGraphLaunch(w.gexec, st);
}

int bfs_work_reserve_many(BfsWork &w, int k, std::string &err)
{
    if (k <= w.outs_cap && k + 1 <= w.evs_cap) return GBFS_OK;
    const int cap = std::max(k, 64);
    if (w.d_outs) cudaFree(w.d_outs);
    if (w.h_outs) cudaFreeHost(w.h_outs);
    w.d_outs = nullptr;
    w.h_outs = nullptr;
    w.outs_cap = 0;
    if (cudaMalloc(&w.d_outs, sizeof(BfsOut) * cap) != cudaSuccess ||
        cudaMallocHost(&w.h_outs, sizeof(BfsOut) * cap) != cudaSuccess) {
        err = "result slots";
        return GBFS_ERR_OOM;
    }
    w.outs_cap = cap;
    if (w.evs) {
        for (int i = 0; i < w.evs_cap; i++) cudaEventDestroy(w.evs[i]);
        delete[] w.evs;
    }
    w.evs = new cudaEvent_t[cap + 1];
    w.evs_cap = cap + 1;
    for (int i = 0; i < w.evs_cap; i++)
        if (cudaEventCreate(&w.evs[i]) != cudaSuccess) {
            err = "events";
            return GBFS_ERR_CUDA;
        }
    return GBFS_OK;
}

int bfs_run(const DeviceCsr &g, const gbfs_params &p, BfsWork &w, const int *d_roots, int k,
            int single_root, int *d_level, cudaStream_t st, BfsResult &res, std::string &err, bool symmetric)
{
    if (g.wide && p.per_level_launch) {
        err = "per-level launch modes need 32-bit row offsets";
        return GBFS_ERR_TOO_LARGE;
    }
    cudaError_t e = cudaSuccess;
    if (p.per_level_launch == 2) {
        // the graph reads its roots from w.roots
        if (d_roots) e = cudaMemcpyAsync(w.roots, d_roots, sizeof(int) * (size_t)k, cudaMemcpyDeviceToDevice, st);
        else e = cudaMemcpyAsync(w.roots, &single_root, sizeof(int), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // single_root lives on this stack frame
    }
    if (e == cudaSuccess) e = cudaEventRecord(w.ev0, st);
    int launches = bfs_launches_per_search(g, p);
    if (p.per_level_launch == 2) {
        if (e == cudaSuccess) e = bfs_graph_launch(g, p, w, d_roots ? k : 1, d_level, st, symmetric);
        launches = -1;  // the graph's own launches: levels + 1, filled in below
    } else if (!p.per_level_launch) {
        if (e == cudaSuccess) e = bfs_enqueue(g, p, w, d_roots, k, single_root, d_level, &w.ctrl->out, st, symmetric);
    } else {
        // The reference's shape: one launch per level, then a device->host
        // read of the loop state before deciding to launch again
        // (1D Partition/src/gpuBFS.cu:66-100).
        for (int resume = 0; e == cudaSuccess; resume = 1, ++launches) {
            e = bfs_enqueue(g, p, w, d_roots, k, single_root, d_level, &w.ctrl->out, st, symmetric, resume, 1);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(&w.h_ctrl->rs, &w.ctrl->rs, sizeof(BfsResume), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            int status = 0;
            e = cudaMemcpy(&status, &w.ctrl->status, sizeof(int), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess || status != DEV_OK || w.h_ctrl->rs.done) break;
        }
    }
    if (e == cudaSuccess) e = cudaEventRecord(w.ev1, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w.h_ctrl, w.ctrl, offsetof(BfsCtrl, t_entry), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        err = std::string("BFS launch: ") + cudaGetErrorString(e);
        return GBFS_ERR_CUDA;
    }
    const BfsCtrl &h = *w.h_ctrl;
    if (h.status != DEV_OK) {
        const int status = h.status;
        cudaMemsetAsync(w.ctrl, 0, sizeof(BfsCtrl), st);
        cudaStreamSynchronize(st);
        if (status == DEV_OVERFLOW) {
            err = "an on-chip frontier queue overflowed";
            return GBFS_ERR_CUDA;
        }
        err = "a device-side wait ran out (grid barrier)";
        return GBFS_ERR_TIMEOUT;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, w.ev0, w.ev1);
    res.ms = ms;
    res.levels = h.out.levels;
    res.td_levels = h.out.td_levels;
    res.bu_levels = h.out.bu_levels;
    res.launches = launches >= 0 ? launches : h.out.levels + 1;
    res.roots = h.out.roots;
    res.reached = (int64_t)h.out.reached;
    res.edges_c = (int64_t)h.out.edges_c;
    return GBFS_OK;
}

}  // namespace gbfs
