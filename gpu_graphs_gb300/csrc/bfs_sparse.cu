// bfs_sparse.cu -- the sparse phase of a single-source BFS on one
// thread-block cluster (sm_103a).
//
// On a high-diameter graph (a road network, a mesh, the perturbed grid) a
// search is thousands of levels whose frontiers hold a few thousand
// vertices.  The persistent grid kernel (bfs.cu) pays for every such level
// with a grid-wide barrier over all of its CTAs, global frontier counters
// and a global queue: about 9 us a level, almost all of it latency.  Once a
// search has run yield_level levels on a graph of small degree, the grid
// kernel parks its level loop and this kernel, queued right behind it,
// continues on ONE cluster of sparse_ctas CTAs (16 SMs of one GPC):
//   * the frontier lives in the CTAs' shared memory: each CTA appends the
//     vertices it claims, with their row bounds, to its own queue, and the
//     CTAs read one another's queues through distributed shared memory;
//   * a level ends with the cluster's hardware barrier instead of a global
//     one, and each CTA learns the level's size from the other CTAs'
//     counters (also in distributed shared memory);
//   * each CTA expands the rows of its own queue when every queue is short
//     or the queues are balanced (the longest within 15 % of the mean);
//     otherwise the level's rows are split evenly over the CTAs (rank order
//     of their queues) and read remotely;
//   * small levels (latency-bound) take one row per lane; larger ones, as in
//     the grid kernel's top-down step, 32 rows per warp as one concatenated
//     edge range; a plain-load filter on the visited bitmap, then the
//     atomicOr claim issued with the row-bound loads of the candidate; the
//     winner writes the level and joins its CTA's queue.
// The visited bitmap and the level array stay in global memory, so the
// result is the same array the grid kernel would write.  When a frontier
// grows past sparse_leave_f vertices (or what the CTAs' queues can hold),
// or the direction rule asks for a bottom-up step, the kernel writes the
// frontier back to the global queue and parks the loop for the grid kernel
// queued after it.
// Replaces, for such graphs, the per-level host loop of gpuBFS::gpuBFS
// (1D Partition/src/gpuBFS.cu:66-100).
#include <algorithm>

#include "bfs.cuh"
#include "bfs_args.cuh"
#include "common.cuh"

namespace gbfs {

namespace {

constexpr int SP_BLOCK = 1024;
constexpr int SP_NW = SP_BLOCK / 32;
constexpr int SP_ILP = 4;        // edges in flight per lane
constexpr unsigned SP_LOCAL_ROWS = 128;  // a CTA expands its own queue when no queue is longer
constexpr unsigned SP_ROW_F = 2048;      // levels up to this size expand one row per lane
constexpr int SP_MAX_CTAS = 16;  // largest cluster tried
constexpr int SP_CAP = 9216;     // queue entries per CTA and level (two levels held: 24 B each)

__device__ __forceinline__ unsigned cluster_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ unsigned cluster_ctas()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

// Address of `p` (this CTA's shared memory) in CTA `rank`'s shared memory.
__device__ __forceinline__ unsigned dsmem_map(const void *p, unsigned rank)
{
    unsigned a;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_addr(p)), "r"(rank));
    return a;
}

__device__ __forceinline__ unsigned ld_dsmem_u32(unsigned a)
{
    unsigned v;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_dsmem_u64(unsigned a)
{
    unsigned long long v;
    asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
    return v;
}

__device__ __forceinline__ int2 ld_dsmem_int2(unsigned a)
{
    int2 v;
    asm volatile("ld.shared::cluster.v2.s32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a) : "memory");
    return v;
}

// The cluster's barrier: every thread of every CTA arrives (releasing its
// shared- and global-memory writes) and waits (acquiring the others').
__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(SP_BLOCK, 1) k_bfs_sparse(BfsArgs a)
{
    extern __shared__ __align__(16) int sp_smem[];
    const int cap = a.sparse_cap;
    // two levels' queues: row bounds (int2) and vertex ids; queue q of a
    // level is qbe0 + q * cap and qv0 + q * cap
    int2 *const qbe0 = reinterpret_cast<int2 *>(sp_smem);
    int *const qv0 = sp_smem + 4 * cap;
    __shared__ unsigned s_cnt[2];
    __shared__ unsigned long long s_deg[2];
    __shared__ unsigned s_off[SP_MAX_CTAS + 1];
    __shared__ unsigned s_maxcnt;
    __shared__ unsigned long long s_mf;
    __shared__ unsigned long long s_red[SP_NW];
    __shared__ int s_stop;

    const unsigned C = cluster_ctas(), r = cluster_rank();
    const unsigned t = threadIdx.x, lane = t & 31, warp = t >> 5;
    BfsCtrl *ctrl = a.ctrl;

    // run only when the grid kernel parked its loop for this kernel
    const BfsResume rs = ctrl->rs;
    if (rs.done || rs.mode != RESUME_SPARSE || ctrl->status != DEV_OK) return;
    long long m_u = rs.m_u;
    unsigned long long prev_nf = rs.prev_nf, reached = rs.reached, edges_c = rs.edges_c, prev_mf = rs.prev_mf;
    const unsigned long long roots = rs.roots;
    int L = rs.L, td_levels = rs.td_levels;
    const int bu_levels = rs.bu_levels;

    auto block_sum = [&](unsigned long long x) -> unsigned long long {
        x = warp_sum(x);
        if (lane == 0) s_red[warp] = x;
        __syncthreads();
        unsigned long long v = 0;
        if (warp == 0) v = warp_sum(lane < SP_NW ? s_red[lane] : 0ull);
        __syncthreads();
        return v;  // thread 0
    };

    // frontier L from the global queue into queue 0, split evenly over the CTAs
    {
        const unsigned long long F0 = cd_count(ctrl->cd[L % 3]);
        const int *qg = (L & 1) ? a.q1 : a.q0;
        const int2 *qbg = a.qb[L & 1];
        const unsigned long long lo = F0 * r / C, hi = F0 * (r + 1) / C;
        unsigned long long my_deg = 0;
        for (unsigned long long i = lo + t; i < hi; i += SP_BLOCK) {
            const int j = (int)(i - lo);
            if (j >= cap) break;  // never: the grid kernel checked the frontier fits
            const int2 be = __ldcg(qbg + i);
            qbe0[j] = be;
            qv0[j] = __ldcg(qg + i);
            my_deg += (unsigned long long)(be.y - be.x);
        }
        const unsigned long long d = block_sum(my_deg);
        if (t == 0) {
            s_cnt[0] = (unsigned)std::min<unsigned long long>(hi - lo, (unsigned long long)cap);
            s_deg[0] = d;
            if (hi - lo > (unsigned long long)cap) atomicCAS(&ctrl->status, DEV_OK, DEV_OVERFLOW);
        }
    }
    cluster_sync_all();

    int buf = 0;
    for (;;) {
        const int nb = buf ^ 1;
        // the level's size: every CTA's count and degree sum, in rank order
        if (warp == 0) {
            unsigned c = 0;
            unsigned long long d = 0;
            if (lane < C) {
                c = ld_dsmem_u32(dsmem_map(&s_cnt[buf], lane));
                d = ld_dsmem_u64(dsmem_map(&s_deg[buf], lane));
            }
            const unsigned incl = warp_incl_scan(c);
            if (lane < C) s_off[lane] = incl - c;
            const unsigned tot = __shfl_sync(FULL, incl, 31);
            const unsigned long long dt = warp_sum(d);
            unsigned mx = c;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
            if (lane == 0) {
                s_off[C] = tot;
                s_maxcnt = mx;
                s_mf = dt;
                s_stop = ld_relaxed_i32(&ctrl->status) != DEV_OK;
            }
        }
        __syncthreads();
        const unsigned long long F = s_off[C], mf = s_mf;
        if (s_stop) {
            // a device error (reported in ctrl->status): leave with the others
            cluster_sync_all();
            return;
        }
        if (F == 0) {
            // the search is complete
            if (r == 0 && t == 0) {
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
                ctrl->t_exit = globaltimer_ns();
            }
            cluster_sync_all();  // no CTA leaves while others may read its queues
            return;
        }
        // Beamer's rule (as the grid kernel applies it after a top-down
        // step), and whether every CTA can hold the next frontier
        const long long m_u_next = m_u - (long long)mf;
        const bool bu = a.direction == GBFS_DIR_OPTIMIZING && a.brow != nullptr && (long long)mf * a.alpha > m_u_next;
        const bool fits = (long long)((F + C - 1) / C) * a.max_degree <= cap;
        if (bu || !fits || F > (unsigned long long)a.sparse_leave_f) {
            // hand the loop back to the grid kernel: frontier L into its
            // global queue (CTA segments in rank order), state parked
            int *qg = (L & 1) ? a.q1 : a.q0;
            int2 *qbg = a.qb[L & 1];
            const unsigned cnt = s_cnt[buf], off = s_off[r];
            for (unsigned j = t; j < cnt; j += SP_BLOCK) {
                qg[off + j] = qv0[buf * cap + j];
                qbg[off + j] = qbe0[buf * cap + j];
            }
            if (r == 0 && t == 0) {
                ctrl->cd[L % 3] = cd_pack(F, mf);
                ctrl->cd[(L + 1) % 3] = 0;
                ctrl->cd[(L + 2) % 3] = 0;
                for (int i = 0; i < 3; i++) ctrl->big[i] = 0;
                BfsResume p;
                p.m_u = m_u;
                p.prev_nf = prev_nf;
                p.reached = reached;
                p.edges_c = edges_c;
                p.roots = roots;
                p.prev_mf = prev_mf;
                p.L = L;
                p.td_levels = td_levels;
                p.bu_levels = bu_levels;
                p.td = 1;
                p.done = 0;
                p.dirty = rs.dirty;
                p.mode = RESUME_HANDBACK;
                p.pad = 0;
                ctrl->rs = p;
            }
            cluster_sync_all();
            return;
        }
        reached += F;
        edges_c += mf;
        m_u = m_u_next;
        prev_nf = F;
        ++td_levels;
        const int nl = L + 1;
        if (t == 0) s_cnt[nb] = 0;  // others read it a level ago, before the last cluster barrier
        __syncthreads();

        // this CTA's rows: its own queue while the queues are balanced (or
        // all small) and each CTA can hold what its rows may find, else rows
        // [F r / C, F (r + 1) / C) of the concatenated queues
        const unsigned maxcnt = s_maxcnt;
        const unsigned long long even = (F + C - 1) / C;
        const bool local = (maxcnt <= SP_LOCAL_ROWS || 20ull * maxcnt <= 23ull * even) &&
                           (long long)maxcnt * a.max_degree <= cap;
        const unsigned long long rlo = local ? 0 : F * r / C;
        const unsigned long long rhi = local ? s_cnt[buf] : F * (r + 1) / C;
        const int2 *lq = qbe0 + buf * cap;
        unsigned long long my_deg = 0;
        auto row_bounds = [&](unsigned long long i) -> int2 {
            if (local) return lq[i];
            int o = 0;  // the owner: the last CTA whose segment starts at or before i
#pragma unroll
            for (int s = SP_MAX_CTAS / 2; s > 0; s >>= 1)
                if (o + s < (int)C && s_off[o + s] <= i) o += s;
            const unsigned idx = (unsigned)(i - s_off[o]);
            return ld_dsmem_int2(dsmem_map(&lq[idx], (unsigned)o));
        };
        // SP_ILP candidate neighbours per lane (w < 0: none): a plain-load
        // filter on the visited bitmap, then the claim and the candidate's
        // row bounds issued together (the bounds of a candidate that loses
        // the claim are not used); winners write their level and join this
        // CTA's queue (warp-aggregated appends)
        auto claim = [&](const int (&w)[SP_ILP]) {
            unsigned word[SP_ILP], old[SP_ILP];
#pragma unroll
            for (int j = 0; j < SP_ILP; j++) word[j] = w[j] >= 0 ? a.visited[w[j] >> 5] : FULL;
            int2 wb[SP_ILP];
#pragma unroll
            for (int j = 0; j < SP_ILP; j++) {
                const unsigned bit = 1u << (w[j] & 31);
                old[j] = FULL;
                wb[j] = make_int2(0, 0);
                if (!(word[j] & bit)) {
                    old[j] = atomicOr(&a.visited[w[j] >> 5], bit);
                    wb[j] = make_int2(__ldg(a.row + w[j]), __ldg(a.row + w[j] + 1));
                }
            }
            bool won[SP_ILP];
#pragma unroll
            for (int j = 0; j < SP_ILP; j++) {
                won[j] = w[j] >= 0 && !((old[j] >> (w[j] & 31)) & 1u);
                if (won[j]) a.level[w[j]] = nl;
            }
#pragma unroll
            for (int j = 0; j < SP_ILP; j++) {
                const unsigned m = __ballot_sync(FULL, won[j]);
                if (!m) continue;
                const int leader = __ffs(m) - 1;
                unsigned pos = 0;
                if ((int)lane == leader) pos = atomicAdd(&s_cnt[nb], (unsigned)__popc(m));
                pos = __shfl_sync(FULL, pos, leader) + __popc(m & lanemask_lt());
                if (won[j]) {
                    if (pos < (unsigned)cap) {
                        qbe0[nb * cap + pos] = wb[j];
                        qv0[nb * cap + pos] = w[j];
                        my_deg += (unsigned long long)(wb[j].y - wb[j].x);
                    } else {
                        atomicCAS(&ctrl->status, DEV_OK, DEV_OVERFLOW);  // never: bounded by the fits rules
                    }
                }
            }
        };
        if (F <= SP_ROW_F) {
            // a small level (latency-bound): one row per lane, its entries
            // SP_ILP at a time
            for (unsigned long long i0 = rlo + (unsigned long long)warp * 32; i0 < rhi;
                 i0 += (unsigned long long)SP_NW * 32) {
                const unsigned long long i = i0 + lane;
                int2 be = make_int2(0, 0);
                if (i < rhi) be = row_bounds(i);
                for (int k0 = be.x; __any_sync(FULL, k0 < be.y); k0 += SP_ILP) {
                    int w[SP_ILP];
#pragma unroll
                    for (int j = 0; j < SP_ILP; j++) w[j] = k0 + j < be.y ? __ldg(a.col + k0 + j) : -1;
                    claim(w);
                }
            }
        } else {
            // a larger level: the warp's 32 rows as one concatenated edge
            // range, SP_ILP edges per lane in flight
            for (unsigned long long i0 = rlo + (unsigned long long)warp * 32; i0 < rhi;
                 i0 += (unsigned long long)SP_NW * 32) {
                const unsigned long long i = i0 + lane;
                int b = 0, e = 0;
                if (i < rhi) {
                    const int2 be = row_bounds(i);
                    b = be.x;
                    e = be.y;
                }
                const int d = e - b;
                const int incl = warp_incl_scan(d);
                const int excl = incl - d;
                const int T = __shfl_sync(FULL, incl, 31);
                for (int e0 = 0; e0 < T; e0 += 32 * SP_ILP) {
                    int w[SP_ILP];
#pragma unroll
                    for (int j = 0; j < SP_ILP; j++) {
                        const int k = e0 + j * 32 + (int)lane;
                        const int kk = min(k, T - 1);
                        int lo = 0;
#pragma unroll
                        for (int s = 16; s > 0; s >>= 1) {
                            const int c = lo + s;
                            if (__shfl_sync(FULL, excl, c) <= kk) lo = c;
                        }
                        const int ob = __shfl_sync(FULL, b, lo);
                        const int oe = __shfl_sync(FULL, excl, lo);
                        w[j] = k < T ? __ldg(a.col + ob + (kk - oe)) : -1;
                    }
                    claim(w);
                }
            }
        }
        const unsigned long long d = block_sum(my_deg);
        if (t == 0) {
            s_deg[nb] = d;
            if (s_cnt[nb] > (unsigned)cap) s_cnt[nb] = (unsigned)cap;
        }
        prev_mf = mf;
        if (r == 0 && t == 0) {
            LevelTrace tr;
            tr.level = L;
            tr.dir = 4;
            tr.frontier = F;
            tr.edges = mf;
            tr.t_ns = globaltimer_ns();
            ctrl->trace[L < TRACE_CAP - 1 ? L : TRACE_CAP - 1] = tr;
        }
        cluster_sync_all();
        buf = nb;
        ++L;
    }
}

size_t sparse_smem(int cap) { return (size_t)cap * (2 * sizeof(int2) + 2 * sizeof(int)); }

}  // namespace

cudaError_t bfs_sparse_shape(int &ctas, int &cap)
{
    static LaunchSetup setup;
    return setup.get(ctas, cap, [](int, int &c_out, int &cap_out) {
        cap_out = SP_CAP;
        c_out = 0;  // 0: no cluster of this shape fits, the sparse phase is not used
        const size_t smem = sparse_smem(SP_CAP);
        cudaError_t r = cudaFuncSetAttribute(k_bfs_sparse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (r == cudaSuccess) r = cudaFuncSetAttribute(k_bfs_sparse, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (r != cudaSuccess) {
            cudaGetLastError();
            return cudaSuccess;
        }
        for (int c = SP_MAX_CTAS; c >= 8; c /= 2) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(SP_BLOCK);
            cfg.dynamicSmemBytes = smem;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, (const void *)k_bfs_sparse, &cfg) == cudaSuccess &&
                nclusters >= 1) {
                c_out = c;
                break;
            }
            cudaGetLastError();
        }
        return cudaSuccess;
    });
}

cudaError_t bfs_sparse_launch(const BfsArgs &args, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(args.sparse_ctas);
    cfg.blockDim = dim3(SP_BLOCK);
    cfg.dynamicSmemBytes = sparse_smem(args.sparse_cap);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = args.sparse_ctas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_bfs_sparse, args);
}

}  // namespace gbfs
