// msbfs.cu -- 64-lane multi-source BFS in one persistent launch (sm_103a).
//
// The reference answers one source per gpuBFS construction
// (1D Partition/src/gpuBFS.cu:13-116).  Here up to 64 searches on the same
// graph share every pass over it: per vertex, uint64 lane masks record
// which searches reached it (vis) and which have it in their frontier
// (cur / nxt).  A lane's level at v is the step in which its bit first
// appears in vis[v], written straight into that lane's int32 level row.
//   push step (sparse frontiers): each frontier vertex ORs its lane mask,
//       minus lanes already visited, into nxt[u] of every neighbour
//       (warp per frontier vertex, coalesced row reads); a second phase
//       filters nxt by vis, records levels and clears the old frontier.
//   pull step (dense frontiers, symmetric graphs): every vertex with
//       unreached lanes ORs cur[] over its row until all those lanes are
//       covered; vertices own their masks, so no atomics.
// One bounded grid barrier separates pull steps; push steps take two.
#include <algorithm>

#include "msbfs.cuh"

namespace gbfs {

namespace {

constexpr int MS_BLOCK = 512;

struct MsArgs {
    int n, n_active, k;
    const int *row, *col;
    unsigned long long *vis, *fa, *fb;
    int *out;
    const int *src;
    MsCtrl *ctrl;
    int pull_allowed, direction, pull_div;
    unsigned long long timeout_ns;
};

template <typename T>
__device__ __forceinline__ T block_reduce_sum(T x, T *s_red)
{
    x = warp_sum(x);
    __syncthreads();
    if (lane_id() == 0) s_red[threadIdx.x >> 5] = x;
    __syncthreads();
    T t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? s_red[threadIdx.x] : 0;
        t = warp_sum(t);
    }
    return t;
}

__device__ __forceinline__ void write_levels(int *out, int n, int u, unsigned long long bits, int nl)
{
    while (bits) {
        const int j = __ffsll((long long)bits) - 1;
        out[(size_t)j * n + u] = nl;
        bits &= bits - 1ull;
    }
}

__global__ void __launch_bounds__(MS_BLOCK) k_msbfs(MsArgs a)
{
    __shared__ unsigned long long s_red[32];
    const int n = a.n;
    const long long gtid = (long long)blockIdx.x * MS_BLOCK + threadIdx.x;
    const long long gthreads = (long long)gridDim.x * MS_BLOCK;
    const unsigned lane = lane_id();
    const unsigned long long all = a.k >= 64 ? ~0ull : ((1ull << a.k) - 1ull);
    MsCtrl *ctrl = a.ctrl;
    unsigned epoch = 0;

    // ---- init ----
    for (long long v = gtid; v < n; v += gthreads) {
        a.vis[v] = 0;
        a.fa[v] = 0;
        a.fb[v] = 0;
    }
    {
        const long long total = (long long)a.k * n;
        if (((uintptr_t)a.out & 15) == 0) {
            int4 *o4 = (int4 *)a.out;
            const long long t4 = total >> 2;
            for (long long i = gtid; i < t4; i += gthreads) o4[i] = make_int4(-1, -1, -1, -1);
            for (long long i = (t4 << 2) + gtid; i < total; i += gthreads) a.out[i] = -1;
        } else {
            for (long long i = gtid; i < total; i += gthreads) a.out[i] = -1;
        }
    }
    if (gtid == 0) {
        ctrl->reached = 0;
        ctrl->edges_c = 0;
    }
    if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
    if (blockIdx.x == 0 && threadIdx.x < (unsigned)a.k) {
        const int s = a.src[threadIdx.x];
        const unsigned long long bit = 1ull << threadIdx.x;
        atomicOr(&a.vis[s], bit);
        const unsigned long long old = atomicOr(&a.fa[s], bit);
        a.out[(size_t)threadIdx.x * n + s] = 0;
        if (old == 0) atomicAdd(&ctrl->cnt[0], 1ull);
    }
    if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;

    int L = 0, push_levels = 0, pull_levels = 0;
    bool last_pull = false;
    for (;;) {
        const unsigned long long nf = ld_relaxed_u64(&ctrl->cnt[L % 3]);
        if (nf == 0) break;
        bool pull;
        if (!a.pull_allowed || a.direction == GBFS_DIR_TOPDOWN) pull = false;
        else if (a.direction == GBFS_DIR_BOTTOMUP) pull = true;
        else pull = (long long)nf * a.pull_div > a.n_active;
        unsigned long long *cur = (L & 1) ? a.fb : a.fa;
        unsigned long long *nxt = (L & 1) ? a.fa : a.fb;
        unsigned long long *cnt_next = &ctrl->cnt[(L + 1) % 3];
        const int nl = L + 1;
        if (gtid == 0) ctrl->cnt[(L + 2) % 3] = 0;
        unsigned long long my_cnt = 0;

        if (pull) {
            ++pull_levels;
            for (long long u = gtid; u < n; u += gthreads) {
                const unsigned long long vu = __ldcg(a.vis + u);
                const unsigned long long need = ~vu & all;
                unsigned long long nw = 0;
                if (need) {
                    const int b = __ldg(a.row + u), e = __ldg(a.row + u + 1);
                    unsigned long long acc = 0;
                    int i = b;
                    for (; i + 1 < e; i += 2) {
                        const int v0 = __ldg(a.col + i), v1 = __ldg(a.col + i + 1);
                        acc |= __ldcg(cur + v0) | __ldcg(cur + v1);
                        if ((acc & need) == need) break;
                    }
                    if (i + 1 == e) acc |= __ldcg(cur + __ldg(a.col + i));
                    nw = acc & need;
                    if (nw) {
                        a.vis[u] = vu | nw;
                        write_levels(a.out, n, (int)u, nw, nl);
                        ++my_cnt;
                    }
                }
                nxt[u] = nw;
            }
        } else {
            ++push_levels;
            if (last_pull) {
                // the array that becomes nxt still holds an old frontier
                for (long long u = gtid; u < n; u += gthreads) nxt[u] = 0;
                if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
            }
            // phase 1: warp per active frontier vertex
            const long long nwarps = gthreads >> 5;
            for (long long base = (gtid >> 5) * 32; base < n; base += nwarps * 32) {
                const long long v = base + lane;
                const unsigned long long c = v < n ? __ldcg(cur + v) : 0ull;
                unsigned act = __ballot_sync(FULL, c != 0);
                while (act) {
                    const int src_lane = __ffs(act) - 1;
                    act &= act - 1;
                    const unsigned long long cv = __shfl_sync(FULL, c, src_lane);
                    const int vv = (int)(base + src_lane);
                    const int b = __ldg(a.row + vv), e = __ldg(a.row + vv + 1);
                    for (int i = b + (int)lane; i < e; i += 32) {
                        const int u = __ldg(a.col + i);
                        const unsigned long long nw = cv & ~__ldcg(a.vis + u);
                        if (nw && (__ldcg(nxt + u) & nw) != nw) atomicOr(nxt + u, nw);
                    }
                }
            }
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
            // phase 2: filter, record, clear the old frontier
            for (long long u = gtid; u < n; u += gthreads) {
                const unsigned long long x = __ldcg(nxt + u);
                cur[u] = 0;
                if (x) {
                    const unsigned long long vu = __ldcg(a.vis + u);
                    const unsigned long long nw = x & ~vu;
                    nxt[u] = nw;
                    if (nw) {
                        a.vis[u] = vu | nw;
                        write_levels(a.out, n, (int)u, nw, nl);
                        ++my_cnt;
                    }
                }
            }
        }
        last_pull = pull;
        const unsigned long long bc = block_reduce_sum(my_cnt, s_red);
        if (threadIdx.x == 0 && bc) atomicAdd(cnt_next, bc);
        if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns, epoch)) return;
        ++L;
    }

    // per-lane totals for GTEPS: reached vertices and their out-edges
    unsigned long long r = 0, ec = 0;
    for (long long u = gtid; u < n; u += gthreads) {
        const int c = __popcll(__ldcg(a.vis + u) & all);
        if (c) {
            r += c;
            ec += (unsigned long long)c * (unsigned long long)(__ldg(a.row + u + 1) - __ldg(a.row + u));
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
        for (int i = 0; i < 3; i++) ctrl->cnt[i] = 0;
    }
    grid_exit(&ctrl->bar);
}

}  // namespace

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
    const size_t b8 = sizeof(unsigned long long) * (size_t)n;
    if (!al((void **)&w.vis, b8) || !al((void **)&w.cur, b8) || !al((void **)&w.nxt, b8) ||
        !al((void **)&w.out, sizeof(int) * (size_t)n * MS_LANES) ||
        !al((void **)&w.src, sizeof(int) * MS_LANES) || !al((void **)&w.ctrl, sizeof(MsCtrl))) {
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
    void *ps[] = {w.vis, w.cur, w.nxt, w.out, w.src, w.ctrl};
    for (void *p : ps)
        if (p) cudaFree(p);
    if (w.h_ctrl) cudaFreeHost(w.h_ctrl);
    if (w.ev0) cudaEventDestroy(w.ev0);
    if (w.ev1) cudaEventDestroy(w.ev1);
    w = MsWork{};
}

int msbfs_run(const DeviceCsr &g, const gbfs_params &p, bool pull_allowed, MsWork &w,
              const int *d_src, int k, int *d_out, cudaStream_t st, MsResult &res, std::string &err)
{
    MsArgs a;
    a.n = g.n;
    a.n_active = (int)std::max<int64_t>(1, g.nonisolated);
    a.k = k;
    a.row = g.row;
    a.col = g.col;
    a.vis = w.vis;
    a.fa = w.cur;
    a.fb = w.nxt;
    a.out = d_out;
    a.src = d_src;
    a.ctrl = w.ctrl;
    a.pull_allowed = pull_allowed ? 1 : 0;
    a.direction = p.direction;
    a.pull_div = 64;
    a.timeout_ns = (unsigned long long)std::max(1, p.timeout_ms) * 1000000ull;

    int dev = 0, sms = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_msbfs, MS_BLOCK, 0);
    if (e == cudaSuccess && occ < 1) e = cudaErrorInvalidConfiguration;
    if (e == cudaSuccess) e = cudaEventRecord(w.ev0, st);
    if (e == cudaSuccess) {
        const int per = std::max(1, std::min(occ, std::max(1, p.blocks_per_sm) * 2));
        void *kargs[] = {&a};
        e = cudaLaunchCooperativeKernel((const void *)k_msbfs, dim3(sms * per), dim3(MS_BLOCK), kargs, 0,
                                        st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(w.ev1, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.h_ctrl, w.ctrl, sizeof(MsCtrl), cudaMemcpyDeviceToHost, st);
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
