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
//   top-down step   frontier queue -> next queue.  Each warp takes 32
//                   frontier vertices; their rows (below big_degree) are
//                   walked as one concatenated edge range (shuffle binary
//                   search per edge, coalesced col_idx reads); rows of
//                   degree >= big_degree are deferred and then split into
//                   512-edge chunks over every warp of the grid, read with
//                   16-byte vector loads.  A vertex is claimed with an
//                   atomicOr on the visited bitmap (after a plain-load
//                   filter), its level written once, and it is appended
//                   through a per-warp shared-memory queue (one global
//                   atomic per flush instead of one per edge).
//   bottom-up step  every unvisited vertex scans its row for a parent in
//                   the frontier bitmap, 4 probes in flight per lane,
//                   stopping at the first hit; each warp owns whole bitmap
//                   words, so visited / next-frontier words are written
//                   without atomics.
//   switching       Beamer's rule: top-down -> bottom-up when the frontier's
//                   out-edges exceed (unexplored edges)/alpha, back when the
//                   frontier has fewer than (non-isolated vertices)/beta
//                   vertices and is shrinking.  A queue <-> bitmap
//                   conversion phase runs at each switch.
// Bottom-up needs in-edges == out-edges, so it is used on symmetric graphs
// only; other graphs run top-down at every level.
#include <algorithm>
#include <cstring>

#include "bfs.cuh"

namespace gbfs {

namespace {

constexpr int QCAP = 256;    // per-warp staging queue entries
constexpr int CHUNK = 512;   // edges per grid-wide chunk of a deferred row

struct BfsArgs {
    int n;
    int n_active;            // non-isolated vertices (for beta)
    long long m;
    const int *row;
    const int *col;
    const unsigned *zmask;
    int *level;
    unsigned *visited;
    unsigned *fb0, *fb1;
    int *q0, *q1;
    int *bigl;
    BfsCtrl *ctrl;
    BfsOut *out;
    const int *roots;
    int nroots;
    int single_root;         // >= 0: fast init for one root
    int alpha, beta, big_degree, direction;
    unsigned long long timeout_ns;
};

struct WarpQ {
    int *buf;
    int n;
};

__device__ __forceinline__ void wq_flush(WarpQ &q, unsigned long long *cnt, int *out)
{
    __syncwarp();
    if (q.n == 0) return;
    unsigned long long base = 0;
    if (lane_id() == 0) base = atomicAdd(cnt, (unsigned long long)q.n);
    base = __shfl_sync(FULL, base, 0);
    for (int i = lane_id(); i < q.n; i += 32) out[base + i] = q.buf[i];
    __syncwarp();
    q.n = 0;
}

__device__ __forceinline__ void wq_push(WarpQ &q, bool has, int v, unsigned long long *cnt, int *out)
{
    unsigned m = __ballot_sync(FULL, has);
    if (!m) return;
    int c = __popc(m);
    if (q.n + c > QCAP) wq_flush(q, cnt, out);
    if (has) q.buf[q.n + __popc(m & lanemask_lt())] = v;
    q.n += c;
}

__device__ __forceinline__ bool td_claim(int w, unsigned *visited, int *level, int nl)
{
    const unsigned bit = 1u << (w & 31);
    unsigned *p = visited + (w >> 5);
    if (__ldcg(p) & bit) return false;
    if (atomicOr(p, bit) & bit) return false;
    level[w] = nl;
    return true;
}

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
    return t;  // thread 0
}

__device__ __forceinline__ int block_excl_scan_int(int x, int *s_warp, int *total)
{
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int incl = warp_incl_scan(x);
    __syncthreads();
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? s_warp[lane] : 0;
        int wi = warp_incl_scan(w);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    *total = s_warp[32];
    return s_warp[warp] + incl - x;
}

// Claim every neighbour in col[s, e) with the whole warp (int4 body).
__device__ __forceinline__ void warp_claim_range(int s, int e, const BfsArgs &a, int nl, WarpQ &q,
                                                 unsigned long long *cnt, int *qn,
                                                 unsigned long long &my_deg)
{
    const int lane = (int)lane_id();
    const int al = min(e, (s + 3) & ~3);
    {
        int k = s + lane;
        bool got = false;
        int w = 0;
        if (k < al) {
            w = __ldg(a.col + k);
            got = td_claim(w, a.visited, a.level, nl);
        }
        if (got) my_deg += __ldg(a.row + w + 1) - __ldg(a.row + w);
        wq_push(q, got, w, cnt, qn);
    }
    const int z = al + ((e - al) & ~3);
    for (int base = al; base < z; base += 128) {
        const int k = base + lane * 4;
        int4 x = make_int4(0, 0, 0, 0);
        const bool ok = k < z;
        if (ok) x = ld_stream_v4(a.col + k);
        bool g0 = ok && td_claim(x.x, a.visited, a.level, nl);
        bool g1 = ok && td_claim(x.y, a.visited, a.level, nl);
        bool g2 = ok && td_claim(x.z, a.visited, a.level, nl);
        bool g3 = ok && td_claim(x.w, a.visited, a.level, nl);
        if (g0) my_deg += __ldg(a.row + x.x + 1) - __ldg(a.row + x.x);
        if (g1) my_deg += __ldg(a.row + x.y + 1) - __ldg(a.row + x.y);
        if (g2) my_deg += __ldg(a.row + x.z + 1) - __ldg(a.row + x.z);
        if (g3) my_deg += __ldg(a.row + x.w + 1) - __ldg(a.row + x.w);
        wq_push(q, g0, x.x, cnt, qn);
        wq_push(q, g1, x.y, cnt, qn);
        wq_push(q, g2, x.z, cnt, qn);
        wq_push(q, g3, x.w, cnt, qn);
    }
    {
        int k = z + lane;
        bool got = false;
        int w = 0;
        if (k < e) {
            w = __ldg(a.col + k);
            got = td_claim(w, a.visited, a.level, nl);
        }
        if (got) my_deg += __ldg(a.row + w + 1) - __ldg(a.row + w);
        wq_push(q, got, w, cnt, qn);
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_bfs(BfsArgs a)
{
    extern __shared__ int smem[];
    __shared__ unsigned long long s_red[32];
    __shared__ int s_warp[33];
    constexpr int NW = BLOCK / 32;
    int *s_q = smem;                       // NW * QCAP
    int *s_cs = smem + NW * QCAP;          // BLOCK + 1 chunk prefix
    int *s_b = s_cs + BLOCK + 1;           // BLOCK row begins
    int *s_e = s_b + BLOCK;                // BLOCK row ends

    const int n = a.n;
    const int W = (n + 31) >> 5;
    const unsigned lane = lane_id();
    const long long gtid = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const long long gthreads = (long long)gridDim.x * BLOCK;
    const long long gwarp = gtid >> 5;
    const long long nwarps = gthreads >> 5;
    BfsCtrl *ctrl = a.ctrl;
    WarpQ q{s_q + (threadIdx.x >> 5) * QCAP, 0};

    // ---- init ----------------------------------------------------------
    {
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
            unsigned z = a.zmask[w];
            if (root >= 0 && w == (root >> 5)) z |= 1u << (root & 31);
            a.visited[w] = z;
            a.fb0[w] = 0;
        }
        if (root >= 0 && gtid == 0) {
            a.q0[0] = root;
            ctrl->cnt[0] = 1;
            ctrl->deg[0] = (unsigned long long)(__ldg(a.row + root + 1) - __ldg(a.row + root));
        }
        if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns)) return;
        if (root >= 0) {
            if (gtid == 0) a.level[root] = 0;
        } else {
            if (blockIdx.x == 0) {
                for (int i = threadIdx.x; i < a.nroots; i += BLOCK) {
                    const int r = a.roots[i];
                    if (atomicCAS(&a.level[r], -1, 0) == -1) {
                        atomicOr(&a.visited[r >> 5], 1u << (r & 31));
                        unsigned long long pos = atomicAdd(&ctrl->cnt[0], 1ull);
                        a.q0[pos] = r;
                        atomicAdd(&ctrl->deg[0],
                                  (unsigned long long)(__ldg(a.row + r + 1) - __ldg(a.row + r)));
                    }
                }
            }
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns)) return;
        }
    }

    // ---- level loop ------------------------------------------------------
    long long m_u = a.m;                 // out-edges of not-yet-reached vertices
    unsigned long long prev_nf = 0, reached = 0, edges_c = 0, roots = 0;
    int L = 0, td_levels = 0, bu_levels = 0;
    bool td = true;
    for (;;) {
        const unsigned long long nf = ld_relaxed_u64(&ctrl->cnt[L % 3]);
        const unsigned long long mf = ld_relaxed_u64(&ctrl->deg[L % 3]);
        if (nf == 0) break;
        if (L == 0) roots = nf;
        reached += nf;
        edges_c += mf;
        m_u -= (long long)mf;
        bool bu;
        if (a.direction == GBFS_DIR_TOPDOWN) bu = false;
        else if (a.direction == GBFS_DIR_BOTTOMUP) bu = true;
        else if (td) bu = (long long)mf * a.alpha > m_u;
        else bu = !((long long)nf * a.beta < a.n_active && nf < prev_nf);
        prev_nf = nf;

        int *qc = (L & 1) ? a.q1 : a.q0;
        int *qn = (L & 1) ? a.q0 : a.q1;
        unsigned *fc = (L & 1) ? a.fb1 : a.fb0;
        unsigned *fn = (L & 1) ? a.fb0 : a.fb1;
        unsigned long long *cnt_next = &ctrl->cnt[(L + 1) % 3];
        unsigned long long *deg_next = &ctrl->deg[(L + 1) % 3];
        const int nl = L + 1;

        if (gtid == 0) {
            ctrl->cnt[(L + 2) % 3] = 0;
            ctrl->deg[(L + 2) % 3] = 0;
            ctrl->big[(L + 1) % 3] = 0;
        }

        if (bu && td) {
            // queue -> bitmap (fc was zeroed by the previous top-down step or init)
            for (long long i = gtid; i < (long long)nf; i += gthreads) {
                const int v = __ldcg(qc + i);
                atomicOr(&fc[v >> 5], 1u << (v & 31));
            }
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns)) return;
        } else if (!bu && !td) {
            // bitmap -> queue (slots from the fill counter, reset by the next
            // top-down step, which is behind the barrier below)
            for (long long w0 = gwarp * 32; w0 < W; w0 += nwarps * 32) {
                const long long w = w0 + lane;
                unsigned bits = w < W ? __ldcg(fc + w) : 0u;
                const int c = __popc(bits);
                const int incl = warp_incl_scan(c);
                const int tot = __shfl_sync(FULL, incl, 31);
                unsigned long long base = 0;
                if (lane == 31 && tot) base = atomicAdd(&ctrl->fill, (unsigned long long)tot);
                base = __shfl_sync(FULL, base, 31);
                unsigned long long pos = base + (unsigned long long)(incl - c);
                while (bits) {
                    const int bpos = __ffs(bits) - 1;
                    qc[pos++] = (int)(w * 32 + bpos);
                    bits &= bits - 1u;
                }
            }
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns)) return;
        }
        td = !bu;

        if (td) {
            ++td_levels;
            if (gtid == 0) ctrl->fill = 0;
            // zero the bitmap the next level would convert into
            for (long long w = gtid; w < W; w += gthreads) fn[w] = 0;
            unsigned long long my_deg = 0;
            for (long long base = gwarp * 32; base < (long long)nf; base += nwarps * 32) {
                const long long i = base + lane;
                int v = 0, b = 0, d = 0;
                if (i < (long long)nf) {
                    v = __ldcg(qc + i);
                    b = __ldg(a.row + v);
                    d = __ldg(a.row + v + 1) - b;
                }
                const bool isbig = d >= a.big_degree;
                const unsigned bm = __ballot_sync(FULL, isbig);
                if (bm) {
                    unsigned pos = 0;
                    const int leader = __ffs(bm) - 1;
                    if ((int)lane == leader) pos = atomicAdd(&ctrl->big[L % 3], (unsigned)__popc(bm));
                    pos = __shfl_sync(FULL, pos, leader);
                    if (isbig) a.bigl[pos + __popc(bm & lanemask_lt())] = v;
                    if (isbig) d = 0;
                }
                const int incl = warp_incl_scan(d);
                const int excl = incl - d;
                const int T = __shfl_sync(FULL, incl, 31);
                for (int e0 = 0; e0 < T; e0 += 32) {
                    const int k = e0 + (int)lane;
                    const int kk = min(k, T - 1);
                    int lo = 0;
#pragma unroll
                    for (int s = 16; s > 0; s >>= 1) {
                        const int c = lo + s;
                        if (__shfl_sync(FULL, excl, c) <= kk) lo = c;
                    }
                    const int ob = __shfl_sync(FULL, b, lo);
                    const int oe = __shfl_sync(FULL, excl, lo);
                    bool got = false;
                    int w = 0;
                    if (k < T) {
                        w = __ldg(a.col + ob + (kk - oe));
                        got = td_claim(w, a.visited, a.level, nl);
                    }
                    if (got) my_deg += __ldg(a.row + w + 1) - __ldg(a.row + w);
                    wq_push(q, got, w, cnt_next, qn);
                }
            }
            wq_flush(q, cnt_next, qn);
            {
                const unsigned long long bd = block_reduce_sum(my_deg, s_red);
                if (threadIdx.x == 0 && bd) atomicAdd(deg_next, bd);
            }
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns)) return;

            // rows deferred as too long for one warp: split over the whole grid
            const int nb = (int)__ldcg(&ctrl->big[L % 3]);
            if (nb > 0) {
                my_deg = 0;
                for (int seg = 0; seg < nb; seg += BLOCK) {
                    const int segn = min(BLOCK, nb - seg);
                    int chunks = 0;
                    if ((int)threadIdx.x < segn) {
                        const int v = __ldcg(a.bigl + seg + threadIdx.x);
                        const int b = __ldg(a.row + v), e = __ldg(a.row + v + 1);
                        s_b[threadIdx.x] = b;
                        s_e[threadIdx.x] = e;
                        chunks = (e - b + CHUNK - 1) / CHUNK;
                    }
                    int total;
                    const int ex = block_excl_scan_int(chunks, s_warp, &total);
                    s_cs[threadIdx.x] = ex;
                    __syncthreads();
                    for (long long c = gwarp; c < total; c += nwarps) {
                        int lo = 0, hi = segn - 1;  // max j with s_cs[j] <= c
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (s_cs[mid] <= c) lo = mid; else hi = mid - 1;
                        }
                        const int s = s_b[lo] + (int)(c - s_cs[lo]) * CHUNK;
                        const int e = min(s + CHUNK, s_e[lo]);
                        warp_claim_range(s, e, a, nl, q, cnt_next, qn, my_deg);
                    }
                    __syncthreads();
                }
                wq_flush(q, cnt_next, qn);
                const unsigned long long bd = block_reduce_sum(my_deg, s_red);
                if (threadIdx.x == 0 && bd) atomicAdd(deg_next, bd);
                if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns)) return;
            }
        } else {
            ++bu_levels;
            unsigned long long my_cnt = 0, my_deg = 0;
            for (long long w = gwarp; w < W; w += nwarps) {
                const unsigned vis = __ldcg(a.visited + w);
                const unsigned valid = (w == W - 1 && (n & 31)) ? ((1u << (n & 31)) - 1u) : FULL;
                const unsigned unv = ~vis & valid;
                if (unv == 0) {
                    if (lane == 0) fn[w] = 0;
                    continue;
                }
                const int v = (int)(w * 32 + lane);
                bool found = false;
                int d = 0;
                if ((unv >> lane) & 1u) {
                    const int b = __ldg(a.row + v), e = __ldg(a.row + v + 1);
                    d = e - b;
                    for (int i = b; i < e; i += 4) {
                        const int u0 = __ldg(a.col + i);
                        const int u1 = i + 1 < e ? __ldg(a.col + i + 1) : u0;
                        const int u2 = i + 2 < e ? __ldg(a.col + i + 2) : u0;
                        const int u3 = i + 3 < e ? __ldg(a.col + i + 3) : u0;
                        const unsigned f = (__ldcg(fc + (u0 >> 5)) >> (u0 & 31)) |
                                           (__ldcg(fc + (u1 >> 5)) >> (u1 & 31)) |
                                           (__ldcg(fc + (u2 >> 5)) >> (u2 & 31)) |
                                           (__ldcg(fc + (u3 >> 5)) >> (u3 & 31));
                        if (f & 1u) {
                            found = true;
                            break;
                        }
                    }
                }
                const unsigned nbm = __ballot_sync(FULL, found);
                if (found) a.level[v] = nl;
                if (lane == 0) {
                    fn[w] = nbm;
                    if (nbm) a.visited[w] = vis | nbm;
                }
                my_cnt += found;
                my_deg += found ? (unsigned long long)d : 0ull;
            }
            const unsigned long long bc = block_reduce_sum(my_cnt, s_red);
            if (threadIdx.x == 0 && bc) atomicAdd(cnt_next, bc);
            const unsigned long long bd = block_reduce_sum(my_deg, s_red);
            if (threadIdx.x == 0 && bd) atomicAdd(deg_next, bd);
            if (!grid_sync(&ctrl->bar, &ctrl->status, a.timeout_ns)) return;
        }
        ++L;
    }

    if (gtid == 0) {
        BfsOut o;
        o.levels = L;
        o.td_levels = td_levels;
        o.bu_levels = bu_levels;
        o.roots = (int)roots;
        o.reached = reached;
        o.edges_c = edges_c;
        *a.out = o;
        for (int i = 0; i < 3; i++) {
            ctrl->cnt[i] = 0;
            ctrl->deg[i] = 0;
            ctrl->big[i] = 0;
        }
        ctrl->fill = 0;
    }
}

template <int BLOCK>
size_t bfs_smem_bytes()
{
    return sizeof(int) * ((size_t)(BLOCK / 32) * QCAP + 3 * (size_t)BLOCK + 1);
}

template <int BLOCK>
cudaError_t bfs_launch(BfsArgs &args, int blocks_per_sm, cudaStream_t st, int &grid_out)
{
    static int sms = 0;
    const size_t smem = bfs_smem_bytes<BLOCK>();
    cudaError_t e;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(k_bfs<BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if (!sms && (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bfs<BLOCK>, BLOCK, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const int per = std::max(1, std::min(blocks_per_sm, occ));
    const int grid = sms * per;
    grid_out = grid;
    void *kargs[] = {&args};
    return cudaLaunchCooperativeKernel((const void *)k_bfs<BLOCK>, dim3(grid), dim3(BLOCK), kargs,
                                       smem, st);
}

}  // namespace

int bfs_work_alloc(BfsWork &w, int32_t n, std::string &err)
{
    if (w.ctrl && w.n == n) return GBFS_OK;
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
        !al((void **)&w.fb0, W * 4) || !al((void **)&w.fb1, W * 4) ||
        !al((void **)&w.q0, bytes_int) || !al((void **)&w.q1, bytes_int) ||
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
    return GBFS_OK;
}

void bfs_work_free(BfsWork &w)
{
    void *ps[] = {w.level, w.visited, w.fb0, w.fb1, w.q0, w.q1, w.big, w.roots, w.ctrl, w.d_outs};
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
    w = BfsWork{};
}

cudaError_t bfs_enqueue(const DeviceCsr &g, const gbfs_params &p, BfsWork &w, const int *d_roots, int k,
                        int single_root, int *d_level, BfsOut *slot, cudaStream_t st)
{
    BfsArgs a;
    a.n = g.n;
    a.n_active = (int)std::max<int64_t>(1, g.nonisolated);
    a.m = g.m;
    a.row = g.row;
    a.col = g.col;
    a.zmask = g.zmask;
    a.level = d_level;
    a.visited = w.visited;
    a.fb0 = w.fb0;
    a.fb1 = w.fb1;
    a.q0 = w.q0;
    a.q1 = w.q1;
    a.bigl = w.big;
    a.ctrl = w.ctrl;
    a.out = slot;
    a.roots = d_roots;
    a.nroots = k;
    a.single_root = single_root;
    a.alpha = std::max(1, p.alpha);
    a.beta = std::max(1, p.beta);
    a.big_degree = std::max(32, p.big_degree);
    a.direction = p.direction;
    a.timeout_ns = (unsigned long long)std::max(1, p.timeout_ms) * 1000000ull;
    int grid = 0;
    switch (p.threads_per_block) {
    case 256: return bfs_launch<256>(a, p.blocks_per_sm, st, grid);
    case 1024: return bfs_launch<1024>(a, p.blocks_per_sm, st, grid);
    default: return bfs_launch<512>(a, p.blocks_per_sm, st, grid);
    }
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
            int single_root, int *d_level, cudaStream_t st, BfsResult &res, std::string &err)
{
    cudaError_t e = cudaEventRecord(w.ev0, st);
    if (e == cudaSuccess) e = bfs_enqueue(g, p, w, d_roots, k, single_root, d_level, &w.ctrl->out, st);
    if (e == cudaSuccess) e = cudaEventRecord(w.ev1, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w.h_ctrl, w.ctrl, sizeof(BfsCtrl), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        err = std::string("BFS launch: ") + cudaGetErrorString(e);
        return GBFS_ERR_CUDA;
    }
    const BfsCtrl &h = *w.h_ctrl;
    if (h.status != DEV_OK) {
        cudaMemsetAsync(w.ctrl, 0, sizeof(BfsCtrl), st);
        cudaStreamSynchronize(st);
        err = "a device-side wait ran out (grid barrier)";
        return GBFS_ERR_TIMEOUT;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, w.ev0, w.ev1);
    res.ms = ms;
    res.levels = h.out.levels;
    res.td_levels = h.out.td_levels;
    res.bu_levels = h.out.bu_levels;
    res.launches = 1;
    res.roots = h.out.roots;
    res.reached = (int64_t)h.out.reached;
    res.edges_c = (int64_t)h.out.edges_c;
    return GBFS_OK;
}

}  // namespace gbfs
