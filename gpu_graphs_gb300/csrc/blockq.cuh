// blockq.cuh -- warp/CTA queue and reduction helpers shared by the
// persistent kernels (bfs.cu, msbfs.cu).
#pragma once

#include "common.cuh"

namespace gbfs {

constexpr int QCAP = 256;    // per-warp staging queue entries

// A warp's staging queue in shared memory (n is warp-uniform).
struct WarpQ {
    int *buf;
    int n;
};

// Append the warp's staged entries to out[] with one global atomic.  The
// queue position is the low 32 bits of the counter (a counter may carry a
// second sum in its high half, see cd_pack in bfs.cuh).
__device__ __forceinline__ void wq_flush(WarpQ &q, unsigned long long *cnt, int *out)
{
    __syncwarp();
    if (q.n == 0) return;
    unsigned long long base = 0;
    if (lane_id() == 0) base = atomicAdd(cnt, (unsigned long long)q.n) & 0xffffffffull;
    base = __shfl_sync(FULL, base, 0);
    for (int i = lane_id(); i < q.n; i += 32) out[base + i] = q.buf[i];
    __syncwarp();
    q.n = 0;
}

// All 32 lanes call; lanes with `has` stage v.
__device__ __forceinline__ void wq_push(WarpQ &q, bool has, int v, unsigned long long *cnt, int *out)
{
    unsigned m = __ballot_sync(FULL, has);
    if (!m) return;
    int c = __popc(m);
    if (q.n + c > QCAP) wq_flush(q, cnt, out);
    if (has) q.buf[q.n + __popc(m & lanemask_lt())] = v;
    q.n += c;
}

// Flush every warp queue of the block with one global atomic (all threads call).
__device__ __forceinline__ void block_flush(WarpQ &q, unsigned long long *cnt, int *out, int *s_wq,
                                            unsigned long long *s_base)
{
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncwarp();
    if (lane_id() == 0) s_wq[w] = q.n;
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int i = 0; i < nw; i++) {
            const int c = s_wq[i];
            s_wq[i] = tot;
            tot += c;
        }
        *s_base = tot ? atomicAdd(cnt, (unsigned long long)tot) : 0ull;
    }
    __syncthreads();
    const unsigned long long base = *s_base + (unsigned long long)s_wq[w];
    for (int i = lane_id(); i < q.n; i += 32) out[base + i] = q.buf[i];
    q.n = 0;
    __syncthreads();
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

}  // namespace gbfs
