// parents.cu -- BFS-tree parents from a finished level array (sm_103a).
//
// The reference's 2D CPU BFS keeps a predecessor per vertex, the frontier
// vertex that happened to discover it first (2D Partition/src/cpuBFS.cpp:16,56);
// its GPU counterpart (d_pred, 2D Partition/include/gpuBFS.cuh:45) inherits
// whatever order the threads ran in.  Here the parent is canonical:
//
//     parent[v] = min { u : edge u -> v, level[u] == level[v] - 1 }
//
// and -1 for the source and for unreached vertices, so one graph and source
// give one parent array and every entry is a valid BFS-tree parent.
//
// Symmetric graphs pull: each reached vertex scans its own row for the
// smallest neighbour one level closer (one thread per light row, one warp
// per row of degree > HEAVY_DEGREE), no atomics.  Directed graphs push: every
// reached u offers itself to the out-neighbours one level further with
// atomicMin, after a plain-load filter (parent values only decrease).
#include <algorithm>
#include <climits>

#include "common.cuh"
#include "parents.cuh"

namespace gbfs {

namespace {

constexpr int PT = 256;

template <typename RT>
__global__ void k_parents_pull_light(const RT *__restrict__ row, const int *__restrict__ col, int n,
                                     const int *__restrict__ level, int *__restrict__ parent)
{
    for (long long v = (long long)blockIdx.x * PT + threadIdx.x; v < n; v += (long long)gridDim.x * PT) {
        const int lv = level[v];
        const RT b = row[v], e = row[v + 1];
        if (lv > 0 && e - b > HEAVY_DEGREE) continue;  // the heavy kernel's row
        int best = -1;
        if (lv > 0) {
            best = INT_MAX;
            for (RT i = b; i < e; i++) {
                const int u = col[i];
                if (u < best && level[u] == lv - 1) best = u;
            }
        }
        parent[v] = best;
    }
}

template <typename RT>
__global__ void k_parents_pull_heavy(const RT *__restrict__ row, const int *__restrict__ col,
                                     const int *__restrict__ heavy, int nheavy, const int *__restrict__ level,
                                     int *__restrict__ parent)
{
    const long long gw = ((long long)blockIdx.x * PT + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * PT) >> 5;
    const int lane = threadIdx.x & 31;
    for (long long h = gw; h < nheavy; h += nw) {
        const int v = heavy[h];
        const int lv = level[v];
        if (lv <= 0) continue;  // written by the light kernel
        int best = INT_MAX;
        for (RT i = row[v] + lane; i < row[v + 1]; i += 32) {
            const int u = col[i];
            if (u < best && level[u] == lv - 1) best = u;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(FULL, best, o));
        if (lane == 0) parent[v] = best;
    }
}

__global__ void k_parents_init(int n, const int *__restrict__ level, int *__restrict__ parent)
{
    for (long long v = (long long)blockIdx.x * PT + threadIdx.x; v < n; v += (long long)gridDim.x * PT)
        parent[v] = level[v] > 0 ? INT_MAX : -1;
}

// one warp per vertex u: offer u to the out-neighbours one level further
template <typename RT>
__global__ void k_parents_push(const RT *__restrict__ row, const int *__restrict__ col, int n,
                               const int *__restrict__ level, int *parent)
{
    const long long gw = ((long long)blockIdx.x * PT + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * PT) >> 5;
    const int lane = threadIdx.x & 31;
    for (long long u = gw; u < n; u += nw) {
        const int lu = level[u];
        if (lu < 0) continue;
        for (RT i = row[u] + lane; i < row[u + 1]; i += 32) {
            const int v = col[i];
            if (level[v] == lu + 1 && parent[v] > (int)u) atomicMin(parent + v, (int)u);
        }
    }
}

int grid_of(long long work, int cap)
{
    long long b = (work + PT - 1) / PT;
    return (int)std::max(1LL, std::min<long long>(b, cap));
}

}  // namespace

namespace {

template <typename RT>
cudaError_t parents_launch(const DeviceCsr &g, const RT *row, bool symmetric, const int *d_level, int *d_parent,
                           cudaStream_t st)
{
    if (symmetric) {
        k_parents_pull_light<RT><<<grid_of(g.n, 152 * 16), PT, 0, st>>>(row, g.col, g.n, d_level, d_parent);
        if (g.nheavy > 0)
            k_parents_pull_heavy<RT><<<grid_of((long long)g.nheavy * 32, 152 * 16), PT, 0, st>>>(
                row, g.col, g.heavy, g.nheavy, d_level, d_parent);
    } else {
        k_parents_init<<<grid_of(g.n, 152 * 16), PT, 0, st>>>(g.n, d_level, d_parent);
        k_parents_push<RT><<<grid_of((long long)g.n * 32, 152 * 16), PT, 0, st>>>(row, g.col, g.n, d_level, d_parent);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t parents_enqueue(const DeviceCsr &g, bool symmetric, const int *d_level, int *d_parent, cudaStream_t st)
{
    if (g.n == 0) return cudaSuccess;
    return g.wide ? parents_launch(g, (const long long *)g.row64, symmetric, d_level, d_parent, st)
                  : parents_launch(g, (const int *)g.row, symmetric, d_level, d_parent, st);
}

}  // namespace gbfs
