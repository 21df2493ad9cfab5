// bfs_args.cuh -- launch arguments shared by the single-source kernels:
// the persistent grid kernel (bfs.cu) and the label-correcting kernel
// (bfs_relax.cu) that finishes long searches on graphs of small degree.
#pragma once

#include "bfs.cuh"

namespace gbfs {

struct BfsArgs {
    int n;
    int n_active;            // non-isolated vertices (for beta)
    long long m;
    int wide;                // 64-bit row offsets: row64 / brow64 / qb64 instead of row / brow / qb
    const int *row;
    const long long *row64;
    const int *col;
    const int *brow, *bcol;  // bottom-up adjacency: in-edges (row/col when symmetric)
    const long long *brow64;
    const int *bfirst;       // first entry of each brow row (-1: empty row)
    const int *bsecond;      // second entries (-1 past the end); null: probe the first alone
    const unsigned *zmask;   // out-degree-0 bitmap, or NULL (directed graphs:
                             // a sink still has in-edges, so it stays claimable)
    int *level;
    unsigned *visited;
    unsigned *fb[3];         // frontier bitmaps, rotating by level
    int *q0, *q1;            // frontier queues
    int2 *qb[2];             // row bounds beside q0 and q1
    longlong2 *qb64[2];      // the same for wide graphs
    int *bigl;
    BfsCtrl *ctrl;
    BfsOut *out;
    const int *roots;
    int nroots;
    int single_root;         // >= 0: fast init for one root
    int resume;              // 1: continue the level loop saved in ctrl->rs
    int max_steps;           // > 0: leave after this many levels (state saved)
    int alpha, beta, big_degree, direction;
    int has_big;             // some row has big_degree entries or more (else none is ever deferred)
    int max_degree;          // largest out-degree
    // the grid kernel may park its level loop for the label-correcting
    // kernel launched right after it: from level yield_level on, at a
    // top-down frontier of at most yield_max_f vertices
    int may_yield;
    int yield_level;
    int yield_max_f;
    unsigned long long timeout_ns;
};

// Row-offset type RT of the kernels (int, or long long on wide graphs): the
// matching row pointers, row-bound pairs and queue bound arrays.
template <typename RT>
struct RowSel;
template <>
struct RowSel<int> {
    using B = int2;
    __device__ static const int *row(const BfsArgs &a) { return a.row; }
    __device__ static const int *brow(const BfsArgs &a) { return a.brow; }
    __device__ static int2 *qb(const BfsArgs &a, int i) { return a.qb[i]; }
    __host__ __device__ static int2 mk(int x, int y) { return make_int2(x, y); }
};
template <>
struct RowSel<long long> {
    using B = longlong2;
    __device__ static const long long *row(const BfsArgs &a) { return a.row64; }
    __device__ static const long long *brow(const BfsArgs &a) { return a.brow64; }
    __device__ static longlong2 *qb(const BfsArgs &a, int i) { return a.qb64[i]; }
    __host__ __device__ static longlong2 mk(long long x, long long y) { return make_longlong2(x, y); }
};
template <typename RT>
using BndT = typename RowSel<RT>::B;

// The label-correcting kernel (bfs_relax.cu), queued after a grid launch
// with may_yield set: it finishes a search the grid launch parked.
cudaError_t bfs_relax_launch(const BfsArgs &args, cudaStream_t st, int max_ctas);

}  // namespace gbfs
