// bfs_args.cuh -- launch arguments shared by the single-source kernels:
// the persistent grid kernel (bfs.cu) and the sparse-phase cluster kernel
// (bfs_sparse.cu), which continue one another's level loop.
#pragma once

#include "bfs.cuh"

namespace gbfs {

struct BfsArgs {
    int n;
    int n_active;            // non-isolated vertices (for beta)
    long long m;
    const int *row;
    const int *col;
    const int *brow, *bcol;  // bottom-up adjacency: in-edges (row/col when symmetric)
    const int *bfirst;       // first entry of each brow row (-1: empty row)
    const int *bsecond;      // second entries (-1 past the end); null: probe the first alone
    const unsigned *zmask;   // out-degree-0 bitmap, or NULL (directed graphs:
                             // a sink still has in-edges, so it stays claimable)
    int *level;
    unsigned *visited;
    unsigned *fb[3];         // frontier bitmaps, rotating by level
    int *q0, *q1;            // frontier queues
    int2 *qb[2];             // row bounds beside q0 and q1
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
    // sparse phase: the grid kernel may hand a run of small top-down
    // frontiers (at most sparse_enter_f vertices) to the cluster kernel
    // launched right after it, from level yield_level on, when each of the
    // cluster's sparse_ctas CTAs can hold the next frontier
    // (ceil(frontier / sparse_ctas) * max_degree entries <= sparse_cap); the
    // cluster kernel hands back frontiers of more than sparse_leave_f
    int may_yield;
    int yield_level;
    int sparse_ctas;
    int sparse_cap;
    int sparse_enter_f;
    int sparse_leave_f;
    unsigned long long timeout_ns;
};

// The sparse-phase cluster kernel (bfs_sparse.cu): its cluster size (0 when
// no such cluster fits this device) and per-CTA queue capacity, and its
// launch (one cluster, after a grid launch with may_yield set).
cudaError_t bfs_sparse_shape(int &ctas, int &cap);
cudaError_t bfs_sparse_launch(const BfsArgs &args, cudaStream_t st);

}  // namespace gbfs
