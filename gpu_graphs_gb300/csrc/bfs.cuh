// bfs.cuh -- single-GPU direction-optimising BFS (host side of bfs.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "common.cuh"
#include "csr_build.cuh"

namespace gbfs {

// Device control block of one traversal context.  Zeroed at allocation; the
// kernel leaves it zeroed on success (the host re-zeroes it after an error).
// One row of the per-level trace (thread 0 writes it after the level's barrier).
struct LevelTrace {
    int level;                   // frontier index L expanded by this step
    int dir;                     // 0 top-down, 1 bottom-up, +2 if a grid-split pass ran,
                                 // 4 one round of the label-correcting kernel (up to
                                 // RX_HOPS levels; `level` counts rounds on from the
                                 // level it took over at)
    unsigned long long frontier; // vertices in frontier L
    unsigned long long edges;    // their out-edges
    unsigned long long t_ns;     // %globaltimer when the step's last barrier completed
};
constexpr int TRACE_CAP = 16384;  // levels kept (the first TRACE_CAP - 1, then the last)

// Results of one traversal, written by the kernel's thread 0.
struct BfsOut {
    int levels, td_levels, bu_levels, roots;   // roots: distinct vertices at level 0
    unsigned long long reached, edges_c;
};

// Who continues a parked level loop (BfsResume::mode).
enum ResumeMode : int {
    RESUME_LEVEL = 0,     // per-level-launch mode: the next grid launch
    RESUME_RELAX = 1,     // the label-correcting kernel (bfs_relax.cu), to the end
};

// Level-loop state kept between launches (per-level-launch mode, and the
// hand-over from the grid kernel to the label-correcting kernel).
struct BfsResume {
    long long m_u;
    unsigned long long prev_nf, reached, edges_c, roots, prev_mf;
    int L, td_levels, bu_levels, td, done, dirty;  // dirty: frontier bitmaps that may hold set bits
    int mode, pad;                                 // mode: ResumeMode
};

// A frontier's vertex count and out-degree sum share one 64-bit word (count
// in the low half, degree sum in the high half: both below 2^31, so the
// halves never carry into each other), so a CTA adds both, and gets its
// queue slots, with one atomic.
__host__ __device__ inline unsigned long long cd_pack(unsigned long long cnt, unsigned long long deg)
{
    return (deg << 32) | cnt;
}
__host__ __device__ inline unsigned long long cd_count(unsigned long long cd) { return cd & 0xffffffffull; }
__host__ __device__ inline unsigned long long cd_degree(unsigned long long cd) { return cd >> 32; }

struct BfsCtrl {
    GridBarrier bar;
    int status;
    int pad0;
    unsigned long long cd[3];    // frontier count | out-degree sum (cd_pack), rotating by level
    unsigned big[3];             // top-down rows deferred to the grid pass
    unsigned pad1;
    unsigned long long fill;     // bitmap -> queue conversion slots
    BfsOut out;                  // results of the last traversal (default slot)
    BfsResume rs;                // per-level-launch mode: state between launches
    unsigned long long rx_reached, rx_edges;  // label-correcting phase: first relaxations
    int rx_max;                  // and the largest level
    int pad4;
    unsigned long long t_entry;  // %globaltimer when CTA 0 started
    unsigned long long t_start;  // %globaltimer after initialisation
    unsigned long long t_end;    // %globaltimer when CTA 0 left the level loop
    unsigned long long t_exit;   // %globaltimer when the last CTA left the kernel
    int trace_len;
    int pad3;
    LevelTrace trace[TRACE_CAP];
};

// Per-graph traversal workspace (allocated on first use, reused).
struct BfsWork {
    int32_t n = 0;
    int *level = nullptr;        // n (used when the caller's buffer is on the host)
    unsigned *visited = nullptr; // W
    unsigned *fb0 = nullptr;     // W frontier bitmaps (three, rotating)
    unsigned *fb1 = nullptr;
    unsigned *fb2 = nullptr;
    int *q0 = nullptr;           // n frontier queues
    int *q1 = nullptr;
    int2 *qb0 = nullptr;         // n row bounds (row[v], row[v + 1]) beside q0 / q1
    int2 *qb1 = nullptr;         // (16-byte longlong2 entries when `wide`)
    bool wide = false;           // sized for a graph with 64-bit row offsets
    int *big = nullptr;          // n deferred rows
    int *roots = nullptr;        // root staging (n)
    BfsCtrl *ctrl = nullptr;
    BfsCtrl *h_ctrl = nullptr;   // pinned mirror for results
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // back-to-back launches: per-launch result slots and events
    BfsOut *d_outs = nullptr;
    BfsOut *h_outs = nullptr;
    int outs_cap = 0;
    cudaEvent_t *evs = nullptr;
    int evs_cap = 0;
    // back-to-back launches with host output: a second level buffer and a
    // copy stream, so the copy of one result overlaps the next traversal
    int *level2 = nullptr;
    cudaStream_t copy_st = nullptr;
    cudaEvent_t ev_ready[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
    // graph-captured per-level launches (per_level_launch == 2): the
    // instantiated graph and the launch arguments / shape it was built for
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    unsigned char graph_key[320] = {};
    int graph_shape[3] = {0, 0, 0};
    int64_t bytes = 0;
};

void bfs_graph_free(BfsWork &w);

// Allocate the second level buffer, the copy stream and its events.
int bfs_work_reserve_overlap(BfsWork &w, std::string &err);

int bfs_work_alloc(BfsWork &w, int32_t n, std::string &err, bool wide = false);
void bfs_work_free(BfsWork &w);

struct BfsResult {
    float ms = 0;
    int levels = 0, td_levels = 0, bu_levels = 0, launches = 0, roots = 0;
    int64_t reached = 0, edges_c = 0;
};

// Enqueues one (multi-root) BFS of `g` writing levels to d_level (device, n
// int32) and its results to *slot (device).  d_roots: device array of k
// roots, or single_root >= 0.  symmetric: in-edges == out-edges (enables the
// zero-degree shortcut; bottom-up must already be off in `p` otherwise).
// Does not synchronise.
cudaError_t bfs_enqueue(const DeviceCsr &g, const gbfs_params &p, BfsWork &w, const int *d_roots, int k,
                        int single_root, int *d_level, BfsOut *slot, cudaStream_t st, bool symmetric,
                        int resume = 0, int max_steps = 0, int max_ctas = 0);

// bfs_enqueue + events + result read-back; synchronises `st`.  With
// p.per_level_launch, one launch per level and a host read-back of the
// level count after each (the reference's loop shape).
int bfs_run(const DeviceCsr &g, const gbfs_params &p, BfsWork &w, const int *d_roots, int k,
            int single_root, int *d_level, cudaStream_t st, BfsResult &res, std::string &err, bool symmetric);

// Whether a search with these parameters on graph g ends in the
// label-correcting kernel, and the kernel launches one search enqueues
// (2 then, else 1).
bool bfs_relax_tail(const DeviceCsr &g, const gbfs_params &p);
int bfs_launches_per_search(const DeviceCsr &g, const gbfs_params &p);

// CTAs of one full-GPU single-source launch with these parameters (0 on error).
int bfs_max_ctas(const gbfs_params &p);

// Grow the per-launch slots / events of `w` to at least `k`.
int bfs_work_reserve_many(BfsWork &w, int k, std::string &err);

}  // namespace gbfs
