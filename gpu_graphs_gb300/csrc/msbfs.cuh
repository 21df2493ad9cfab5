// msbfs.cuh -- 64-lane multi-source BFS (host side of msbfs.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "common.cuh"
#include "bfs.cuh"
#include "csr_build.cuh"

namespace gbfs {

constexpr int MS_LANES = 64;
constexpr int MS_PIECE = 2048;           // edges of a huge row one warp takes in a pull step
constexpr int MS_HUGE = 2 * MS_PIECE;    // rows longer than this are split into pieces

struct MsCtrl {
    GridBarrier bar;
    int status;
    int pad0;
    unsigned long long qcnt[4];  // active-queue lengths, rotating by level
    unsigned long long alive[4]; // lanes with a non-empty frontier, rotating by level
    unsigned long long big[2];   // long rows a push step deferred to its grid-wide pass
    int levels, push_levels, pull_levels, trace_len;
    unsigned long long reached, edges_c;
    unsigned long long t_entry, t_start, t_end;
    unsigned long long t_exit;     // the last CTA leaving the kernel (after the closing pass)
    LevelTrace trace[TRACE_CAP];   // per level: frontier = active vertices
};

struct MsWork {
    int32_t n = 0;
    unsigned long long *vis = nullptr;   // n lane masks: lanes that reached v
    unsigned long long *F[3] = {nullptr, nullptr, nullptr};  // frontier masks, rotating
    int *Q[4] = {nullptr, nullptr, nullptr, nullptr};        // active queues, rotating
    unsigned long long *hacc = nullptr;  // n: per huge row, lanes its pull pieces found
    unsigned *hcnt = nullptr;            // n: per huge row, pieces done this level
    unsigned char *lv8 = nullptr;        // MS_LANES * n levels as bytes while the search runs
    int *bigl = nullptr;                 // n: long rows deferred by a push step
    int *out = nullptr;                  // MS_LANES * n levels (host-bound results)
    int *src = nullptr;                  // MS_LANES sources
    MsCtrl *ctrl = nullptr;
    MsCtrl *h_ctrl = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int64_t bytes = 0;
};

// Split the huge rows into pull pieces (DeviceCsr::pieces, and tpieces for
// the transpose once it exists); a no-op once built.  Synchronises st.
int ms_prepare(DeviceCsr &g, cudaStream_t st, std::string &err);
// Device bytes ms_prepare adds to a graph (`transpose`: count the pieces of
// the transpose too, built or about to be).
int64_t ms_prepare_bytes(const DeviceCsr &g, bool transpose);

// Device bytes ms_work_alloc takes for n vertices.
int64_t ms_work_bytes(int64_t n);

int ms_work_alloc(MsWork &w, int32_t n, std::string &err);
void ms_work_free(MsWork &w);

struct MsResult {
    float ms = 0;
    int levels = 0, push_levels = 0, pull_levels = 0;
    int64_t reached = 0, edges_c = 0;
};

// Enqueue one launch: k <= 64 sources (device array d_src); d_out: k*n
// int32, row i = levels of source i; results land in w.ctrl.  max_ctas > 0
// caps the grid (concurrent launches on several streams must fit on the GPU
// together, since every launch waits on all of its own CTAs).  Pull steps
// gather over in-edges: the rows themselves when `symmetric`, else the
// transpose if it has been built (top-down only without it).  No sync.
cudaError_t msbfs_enqueue(const DeviceCsr &g, const gbfs_params &p, bool symmetric, MsWork &w,
                          const int *d_src, int k, int *d_out, cudaStream_t st, int max_ctas);

// CTAs of one full-GPU multi-source launch (0 on error).
int ms_max_ctas();

// msbfs_enqueue + read-back.  Synchronises `st`.
int msbfs_run(const DeviceCsr &g, const gbfs_params &p, bool symmetric, MsWork &w,
              const int *d_src, int k, int *d_out, cudaStream_t st, MsResult &res,
              std::string &err);

}  // namespace gbfs
