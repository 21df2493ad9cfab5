// csr_build.cuh -- on-device edge list -> CSR builder.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace gbfs {

// A CSR resident in HBM.  Rows of graphs built from edges are sorted
// ascending.  zmask bit v is set when out-degree(v) == 0.
struct DeviceCsr {
    int32_t n = 0;
    int64_t m = 0;
    int *row = nullptr;        // n+1 (null when wide)
    long long *row64 = nullptr;  // n+1, wide graphs only: 64-bit row offsets (more than 2^31-1 edges)
    bool wide = false;
    int *col = nullptr;        // m
    unsigned *zmask = nullptr; // (n+31)/32
    int32_t max_degree = 0;
    int64_t nonisolated = 0;
    int *heavy = nullptr;      // vertices of out-degree > HEAVY_DEGREE (any order)
    int32_t nheavy = 0;
    // each row's first and second entries, -1 where the row is shorter (with
    // hub-first rows, the first is the highest-degree neighbour): bottom-up's
    // first probe, read coalesced
    int *first = nullptr;      // n
    int *second = nullptr;     // n; not allocated for hub-first rows (probed at the first entry alone)
    bool hub_rows = false;     // rows are hub-first (csr_hub_first ran)
    // multi-source pull pieces (built on demand by ms_prepare): every row of
    // degree > 2 * MS_PIECE contributes {vertex, j} for its j-th MS_PIECE edges
    int2 *pieces = nullptr;
    int32_t npieces = 0;
    bool pieces_built = false;
    // transpose (in-edges), built on demand for bottom-up steps on graphs
    // whose in-edges differ from their out-edges; rows unsorted
    int *trow = nullptr;       // n+1
    int *tcol = nullptr;       // m
    int *tfirst = nullptr;     // n: the transpose's first entries (its rows are hub-first)
    int *theavy = nullptr;     // vertices of in-degree > HEAVY_DEGREE (built with the transpose)
    int32_t ntheavy = 0;
    // multi-source pull pieces over the transpose (ms_prepare, once trow exists)
    int2 *tpieces = nullptr;
    int32_t ntpieces = 0;
    bool tpieces_built = false;
};

// Rows longer than this are walked by a whole warp in multi-source passes.
constexpr int HEAVY_DEGREE = 64;

// Build from device edge arrays (m entries each).  Returns a GBFS_* status;
// on failure `err` says why.  All work is ordered on `st`; the call
// synchronises `st` before returning.  The row offsets are 64-bit (`wide`)
// when the edges to store could exceed 2^31-1, or with GBFS_WIDE_ROWS.
int csr_build_from_edges(int32_t n, int64_t m, const int *d_src, const int *d_dst,
                         unsigned flags, cudaStream_t st, DeviceCsr &out, std::string &err);

// Take an existing device CSR (row n+1, col m; ownership moves to `out`),
// validate it and compute zmask / max_degree / nonisolated.
int csr_adopt(int32_t n, int64_t m, int *d_row, int *d_col, cudaStream_t st, DeviceCsr &out,
              std::string &err);
// The same with 64-bit row offsets (a wide graph).
int csr_adopt64(int32_t n, int64_t m, long long *d_row, int *d_col, cudaStream_t st, DeviceCsr &out,
                std::string &err);

// in-edges == out-edges?  Rows need not be sorted (a sorted copy is checked).
int csr_check_symmetric(const DeviceCsr &c, cudaStream_t st, bool &sym, std::string &err);

// Move each row's highest-degree neighbour to the row's front.
int csr_hub_first(DeviceCsr &c, cudaStream_t st, std::string &err);

// Build c.trow / c.tcol (the in-edge CSR, rows hub-first) with c.tfirst and
// c.theavy; a no-op once built.  Synchronises st.  Not for wide graphs
// (GBFS_ERR_TOO_LARGE: their searches stay top-down).
int csr_build_transpose(DeviceCsr &c, cudaStream_t st, std::string &err);

// (Re)compute c.first / c.second from the rows as they are now.  Synchronises st.
int csr_build_first(DeviceCsr &c, cudaStream_t st, std::string &err);

// Device bytes held by the CSR and everything built on it.
int64_t csr_device_bytes(const DeviceCsr &c);

void csr_free(DeviceCsr &c);

}  // namespace gbfs
