// scan.cuh -- single-pass exclusive prefix sum with decoupled look-back.
//
// Replaces the reference's three-launch recursive Blelloch scan
// (2D Partition/src/prefixSum.cu:15-224, which cudaMallocs and frees its
// block-sum arrays on every call) with one launch: each tile of
// SCAN_THREADS * SCAN_ITEMS elements is staged through shared memory (loads
// and stores coalesced), scans itself with warp shuffles, publishes its
// aggregate, looks back over its predecessors' published aggregates /
// inclusive prefixes 32 at a time (one warp), and publishes its inclusive
// prefix.
// Tiles take ids from an atomic counter in launch order, so a tile only
// ever waits on tiles that are already running.  The scratch is
// self-cleaning (epoch-tagged flags, counters reset by the last tile), so
// repeated calls need no memset.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbfs {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

struct ScanScratch {
    unsigned *flags = nullptr;      // per tile: (epoch << 2) | {1 agg, 2 inclusive}
    long long *agg = nullptr;       // per tile aggregate
    long long *inc = nullptr;       // per tile inclusive prefix
    unsigned *ctl = nullptr;        // [0] tile ticket, [1] tiles done, [2] status
    int64_t max_tiles = 0;
    unsigned epoch = 0;             // host-side call counter
};

// Bytes of scratch for up to `max_tiles` tiles (one allocation, carved).
size_t scan_scratch_bytes(int64_t max_tiles);
// Carve `mem` (scan_scratch_bytes(max_tiles) bytes, zeroed once) into s.
void scan_scratch_carve(void *mem, int64_t max_tiles, ScanScratch &s);
inline int64_t scan_tiles(int64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

// out[i] = sum(in[0..i)); *total_out (nullable, device) = sum(in[0..n)).
cudaError_t scan_exclusive_i32_i32(const int *in, int *out, int64_t n, int *total_out,
                                   ScanScratch &s, cudaStream_t st);
cudaError_t scan_exclusive_i32_i64(const int *in, long long *out, int64_t n,
                                   long long *total_out, ScanScratch &s, cudaStream_t st);

}  // namespace gbfs
