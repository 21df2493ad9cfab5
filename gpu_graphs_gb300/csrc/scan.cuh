// scan.cuh -- single-pass exclusive prefix sum with decoupled look-back.
//
// Replaces the reference's three-launch recursive Blelloch scan
// (2D Partition/src/prefixSum.cu:15-224, which cudaMallocs and frees its
// block-sum arrays on every call) with one launch, one CTA per tile of
// SCAN_TILE elements: the tile is bulk-copied (TMA) into shared memory, each
// warp reads its run of consecutive elements as 16-byte vectors interleaved
// by lane, the tile publishes its aggregate, looks back over its
// predecessors' published aggregates / inclusive prefixes (the whole CTA,
// 256 predecessors per step, one round trip each: value and status share a
// 16-byte word), publishes its inclusive prefix and writes its outputs from
// registers as 16-byte coalesced stores.  Small shared memory and few
// registers keep several tiles in flight per SM.
// A tile waits only on tiles with smaller indices, which start first.  The
// tile states carry a call number (epoch), so repeated calls need no
// clearing of them.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbfs {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 32;      // elements per thread (SCAN_TILE = 8192)
constexpr int SCAN_MIN_BLOCKS = 6;  // CTAs per SM the register budget is sized for
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// A tile's published aggregate or inclusive prefix and its status,
// (call number << 2) | {1 aggregate, 2 inclusive}, in one 16-byte word.
struct alignas(16) ScanDesc {
    long long value;
    unsigned long long status;
};

struct ScanScratch {
    ScanDesc *desc = nullptr;       // per tile
    unsigned *ctl = nullptr;        // [2] status (a bounded wait ran out); [0], [1] unused
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
