// parents.cuh -- canonical BFS-tree parents from a level array.
#pragma once

#include <cuda_runtime.h>

#include "csr_build.cuh"

namespace gbfs {

// parent[v] = smallest u with an edge u -> v and level[u] == level[v] - 1;
// -1 for level <= 0 (the source, unreached).  d_level must be a complete BFS
// level array of g.  Enqueued on st; no sync.
cudaError_t parents_enqueue(const DeviceCsr &g, bool symmetric, const int *d_level, int *d_parent, cudaStream_t st);

}  // namespace gbfs
