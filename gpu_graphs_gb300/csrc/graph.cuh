// graph.cuh -- the opaque handle types behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "bfs.cuh"
#include "csr_build.cuh"
#include "msbfs.cuh"

struct gbfs_graphset;

struct gbfs_graph {
    gbfs::DeviceCsr csr;
    gbfs_params params{};        // read and written only under pmu (graph_params / set)
    mutable std::mutex pmu;
    gbfs::BfsWork work;
    gbfs::MsWork ms;
    cudaStream_t stream = nullptr;
    int device = 0;
    bool symmetric = false;      // in-edges == out-edges (bottom-up allowed)
    bool last_multi = false;     // the last traversal was multi-source (trace source)
    std::mutex mu;
    // graph set cached by gbfs_bfs_batch_graphs (keyed by the handle list)
    std::vector<const gbfs_graph *> batch_key;
    gbfs_graphset *batch_set = nullptr;
};

struct gbfs_graphset {
    gbfs_graph *g = nullptr;           // the disjoint union
    std::vector<int64_t> offsets;      // count+1 vertex offsets
    std::vector<int32_t> sizes;        // n of each member
};

namespace gbfs {

// A copy of the graph's traversal parameters (other threads may set them).
inline gbfs_params graph_params(const gbfs_graph *g)
{
    std::lock_guard<std::mutex> lk(g->pmu);
    return g->params;
}

inline void graph_set_params(gbfs_graph *g, const gbfs_params &p)
{
    std::lock_guard<std::mutex> lk(g->pmu);
    g->params = p;
}

// thread-local error detail
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
bool is_device_ptr(const void *p);
int cuda_fail(cudaError_t e, const char *what);

// Make a handle around a built CSR (takes ownership of csr).
int graph_wrap(DeviceCsr &csr, bool symmetric_known, bool symmetric, cudaStream_t st,
               gbfs_graph **out);

}  // namespace gbfs
