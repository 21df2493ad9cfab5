/*
 * gbfs_graphbfs.hpp -- the reference's host classes over the gbfs C ABI.
 *
 * Header-only C++ mirror of the graphBFS host interface of YKMorsy/GPU_Graphs:
 *   csr(const char* filename)      1D Partition/include/csr.h:9-23
 *   gpuBFS(csr& graph, int source) 1D Partition/include/gpuBFS.cuh:9-54
 * with the same public members, so the reference's drivers
 * (1D Partition/main.cu:10-82) compile against it unchanged in spirit:
 *   csr graph(file);  gpuBFS bfs(graph, source);  bfs.host_distance[v] ...
 * Differences, on purpose: ids in the file are 1-based and converted like
 * 2D Partition/src/csc.cpp:24 (the 1D loader skips that conversion and
 * writes out of bounds); unreachable vertices are -1; errors throw
 * gbfs::error instead of exit(EXIT_FAILURE); a missing file prints the
 * reference's "Error: Unable to open file" line and then throws.
 */
#ifndef GBFS_GRAPHBFS_HPP
#define GBFS_GRAPHBFS_HPP

#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>

#include "gbfs.h"

namespace gbfs {

struct error : std::runtime_error {
    int code;
    error(int c, const std::string &where)
        : std::runtime_error(where + ": " + gbfs_strerror(c) + " (" + gbfs_last_error() + ")"), code(c) {}
};

inline void check(int rc, const char *where)
{
    if (rc != GBFS_OK) throw error(rc, where);
}

class csr {
public:
    explicit csr(const char *filename, uint32_t flags = 0)
    {
        int32_t *src = nullptr, *dst = nullptr;
        int64_t m = 0;
        int rc = gbfs_read_edge_list(filename, 1, &num_nodes, &m, &src, &dst);
        if (rc == GBFS_ERR_IO && std::string(gbfs_last_error()).rfind("Unable to open", 0) == 0)
            std::cerr << "Error: Unable to open file " << filename << "\n";
        check(rc, "gbfs_read_edge_list");
        rc = gbfs_graph_from_edges(num_nodes, m, src, dst, flags, &graph);
        gbfs_free(src);
        gbfs_free(dst);
        check(rc, "gbfs_graph_from_edges");
        gbfs_graph_info info;
        check(gbfs_graph_get_info(graph, &info), "gbfs_graph_get_info");
        if (info.wide) {  // the reference's int members cannot hold it: use the C ABI (gbfs_graph_get_csr64)
            gbfs_graph_destroy(graph);
            graph = nullptr;
            throw error(GBFS_ERR_TOO_LARGE, "csr: more than 2^31-1 edges");
        }
        num_edges = (int)info.m;
        row_offset = (int *)malloc(sizeof(int) * ((size_t)num_nodes + 1));
        col_idx = (int *)malloc(sizeof(int) * (size_t)(num_edges > 0 ? num_edges : 1));
        check(gbfs_graph_get_csr(graph, row_offset, col_idx), "gbfs_graph_get_csr");
    }
    ~csr()
    {
        free(col_idx);
        free(row_offset);
        gbfs_graph_destroy(graph);
    }
    csr(const csr &) = delete;
    csr &operator=(const csr &) = delete;

    int *col_idx = nullptr;
    int *row_offset = nullptr;
    int num_nodes = 0;
    int num_edges = 0;
    gbfs_graph *graph = nullptr;  // the device CSR behind the host arrays
};

class gpuBFS {
public:
    gpuBFS(csr &g, int source)
    {
        host_distance = (int *)malloc(sizeof(int) * (size_t)g.num_nodes);
        gbfs_stats st;
        int rc = gbfs_bfs(g.graph, source, host_distance, &st);
        if (rc != GBFS_OK) {
            free(host_distance);
            host_distance = nullptr;
            throw error(rc, "gbfs_bfs");
        }
        exec_time = st.ms;
        total_edges_traversed = (int)st.edges_traversed;
        iteration = st.levels;
    }
    ~gpuBFS() { free(host_distance); }
    gpuBFS(const gpuBFS &) = delete;
    gpuBFS &operator=(const gpuBFS &) = delete;

    int *host_distance = nullptr;
    float exec_time = 0;
    int total_edges_traversed = 0;
    int iteration = 0;
};

}  // namespace gbfs

#endif /* GBFS_GRAPHBFS_HPP */
