// batch.cu -- many small graphs, one fused launch.
//
// A graph set is the disjoint union of its members in one CSR (member i's
// vertex v becomes offsets[i] + v) plus the offset table.  One BFS per
// member then runs as a single multi-root launch of the persistent kernel
// with member i's source as its root: components of a disjoint union never
// meet, so every vertex's level in the union equals its level in its own
// member's single-source BFS, bit for bit, and -1 stays -1.  The union
// load-balances graphs of uneven size across the whole GPU for free.
#include <algorithm>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "graph.cuh"

using namespace gbfs;

namespace {

__global__ void k_offset_copy(const int *__restrict__ src, int *__restrict__ dst, int64_t count, int add)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
        dst[i] = src[i] + add;
}

int make_set(gbfs_graph *g, int32_t count, const std::vector<int64_t> &offsets, gbfs_graphset **out)
{
    gbfs_graphset *s = new (std::nothrow) gbfs_graphset();
    if (!s) {
        gbfs_graph_destroy(g);
        return fail(GBFS_ERR_OOM, "host allocation failed");
    }
    s->g = g;
    s->offsets = offsets;
    s->sizes.resize(count);
    for (int32_t i = 0; i < count; i++) s->sizes[i] = (int32_t)(offsets[i + 1] - offsets[i]);
    *out = s;
    return GBFS_OK;
}

}  // namespace

extern "C" int gbfs_graphset_from_edges(int32_t count, const int32_t *n, const int64_t *m,
                                        const int32_t *const *src, const int32_t *const *dst, uint32_t flags,
                                        gbfs_graphset **out)
{
    if (!out || count < 1 || !n || !m || !src || !dst) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    *out = nullptr;
    std::vector<int64_t> voff(count + 1, 0), eoff(count + 1, 0);
    for (int32_t i = 0; i < count; i++) {
        if (n[i] < 1 || m[i] < 0 || (m[i] > 0 && (!src[i] || !dst[i])))
            return fail(GBFS_ERR_INVALID_ARG, "bad member graph " + std::to_string(i));
        voff[i + 1] = voff[i] + n[i];
        eoff[i + 1] = eoff[i] + m[i];
    }
    if (voff[count] > INT32_MAX - 1) return fail(GBFS_ERR_TOO_LARGE, "union has more than 2^31-2 vertices");
    // Union edge list on the host (device member arrays are fetched first).
    std::vector<int32_t> us, ud;
    try {
        us.resize((size_t)eoff[count]);
        ud.resize((size_t)eoff[count]);
    } catch (const std::bad_alloc &) {
        return fail(GBFS_ERR_OOM, "host allocation failed for the union edge list");
    }
    for (int32_t i = 0; i < count; i++) {
        const int64_t mi = m[i];
        if (mi == 0) continue;
        int32_t *ps = us.data() + eoff[i], *pd = ud.data() + eoff[i];
        for (int which = 0; which < 2; which++) {
            const int32_t *in = which ? dst[i] : src[i];
            int32_t *o = which ? pd : ps;
            if (is_device_ptr(in)) {
                cudaError_t e = cudaMemcpy(o, in, sizeof(int32_t) * (size_t)mi, cudaMemcpyDeviceToHost);
                if (e != cudaSuccess) return cuda_fail(e, "member edges D2H");
            } else {
                memcpy(o, in, sizeof(int32_t) * (size_t)mi);
            }
        }
        const int32_t off = (int32_t)voff[i], ni = n[i];
        for (int64_t j = 0; j < mi; j++) {
            if (ps[j] < 0 || ps[j] >= ni || pd[j] < 0 || pd[j] >= ni)
                return fail(GBFS_ERR_INVALID_ARG, "edge endpoint outside its member graph");
            ps[j] += off;
            pd[j] += off;
        }
    }
    gbfs_graph *g = nullptr;
    int rc = gbfs_graph_from_edges((int32_t)voff[count], eoff[count], us.data(), ud.data(), flags, &g);
    if (rc) return rc;
    return make_set(g, count, voff, out);
}

extern "C" int gbfs_graphset_from_graphs(int32_t count, gbfs_graph *const *graphs, gbfs_graphset **out)
{
    if (!out || count < 1 || !graphs) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    *out = nullptr;
    std::vector<int64_t> voff(count + 1, 0), eoff(count + 1, 0);
    bool sym = true;
    for (int32_t i = 0; i < count; i++) {
        if (!graphs[i]) return fail(GBFS_ERR_INVALID_ARG, "NULL member graph");
        if (graphs[i]->csr.wide) return fail(GBFS_ERR_TOO_LARGE, "member graph with 64-bit row offsets");
        voff[i + 1] = voff[i] + graphs[i]->csr.n;
        eoff[i + 1] = eoff[i] + graphs[i]->csr.m;
        sym = sym && graphs[i]->symmetric;
    }
    if (voff[count] > INT32_MAX - 1 || eoff[count] > INT32_MAX)
        return fail(GBFS_ERR_TOO_LARGE, "union exceeds the int32 CSR limits");
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    int *row = nullptr, *col = nullptr;
    e = cudaMalloc(&row, sizeof(int) * ((size_t)voff[count] + 1));
    if (e == cudaSuccess) e = cudaMalloc(&col, sizeof(int) * (size_t)std::max<int64_t>(eoff[count], 1));
    for (int32_t i = 0; i < count && e == cudaSuccess; i++) {
        gbfs_graph *gi = graphs[i];
        std::lock_guard<std::mutex> lk(gi->mu);
        cudaStreamSynchronize(gi->stream);
        const int64_t ni = gi->csr.n, mi = gi->csr.m;
        int grid = (int)std::max<int64_t>(1, std::min<int64_t>(1024, (ni + 255) / 256));
        k_offset_copy<<<grid, 256, 0, st>>>(gi->csr.row, row + voff[i], ni, (int)eoff[i]);
        if (mi > 0) {
            grid = (int)std::max<int64_t>(1, std::min<int64_t>(1024, (mi + 255) / 256));
            k_offset_copy<<<grid, 256, 0, st>>>(gi->csr.col, col + eoff[i], mi, (int)voff[i]);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        const int last = (int)eoff[count];
        e = cudaMemcpyAsync(row + voff[count], &last, sizeof(int), cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        if (row) cudaFree(row);
        if (col) cudaFree(col);
        cudaStreamDestroy(st);
        return cuda_fail(e, "graph set assembly");
    }
    DeviceCsr csr;
    std::string err;
    int rc = csr_adopt((int32_t)voff[count], eoff[count], row, col, st, csr, err);
    if (rc) {
        cudaStreamDestroy(st);
        return fail(rc, err);
    }
    gbfs_graph *g = nullptr;
    rc = graph_wrap(csr, sym, sym, st, &g);
    if (rc) return rc;
    return make_set(g, count, voff, out);
}

extern "C" void gbfs_graphset_destroy(gbfs_graphset *s)
{
    if (!s) return;
    gbfs_graph_destroy(s->g);
    delete s;
}

extern "C" int gbfs_graphset_vertex_offsets(const gbfs_graphset *s, int64_t *offsets)
{
    if (!s || !offsets) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    std::copy(s->offsets.begin(), s->offsets.end(), offsets);
    return GBFS_OK;
}

extern "C" int gbfs_bfs_batch(gbfs_graphset *s, const int32_t *sources, int32_t *const *levels_out,
                              gbfs_stats *stats)
{
    if (!s || !sources || !levels_out) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    const int32_t count = (int32_t)s->sizes.size();
    std::vector<int32_t> roots(count);
    for (int32_t i = 0; i < count; i++) {
        if (!levels_out[i]) return fail(GBFS_ERR_INVALID_ARG, "NULL level buffer");
        if (sources[i] < 0 || sources[i] >= s->sizes[i]) return fail(GBFS_ERR_INVALID_ARG, "source outside its graph");
        roots[i] = (int32_t)(s->offsets[i] + sources[i]);
    }
    gbfs_graph *g = s->g;
    gbfs_stats st{};
    // Run into the union's own device level array, then scatter the slices.
    {
        std::string err;
        std::lock_guard<std::mutex> lk(g->mu);
        int rc = bfs_work_alloc(g->work, g->csr.n, err, g->csr.wide);
        if (rc) return fail(rc, err);
    }
    int rc = gbfs_bfs_multiroot(g, roots.data(), count, g->work.level, &st);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g->mu);
    bool any_host = false;
    for (int32_t i = 0; i < count; i++) any_host = any_host || !is_device_ptr(levels_out[i]);
    cudaError_t e = cudaSuccess;
    if (any_host) {
        // one D2H of the whole union, then host copies
        int32_t *stage = nullptr;
        e = cudaMallocHost(&stage, sizeof(int32_t) * (size_t)g->csr.n);
        if (e != cudaSuccess) return cuda_fail(e, "pinned staging");
        e = cudaMemcpyAsync(stage, g->work.level, sizeof(int32_t) * (size_t)g->csr.n, cudaMemcpyDeviceToHost,
                            g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        if (e == cudaSuccess)
            for (int32_t i = 0; i < count; i++)
                if (!is_device_ptr(levels_out[i]))
                    memcpy(levels_out[i], stage + s->offsets[i], sizeof(int32_t) * (size_t)s->sizes[i]);
        cudaFreeHost(stage);
    }
    for (int32_t i = 0; i < count && e == cudaSuccess; i++)
        if (is_device_ptr(levels_out[i]))
            e = cudaMemcpyAsync(levels_out[i], g->work.level + s->offsets[i], sizeof(int32_t) * (size_t)s->sizes[i],
                                cudaMemcpyDeviceToDevice, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch levels copy-out");
    if (stats) *stats = st;
    return GBFS_OK;
}

extern "C" int gbfs_bfs_batch_graphs(gbfs_graph *const *graphs, const int32_t *sources, int32_t count,
                                     int32_t *const *levels_out, gbfs_stats *stats)
{
    if (!graphs || count < 1 || !graphs[0]) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    gbfs_graph *head = graphs[0];
    std::vector<const gbfs_graph *> key(graphs, graphs + count);
    gbfs_graphset *set = nullptr;
    {
        std::lock_guard<std::mutex> lk(head->mu);
        if (head->batch_set && head->batch_key == key) set = head->batch_set;
    }
    if (!set) {
        int rc = gbfs_graphset_from_graphs(count, graphs, &set);
        if (rc) return rc;
        std::lock_guard<std::mutex> lk(head->mu);
        if (head->batch_set) gbfs_graphset_destroy(head->batch_set);
        head->batch_set = set;
        head->batch_key = key;
    }
    return gbfs_bfs_batch(set, sources, levels_out, stats);
}
