// api.cu -- the extern "C" entry points of libgbfs.so (see include/gbfs.h).
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/gbfs.h"
#include "graph.cuh"
#include "parents.cuh"
#include "scan.cuh"

namespace gbfs {

static thread_local std::string tl_error;

void set_error(const std::string &msg) { tl_error = msg; }

int fail(int code, const std::string &msg)
{
    tl_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    tl_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GBFS_ERR_OOM : GBFS_ERR_CUDA;
}

bool is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int graph_wrap(DeviceCsr &csr, bool symmetric_known, bool symmetric, cudaStream_t st, gbfs_graph **out)
{
    gbfs_graph *g = new (std::nothrow) gbfs_graph();
    if (!g) {
        csr_free(csr);
        if (st) cudaStreamDestroy(st);
        return fail(GBFS_ERR_OOM, "host allocation failed");
    }
    g->csr = csr;
    csr = DeviceCsr{};
    g->stream = st;
    cudaGetDevice(&g->device);
    gbfs_default_params(&g->params);
    {
        std::string err;
        const int rc = csr_build_first(g->csr, st, err);  // after any row reordering
        if (rc != GBFS_OK) {
            gbfs_graph_destroy(g);
            return fail(rc, err);
        }
    }
    if (symmetric_known) {
        g->symmetric = symmetric;
    } else {
        bool s = false;
        std::string err;
        int rc = csr_check_symmetric(g->csr, st, s, err);
        if (rc != GBFS_OK) {
            gbfs_graph_destroy(g);
            return fail(rc, err);
        }
        g->symmetric = s;
    }
    *out = g;
    return GBFS_OK;
}

}  // namespace gbfs

using namespace gbfs;

// ---- status -----------------------------------------------------------------

extern "C" const char *gbfs_strerror(int status)
{
    switch (status) {
    case GBFS_OK: return "ok";
    case GBFS_ERR_INVALID_ARG: return "invalid argument";
    case GBFS_ERR_OOM: return "out of memory";
    case GBFS_ERR_CUDA: return "CUDA error";
    case GBFS_ERR_TIMEOUT: return "device-side wait timed out";
    case GBFS_ERR_TOO_LARGE: return "graph too large for this path (size limit, or 64-bit row offsets)";
    case GBFS_ERR_IO: return "file missing or malformed";
    case GBFS_ERR_BUDGET: return "memory budget exceeded";
    case GBFS_ERR_NOT_FOUND: return "unknown graph id or ticket";
    case GBFS_ERR_SHUTDOWN: return "server is shutting down";
    default: return "unknown status";
    }
}

extern "C" const char *gbfs_last_error(void) { return tl_error.c_str(); }

extern "C" const char *gbfs_version(void) { return "gbfs 0.1 (sm_103a)"; }

extern "C" void gbfs_free(void *p) { free(p); }

// ---- params -------------------------------------------------------------------

extern "C" int gbfs_default_params(gbfs_params *p)
{
    if (!p) return fail(GBFS_ERR_INVALID_ARG, "params is NULL");
    p->threads_per_block = 512;
    p->blocks_per_sm = 2;
    p->alpha = 14;
    p->beta = 24;
    p->big_degree = 256;
    p->direction = GBFS_DIR_OPTIMIZING;
    p->per_level_launch = 0;
    p->timeout_ms = 2000;
    return GBFS_OK;
}

static int validate_params(const gbfs_params *p)
{
    if (!p) return fail(GBFS_ERR_INVALID_ARG, "params is NULL");
    if (p->threads_per_block != 256 && p->threads_per_block != 512 && p->threads_per_block != 1024)
        return fail(GBFS_ERR_INVALID_ARG, "threads_per_block must be 256, 512 or 1024");
    if (p->blocks_per_sm < 1 || p->blocks_per_sm > 32)
        return fail(GBFS_ERR_INVALID_ARG, "blocks_per_sm must be in [1, 32]");
    if (p->alpha < 1 || p->beta < 1) return fail(GBFS_ERR_INVALID_ARG, "alpha and beta must be >= 1");
    if (p->big_degree < 32) return fail(GBFS_ERR_INVALID_ARG, "big_degree must be >= 32");
    if (p->direction < 0 || p->direction > 2) return fail(GBFS_ERR_INVALID_ARG, "bad direction");
    if (p->per_level_launch < 0 || p->per_level_launch > 2)
        return fail(GBFS_ERR_INVALID_ARG, "per_level_launch must be 0, 1 or 2");
    if (p->timeout_ms < 1) return fail(GBFS_ERR_INVALID_ARG, "timeout_ms must be >= 1");
    return GBFS_OK;
}

extern "C" int gbfs_get_params(const gbfs_graph *g, gbfs_params *p)
{
    if (!g || !p) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    *p = graph_params(g);
    return GBFS_OK;
}

extern "C" int gbfs_set_params(gbfs_graph *g, const gbfs_params *p)
{
    if (!g) return fail(GBFS_ERR_INVALID_ARG, "graph is NULL");
    int rc = validate_params(p);
    if (rc) return rc;
    graph_set_params(g, *p);
    return GBFS_OK;
}

// ---- graph construction ----------------------------------------------------

static int make_stream(cudaStream_t *st)
{
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(GBFS_ERR_CUDA, "no CUDA device available");
    }
    e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    return GBFS_OK;
}

// Copy `count` ints from host or device `p` into a new device buffer.
static int to_device(const int32_t *p, int64_t count, cudaStream_t st, int **out, bool *owned)
{
    *owned = false;
    if (count == 0) {
        *out = nullptr;
        return GBFS_OK;
    }
    if (is_device_ptr(p)) {
        *out = const_cast<int *>(p);
        return GBFS_OK;
    }
    cudaError_t e = cudaMalloc(out, sizeof(int) * (size_t)count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    *owned = true;
    e = cudaMemcpyAsync(*out, p, sizeof(int) * (size_t)count, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy H2D");
    return GBFS_OK;
}

extern "C" int gbfs_graph_from_edges(int32_t n, int64_t m, const int32_t *src, const int32_t *dst,
                                     uint32_t flags, gbfs_graph **out)
{
    if (!out) return fail(GBFS_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (n < 1 || n > INT32_MAX - 1) return fail(GBFS_ERR_INVALID_ARG, "n must be in [1, 2^31-2]");
    if (m < 0 || (m > 0 && (!src || !dst))) return fail(GBFS_ERR_INVALID_ARG, "bad edge arrays");
    if (flags & ~31u) return fail(GBFS_ERR_INVALID_ARG, "unknown flag bits");
    cudaStream_t st = nullptr;
    int rc = make_stream(&st);
    if (rc) return rc;
    int *d_src = nullptr, *d_dst = nullptr;
    bool own_s = false, own_d = false;
    DeviceCsr csr;
    std::string err;
    rc = to_device(src, m, st, &d_src, &own_s);
    if (!rc) rc = to_device(dst, m, st, &d_dst, &own_d);
    if (!rc) {
        rc = csr_build_from_edges(n, m, d_src, d_dst, flags & (7u | GBFS_WIDE_ROWS), st, csr, err);
        if (!rc && (flags & GBFS_HUB_FIRST)) rc = csr_hub_first(csr, st, err);
        if (rc) set_error(err);
    }
    cudaStreamSynchronize(st);
    if (own_s) cudaFree(d_src);
    if (own_d) cudaFree(d_dst);
    if (rc) {
        cudaStreamDestroy(st);
        return rc;
    }
    return graph_wrap(csr, (flags & GBFS_SYMMETRIZE) != 0, true, st, out);
}

extern "C" int gbfs_graph_from_csr(int32_t n, int64_t m, const int32_t *row_offset,
                                   const int32_t *col_idx, gbfs_graph **out)
{
    if (!out) return fail(GBFS_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (n < 1 || n > INT32_MAX - 1) return fail(GBFS_ERR_INVALID_ARG, "n must be in [1, 2^31-2]");
    if (m < 0 || m > INT32_MAX) return fail(m < 0 ? GBFS_ERR_INVALID_ARG : GBFS_ERR_TOO_LARGE, "bad m");
    if (!row_offset || (m > 0 && !col_idx)) return fail(GBFS_ERR_INVALID_ARG, "NULL CSR array");
    cudaStream_t st = nullptr;
    int rc = make_stream(&st);
    if (rc) return rc;
    int *d_row = nullptr, *d_col = nullptr;
    cudaError_t e = cudaMalloc(&d_row, sizeof(int) * ((size_t)n + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_col, sizeof(int) * (size_t)std::max<int64_t>(m, 1));
    const cudaMemcpyKind kr = is_device_ptr(row_offset) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind kc = is_device_ptr(col_idx) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_row, row_offset, sizeof(int) * ((size_t)n + 1), kr, st);
    if (e == cudaSuccess && m > 0) e = cudaMemcpyAsync(d_col, col_idx, sizeof(int) * (size_t)m, kc, st);
    if (e != cudaSuccess) {
        if (d_row) cudaFree(d_row);
        if (d_col) cudaFree(d_col);
        cudaStreamDestroy(st);
        return cuda_fail(e, "CSR upload");
    }
    DeviceCsr csr;
    std::string err;
    rc = csr_adopt(n, m, d_row, d_col, st, csr, err);
    if (rc) {
        set_error(err);
        cudaStreamDestroy(st);
        return rc;
    }
    return graph_wrap(csr, false, false, st, out);
}

extern "C" void gbfs_graph_destroy(gbfs_graph *g)
{
    if (!g) return;
    if (g->batch_set) gbfs_graphset_destroy(g->batch_set);
    if (g->stream) cudaStreamSynchronize(g->stream);
    bfs_work_free(g->work);
    ms_work_free(g->ms);
    csr_free(g->csr);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

extern "C" int gbfs_graph_get_info(const gbfs_graph *g, gbfs_graph_info *info)
{
    if (!g || !info) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    info->n = g->csr.n;
    info->m = g->csr.m;
    info->max_degree = g->csr.max_degree;
    info->nonisolated = g->csr.nonisolated;
    info->device_bytes = csr_device_bytes(g->csr) + g->work.bytes + g->ms.bytes;
    info->wide = g->csr.wide ? 1 : 0;
    info->reserved = 0;
    return GBFS_OK;
}

extern "C" int gbfs_graph_get_csr(const gbfs_graph *g, int32_t *row_offset, int32_t *col_idx)
{
    if (!g || !row_offset || (g->csr.m > 0 && !col_idx)) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    if (g->csr.wide) return fail(GBFS_ERR_TOO_LARGE, "64-bit row offsets: use gbfs_graph_get_csr64");
    gbfs_graph *gg = const_cast<gbfs_graph *>(g);
    std::lock_guard<std::mutex> lk(gg->mu);
    const cudaMemcpyKind kr = is_device_ptr(row_offset) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const cudaMemcpyKind kc = is_device_ptr(col_idx) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaError_t e = cudaMemcpyAsync(row_offset, g->csr.row, sizeof(int) * ((size_t)g->csr.n + 1), kr, g->stream);
    if (e == cudaSuccess && g->csr.m > 0)
        e = cudaMemcpyAsync(col_idx, g->csr.col, sizeof(int) * (size_t)g->csr.m, kc, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "CSR download");
    return GBFS_OK;
}

extern "C" int gbfs_graph_get_csr64(const gbfs_graph *g, int64_t *row_offset, int32_t *col_idx)
{
    if (!g || !row_offset) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    gbfs_graph *gg = const_cast<gbfs_graph *>(g);
    std::lock_guard<std::mutex> lk(gg->mu);
    const size_t nr = (size_t)g->csr.n + 1;
    const bool dev_row = is_device_ptr(row_offset);
    const cudaMemcpyKind kc = is_device_ptr(col_idx) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaError_t e = cudaSuccess;
    if (g->csr.wide) {
        e = cudaMemcpyAsync(row_offset, g->csr.row64, sizeof(int64_t) * nr,
                            dev_row ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, g->stream);
    } else {
        // 32-bit offsets widened on the host
        std::vector<int32_t> r32;
        std::vector<int64_t> r64;
        try {
            r32.resize(nr);
            r64.resize(nr);
        } catch (const std::bad_alloc &) {
            return fail(GBFS_ERR_OOM, "host allocation failed for the row offsets");
        }
        e = cudaMemcpyAsync(r32.data(), g->csr.row, sizeof(int32_t) * nr, cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        if (e == cudaSuccess) {
            std::copy(r32.begin(), r32.end(), r64.begin());
            e = cudaMemcpy(row_offset, r64.data(), sizeof(int64_t) * nr,
                           dev_row ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost);
        }
    }
    if (e == cudaSuccess && g->csr.m > 0 && col_idx)
        e = cudaMemcpyAsync(col_idx, g->csr.col, sizeof(int) * (size_t)g->csr.m, kc, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "CSR download");
    return GBFS_OK;
}

// ---- traversal ------------------------------------------------------------------

static void fill_stats(gbfs_stats *s, const BfsResult &r, int64_t nsources)
{
    if (!s) return;
    s->ms = r.ms;
    s->levels = r.levels;
    s->td_levels = r.td_levels;
    s->bu_levels = r.bu_levels;
    s->launches = r.launches;
    s->vertices_reached = r.reached;
    s->edges_in_component = r.edges_c;
    s->edges_traversed = r.reached - nsources;
}

// Parameters for a traversal of g: bottom-up steps need in-edges, so a
// graph whose in-edges differ from its out-edges gets its transpose built
// here on first use (top-down only if that fails for lack of memory).
// Caller holds g->mu.
static gbfs_params effective_params(gbfs_graph *g)
{
    gbfs_params p = graph_params(g);
    if (!g->symmetric && p.direction != GBFS_DIR_TOPDOWN && !g->csr.trow) {
        std::string err;
        if (csr_build_transpose(g->csr, g->stream, err) != GBFS_OK) cudaGetLastError();
    }
    if (!g->symmetric && !g->csr.trow) p.direction = GBFS_DIR_TOPDOWN;
    return p;
}

// Runs a BFS into the graph's workspace or the caller's device buffer, then
// copies to the caller's host buffer if needed.  Caller holds g->mu.
static int run_bfs_locked(gbfs_graph *g, const int *d_roots, int k, int single_root, int32_t *levels_out,
                          BfsResult &res)
{
    std::string err;
    int rc = bfs_work_alloc(g->work, g->csr.n, err, g->csr.wide);
    if (rc) return fail(rc, err);
    const bool dev_out = is_device_ptr(levels_out);
    int *d_level = dev_out ? levels_out : g->work.level;
    gbfs_params p = effective_params(g);
    g->last_multi = false;
    rc = bfs_run(g->csr, p, g->work, d_roots, k, single_root, d_level, g->stream, res, err, g->symmetric);
    if (rc) return fail(rc, err);
    if (!dev_out) {
        cudaError_t e = cudaMemcpyAsync(levels_out, d_level, sizeof(int) * (size_t)g->csr.n,
                                        cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) return cuda_fail(e, "levels D2H");
    }
    return GBFS_OK;
}

extern "C" int gbfs_bfs(gbfs_graph *g, int32_t source, int32_t *levels_out, gbfs_stats *stats)
{
    if (!g || !levels_out) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    if (source < 0 || source >= g->csr.n) return fail(GBFS_ERR_INVALID_ARG, "source outside [0, n)");
    std::lock_guard<std::mutex> lk(g->mu);
    BfsResult res;
    int rc = run_bfs_locked(g, nullptr, 1, source, levels_out, res);
    if (rc) return rc;
    fill_stats(stats, res, 1);
    return GBFS_OK;
}

extern "C" int gbfs_bfs_parents(gbfs_graph *g, int32_t source, int32_t *levels_out, int32_t *parents_out,
                                gbfs_stats *stats)
{
    if (!g || !parents_out) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    if (source < 0 || source >= g->csr.n) return fail(GBFS_ERR_INVALID_ARG, "source outside [0, n)");
    std::lock_guard<std::mutex> lk(g->mu);
    std::string err;
    int rc = bfs_work_alloc(g->work, g->csr.n, err, g->csr.wide);
    if (rc) return fail(rc, err);
    BfsWork &w = g->work;
    const size_t n = (size_t)g->csr.n;
    const bool dev_lv = levels_out && is_device_ptr(levels_out);
    const bool dev_par = is_device_ptr(parents_out);
    int *d_level = dev_lv ? levels_out : w.level;
    // the traversal's queues are free once it has finished
    int *d_parent = dev_par ? parents_out : w.q0;
    gbfs_params p = effective_params(g);
    g->last_multi = false;
    BfsResult res;
    rc = bfs_run(g->csr, p, w, nullptr, 1, source, d_level, g->stream, res, err, g->symmetric);
    if (rc) return fail(rc, err);
    cudaError_t e = parents_enqueue(g->csr, g->symmetric, d_level, d_parent, g->stream);
    if (e == cudaSuccess && !dev_par)
        e = cudaMemcpyAsync(parents_out, d_parent, sizeof(int) * n, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess && levels_out && !dev_lv)
        e = cudaMemcpyAsync(levels_out, d_level, sizeof(int) * n, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "parents");
    fill_stats(stats, res, 1);
    return GBFS_OK;
}

extern "C" int gbfs_bfs_many(gbfs_graph *g, const int32_t *sources, int32_t k, int32_t *levels_out,
                             gbfs_stats *stats)
{
    if (!g || !sources || k < 1) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    std::vector<int32_t> hsrc((size_t)k);
    if (is_device_ptr(sources)) {
        cudaError_t e = cudaMemcpy(hsrc.data(), sources, sizeof(int32_t) * (size_t)k, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "sources D2H");
    } else {
        std::copy(sources, sources + k, hsrc.begin());
    }
    for (int32_t i = 0; i < k; i++)
        if (hsrc[i] < 0 || hsrc[i] >= g->csr.n) return fail(GBFS_ERR_INVALID_ARG, "source outside [0, n)");
    std::lock_guard<std::mutex> lk(g->mu);
    std::string err;
    int rc = bfs_work_alloc(g->work, g->csr.n, err, g->csr.wide);
    if (!rc) rc = bfs_work_reserve_many(g->work, k, err);
    if (rc) return fail(rc, err);
    BfsWork &w = g->work;
    const size_t n = (size_t)g->csr.n;
    const bool dev_out = levels_out && is_device_ptr(levels_out);
    const gbfs_params p = effective_params(g);
    if (p.per_level_launch) {  // host loop per level: one source at a time
        for (int32_t i = 0; i < k; i++) {
            BfsResult r;
            int32_t *dst = levels_out ? levels_out + n * i : nullptr;
            int *d_level = dev_out ? dst : w.level;
            rc = bfs_run(g->csr, p, w, nullptr, 1, hsrc[i], d_level, g->stream, r, err, g->symmetric);
            if (rc) return fail(rc, err);
            if (dst && !dev_out) {
                cudaError_t e2 = cudaMemcpy(dst, w.level, sizeof(int) * n, cudaMemcpyDeviceToHost);
                if (e2 != cudaSuccess) return cuda_fail(e2, "levels D2H");
            }
            if (stats) fill_stats(&stats[i], r, 1);
        }
        return GBFS_OK;
    }
    const bool host_out = levels_out && !dev_out;
    if (host_out) {
        rc = bfs_work_reserve_overlap(w, err);
        if (rc) return fail(rc, err);
    }
    cudaError_t e = cudaSuccess;
    for (int32_t i = 0; i < k && e == cudaSuccess; i++) {
        // host output: results alternate between two device buffers and are
        // copied on a second stream while the next traversal runs; launch i
        // waits for the copy that last used its buffer (launch i - 2)
        int *d_level = dev_out ? levels_out + n * i : (host_out && (i & 1)) ? w.level2 : w.level;
        if (host_out && i >= 2) e = cudaStreamWaitEvent(g->stream, w.ev_copied[i & 1], 0);
        if (e == cudaSuccess) e = cudaEventRecord(w.evs[i], g->stream);
        if (e == cudaSuccess)
            e = bfs_enqueue(g->csr, p, w, nullptr, 1, hsrc[i], d_level, w.d_outs + i, g->stream, g->symmetric);
        if (e == cudaSuccess && host_out) {
            e = cudaEventRecord(w.ev_ready[i & 1], g->stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(w.copy_st, w.ev_ready[i & 1], 0);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(levels_out + n * i, d_level, sizeof(int) * n, cudaMemcpyDeviceToHost, w.copy_st);
            if (e == cudaSuccess) e = cudaEventRecord(w.ev_copied[i & 1], w.copy_st);
        }
    }
    if (e == cudaSuccess) e = cudaEventRecord(w.evs[k], g->stream);
    if (e == cudaSuccess && host_out) e = cudaStreamSynchronize(w.copy_st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w.h_outs, w.d_outs, sizeof(BfsOut) * (size_t)k, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w.h_ctrl, w.ctrl, offsetof(BfsCtrl, t_entry), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "BFS launches");
    if (w.h_ctrl->status != DEV_OK) {
        cudaMemsetAsync(w.ctrl, 0, sizeof(BfsCtrl), g->stream);
        cudaStreamSynchronize(g->stream);
        return fail(GBFS_ERR_TIMEOUT, "a device-side wait ran out (grid barrier)");
    }
    if (stats)
        for (int32_t i = 0; i < k; i++) {
            BfsResult r;
            cudaEventElapsedTime(&r.ms, w.evs[i], w.evs[i + 1]);
            const BfsOut &o = w.h_outs[i];
            r.levels = o.levels;
            r.td_levels = o.td_levels;
            r.bu_levels = o.bu_levels;
            r.launches = bfs_launches_per_search(g->csr, p);
            r.reached = (int64_t)o.reached;
            r.edges_c = (int64_t)o.edges_c;
            fill_stats(&stats[i], r, 1);
        }
    return GBFS_OK;
}

extern "C" int gbfs_last_trace(gbfs_graph *g, gbfs_level_trace *rows, int32_t cap)
{
    if (!g || (cap > 0 && !rows) || cap < 0) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    std::lock_guard<std::mutex> lk(g->mu);
    unsigned long long t_entry, t_start, t_end, t_exit;
    int trace_len;
    const LevelTrace *trace;
    cudaError_t e;
    if (g->last_multi) {
        if (!g->ms.ctrl) return 0;
        MsCtrl *h = g->ms.h_ctrl;
        e = cudaMemcpyAsync(&h->t_entry, &g->ms.ctrl->t_entry, sizeof(MsCtrl) - offsetof(MsCtrl, t_entry),
                            cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h->trace_len, &g->ms.ctrl->trace_len, sizeof(int),
                                                  cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) return cuda_fail(e, "trace D2H");
        t_entry = h->t_entry; t_start = h->t_start; t_end = h->t_end; t_exit = h->t_exit;
        trace_len = h->trace_len; trace = h->trace;
    } else {
        if (!g->work.ctrl) return 0;
        BfsCtrl *h = g->work.h_ctrl;
        e = cudaMemcpyAsync(&h->t_entry, &g->work.ctrl->t_entry, sizeof(BfsCtrl) - offsetof(BfsCtrl, t_entry),
                            cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) return cuda_fail(e, "trace D2H");
        t_entry = h->t_entry; t_start = h->t_start; t_end = h->t_end; t_exit = h->t_exit;
        trace_len = h->trace_len; trace = h->trace;
    }
    const int len = std::min<int>(std::min<int>(trace_len, TRACE_CAP), cap - 3);
    if (len < 0) return 0;
    // row 0: initialisation (level -1), from CTA 0's entry to the first level
    rows[0].level = -1;
    rows[0].direction = -1;
    rows[0].frontier_vertices = 0;
    rows[0].frontier_edges = 0;
    rows[0].t_us = -(double)(t_start - t_entry) / 1000.0;
    rows++;
    for (int i = 0; i < len; i++) {
        const LevelTrace &t = trace[i];
        rows[i].level = t.level;
        rows[i].direction = t.dir;
        rows[i].frontier_vertices = (int64_t)t.frontier;
        rows[i].frontier_edges = (int64_t)t.edges;
        rows[i].t_us = (double)(t.t_ns - t_start) / 1000.0;
    }
    // last row: the end of the level loop (the termination check included)
    rows[len].level = -2;
    rows[len].direction = -2;
    rows[len].frontier_vertices = 0;
    rows[len].frontier_edges = 0;
    rows[len].t_us = (double)(t_end - t_start) / 1000.0;
    // then the last CTA's exit: closing passes (unreached lanes, totals) done
    rows[len + 1].level = -3;
    rows[len + 1].direction = -3;
    rows[len + 1].frontier_vertices = 0;
    rows[len + 1].frontier_edges = 0;
    rows[len + 1].t_us = (double)(t_exit - t_start) / 1000.0;
    return len + 3;
}

extern "C" void *gbfs_graph_stream(const gbfs_graph *g) { return g ? (void *)g->stream : nullptr; }

extern "C" int gbfs_bfs_multiroot(gbfs_graph *g, const int32_t *sources, int32_t k, int32_t *levels_out,
                                  gbfs_stats *stats)
{
    if (!g || !levels_out || !sources || k < 1) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    if (k > g->csr.n) return fail(GBFS_ERR_INVALID_ARG, "more roots than vertices");
    const bool dev_src = is_device_ptr(sources);
    if (!dev_src)
        for (int32_t i = 0; i < k; i++)
            if (sources[i] < 0 || sources[i] >= g->csr.n) return fail(GBFS_ERR_INVALID_ARG, "root outside [0, n)");
    std::lock_guard<std::mutex> lk(g->mu);
    std::string err;
    int rc = bfs_work_alloc(g->work, g->csr.n, err, g->csr.wide);
    if (rc) return fail(rc, err);
    cudaError_t e = cudaMemcpyAsync(g->work.roots, sources, sizeof(int) * (size_t)k,
                                    dev_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "roots upload");
    BfsResult res;
    rc = run_bfs_locked(g, g->work.roots, k, -1, levels_out, res);
    if (rc) return rc;
    fill_stats(stats, res, res.roots);
    return GBFS_OK;
}

extern "C" int gbfs_bfs_multi(gbfs_graph *g, const int32_t *sources, int32_t k, int32_t *levels_out,
                              gbfs_stats *stats)
{
    if (!g || !levels_out || !sources || k < 1) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    const bool dev_src = is_device_ptr(sources);
    std::vector<int32_t> hsrc;
    if (dev_src) {
        hsrc.resize(k);
        cudaError_t e = cudaMemcpy(hsrc.data(), sources, sizeof(int) * (size_t)k, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "sources D2H");
    } else {
        hsrc.assign(sources, sources + k);
    }
    for (int32_t i = 0; i < k; i++)
        if (hsrc[i] < 0 || hsrc[i] >= g->csr.n) return fail(GBFS_ERR_INVALID_ARG, "source outside [0, n)");
    if (g->csr.wide) return fail(GBFS_ERR_TOO_LARGE, "multi-source search needs 32-bit row offsets");
    std::lock_guard<std::mutex> lk(g->mu);
    std::string err;
    int rc = ms_work_alloc(g->ms, g->csr.n, err);
    if (rc) return fail(rc, err);
    const gbfs_params p = effective_params(g);  // builds the transpose a directed graph's pull steps need
    rc = ms_prepare(g->csr, g->stream, err);
    if (rc) return fail(rc, err);
    const bool dev_out = is_device_ptr(levels_out);
    const size_t n = (size_t)g->csr.n;
    MsResult tot;
    g->last_multi = true;
    for (int32_t b0 = 0; b0 < k; b0 += MS_LANES) {
        const int kk = std::min<int>(MS_LANES, k - b0);
        cudaError_t e = cudaMemcpyAsync(g->ms.src, hsrc.data() + b0, sizeof(int) * kk, cudaMemcpyHostToDevice,
                                        g->stream);
        if (e != cudaSuccess) return cuda_fail(e, "sources H2D");
        int *d_out = dev_out ? levels_out + (size_t)b0 * n : g->ms.out;
        MsResult r;
        rc = msbfs_run(g->csr, p, g->symmetric, g->ms, g->ms.src, kk, d_out, g->stream, r, err);
        if (rc) return fail(rc, err);
        if (!dev_out) {
            e = cudaMemcpyAsync(levels_out + (size_t)b0 * n, d_out, sizeof(int) * n * kk, cudaMemcpyDeviceToHost,
                                g->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
            if (e != cudaSuccess) return cuda_fail(e, "levels D2H");
        }
        tot.ms += r.ms;
        tot.levels = std::max(tot.levels, r.levels);
        tot.push_levels += r.push_levels;
        tot.pull_levels += r.pull_levels;
        tot.reached += r.reached;
        tot.edges_c += r.edges_c;
    }
    if (stats) {
        stats->ms = tot.ms;
        stats->levels = tot.levels;
        stats->td_levels = tot.push_levels;
        stats->bu_levels = tot.pull_levels;
        stats->launches = (k + MS_LANES - 1) / MS_LANES;
        stats->vertices_reached = tot.reached;
        stats->edges_in_component = tot.edges_c;
        stats->edges_traversed = tot.reached - k;
    }
    return GBFS_OK;
}

// ---- scan primitive --------------------------------------------------------------

namespace {
struct ScanPool {
    std::mutex mu;
    void *mem = nullptr;
    int64_t tiles = 0;
    ScanScratch s;
    int device = -1;
};
ScanPool g_scan_pool[64];
}  // namespace

extern "C" int gbfs_exclusive_scan_i32(const int32_t *d_in, int64_t *d_out, int64_t n, void *stream)
{
    if (n < 0 || (n > 0 && (!d_in || !d_out))) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    if (n == 0) return GBFS_OK;
    if (!is_device_ptr(d_in) || !is_device_ptr(d_out))
        return fail(GBFS_ERR_INVALID_ARG, "d_in and d_out must be device pointers");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    ScanPool &pool = g_scan_pool[dev & 63];
    std::lock_guard<std::mutex> lk(pool.mu);
    const int64_t tiles = scan_tiles(n);
    cudaStream_t st = (cudaStream_t)stream;
    if (pool.tiles < tiles) {
        if (pool.mem) {
            cudaDeviceSynchronize();
            cudaFree(pool.mem);
            pool.mem = nullptr;
        }
        const int64_t want = std::max<int64_t>(tiles, 1024);
        e = cudaMalloc(&pool.mem, scan_scratch_bytes(want));
        if (e != cudaSuccess) {
            pool.tiles = 0;
            return cuda_fail(e, "scan scratch");
        }
        e = cudaMemset(pool.mem, 0, scan_scratch_bytes(want));
        if (e != cudaSuccess) return cuda_fail(e, "scan scratch");
        scan_scratch_carve(pool.mem, want, pool.s);
        pool.tiles = want;
        pool.s.epoch = 0;
    }
    e = scan_exclusive_i32_i64(d_in, (long long *)d_out, n, nullptr, pool.s, st);
    if (e != cudaSuccess) return cuda_fail(e, "scan launch");
    unsigned status = 0;
    e = cudaMemcpyAsync(&status, pool.s.ctl + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "scan");
    if (status != 0) {
        unsigned zero = 0;
        cudaMemcpy(pool.s.ctl + 2, &zero, sizeof(unsigned), cudaMemcpyHostToDevice);
        return fail(GBFS_ERR_TIMEOUT, "scan look-back wait ran out");
    }
    return GBFS_OK;
}

// ---- file format ------------------------------------------------------------------

namespace gbfs {
// edge_list.cpp: mapped, parsed in parallel, with the semantics of the
// reference's `while (infile >> from >> to)` loop
int read_edge_list_text(const char *path, int32_t one_based, int32_t *n, int64_t *m, int32_t **src, int32_t **dst);
}  // namespace gbfs

extern "C" int gbfs_read_edge_list(const char *path, int32_t one_based, int32_t *n, int64_t *m, int32_t **src,
                                   int32_t **dst)
{
    if (!path || !n || !m || !src || !dst) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    *src = *dst = nullptr;
    return gbfs::read_edge_list_text(path, one_based, n, m, src, dst);
}

// File layout: int32 n, int64 m, row offsets (n + 1), int32 col (m).  The
// offsets are int32; a wide graph stores -n and int64 offsets (a reader
// that only knows the int32 layout rejects the negative count).
extern "C" int gbfs_graph_save(const gbfs_graph *g, const char *path)
{
    if (!g || !path) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    const bool wide = g->csr.wide;
    std::vector<int32_t> row32, col;
    std::vector<int64_t> row64;
    try {
        row32.resize(wide ? 0 : (size_t)g->csr.n + 1);
        col.resize((size_t)std::max<int64_t>(g->csr.m, 1));
        row64.resize(wide ? (size_t)g->csr.n + 1 : 0);
    } catch (const std::bad_alloc &) {
        return fail(GBFS_ERR_OOM, "host allocation failed for the CSR copy");
    }
    int rc = wide ? gbfs_graph_get_csr64(g, row64.data(), col.data()) : gbfs_graph_get_csr(g, row32.data(), col.data());
    if (rc) return rc;
    FILE *f = fopen(path, "wb");
    if (!f) return fail(GBFS_ERR_IO, std::string("cannot write ") + path);
    int32_t n = wide ? -g->csr.n : g->csr.n;
    int64_t m = g->csr.m;
    bool ok = fwrite(&n, 4, 1, f) == 1 && fwrite(&m, 8, 1, f) == 1 &&
              (wide ? fwrite(row64.data(), 8, row64.size(), f) == row64.size()
                    : fwrite(row32.data(), 4, row32.size(), f) == row32.size()) &&
              (m == 0 || fwrite(col.data(), 4, (size_t)m, f) == (size_t)m);
    ok = (fclose(f) == 0) && ok;
    return ok ? GBFS_OK : fail(GBFS_ERR_IO, "short write");
}

extern "C" int gbfs_graph_load(const char *path, gbfs_graph **out)
{
    if (!path || !out) return fail(GBFS_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return fail(GBFS_ERR_IO, std::string("cannot open ") + path);
    int32_t n = 0;
    int64_t m = 0;
    if (fread(&n, 4, 1, f) != 1 || fread(&m, 8, 1, f) != 1) {
        fclose(f);
        return fail(GBFS_ERR_IO, "bad CSR header");
    }
    const bool wide = n < 0;
    if (wide) n = n == INT32_MIN ? 0 : -n;
    if (n < 1 || n > INT32_MAX - 1 || m < 0 || (!wide && m > INT32_MAX) || m > (int64_t)1 << 40) {
        fclose(f);
        return fail(GBFS_ERR_IO, "bad CSR header");
    }
    // the file must hold exactly what its header announces: a corrupt or
    // foreign header is refused before anything is allocated for it
    const int64_t want = 12 + ((int64_t)n + 1) * (wide ? 8 : 4) + 4 * m;
    if (fseeko(f, 0, SEEK_END) != 0 || ftello(f) != (off_t)want || fseeko(f, 12, SEEK_SET) != 0) {
        fclose(f);
        return fail(GBFS_ERR_IO, "CSR file size does not match its header (" + std::to_string(want) + " bytes expected)");
    }
    std::vector<int32_t> row32, col;
    std::vector<int64_t> row64;
    try {
        row32.resize(wide ? 0 : (size_t)n + 1);
        col.resize((size_t)std::max<int64_t>(m, 1));
        row64.resize(wide ? (size_t)n + 1 : 0);
    } catch (const std::bad_alloc &) {
        fclose(f);
        return fail(GBFS_ERR_OOM, "host allocation failed for the CSR file");
    }
    bool ok = (wide ? fread(row64.data(), 8, row64.size(), f) == row64.size()
                    : fread(row32.data(), 4, row32.size(), f) == row32.size()) &&
              (m == 0 || fread(col.data(), 4, (size_t)m, f) == (size_t)m);
    fclose(f);
    if (!ok) return fail(GBFS_ERR_IO, "truncated CSR file");
    if (!wide) return gbfs_graph_from_csr(n, m, row32.data(), col.data(), out);
    // a wide CSR: upload and adopt with 64-bit offsets
    cudaStream_t st = nullptr;
    int rc = make_stream(&st);
    if (rc) return rc;
    long long *d_row = nullptr;
    int *d_col = nullptr;
    cudaError_t e = cudaMalloc(&d_row, sizeof(long long) * ((size_t)n + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d_col, sizeof(int) * (size_t)std::max<int64_t>(m, 1));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_row, row64.data(), sizeof(long long) * ((size_t)n + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && m > 0)
        e = cudaMemcpyAsync(d_col, col.data(), sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        if (d_row) cudaFree(d_row);
        if (d_col) cudaFree(d_col);
        cudaStreamDestroy(st);
        return cuda_fail(e, "CSR upload");
    }
    DeviceCsr csr;
    std::string err;
    rc = csr_adopt64(n, m, d_row, d_col, st, csr, err);
    if (rc) {
        set_error(err);
        cudaStreamDestroy(st);
        return rc;
    }
    return graph_wrap(csr, false, false, st, out);
}
