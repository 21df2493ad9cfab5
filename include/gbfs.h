/*
 * gbfs.h -- C ABI of the GB300-native BFS engine (libgbfs.so).
 *
 * The engine keeps the reference's graphBFS host path -- edge list in, CSR
 * build, BFS from a source, per-vertex int32 level array out (-1 =
 * unreachable) -- on one GPU, behind plain C entry points: pointers, sizes
 * and status codes, no C++ or torch types.  Every call returns GBFS_OK (0)
 * or a negative status; the library never exits the process.
 *
 * Reference interfaces replaced (paths relative to the YKMorsy/GPU_Graphs
 * project root):
 *   csr::csr(const char*)          1D Partition/include/csr.h:9-23,
 *                                  1D Partition/src/csr.cpp:3-67
 *   csc::csc(const char*, R, C)    2D Partition/include/csc.h:12-25,
 *                                  2D Partition/src/csc.cpp:3-94
 *   gpuBFS::gpuBFS(csr&, int)      1D Partition/include/gpuBFS.cuh:9-54,
 *                                  1D Partition/src/gpuBFS.cu:13-116
 *   gpuBFS::gpuBFS(csc&, int,R,C)  2D Partition/include/gpuBFS.cuh:12-63,
 *                                  2D Partition/src/gpuBFS.cu:189-345
 *   PrefixSum::sum_scan_blelloch   2D Partition/include/prefixSum.cuh:4-10
 *
 * Pointers marked "host or device" are classified with
 * cudaPointerGetAttributes; device pointers must be on the current device.
 * Thread safety: calls on one graph handle are serialised by a per-graph
 * lock; different handles may be used from different threads at once.
 * The library keeps per-device launch settings for the life of the
 * process: cudaDeviceReset while it is in use is not supported.
 */
#ifndef GBFS_H
#define GBFS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GBFS_OK                0
#define GBFS_ERR_INVALID_ARG  -1  /* bad pointer, size, id or source        */
#define GBFS_ERR_OOM          -2  /* device or host allocation failed       */
#define GBFS_ERR_CUDA         -3  /* a CUDA runtime call failed / no device */
#define GBFS_ERR_TIMEOUT      -4  /* a bounded device-side wait ran out     */
#define GBFS_ERR_TOO_LARGE    -5  /* size limit, or a path without 64-bit rows */
#define GBFS_ERR_IO           -6  /* file missing or malformed              */
#define GBFS_ERR_BUDGET       -7  /* serving: memory budget refuses it      */
#define GBFS_ERR_NOT_FOUND    -8  /* serving: unknown graph id or ticket    */
#define GBFS_ERR_SHUTDOWN     -9  /* serving: server is shutting down       */

/* Text for a status code (static storage). */
const char *gbfs_strerror(int status);
/* Detail message of the last failing call on this thread ("" if none). */
const char *gbfs_last_error(void);
/* Library version string. */
const char *gbfs_version(void);

/* ---- graph construction ---------------------------------------------- */
/* Build flags.  With 0 the CSR keeps the edges as stored, like the
 * reference loaders (directed, duplicates and self-loops kept). */
#define GBFS_SYMMETRIZE       1u  /* add (v,u) for every (u,v)              */
#define GBFS_DEDUP            2u  /* drop repeated (u,v)                     */
#define GBFS_DROP_SELF_LOOPS  4u  /* drop (u,u)                              */
#define GBFS_UNDIRECTED (GBFS_SYMMETRIZE | GBFS_DEDUP | GBFS_DROP_SELF_LOOPS)
/* Layout option: after the build, each row's highest-degree neighbour is
 * moved to the row's front (the rest stays ascending).  Bottom-up steps
 * probe it first, which resolves most unvisited vertices with one probe on
 * power-law graphs.  Levels are unaffected. */
#define GBFS_HUB_FIRST        8u
/* Store 64-bit row offsets even when 32-bit ones would do (graphs whose
 * stored edges can exceed 2^31-1 get them anyway). */
#define GBFS_WIDE_ROWS       16u

typedef struct gbfs_graph gbfs_graph;

/*
 * Edge list -> device CSR, built on the GPU (degree count, look-back scan,
 * scatter, per-row sort, dedup, compaction).  Rows come out sorted
 * ascending (see GBFS_HUB_FIRST for the one exception).  src/dst: m int32 vertex ids in [0, n), host or device.
 * Replaces csr::csr / csc::csc (which parse a file into host CSR; the file
 * parser is gbfs_read_edge_list below).  Limits: n <= 2^31-2; a graph
 * whose stored directed edges can exceed 2^31-1 (counted before
 * deduplication) gets 64-bit row offsets ("wide", also with
 * GBFS_WIDE_ROWS).  A wide graph supports single-source searches (top-down
 * and, when built symmetric, direction-optimising), parents, the trace,
 * gbfs_graph_get_csr64 and the binary cache; multi-source searches, graph sets,
 * the server, per-level launch modes and the transpose of a directed wide
 * graph return GBFS_ERR_TOO_LARGE.
 */
int gbfs_graph_from_edges(int32_t n, int64_t m, const int32_t *src,
                          const int32_t *dst, uint32_t flags,
                          gbfs_graph **out);

/*
 * Existing CSR -> device graph, taken as is (rows need not be sorted).
 * row_offset: n+1 int32 (row_offset[0]==0, non-decreasing, [n]==m);
 * col_idx: m int32 in [0, n).  Host or device.  Mirrors the public
 * int* row_offset / int* col_idx of csr (1D Partition/include/csr.h:15-16).
 */
int gbfs_graph_from_csr(int32_t n, int64_t m, const int32_t *row_offset,
                        const int32_t *col_idx, gbfs_graph **out);

void gbfs_graph_destroy(gbfs_graph *g);

typedef struct gbfs_graph_info {
    int32_t n;                  /* vertices                                  */
    int32_t max_degree;
    int64_t m;                  /* stored directed edges                     */
    int64_t nonisolated;        /* vertices with out-degree > 0              */
    int64_t device_bytes;       /* CSR and what is built on it (first-entry
                                   arrays, pull pieces, transpose) + per-graph
                                   search workspace                          */
    int32_t wide;               /* 1: 64-bit row offsets                     */
    int32_t reserved;
} gbfs_graph_info;

int gbfs_graph_get_info(const gbfs_graph *g, gbfs_graph_info *info);

/* Copy the device CSR out: row_offset n+1, col_idx m (host or device).
 * GBFS_ERR_TOO_LARGE for a wide graph (64-bit row offsets). */
int gbfs_graph_get_csr(const gbfs_graph *g, int32_t *row_offset,
                       int32_t *col_idx);
/* The same with 64-bit row offsets, for any graph; col_idx may be NULL
 * (the offsets alone). */
int gbfs_graph_get_csr64(const gbfs_graph *g, int64_t *row_offset,
                         int32_t *col_idx);

/* ---- traversal parameters (autotuned) --------------------------------- */
/* Bottom-up steps probe in-edges: on a directed graph the first traversal
 * that may take one builds the transpose (4(3n+1) + 4m device bytes) and
 * keeps it with the graph; if that allocation fails the search is top-down. */
#define GBFS_DIR_OPTIMIZING   0   /* Beamer top-down / bottom-up switching  */
#define GBFS_DIR_TOPDOWN      1
#define GBFS_DIR_BOTTOMUP     2

typedef struct gbfs_params {
    int32_t threads_per_block;  /* 256, 512 or 1024                         */
    int32_t blocks_per_sm;      /* persistent CTAs per SM (capped by occupancy) */
    int32_t alpha;              /* TD->BU when frontier edges > unexplored/alpha */
    int32_t beta;               /* BU->TD when frontier vertices < n/beta    */
    int32_t big_degree;         /* TD rows >= this are split across the grid */
    int32_t direction;          /* GBFS_DIR_*                               */
    int32_t per_level_launch;   /* 0: one persistent launch per search;
                                   1: one launch per level with a host loop
                                   (the reference's shape); 2: one launch per
                                   level replayed by a CUDA graph with a
                                   device-side while loop (no host round
                                   trip between levels)                     */
    int32_t timeout_ms;         /* bound on every device-side wait          */
} gbfs_params;

/* Built-in defaults (before any autotuning). */
int gbfs_default_params(gbfs_params *p);
int gbfs_get_params(const gbfs_graph *g, gbfs_params *p);
int gbfs_set_params(gbfs_graph *g, const gbfs_params *p);

/*
 * Autotuner: times a grid of candidate parameters (block size, CTAs per SM,
 * alpha, beta, big_degree) on up to 16 of `nsources` sources of this graph
 * (pass 16 or more: per-source times vary widely), keeps a candidate only
 * if it is more than 2 % faster than the best so far and its levels equal
 * the default's, stores the result in the graph and returns it in *best
 * (nullable).  A process-wide cache keyed by the graph's size/degree
 * signature makes repeated calls cheap.
 */
int gbfs_autotune(gbfs_graph *g, const int32_t *sources, int32_t nsources,
                  gbfs_params *best);

/* ---- single-source BFS ------------------------------------------------ */
typedef struct gbfs_stats {
    float   ms;                 /* device time of the traversal (events)    */
    int32_t levels;             /* number of BFS levels (max level + 1)     */
    int32_t td_levels;          /* levels expanded top-down                 */
    int32_t bu_levels;          /* levels expanded bottom-up                */
    int32_t launches;           /* kernel launches this call queued per
                                   search: 1; 2 on graphs of out-degree
                                   <= 16 (the grid launch and the
                                   label-correcting launch that finishes a
                                   long search, returning at once when the
                                   search is already done); one per level
                                   (+1) with per_level_launch              */
    int64_t vertices_reached;   /* vertices with level >= 0 (all sources)   */
    int64_t edges_in_component; /* out-edges of reached vertices (E_c)      */
    int64_t edges_traversed;    /* reference convention: discovered vertices
                                   (2D Partition/src/cpuBFS.cpp:59)         */
} gbfs_stats;

/*
 * BFS from `source`; levels_out receives n int32 (host or device), -1 for
 * unreachable.  Replaces gpuBFS::gpuBFS(csr&, int) and its host_distance /
 * exec_time / total_edges_traversed / iteration members.  stats nullable.
 */
int gbfs_bfs(gbfs_graph *g, int32_t source, int32_t *levels_out,
             gbfs_stats *stats);

/*
 * BFS plus a BFS tree.  parents_out (n int32, host or device) receives the
 * canonical parent of every vertex: the smallest u with an edge u -> v and
 * level[u] == level[v] - 1, or -1 for the source and unreached vertices.
 * Replaces the predecessor array of the reference's 2D BFS (`pred`,
 * 2D Partition/src/cpuBFS.cpp:16,56; `d_pred`, 2D Partition/include/gpuBFS.cuh:45),
 * whose entries depend on the order the frontier is walked; any of those is
 * a valid parent, this one is unique.  levels_out: n int32 or NULL.
 * stats.ms covers the traversal only.
 */
int gbfs_bfs_parents(gbfs_graph *g, int32_t source, int32_t *levels_out,
                     int32_t *parents_out, gbfs_stats *stats);

/*
 * k single-source searches run back to back, one launch each, queued on the
 * graph's stream with no host round trip in between (the plain
 * one-query-per-launch BFS).  levels_out: k*n int32 (host or device; row i
 * for sources[i]) or NULL to discard the levels.  With levels_out on the
 * host, results alternate between two device buffers and each is copied
 * on a second stream while the next search runs.  stats: k entries
 * (nullable); stats[i].ms spans launch i on the graph's stream (with host
 * output, plus any wait for the copy two launches back to free its buffer).
 */
int gbfs_bfs_many(gbfs_graph *g, const int32_t *sources, int32_t k,
                  int32_t *levels_out, gbfs_stats *stats);

/* Per-level trace of the graph's last traversal, single-source,
 * multi-root or multi-source (thread 0 stamps %globaltimer after each
 * level's barrier; for multi-source, frontier_vertices counts vertices
 * active in any lane, direction 0 push / 1 pull, frontier_edges 0). */
typedef struct gbfs_level_trace {
    int32_t level;              /* frontier expanded by this step            */
    int32_t direction;          /* 0 top-down, 1 bottom-up, 2 top-down with
                                   a grid-split pass over long rows, 4 one
                                   round of the label-correcting phase of
                                   long searches on small-degree graphs (up
                                   to 64 levels; from the level it took
                                   over at, `level` counts rounds)         */
    int64_t frontier_vertices;
    int64_t frontier_edges;     /* out-edges of the frontier                 */
    double  t_us;               /* end of the step, us after initialisation  */
} gbfs_level_trace;

/* Copies up to cap rows (up to 16,384 levels are kept: the first 16,383
 * and the last); returns the number of rows (>= 0) or a status.
 * Row 0 describes initialisation: level -1, t_us = minus its duration
 * (from the first CTA's entry to the first level).  Then one row per level,
 * then a row with level -2 marking the end of the level loop (termination
 * check included) and a last row with level -3: the moment the last CTA
 * left the kernel, after the closing passes. */
int gbfs_last_trace(gbfs_graph *g, gbfs_level_trace *rows, int32_t cap);

/* The CUDA stream (cudaStream_t) the graph's work is ordered on, for
 * callers that record their own events around it. */
void *gbfs_graph_stream(const gbfs_graph *g);

/*
 * Multi-root BFS: every vertex in sources[0..k) starts at level 0 and a
 * vertex's level is its distance to the nearest root.  levels_out: n int32.
 */
int gbfs_bfs_multiroot(gbfs_graph *g, const int32_t *sources, int32_t k,
                       int32_t *levels_out, gbfs_stats *stats);

/*
 * Multi-source BFS: k independent searches on one graph, 64 per launch in
 * uint64 per-vertex lane masks.  levels_out: k*n int32, row i = the level
 * array of sources[i].  stats (nullable) sums over all searches.
 */
int gbfs_bfs_multi(gbfs_graph *g, const int32_t *sources, int32_t k,
                   int32_t *levels_out, gbfs_stats *stats);

/* ---- many small graphs, one fused launch ------------------------------ */
typedef struct gbfs_graphset gbfs_graphset;

/*
 * `count` edge lists -> one device graph set (the disjoint union in one CSR
 * plus a per-graph vertex offset table).  n[i], m[i], src[i], dst[i] as in
 * gbfs_graph_from_edges; ids are local to each graph.
 */
int gbfs_graphset_from_edges(int32_t count, const int32_t *n,
                             const int64_t *m, const int32_t *const *src,
                             const int32_t *const *dst, uint32_t flags,
                             gbfs_graphset **out);
/* Same, from graphs already on the device (their CSRs are copied). */
int gbfs_graphset_from_graphs(int32_t count, gbfs_graph *const *graphs,
                              gbfs_graphset **out);
void gbfs_graphset_destroy(gbfs_graphset *s);
int gbfs_graphset_vertex_offsets(const gbfs_graphset *s, int64_t *offsets);

/*
 * One BFS per graph (sources[i] local to graph i), all in one persistent
 * launch.  levels_out[i]: n[i] int32 (host or device).
 */
int gbfs_bfs_batch(gbfs_graphset *s, const int32_t *sources,
                   int32_t *const *levels_out, gbfs_stats *stats);

/* Convenience over separate handles: builds (and caches on the first
 * handle) a graph set, then runs gbfs_bfs_batch. */
int gbfs_bfs_batch_graphs(gbfs_graph *const *graphs, const int32_t *sources,
                          int32_t count, int32_t *const *levels_out,
                          gbfs_stats *stats);

/* ---- scan primitive ---------------------------------------------------- */
/*
 * Exclusive prefix sum of n int32 on the device (single-pass decoupled
 * look-back), 64-bit output.  d_in, d_out device pointers; stream may be
 * NULL (legacy default stream).  Replaces PrefixSum::sum_scan_blelloch
 * (2D Partition/src/prefixSum.cu:136-224), which allocates and frees its
 * scratch on every call; this one keeps a per-device scratch pool.
 */
int gbfs_exclusive_scan_i32(const int32_t *d_in, int64_t *d_out, int64_t n,
                            void *stream);

/*
 * Allocation-free variant of gbfs_exclusive_scan_i32 (no counterpart in the
 * reference).  For callers that cannot let a library allocate device memory
 * while they run: processes that reserve all of HBM up front in their own
 * pools, loops that must not take the driver's allocation locks (cudaMalloc
 * and cudaFree may synchronise the device), allocators calling in from their
 * own critical section.  The look-back scratch is a fixed array compiled
 * into the library (under 1 MB, held on every GPU that loads the library
 * until the process exits), so this call makes no cudaMalloc, cudaFree or
 * other allocating call.  Limits and rules:
 *   - n <= GBFS_SCAN_NOALLOC_MAX_N, else GBFS_ERR_TOO_LARGE;
 *   - the first call on a device looks the array's address up once (with
 *     that device current); make that first call before any stream capture;
 *   - do not call cudaDeviceReset between calls: the library keeps that
 *     address (and its other per-device launch settings) for the process;
 *   - all calls share the array: calls whose work overlaps on the GPU
 *     (different streams or threads) race; serialise them;
 *   - the call synchronises `stream` to report the scan's status.
 * Same result as gbfs_exclusive_scan_i32 otherwise.
 */
#define GBFS_SCAN_NOALLOC_MAX_N (1LL << 26)
int gbfs_exclusive_scan_i32_noalloc(const int32_t *d_in, int64_t *d_out,
                                    int64_t n, void *stream);

/*
 * Failure-detection self-test (no counterpart in the reference): launches a
 * two-CTA cooperative kernel whose second CTA never reaches the grid
 * barrier, so the first CTA's bounded wait runs out after timeout_ms
 * (1..10000).  Returns GBFS_ERR_TIMEOUT when the wait reported its timeout
 * and the context is still usable; any other status is a failure.
 */
int gbfs_selftest_wait_timeout(int32_t timeout_ms);

/* ---- file format and workload generators ------------------------------ */
/*
 * Read the reference's text format: "n", "m", then whitespace-separated
 * "from to" pairs until end of file (1D Partition/src/csr.cpp:14-29,
 * 2D Partition/src/csc.cpp:14-25).  one_based=1 subtracts 1 from every id
 * like csc.cpp:24.  *src / *dst are malloc'd; free with gbfs_free.
 * Ids outside [0, n) are an error (the reference writes out of bounds).
 */
int gbfs_read_edge_list(const char *path, int32_t one_based, int32_t *n,
                        int64_t *m, int32_t **src, int32_t **dst);
void gbfs_free(void *p);

/* Binary CSR cache: int32 n, int64 m, int32 row_offset[n+1], int32 col[m]
 * (a wide graph: int32 -n, int64 m, int64 row_offset[n+1], int32 col[m]).
 * Loading refuses (GBFS_ERR_IO) a file whose size is not exactly what its
 * header announces, before allocating anything for it. */
int gbfs_graph_save(const gbfs_graph *g, const char *path);
int gbfs_graph_load(const char *path, gbfs_graph **out);

/*
 * Seeded, thread-count-independent workload generators (host).  Each
 * returns the number of edges written, or a negative status if `cap` is too
 * small.  Edges are undirected pairs, to be built with GBFS_UNDIRECTED.
 *   er:   `pairs` uniform (u,v) pairs over n vertices
 *   rmat: 2^scale vertices, edge_factor*2^scale edges, quadrant
 *         probabilities a,b,c (d = 1-a-b-c), ids permuted by the seed
 *   grid: side x side 4-neighbour grid (row-major ids), each edge dropped
 *         with probability drop, plus round(extra * 2*side*(side-1)) edges
 *         from a uniform vertex to a uniform vertex within Manhattan radius
 *         `radius` (a draw that finds no in-grid target in 64 tries becomes
 *         a self-loop, removed by GBFS_DROP_SELF_LOOPS)
 */
int64_t gbfs_gen_er(int32_t n, int64_t pairs, uint64_t seed, int32_t *src,
                    int32_t *dst, int64_t cap);
int64_t gbfs_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b,
                      double c, uint64_t seed, int32_t *src, int32_t *dst,
                      int64_t cap);
int64_t gbfs_gen_grid(int32_t side, double drop, double extra, int32_t radius,
                      uint64_t seed, int32_t *src, int32_t *dst, int64_t cap);
/* Upper bound of gbfs_gen_grid's edge count for the same arguments. */
int64_t gbfs_gen_grid_capacity(int32_t side, double extra);

/* ---- serving loop (no counterpart in the reference) --------------------
 * A server keeps graphs resident, admits them against an HBM budget and
 * answers BFS queries with continuous batching: same-graph queries that
 * arrive while others run are packed into 64-lane multi-source launches as
 * slots (streams with their own workspace) free up.  On a graph of
 * out-degree <= 16 (meshes, grids, road networks: long searches of small
 * frontiers) each slot instead runs up to 4 queries at once as
 * single-source searches on its own streams, each with a quarter of the
 * slot's CTAs, and starts the next waiting query as soon as any of them
 * ends (batch_lanes then counts the slot's searches running at its start;
 * a query alone in the server gets the slot's whole CTA share).
 * These run concurrently only with enough hardware work queues: start the
 * process with CUDA_DEVICE_MAX_CONNECTIONS of at least 4 * num_slots + 2
 * (CUDA's default of 8 lets about four searches progress at a time). */
typedef struct gbfs_server gbfs_server;

typedef struct gbfs_server_config {
    int64_t mem_budget_bytes;   /* HBM the server may hold: graphs + slots  */
    int32_t num_slots;          /* concurrent in-flight launches (streams)  */
    int32_t max_lanes;          /* sources per multi-source launch (<= 64)  */
    int32_t batch_window_us;    /* wait this long for same-graph arrivals   */
    int32_t timeout_ms;         /* device wait bound for each launch        */
    int32_t window_pct;         /* ...or up to this percentage of the graph's
                                   recent launch time, if longer (0: fixed
                                   window).  A launch costs about the same
                                   for 1 or 64 sources, so on slow graphs a
                                   longer wait buys throughput.             */
} gbfs_server_config;

typedef struct gbfs_query_info {
    double  latency_ms;         /* submit -> result in the caller's buffer  */
    double  queue_ms;           /* submit -> launch                         */
    int32_t batch_lanes;        /* sources that shared the launch           */
    int32_t status;             /* GBFS_OK or the launch's error            */
} gbfs_query_info;

typedef struct gbfs_server_stats {      /* since the last reset; the latency
                                           percentiles cover the most recent
                                           131,072 completed queries          */
    int64_t completed;
    int64_t launches;
    int64_t rejected;           /* admissions refused by the budget         */
    double  p50_ms, p99_ms, mean_ms, max_ms;
    double  mean_batch_lanes;
    int64_t resident_bytes;     /* graphs admitted                          */
    int64_t peak_bytes;         /* high-water mark of graphs + slots        */
} gbfs_server_stats;

int gbfs_server_create(const gbfs_server_config *cfg, gbfs_server **out);
/* Stops admission, drains in-flight work, frees slots (not the graphs). */
void gbfs_server_destroy(gbfs_server *s);
/* Admit a resident graph (borrowed; must outlive the server or be removed).
 * A directed graph whose direction is not GBFS_DIR_TOPDOWN gets its
 * transpose (in-edge rows, for bottom-up and pull steps) built here and
 * counted in the budget.  GBFS_ERR_BUDGET if its CSR plus one slot's
 * workspace does not fit.  Concurrent calls are serialised (each sees the
 * bytes the others admitted). */
int gbfs_server_add_graph(gbfs_server *s, gbfs_graph *g, int32_t *graph_id);
int gbfs_server_remove_graph(gbfs_server *s, int32_t graph_id);
/* Queue one query; levels_out (host, n int32) is written before completion
 * is reported.  Returns at once with a ticket. */
int gbfs_server_submit(gbfs_server *s, int32_t graph_id, int32_t source,
                       int32_t *levels_out, int64_t *ticket);
/* Wait for a ticket (timeout_ms < 0: forever).  GBFS_ERR_TIMEOUT if it is
 * still pending; otherwise the query's own status.  info nullable.  The
 * ticket is released when a wait returns its result: threads already
 * waiting on it all get the result, later waits get GBFS_ERR_NOT_FOUND. */
int gbfs_server_wait(gbfs_server *s, int64_t ticket, int32_t timeout_ms,
                     gbfs_query_info *info);
int gbfs_server_get_stats(gbfs_server *s, gbfs_server_stats *st);
void gbfs_server_reset_stats(gbfs_server *s);

#ifdef __cplusplus
}
#endif
#endif /* GBFS_H */
