/*
 * oracle.h -- CPU oracle for the gbfs BFS engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker, never the product: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
 * arm load liboracle.so.  The engine (gpu_graphs_gb300/libgbfs.so) neither
 * links nor calls anything here and has no CPU fallback.
 *
 * Each function restates one piece of the reference's CPU path in plain C
 * and cites the reference file:line it follows (paths are relative to the
 * YKMorsy/GPU_Graphs project root).  Pinning: tests/golden/ holds level
 * arrays produced by the reference's own CPU BFS (compiled from its sources
 * by oracle/Makefile into oracle/_ref/) and tests/test_oracle.py checks this
 * restatement against every one of them.
 */
#ifndef GBFS_ORACLE_H
#define GBFS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Build flags (same bit values as the engine's GBFS_* flags). */
#define ORACLE_SYMMETRIZE      1u
#define ORACLE_DEDUP           2u
#define ORACLE_DROP_SELF_LOOPS 4u

/*
 * Edge list -> CSR, following the reference loader
 * (2D Partition/src/csc.cpp:14-25 adjacency lists in input order, then
 * :64-89 offsets by prefix sum and flattening, i.e. csc(file, 1, 1)).
 * With flags == 0 the result is exactly the reference's CSR: directed as
 * stored, duplicates and self-loops kept, rows in input order.  The flags
 * add what the reference does not have: SYMMETRIZE appends (v,u) right after
 * each (u,v); DROP_SELF_LOOPS skips u==v; DEDUP sorts every row ascending
 * and removes repeats.
 * row_offset: n+1 entries.  col_idx: capacity >= m (2m with SYMMETRIZE).
 * Returns the number of directed edges stored, or -1 on an id outside [0,n).
 */
int64_t oracle_csr_build(int32_t n, int64_t m, const int32_t *src,
                         const int32_t *dst, uint32_t flags,
                         int64_t *row_offset, int32_t *col_idx);

/*
 * Level-synchronous BFS of the 2D reference CPU path
 * (2D Partition/src/cpuBFS.cpp:3-73): per level, gather (u, v) for every
 * frontier edge, then the first v with bmap[v]==0 in that order gets
 * distance=iteration and pred=u.  Unreachable = -1.  pred may be NULL.
 * Returns the reference's total_edges_traversed (discovered vertices,
 * cpuBFS.cpp:59) or -1 on a bad source.
 */
int64_t oracle_bfs_levelsync(int32_t n, const int64_t *row_offset,
                             const int32_t *col_idx, int32_t source,
                             int32_t *level, int32_t *pred);

/*
 * FIFO-queue BFS of the single-GPU migration CPU path
 * (1D Partition/migration/GPU_Graphs/include/cpu/cpuBFS.cpp:3-49):
 * distance[nb] = distance[cur] + 1 on first sight.  Unreachable = -1.
 * Returns 0, or -1 on a bad source.
 */
int oracle_bfs_queue(int32_t n, const int64_t *row_offset,
                     const int32_t *col_idx, int32_t source, int32_t *level);

/*
 * oracle_bfs_queue with the reference's own timing around it: clock() at
 * entry and exit, exec_ms = (end - start) / CLOCKS_PER_SEC * 1000
 * (migration cpuBFS.cpp:5-6,51-53; the same formula in
 * 2D Partition/src/cpuBFS.cpp:5-6,71-72).  clock() counts the CPU time of
 * the whole process, so exec_ms is meaningful only when no other thread
 * runs meanwhile.  Also returns the reference's edge count convention, the
 * number of discovered vertices (2D Partition/src/cpuBFS.cpp:59), in
 * *discovered.  Returns 0, or -1 on a bad source.
 */
int oracle_bfs_queue_clock(int32_t n, const int64_t *row_offset,
                           const int32_t *col_idx, int32_t source,
                           int32_t *level, double *exec_ms,
                           int64_t *discovered);

/*
 * Exclusive prefix sum, the contract of PrefixSum::sum_scan_blelloch
 * (2D Partition/src/prefixSum.cu:136-224: out[0]=0, out[i]=sum in[0..i-1]).
 * 64-bit accumulation.
 */
void oracle_exclusive_scan_i32(const int32_t *in, int64_t *out, int64_t n);

/*
 * Number of directed edges leaving reached vertices (sum of out-degrees of
 * every v with level[v] >= 0): the E_c of the GTEPS / roofline formulas.
 */
int64_t oracle_component_edges(int32_t n, const int64_t *row_offset,
                               const int32_t *level);

/*
 * Canonical BFS-tree parents from a level array: parent[v] = the smallest u
 * with an edge u -> v and level[u] == level[v] - 1; -1 where level[v] <= 0.
 * The reference's predecessor (pred, 2D Partition/src/cpuBFS.cpp:16,56) is
 * the first such u in its frontier order; oracle_bfs_levelsync returns that
 * one.  Both are valid parents; this one does not depend on any order.
 */
void oracle_bfs_min_parents(int32_t n, const int64_t *row_offset,
                            const int32_t *col_idx, const int32_t *level,
                            int32_t *parent);

#ifdef __cplusplus
}
#endif
#endif /* GBFS_ORACLE_H */
