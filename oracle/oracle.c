/*
 * oracle.c -- CPU oracle for the gbfs BFS engine (TEST INFRASTRUCTURE ONLY).
 *
 * Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU legs as
 * the checker; the engine never calls it.  See oracle.h for the contract of
 * each function and the reference lines each one restates.
 */
#include "oracle.h"

#include <stdlib.h>
#include <time.h>
#include <string.h>

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* Reference: 2D Partition/src/csc.cpp:14-25 (push_back per input line into
 * adjList[from]) and :64-89 (col_offset[col+1] = size, prefix sum, copy rows
 * in order).  A stable counting sort by source gives the same rows. */
int64_t oracle_csr_build(int32_t n, int64_t m, const int32_t *src,
                         const int32_t *dst, uint32_t flags,
                         int64_t *row_offset, int32_t *col_idx)
{
    const int sym = (flags & ORACLE_SYMMETRIZE) != 0;
    const int noself = (flags & ORACLE_DROP_SELF_LOOPS) != 0;
    int64_t i;

    for (i = 0; i < m; i++)
        if (src[i] < 0 || src[i] >= n || dst[i] < 0 || dst[i] >= n)
            return -1;

    memset(row_offset, 0, sizeof(int64_t) * ((size_t)n + 1));
    for (i = 0; i < m; i++) {
        int32_t u = src[i], v = dst[i];
        if (noself && u == v) continue;
        row_offset[u + 1]++;
        if (sym) row_offset[v + 1]++;
    }
    for (i = 0; i < n; i++) row_offset[i + 1] += row_offset[i];

    int64_t *cursor = (int64_t *)malloc(sizeof(int64_t) * ((size_t)n + 1));
    if (!cursor) return -1;
    memcpy(cursor, row_offset, sizeof(int64_t) * (size_t)n);
    for (i = 0; i < m; i++) {
        int32_t u = src[i], v = dst[i];
        if (noself && u == v) continue;
        col_idx[cursor[u]++] = v;          /* (u,v) in input order */
        if (sym) col_idx[cursor[v]++] = u; /* then its reverse */
    }
    free(cursor);

    if (flags & ORACLE_DEDUP) {
        int64_t w = 0, r;
        for (r = 0; r < n; r++) {
            int64_t b = row_offset[r], e = row_offset[r + 1], k;
            qsort(col_idx + b, (size_t)(e - b), sizeof(int32_t), cmp_i32);
            row_offset[r] = w;
            for (k = b; k < e; k++)
                if (k == b || col_idx[k] != col_idx[k - 1]) col_idx[w++] = col_idx[k];
        }
        row_offset[n] = w;
    }
    return row_offset[n];
}

/* Reference: 2D Partition/src/cpuBFS.cpp:3-73.  The reference first builds
 * frontier_edges (:33-45) and then scans it (:49-61); scanning each
 * frontier vertex's row right away visits the same (u, v) pairs in the same
 * order, so distance and pred come out identical. */
int64_t oracle_bfs_levelsync(int32_t n, const int64_t *row_offset,
                             const int32_t *col_idx, int32_t source,
                             int32_t *level, int32_t *pred)
{
    if (source < 0 || source >= n) return -1;
    int32_t *frontier = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *next = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    unsigned char *bmap = (unsigned char *)calloc((size_t)n, 1);
    if (!frontier || !next || !bmap) {
        free(frontier); free(next); free(bmap);
        return -1;
    }
    int32_t i;
    for (i = 0; i < n; i++) level[i] = -1;          /* :13 distance(-1) */
    if (pred) for (i = 0; i < n; i++) pred[i] = -1; /* :16 pred(-1) */

    int64_t nf = 0, nn, total = 0, f;
    frontier[nf++] = source;                        /* :20-22 */
    level[source] = 0;
    bmap[source] = 1;
    int32_t iteration = 1;                          /* :24 */
    for (;;) {
        nn = 0;
        for (f = 0; f < nf; f++) {
            int32_t u = frontier[f];
            int64_t e;
            for (e = row_offset[u]; e < row_offset[u + 1]; e++) {
                int32_t v = col_idx[e];
                if (!bmap[v]) {                     /* :53-60 */
                    bmap[v] = 1;
                    if (pred) pred[v] = u;
                    level[v] = iteration;
                    next[nn++] = v;
                    total++;
                }
            }
        }
        iteration++;                                /* :64 */
        if (nn == 0) break;                         /* :66-69 */
        int32_t *t = frontier; frontier = next; next = t;
        nf = nn;
    }
    free(frontier); free(next); free(bmap);
    return total;
}

/* Reference: 1D Partition/migration/GPU_Graphs/include/cpu/cpuBFS.cpp:3-49
 * (std::queue; distance[neighbor] = distance[cur_node] + 1 when it is -1). */
int oracle_bfs_queue(int32_t n, const int64_t *row_offset,
                     const int32_t *col_idx, int32_t source, int32_t *level)
{
    if (source < 0 || source >= n) return -1;
    int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    if (!queue) return -1;
    int32_t i;
    for (i = 0; i < n; i++) level[i] = -1;          /* :9-13 */
    int64_t head = 0, tail = 0;
    queue[tail++] = source;                         /* :16-17 */
    level[source] = 0;
    while (head < tail) {                           /* :21 */
        int32_t cur = queue[head++];
        int64_t e;
        for (e = row_offset[cur]; e < row_offset[cur + 1]; e++) {
            int32_t nb = col_idx[e];
            if (level[nb] == -1) {                  /* :40-45 */
                queue[tail++] = nb;
                level[nb] = level[cur] + 1;
            }
        }
    }
    free(queue);
    return 0;
}

/* Timing of migration cpuBFS.cpp:5-6,51-53 around the queue BFS above. */
int oracle_bfs_queue_clock(int32_t n, const int64_t *row_offset,
                           const int32_t *col_idx, int32_t source,
                           int32_t *level, double *exec_ms,
                           int64_t *discovered)
{
    clock_t start = clock();
    int r = oracle_bfs_queue(n, row_offset, col_idx, source, level);
    clock_t end = clock();
    if (exec_ms) *exec_ms = ((double)(end - start)) / CLOCKS_PER_SEC * 1000.0;
    if (discovered) {
        int64_t d = 0;
        int32_t v;
        if (r == 0)
            for (v = 0; v < n; v++) d += level[v] > 0;
        *discovered = d;
    }
    return r;
}

/* Reference contract: 2D Partition/src/prefixSum.cu:136-224 (exclusive). */
void oracle_exclusive_scan_i32(const int32_t *in, int64_t *out, int64_t n)
{
    int64_t acc = 0, i;
    for (i = 0; i < n; i++) {
        out[i] = acc;
        acc += in[i];
    }
}

int64_t oracle_component_edges(int32_t n, const int64_t *row_offset,
                               const int32_t *level)
{
    int64_t s = 0;
    int32_t v;
    for (v = 0; v < n; v++)
        if (level[v] >= 0) s += row_offset[v + 1] - row_offset[v];
    return s;
}

void oracle_bfs_min_parents(int32_t n, const int64_t *row_offset,
                            const int32_t *col_idx, const int32_t *level,
                            int32_t *parent)
{
    int32_t u, v;
    int64_t i;
    for (v = 0; v < n; v++) parent[v] = level[v] > 0 ? INT32_MAX : -1;
    for (u = 0; u < n; u++) {
        if (level[u] < 0) continue;
        for (i = row_offset[u]; i < row_offset[u + 1]; i++) {
            v = col_idx[i];
            if (level[v] == level[u] + 1 && u < parent[v]) parent[v] = u;
        }
    }
}
