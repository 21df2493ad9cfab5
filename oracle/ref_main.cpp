// ref_main.cpp -- driver around the reference's own CPU BFS (TEST
// INFRASTRUCTURE ONLY).  oracle/Makefile compiles this file twice against
// the reference sources, unmodified, where they lie:
//   -DREF_C9 : 2D Partition/src/{csc,cpuBFS}.cpp  (level-synchronous BFS)
//   -DREF_C10: 1D Partition/migration/GPU_Graphs/include/{csr/csr,cpu/cpuBFS}.cpp
//              (FIFO-queue BFS)
// The binaries land in oracle/_ref/ and are used to pin the C restatement
// (oracle.c) and to generate tests/golden/.
//
// usage:
//   ref_cXX text <graph.txt> <source> <levels.bin>
//       load through the reference's own text loader (1-based "n m u v ..")
//   ref_cXX csrdump <graph.txt> <out.csr>
//       load through the reference's text loader and write its CSR
//   ref_cXX csr <graph.csr> <source> <levels.bin> [reps]
//       inject a binary CSR (int32 n, int64 m, int32 row[n+1], int32 col[m])
//       through the reference object's public members, then run the BFS
// stdout: "n=<n> m=<m> exec_ms=<clock() ms> wall_ms=<steady_clock ms>"
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <unistd.h>

#ifdef REF_C9
#include "csc.h"
#include "cpuBFS.h"
typedef csc graph_t;
static graph_t *load_text(const char *path) { return new csc(path, 1, 1); }
static int graph_n(graph_t *g) { return g->num_nodes; }
static long long graph_m(graph_t *g) { return (long long)g->csc_vect[0].second.size(); }
static void inject(graph_t *g, int n, long long m, std::vector<int> &row, std::vector<int> &col)
{
    g->num_nodes = n;
    g->num_edges = (int)m;
    g->csc_vect[0].first = row;   // public members (2D Partition/include/csc.h:12-25)
    g->csc_vect[0].second = col;
}
static const int *levels_of(cpuBFS &b) { return b.distance.data(); }
static void get_csr(graph_t *g, std::vector<int> &row, std::vector<int> &col)
{
    row = g->csc_vect[0].first;
    col = g->csc_vect[0].second;
}
#else
#include "csr/csr.h"
#include "cpu/cpuBFS.h"
typedef csr graph_t;
static graph_t *load_text(const char *path) { return new csr(path); }
static int graph_n(graph_t *g) { return g->num_nodes; }
static long long graph_m(graph_t *g) { return g->row_offset[g->num_nodes]; }
static void inject(graph_t *g, int n, long long m, std::vector<int> &row, std::vector<int> &col)
{
    // public malloc'd members (migration/.../include/csr/csr.h:6-16), freed by ~csr
    free(g->row_offset);
    free(g->col_idx);
    g->row_offset = (int *)malloc(sizeof(int) * (n + 1));
    g->col_idx = (int *)malloc(sizeof(int) * (m > 0 ? m : 1));
    memcpy(g->row_offset, row.data(), sizeof(int) * (n + 1));
    if (m) memcpy(g->col_idx, col.data(), sizeof(int) * m);
    g->num_nodes = n;
    g->num_edges = (int)m;
}
// distance is reserve()d and written through operator[] (cpuBFS.cpp:9-13),
// so size() stays 0: read it through data().
static const int *levels_of(cpuBFS &b) { return b.distance.data(); }
static void get_csr(graph_t *g, std::vector<int> &row, std::vector<int> &col)
{
    row.assign(g->row_offset, g->row_offset + g->num_nodes + 1);
    col.assign(g->col_idx, g->col_idx + g->row_offset[g->num_nodes]);
}
#endif

static graph_t *load_csr(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f) { perror(path); exit(2); }
    int n; long long m;
    if (fread(&n, 4, 1, f) != 1 || fread(&m, 8, 1, f) != 1) { fprintf(stderr, "bad csr\n"); exit(2); }
    std::vector<int> row(n + 1), col(m);
    if (fread(row.data(), 4, n + 1, f) != (size_t)(n + 1)) { fprintf(stderr, "bad csr\n"); exit(2); }
    if (m && fread(col.data(), 4, m, f) != (size_t)m) { fprintf(stderr, "bad csr\n"); exit(2); }
    fclose(f);
    // The reference objects can only be built from a file: make a 1-vertex one.
    char tmpl[] = "/tmp/gbfs_ref_XXXXXX";
    int fd = mkstemp(tmpl);
    if (fd < 0) { perror("mkstemp"); exit(2); }
    if (write(fd, "1\n0\n", 4) != 4) { perror("write"); exit(2); }
    close(fd);
    graph_t *g = load_text(tmpl);
    unlink(tmpl);
    inject(g, n, m, row, col);
    return g;
}

int main(int argc, char **argv)
{
    if (argc < 4 || (strcmp(argv[1], "csrdump") != 0 && argc < 5)) {
        fprintf(stderr, "usage: %s text|csr <graph> <source> <levels.bin> [reps]\n", argv[0]);
        return 2;
    }
    if (strcmp(argv[1], "csrdump") == 0) {
        graph_t *g = load_text(argv[2]);
        std::vector<int> row, col;
        get_csr(g, row, col);
        FILE *f = fopen(argv[3], "wb");
        if (!f) { perror(argv[3]); return 2; }
        int n = graph_n(g);
        long long m = (long long)col.size();
        fwrite(&n, 4, 1, f);
        fwrite(&m, 8, 1, f);
        fwrite(row.data(), 4, row.size(), f);
        fwrite(col.data(), 4, col.size(), f);
        fclose(f);
        delete g;
        return 0;
    }
    graph_t *g = strcmp(argv[1], "text") == 0 ? load_text(argv[2]) : load_csr(argv[2]);
    int source = std::stoi(argv[3]);
    int reps = argc > 5 ? std::stoi(argv[5]) : 1;
    int n = graph_n(g);
    std::vector<int> out(n);
    double exec_ms = 0, wall_ms = 0;
    for (int r = 0; r < reps; r++) {
        auto t0 = std::chrono::steady_clock::now();
        cpuBFS b(*g, source);
        auto t1 = std::chrono::steady_clock::now();
        exec_ms += b.exec_time;
        wall_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        if (r == 0) memcpy(out.data(), levels_of(b), sizeof(int) * n);
    }
    FILE *f = fopen(argv[4], "wb");
    if (!f) { perror(argv[4]); return 2; }
    fwrite(out.data(), 4, n, f);
    fclose(f);
    printf("n=%d m=%lld exec_ms=%.6f wall_ms=%.6f\n", n, graph_m(g), exec_ms / reps, wall_ms / reps);
    delete g;
    return 0;
}
