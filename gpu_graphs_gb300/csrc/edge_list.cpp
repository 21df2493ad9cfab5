// edge_list.cpp -- the text edge-list reader behind gbfs_read_edge_list.
//
// The reference reads "n m" and then pairs with
//     while (infile >> from >> to) { ... }
// (2D Partition/src/csc.cpp:14-25; 1D Partition/src/csr.cpp:14-29):
// integers separated by whitespace, pairs until the end of the file or the
// first token that is not an integer, a trailing unpaired integer ignored.
// This reader keeps those semantics and parses in parallel.  Where the
// reference indexes its adjacency list with an endpoint outside [0, n)
// (undefined behaviour there), this reader returns an error, for the pairs
// it reads; an integer too large for the reference's `int` (where its
// extraction would fail and end the loop) is such an endpoint too.  In
// parallel: the file is mapped, cut into chunks at whitespace, each chunk's
// integers are parsed by its own thread, and the chunks are joined in file
// order up to the first chunk that met a non-integer token.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gbfs.h"

namespace gbfs {

int fail(int code, const std::string &msg);

namespace {

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

// One integer as the reference's `>>` and scanf's %lld take it (optional
// sign, decimal digits), starting at p (whitespace already skipped).
// Returns false if there is no digit.  Values beyond +-2^62 saturate (they
// are outside any vertex range anyway).
inline bool parse_int(const char *&p, const char *end, long long &v)
{
    const char *q = p;
    bool neg = false;
    if (q < end && (*q == '+' || *q == '-')) neg = *q++ == '-';
    if (q == end || *q < '0' || *q > '9') return false;
    unsigned long long x = 0;
    constexpr unsigned long long SAT = 1ull << 62;
    while (q < end && *q >= '0' && *q <= '9') {
        if (x < SAT) x = x * 10 + (unsigned long long)(*q - '0');
        ++q;
    }
    if (x > SAT) x = SAT;
    v = neg ? -(long long)x : (long long)x;
    p = q;
    return true;
}

inline void skip_space(const char *&p, const char *end)
{
    while (p < end && is_space(*p)) ++p;
}

// A chunk's integers, already shifted by the id offset; bad_at is the index
// of its first value outside [0, n), -1 if none; stopped: it met a token
// that is not an integer (parsing stopped there).
struct Chunk {
    const char *begin = nullptr, *end = nullptr;
    std::vector<int32_t> vals;
    long long bad_at = -1;
    bool stopped = false;
    bool oom = false;
};

void parse_chunk(Chunk &c, long long off, long long n)
{
    try {
        c.vals.reserve((size_t)((c.end - c.begin) / 8 + 16));
        const char *p = c.begin;
        for (;;) {
            skip_space(p, c.end);
            if (p == c.end) return;
            long long v;
            if (!parse_int(p, c.end, v)) {
                c.stopped = true;
                return;
            }
            v -= off;
            if ((v < 0 || v >= n) && c.bad_at < 0) c.bad_at = (long long)c.vals.size();
            c.vals.push_back(v >= 0 && v < n ? (int32_t)v : 0);
        }
    } catch (const std::bad_alloc &) {
        c.oom = true;
    }
}

// The file's bytes: mapped, or read into `buf` where mapping is not possible.
struct FileBytes {
    const char *data = nullptr;
    size_t size = 0;
    void *map = nullptr;
    std::vector<char> buf;
    ~FileBytes()
    {
        if (map) munmap(map, size);
    }
};

int load_bytes(const char *path, FileBytes &fb)
{
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return fail(GBFS_ERR_IO, std::string("Unable to open file ") + path);
    struct stat st;
    if (fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
        void *m = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
        if (m != MAP_FAILED) {
            fb.map = m;
            fb.data = static_cast<const char *>(m);
            fb.size = (size_t)st.st_size;
            close(fd);
            return GBFS_OK;
        }
    }
    // not mappable (empty, a pipe, ...): read it whole
    try {
        char tmp[1 << 16];
        for (;;) {
            const ssize_t r = read(fd, tmp, sizeof(tmp));
            if (r < 0) {
                close(fd);
                return fail(GBFS_ERR_IO, std::string("read error in ") + path);
            }
            if (r == 0) break;
            fb.buf.insert(fb.buf.end(), tmp, tmp + r);
        }
    } catch (const std::bad_alloc &) {
        close(fd);
        return fail(GBFS_ERR_OOM, "host allocation failed while reading the edge list");
    }
    close(fd);
    fb.data = fb.buf.data();
    fb.size = fb.buf.size();
    return GBFS_OK;
}

}  // namespace

int read_edge_list_text(const char *path, int32_t one_based, int32_t *n_out, int64_t *m_out, int32_t **src,
                        int32_t **dst)
{
    FileBytes fb;
    int rc = load_bytes(path, fb);
    if (rc) return rc;
    const char *p = fb.data, *end = fb.data + fb.size;
    long long hn = 0, hm = 0;
    skip_space(p, end);
    bool ok = parse_int(p, end, hn);
    if (ok) {
        skip_space(p, end);
        ok = parse_int(p, end, hm);
    }
    if (!ok || hn < 1 || hn > INT32_MAX - 1 || hm < 0)
        return fail(GBFS_ERR_IO, "bad header (expected vertex and edge counts)");
    // chunks of at least 4 MB, cut at whitespace so no token is split
    const size_t body = (size_t)(end - p);
    size_t nthreads = std::max(1u, std::thread::hardware_concurrency());
    nthreads = std::min<size_t>({nthreads, 64, body / (4u << 20) + 1});
    std::vector<Chunk> chunks;
    try {
        chunks.resize(nthreads);
    } catch (const std::bad_alloc &) {
        return fail(GBFS_ERR_OOM, "host allocation failed while reading the edge list");
    }
    const char *cut = p;
    for (size_t i = 0; i < nthreads; i++) {
        const char *e = i + 1 == nthreads ? end : std::max(cut, p + body * (i + 1) / nthreads);
        while (e < end && !is_space(*e)) ++e;
        chunks[i].begin = cut;
        chunks[i].end = e;
        cut = e;
    }
    const long long off = one_based ? 1 : 0;
    if (nthreads == 1) {
        parse_chunk(chunks[0], off, hn);
    } else {
        std::vector<std::thread> th;
        try {
            th.reserve(nthreads);
            for (size_t i = 0; i < nthreads; i++) th.emplace_back(parse_chunk, std::ref(chunks[i]), off, hn);
        } catch (const std::exception &) {
            // threads could not start: parse the rest on this thread
            for (size_t i = th.size(); i < nthreads; i++) parse_chunk(chunks[i], off, hn);
        }
        for (auto &t : th) t.join();
    }
    // join in file order, up to the first chunk that stopped at a
    // non-integer token; a final unpaired integer is dropped
    size_t used = 0;
    long long total = 0, first_bad = -1;
    for (; used < nthreads; used++) {
        const Chunk &c = chunks[used];
        if (c.oom) return fail(GBFS_ERR_OOM, "host allocation failed while reading the edge list");
        if (c.bad_at >= 0 && first_bad < 0) first_bad = total + c.bad_at;
        total += (long long)c.vals.size();
        if (c.stopped) {
            ++used;
            break;
        }
    }
    const long long pairs_vals = total & ~1LL;
    if (first_bad >= 0 && first_bad < pairs_vals)
        return fail(GBFS_ERR_IO, "edge endpoint outside the declared vertex range");
    const size_t cnt = (size_t)(pairs_vals / 2);
    int32_t *s = (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(cnt, 1));
    int32_t *d = (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(cnt, 1));
    if (!s || !d) {
        free(s);
        free(d);
        return fail(GBFS_ERR_OOM, "host allocation failed");
    }
    long long g = 0;
    for (size_t i = 0; i < used; i++)
        for (int32_t v : chunks[i].vals) {
            if (g >= pairs_vals) break;
            (g & 1 ? d : s)[g >> 1] = v;
            ++g;
        }
    *src = s;
    *dst = d;
    *n_out = (int32_t)hn;
    *m_out = (int64_t)cnt;
    return GBFS_OK;
}

}  // namespace gbfs
