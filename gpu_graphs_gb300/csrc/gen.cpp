// gen.cpp -- seeded synthetic workload generators (host side).
//
// The reference reads its graphs from text files only; these generators
// make the synthetic stand-ins for its inputs (Erdos-Renyi, RMAT/Kronecker
// in the Graph500 shape, perturbed 2D grids).  Every edge is a pure
// function of (seed, edge index) through a counter-based splitmix64
// stream, so the output does not depend on the number of threads or the
// machine (x86_64 and aarch64 give the same bytes).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/gbfs.h"

namespace {

inline uint64_t mix64(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// Independent stream `stream` of `seed`; draw(i) is its i-th 64-bit word.
struct Stream {
    uint64_t key;
    Stream(uint64_t seed, uint64_t stream) : key(mix64(seed ^ mix64(stream * 0xd1b54a32d192ed03ULL))) {}
    uint64_t draw(uint64_t i) const { return mix64(key + i * 0x9e3779b97f4a7c15ULL); }
};

// Uniform integer in [0, n) from the top 32 bits (multiply-shift).
inline uint32_t bounded(uint64_t r, uint32_t n) { return (uint32_t)(((r >> 32) * (uint64_t)n) >> 32); }

inline uint32_t threshold32(double p)
{
    if (p <= 0) return 0;
    if (p >= 1) return 0xffffffffu;
    return (uint32_t)std::floor(p * 4294967296.0);
}

template <typename F>
void parallel_chunks(int64_t total, F fn)
{
    unsigned hw = std::thread::hardware_concurrency();
    int nt = (int)std::min<int64_t>(std::max(1u, std::min(hw, 64u)), std::max<int64_t>(1, total / 65536));
    if (nt <= 1) { fn(0, (int64_t)0, total); return; }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) {
        int64_t b = total * t / nt, e = total * (t + 1) / nt;
        th.emplace_back([=] { fn(t, b, e); });
    }
    for (auto &x : th) x.join();
}

}  // namespace

extern "C" int64_t gbfs_gen_er(int32_t n, int64_t pairs, uint64_t seed, int32_t *src,
                               int32_t *dst, int64_t cap)
{
    if (n <= 0 || pairs < 0 || !src || !dst) return GBFS_ERR_INVALID_ARG;
    if (cap < pairs) return GBFS_ERR_INVALID_ARG;
    Stream s(seed, 1);
    parallel_chunks(pairs, [&](int, int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            src[i] = (int32_t)bounded(s.draw(2 * (uint64_t)i), (uint32_t)n);
            dst[i] = (int32_t)bounded(s.draw(2 * (uint64_t)i + 1), (uint32_t)n);
        }
    });
    return pairs;
}

extern "C" int64_t gbfs_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b,
                                 double c, uint64_t seed, int32_t *src, int32_t *dst,
                                 int64_t cap)
{
    if (scale < 1 || scale > 30 || edge_factor < 1 || !src || !dst) return GBFS_ERR_INVALID_ARG;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return GBFS_ERR_INVALID_ARG;
    const int64_t nv = int64_t(1) << scale;
    const int64_t m = nv * edge_factor;
    if (cap < m) return GBFS_ERR_INVALID_ARG;
    const uint32_t ta = threshold32(a), tab = threshold32(a + b), tabc = threshold32(a + b + c);

    // Seeded vertex permutation (Fisher-Yates on stream 3).
    std::vector<int32_t> perm((size_t)nv);
    for (int64_t i = 0; i < nv; i++) perm[i] = (int32_t)i;
    Stream ps(seed, 3);
    for (int64_t i = nv - 1; i > 0; i--) {
        int64_t j = (int64_t)bounded(ps.draw((uint64_t)i), (uint32_t)(i + 1));
        std::swap(perm[i], perm[j]);
    }

    Stream s(seed, 2);
    const int words = (scale + 1) / 2;  // two 32-bit decisions per 64-bit draw
    parallel_chunks(m, [&](int, int64_t bgn, int64_t end) {
        for (int64_t i = bgn; i < end; i++) {
            uint32_t u = 0, v = 0;
            for (int w = 0; w < words; w++) {
                uint64_t r = s.draw((uint64_t)i * words + w);
                for (int h = 0; h < 2; h++) {
                    if (2 * w + h >= scale) break;
                    uint32_t x = h ? (uint32_t)(r >> 32) : (uint32_t)r;
                    uint32_t bu, bv;
                    if (x < ta)        { bu = 0; bv = 0; }
                    else if (x < tab)  { bu = 0; bv = 1; }
                    else if (x < tabc) { bu = 1; bv = 0; }
                    else               { bu = 1; bv = 1; }
                    u = (u << 1) | bu;
                    v = (v << 1) | bv;
                }
            }
            src[i] = perm[u];
            dst[i] = perm[v];
        }
    });
    return m;
}

static int64_t grid_extra_count(int32_t side, double extra)
{
    double base = 2.0 * (double)side * (double)(side - 1);
    return (int64_t)std::llround(extra * base);
}

extern "C" int64_t gbfs_gen_grid_capacity(int32_t side, double extra)
{
    if (side < 1 || extra < 0) return GBFS_ERR_INVALID_ARG;
    return 2 * (int64_t)side * (side - 1) + grid_extra_count(side, extra);
}

extern "C" int64_t gbfs_gen_grid(int32_t side, double drop, double extra, int32_t radius,
                                 uint64_t seed, int32_t *src, int32_t *dst, int64_t cap)
{
    if (side < 1 || (int64_t)side * side > INT32_MAX || drop < 0 || drop > 1 || extra < 0 ||
        radius < 1 || !src || !dst)
        return GBFS_ERR_INVALID_ARG;
    const int64_t H = (int64_t)side * (side - 1);  // horizontal edges
    const int64_t G = 2 * H;                       // + vertical edges
    const int64_t X = grid_extra_count(side, extra);
    if (cap < G + X) return GBFS_ERR_INVALID_ARG;
    // Drop decision per grid edge: keep if draw >= drop * 2^64.
    const uint64_t tdrop = drop >= 1 ? ~0ULL : (uint64_t)std::floor(drop * 18446744073709551616.0);
    Stream sd(seed, 4);
    auto endpoints = [&](int64_t e, int32_t &u, int32_t &v) {
        if (e < H) {  // (r, c) - (r, c+1)
            int64_t r = e / (side - 1), c = e % (side - 1);
            u = (int32_t)(r * side + c);
            v = u + 1;
        } else {      // (r, c) - (r+1, c)
            int64_t k = e - H;
            int64_t r = k / side, c = k % side;
            u = (int32_t)(r * side + c);
            v = u + side;
        }
    };
    // Pass 1: kept-edge count per chunk; pass 2: write at scanned offsets.
    const int chunks = 256;
    std::vector<int64_t> cnt(chunks + 1, 0);
    auto chunk_range = [&](int k, int64_t &b, int64_t &e) { b = G * k / chunks; e = G * (k + 1) / chunks; };
    parallel_chunks(chunks, [&](int, int64_t kb, int64_t ke) {
        for (int64_t k = kb; k < ke; k++) {
            int64_t b, e, c = 0;
            chunk_range((int)k, b, e);
            for (int64_t i = b; i < e; i++) c += sd.draw((uint64_t)i) >= tdrop;
            cnt[k + 1] = c;
        }
    });
    for (int k = 0; k < chunks; k++) cnt[k + 1] += cnt[k];
    parallel_chunks(chunks, [&](int, int64_t kb, int64_t ke) {
        for (int64_t k = kb; k < ke; k++) {
            int64_t b, e, w = cnt[k];
            chunk_range((int)k, b, e);
            for (int64_t i = b; i < e; i++) {
                if (sd.draw((uint64_t)i) < tdrop) continue;
                int32_t u, v;
                endpoints(i, u, v);
                src[w] = u;
                dst[w] = v;
                w++;
            }
        }
    });
    const int64_t kept = cnt[chunks];
    // Extra edges: uniform vertex, uniform offset in the Manhattan diamond
    // 1 <= |dx|+|dy| <= radius, rejection-sampled on the edge's own substream;
    // an edge with no accepted draw in 64 tries becomes a self-loop (dropped
    // by GBFS_DROP_SELF_LOOPS), so the count stays fixed.
    Stream sx(seed, 5);
    const int span = 2 * radius + 1;
    parallel_chunks(X, [&](int, int64_t b, int64_t e) {
        for (int64_t j = b; j < e; j++) {
            Stream sub(sx.draw((uint64_t)j), 7);
            uint32_t u = bounded(sub.draw(0), (uint32_t)((int64_t)side * side));
            int64_t ur = u / side, uc = u % side;
            uint32_t v = u;
            for (int t = 0; t < 64; t++) {
                uint64_t r = sub.draw(1 + (uint64_t)t);
                int dx = (int)bounded(r, (uint32_t)span) - radius;
                int dy = (int)bounded(r << 32, (uint32_t)span) - radius;
                int d = std::abs(dx) + std::abs(dy);
                if (d < 1 || d > radius) continue;
                int64_t vr = ur + dy, vc = uc + dx;
                if (vr < 0 || vr >= side || vc < 0 || vc >= side) continue;
                v = (uint32_t)(vr * side + vc);
                break;
            }
            src[kept + j] = (int32_t)u;
            dst[kept + j] = (int32_t)v;
        }
    });
    return kept + X;
}
