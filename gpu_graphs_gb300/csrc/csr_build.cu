// csr_build.cu -- on-device edge list -> CSR (sm_103a).
//
// The reference builds CSR on the host: vector<vector<int>> adjacency lists
// filled line by line, then flattened (1D Partition/src/csr.cpp:25-65,
// 2D Partition/src/csc.cpp:18-89), with no dedup, no self-loop removal and
// no symmetrisation.  Here the same CSR (rows sorted, which does not change
// BFS levels) is built in HBM:
//   1. k_count   degree histogram (warp-aggregated atomics: match_any groups
//                lanes with the same source so hubs take one atomic)
//   2. scan      decoupled look-back exclusive scan -> row offsets
//   3. k_scatter each edge to its row (aggregated atomic cursors)
//   4. k_bin + k_sort_small / k_sort_medium / k_sort_large
//                per-row sort: rows <= 32 in registers (warp bitonic), rows
//                <= 4096 in shared memory (CTA bitonic), longer rows with a
//                CTA-wide stable LSD radix sort; each row also counts (and
//                packs to its front) its distinct values when deduplicating
//   5. scan + k_compact   packed rows -> final col_idx (dedup only)
//   6. k_finalize zero-degree bitmap, max degree, non-isolated count
#include <algorithm>
#include <climits>
#include <cstdio>

#include "common.cuh"
#include "csr_build.cuh"
#include "scan.cuh"

namespace gbfs {

namespace {

constexpr int W4_MAX = 128;       // rows up to this length: warp sort, 4 values per lane
constexpr int W16_MAX = 512;      // rows up to this length: warp sort, 16 values per lane
constexpr int MED_MAX = 4096;     // rows up to this length sort in shared memory
constexpr int MED_THREADS = 512;
constexpr int LARGE_THREADS = 1024;
constexpr int BIN_THREADS = 1024;

#define CK(call)                                                                 \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) {                                                 \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
            rc = (e_ == cudaErrorMemoryAllocation) ? GBFS_ERR_OOM : GBFS_ERR_CUDA; \
            goto done;                                                           \
        }                                                                        \
    } while (0)

__device__ __forceinline__ int atomic_add_t(int *p, int v) { return atomicAdd(p, v); }
__device__ __forceinline__ long long atomic_add_t(long long *p, long long v)
{
    return (long long)atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}

// All 32 lanes call; key < 0 means "no increment".  Returns the old value of
// arr[key] plus this lane's rank among lanes with the same key.
template <typename T>
__device__ __forceinline__ T agg_atomic_add(T *arr, int key)
{
    unsigned peers = __match_any_sync(FULL, key);
    int leader = __ffs(peers) - 1;
    T old = 0;
    if (key >= 0 && (int)lane_id() == leader) old = atomic_add_t(&arr[key], (T)__popc(peers));
    old = __shfl_sync(FULL, old, leader);
    return old + (T)__popc(peers & lanemask_lt());
}

template <typename T>
__device__ __forceinline__ T block_sum(T x, T *s_red)
{
    x = warp_sum(x);
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s_red[warp] = x;
    __syncthreads();
    T t = 0;
    if (warp == 0) {
        t = lane < (blockDim.x >> 5) ? s_red[lane] : 0;
        t = warp_sum(t);
    }
    return t;  // valid in thread 0
}

// Exclusive block scan (blockDim.x <= 1024); returns the prefix, *total set.
__device__ __forceinline__ int block_excl_scan(int x, int *s_warp, int *total)
{
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int incl = warp_incl_scan(x);
    __syncthreads();
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? s_warp[lane] : 0;
        int wi = warp_incl_scan(w);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    *total = s_warp[32];
    return s_warp[warp] + incl - x;
}

__global__ void k_count(const int *__restrict__ src, const int *__restrict__ dst, int64_t m,
                        int n, unsigned flags, int *deg, unsigned long long *total, int *status)
{
    __shared__ unsigned long long s_red[32];
    const bool sym = flags & GBFS_SYMMETRIZE, noself = flags & GBFS_DROP_SELF_LOOPS;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long mine = 0;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < m;
         base += stride) {
        int64_t i = base + lane_id();
        int u = -1, v = -1;
        if (i < m) {
            u = src[i];
            v = dst[i];
            if ((unsigned)u >= (unsigned)n || (unsigned)v >= (unsigned)n) {
                atomicExch(status, DEV_BAD_ID);
                u = v = -1;
            } else if (noself && u == v) {
                u = v = -1;
            }
        }
        // (every lane calls agg_atomic_add); a row of 2^30 edges or more
        // would overflow the int32 degrees
        const int cu = agg_atomic_add(deg, u);
        if (u >= 0 && cu >= (1 << 30)) atomicExch(status, DEV_OVERFLOW);
        mine += u >= 0;
        if (sym) {
            const int cv = agg_atomic_add(deg, v);
            if (v >= 0 && cv >= (1 << 30)) atomicExch(status, DEV_OVERFLOW);
            mine += v >= 0;
        }
    }
    unsigned long long t = block_sum(mine, s_red);
    if (threadIdx.x == 0 && t) atomicAdd(total, t);
}

template <typename RT>
__global__ void k_scatter(const int *__restrict__ src, const int *__restrict__ dst, int64_t m,
                          int n, unsigned flags, RT *cursor, int *tmp)
{
    const bool sym = flags & GBFS_SYMMETRIZE, noself = flags & GBFS_DROP_SELF_LOOPS;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < m;
         base += stride) {
        int64_t i = base + lane_id();
        int u = -1, v = -1;
        if (i < m) {
            u = src[i];
            v = dst[i];
            if ((unsigned)u >= (unsigned)n || (unsigned)v >= (unsigned)n || (noself && u == v))
                u = v = -1;
        }
        const RT p = agg_atomic_add(cursor, u);
        if (u >= 0) tmp[p] = v;
        if (sym) {
            const RT q = agg_atomic_add(cursor, v);
            if (v >= 0) tmp[q] = u;
        }
    }
}

// Rows longer than 32 go to one of four lists by length: up to W4_MAX and
// up to W16_MAX (warp sorts in registers), up to MED_MAX (CTA sort in shared
// memory), longer (radix sort).  cnt[0] medium, [1] large, [2] W4, [3] W16.
template <typename RT>
__global__ void k_bin(const RT *__restrict__ row, int n, int *med, int *large, int *w4, int *w16, unsigned *cnt)
{
    __shared__ int s_warp[33];
    __shared__ int s_base[4];
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n;
         base += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = base + threadIdx.x;
        int d = r < n ? (int)(row[r + 1] - row[r]) : 0;
        const int cls = d <= 32 ? -1 : d <= W4_MAX ? 2 : d <= W16_MAX ? 3 : d <= MED_MAX ? 0 : 1;
        int tot[4], off[4];
#pragma unroll
        for (int c = 0; c < 4; c++) off[c] = block_excl_scan(cls == c, s_warp, &tot[c]);
        if (threadIdx.x == 0)
            for (int c = 0; c < 4; c++) s_base[c] = tot[c] ? (int)atomicAdd(&cnt[c], (unsigned)tot[c]) : 0;
        __syncthreads();
        if (cls >= 0) {
            int *dst = cls == 0 ? med : cls == 1 ? large : cls == 2 ? w4 : w16;
            dst[s_base[cls] + off[cls]] = (int)r;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ int warp_bitonic_sort(int x)
{
    const unsigned lane = lane_id();
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            int y = __shfl_xor_sync(FULL, x, j);
            bool up = (lane & k) == 0;
            bool lower = (lane & j) == 0;
            x = (lower == up) ? min(x, y) : max(x, y);
        }
    }
    return x;
}

// Rows of length <= 32, one warp per row: sort in registers, pack distinct
// values.  A warp loads the offsets of 32 consecutive rows at once, then
// sorts those of them that are short, one after another.
template <typename RT>
__global__ void k_sort_small(const RT *__restrict__ row, int n, int *tmp, int dedup, int *ucnt)
{
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned lane = lane_id();
    for (int64_t r0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; r0 < n; r0 += warps * 32) {
        RT bl = 0;
        int dl = 33;  // rows past n are skipped as long ones
        if (r0 + lane < n) {
            bl = row[r0 + lane];
            dl = (int)(row[r0 + lane + 1] - bl);
        }
        for (int j = 0; j < 32; j++) {
            const int64_t r = r0 + j;
            const RT b = __shfl_sync(FULL, bl, j);
            const int d = __shfl_sync(FULL, dl, j);
            if (d > 32) continue;
            if (d <= 1) {
                if (lane == 0) ucnt[r] = d;
                continue;
            }
            int x = (int)lane < d ? tmp[b + lane] : INT_MAX;
            x = warp_bitonic_sort(x);
            if (dedup) {
                int prev = __shfl_up_sync(FULL, x, 1);
                bool uniq = (int)lane < d && (lane == 0 || x != prev);
                unsigned mask = __ballot_sync(FULL, uniq);
                if (uniq) tmp[b + __popc(mask & lanemask_lt())] = x;
                if (lane == 0) ucnt[r] = __popc(mask);
            } else {
                if ((int)lane < d) tmp[b + lane] = x;
                if (lane == 0) ucnt[r] = d;
            }
        }
    }
}

// Bitonic sort of 32*E values held E per lane (element i = lane i%32,
// register i/32), ascending.  Compare-exchange distances below 32 go
// through shuffles, larger ones between a lane's own registers; all loops
// unroll, so the registers stay registers.
template <int E>
__device__ __forceinline__ void warp_bitonic_sort_regs(int (&v)[E])
{
    const int lane = (int)lane_id();
#pragma unroll
    for (int k = 2; k <= 32 * E; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
#pragma unroll
                for (int r = 0; r < E; r++) {
                    const int r2 = r ^ (j >> 5);
                    if (r2 > r) {
                        const bool up = ((r * 32 + lane) & k) == 0;
                        const int a = v[r], c = v[r2];
                        if ((a > c) == up) {
                            v[r] = c;
                            v[r2] = a;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < E; r++) {
                    const int y = __shfl_xor_sync(FULL, v[r], j);
                    const bool up = ((r * 32 + lane) & k) == 0;
                    const bool lower = (lane & j) == 0;
                    v[r] = (lower == up) ? min(v[r], y) : max(v[r], y);
                }
            }
        }
    }
}

// One warp per listed row of length 33..32*E: sort in registers, pack the
// distinct values (dedup) or all of them back in place, record the count.
template <int E, typename RT>
__global__ void k_sort_warp(const RT *__restrict__ row, const int *__restrict__ list, const unsigned *cnt,
                            int *tmp, int dedup, int *ucnt)
{
    const int count = (int)*cnt;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = (int)lane_id();
    for (int64_t li = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < count; li += warps) {
        const int r = list[li];
        const RT b = row[r];
        const int d = (int)(row[r + 1] - b);
        int v[E];
#pragma unroll
        for (int k = 0; k < E; k++) {
            const int i = k * 32 + lane;
            v[k] = i < d ? tmp[b + i] : INT_MAX;
        }
        warp_bitonic_sort_regs<E>(v);
        int base = 0;
#pragma unroll
        for (int k = 0; k < E; k++) {
            const int i = k * 32 + lane;
            int prev = __shfl_up_sync(FULL, v[k], 1);
            if (k > 0) {
                const int last = __shfl_sync(FULL, v[k - 1], 31);
                if (lane == 0) prev = last;
            }
            const bool keep = i < d && (!dedup || i == 0 || v[k] != prev);
            const unsigned mk = __ballot_sync(FULL, keep);
            if (keep) tmp[b + base + __popc(mk & lanemask_lt())] = v[k];
            base += __popc(mk);
        }
        if (lane == 0) ucnt[r] = base;
    }
}

// One CTA per row of length W16_MAX+1..MED_MAX: bitonic sort in shared memory.
template <typename RT>
__global__ void __launch_bounds__(MED_THREADS)
k_sort_medium(const RT *__restrict__ row, const int *__restrict__ list, const unsigned *cnt,
              int *tmp, int dedup, int *ucnt)
{
    __shared__ int s[MED_MAX];
    __shared__ int s_warp[33];
    const int count = (int)cnt[0];
    for (int li = blockIdx.x; li < count; li += gridDim.x) {
        const int r = list[li];
        const RT b = row[r];
        const int d = (int)(row[r + 1] - b);
        int P = 64;
        while (P < d) P <<= 1;
        for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < d ? tmp[b + i] : INT_MAX;
        __syncthreads();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = threadIdx.x; i < P; i += blockDim.x) {
                    int ixj = i ^ j;
                    if (ixj > i) {
                        int a = s[i], c = s[ixj];
                        bool up = (i & k) == 0;
                        if ((a > c) == up) {
                            s[i] = c;
                            s[ixj] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        // Each thread owns a contiguous run of ceil(P/blockDim) slots.
        const int per = (P + blockDim.x - 1) / blockDim.x;
        const int lo = threadIdx.x * per, hi = min(lo + per, d);
        int c = 0;
        for (int i = lo; i < hi; i++) c += !dedup || i == 0 || s[i] != s[i - 1];
        int total;
        int off = block_excl_scan(c, s_warp, &total);
        int vals[8];
        int nv = 0;
        for (int i = lo; i < hi; i++)
            if (!dedup || i == 0 || s[i] != s[i - 1]) vals[nv++] = s[i];
        __syncthreads();
        for (int k = 0; k < nv; k++) tmp[b + off + k] = vals[k];
        if (threadIdx.x == 0) ucnt[r] = total;
        __syncthreads();
    }
}

// One CTA per row longer than MED_MAX: stable LSD radix sort (8-bit digits)
// ping-ponging between tmp and tmp2 over the row's own range, then packing
// distinct values into tmp.  Stability within a 1024-element tile comes
// from match_any ranks inside each warp and per-digit prefixes across warps
// in warp order.
template <typename RT>
__global__ void __launch_bounds__(LARGE_THREADS)
k_sort_large(const RT *__restrict__ row, const int *__restrict__ list, const unsigned *cnt,
             int *tmp, int *tmp2, int key_bits, int dedup, int *ucnt)
{
    __shared__ int s_hist[256];
    __shared__ int s_base[256];
    __shared__ int s_tile[256];
    __shared__ unsigned short s_wcnt[LARGE_THREADS / 32][256];
    __shared__ int s_warp[33];
    const int count = (int)cnt[1];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    for (int li = blockIdx.x; li < count; li += gridDim.x) {
        const int r = list[li];
        const RT b = row[r];
        const int d = (int)(row[r + 1] - b);
        int *from = tmp + b, *to = tmp2 + b;
        for (int shift = 0; shift < key_bits; shift += 8) {
            for (int i = threadIdx.x; i < 256; i += blockDim.x) s_hist[i] = 0;
            __syncthreads();
            for (int i = threadIdx.x; i < d; i += blockDim.x)
                atomicAdd(&s_hist[((unsigned)from[i] >> shift) & 255u], 1);
            __syncthreads();
            if (warp == 0) {  // exclusive scan of 256 bins, 8 per lane
                int v[8], t = 0;
                for (int k = 0; k < 8; k++) { v[k] = s_hist[lane * 8 + k]; t += v[k]; }
                int incl = warp_incl_scan(t);
                int run = incl - t;
                for (int k = 0; k < 8; k++) { s_base[lane * 8 + k] = run; run += v[k]; }
            }
            __syncthreads();
            for (int t0 = 0; t0 < d; t0 += blockDim.x) {
                const int i = t0 + threadIdx.x;
                const bool ok = i < d;
                const int x = ok ? from[i] : 0;
                const int dig = ok ? (int)(((unsigned)x >> shift) & 255u) : 256;
                for (int k = threadIdx.x; k < nwarps * 256; k += blockDim.x)
                    s_wcnt[k >> 8][k & 255] = 0;
                __syncthreads();
                unsigned peers = __match_any_sync(FULL, dig);
                int rank = __popc(peers & lanemask_lt());
                if (ok && (int)lane == __ffs(peers) - 1) s_wcnt[warp][dig] = (unsigned short)__popc(peers);
                __syncthreads();
                for (int k = threadIdx.x; k < 256; k += blockDim.x) {
                    int run = 0;
                    for (int w = 0; w < nwarps; w++) {
                        int c = s_wcnt[w][k];
                        s_wcnt[w][k] = (unsigned short)run;
                        run += c;
                    }
                    s_tile[k] = run;
                }
                __syncthreads();
                if (ok) to[s_base[dig] + s_wcnt[warp][dig] + rank] = x;
                __syncthreads();
                for (int k = threadIdx.x; k < 256; k += blockDim.x) s_base[k] += s_tile[k];
                __syncthreads();
            }
            int *t = from; from = to; to = t;
        }
        // Sorted values are in `from`; pack (distinct) values into tmp.
        if (from == tmp + b) {
            for (int i = threadIdx.x; i < d; i += blockDim.x) tmp2[b + i] = from[i];
            __syncthreads();
            from = tmp2 + b;
        }
        int written = 0;
        for (int t0 = 0; t0 < d; t0 += blockDim.x) {
            const int i = t0 + threadIdx.x;
            const int x = i < d ? from[i] : 0;
            const int keep = i < d && (!dedup || i == 0 || x != from[i - 1]);
            int total;
            int off = block_excl_scan(keep, s_warp, &total);
            if (keep) tmp[b + written + off] = x;
            written += total;
            __syncthreads();
        }
        if (threadIdx.x == 0) ucnt[r] = written;
        __syncthreads();
    }
}

// Copy the packed distinct prefix of each row.  A warp loads the offsets
// of 32 consecutive rows at once (one coalesced load per array instead of
// a dependent pair per row), then copies the 32 rows one after another.
template <typename RT>
__global__ void k_compact(const RT *__restrict__ row, const RT *__restrict__ row2, int n,
                          const int *__restrict__ tmp, int *col)
{
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = (int)lane_id();
    for (int64_t r0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; r0 < n; r0 += warps * 32) {
        const int64_t r = r0 + lane;
        RT b = 0, o = 0;
        int c = 0;
        // rows longer than MED_MAX before deduplication: k_compact_long
        if (r < n && row[r + 1] - row[r] <= MED_MAX) {
            b = row[r];
            o = row2[r];
            c = (int)(row2[r + 1] - o);
        }
#pragma unroll 4
        for (int j = 0; j < 32; j++) {
            const RT bj = __shfl_sync(FULL, b, j), oj = __shfl_sync(FULL, o, j);
            const int cj = __shfl_sync(FULL, c, j);
            for (int i = lane; i < cj; i += 32) col[oj + i] = tmp[bj + i];
        }
    }
}

// The rows of list[0, cnt[1]) (longer than MED_MAX before deduplication),
// one CTA per row: a long hub row copied by one warp would set the whole
// pass's time.
template <typename RT>
__global__ void k_compact_long(const RT *__restrict__ row, const RT *__restrict__ row2, const int *__restrict__ list,
                               const unsigned *cnt, const int *__restrict__ tmp, int *col)
{
    const int count = (int)cnt[1];
    for (int li = blockIdx.x; li < count; li += gridDim.x) {
        const int r = list[li];
        const RT b = row[r], o = row2[r];
        const int c = (int)(row2[r + 1] - o);
#pragma unroll 4
        for (int i = threadIdx.x; i < c; i += blockDim.x) col[o + i] = tmp[b + i];
    }
}

template <typename RT>
__global__ void k_finalize(const RT *__restrict__ row, int n, unsigned *zmask, int *maxdeg,
                           unsigned long long *nonisolated)
{
    __shared__ unsigned long long s_red[32];
    __shared__ int s_max[32];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long mine = 0;
    int mx = 0;
    const int W = (n + 31) >> 5;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < (int64_t)W * 32;
         base += stride) {
        int64_t v = base + lane_id();
        int d = v < n ? (int)(row[v + 1] - row[v]) : 0;
        unsigned z = __ballot_sync(FULL, d == 0);  // out-of-range bits count as zero-degree
        if (lane_id() == 0) zmask[v >> 5] = z;
        mine += d > 0;
        mx = max(mx, d);
    }
    unsigned long long t = block_sum(mine, s_red);
    if (threadIdx.x == 0 && t) atomicAdd(nonisolated, t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
    __syncthreads();
    if (lane_id() == 0) s_max[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned w = 1; w < (blockDim.x >> 5); w++) mx = max(mx, s_max[w]);
        atomicMax(maxdeg, mx);
    }
}

template <typename RT>
__global__ void k_heavy_list(const RT *__restrict__ row, int n, int *heavy, unsigned *cnt)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const int64_t v = base + lane_id();
        const bool h = v < n && row[v + 1] - row[v] > HEAVY_DEGREE;
        const unsigned m = __ballot_sync(FULL, h);
        if (!m) continue;
        unsigned pos = 0;
        if (lane_id() == 0) pos = atomicAdd(cnt, (unsigned)__popc(m));
        pos = __shfl_sync(FULL, pos, 0);
        if (h) heavy[pos + __popc(m & lanemask_lt())] = (int)v;
    }
}

template <typename RT>
__global__ void k_validate_csr(const RT *__restrict__ row, const int *__restrict__ col, int n,
                               int64_t m, int *status)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m || i < n; i += stride) {
        if (i < n && row[i + 1] < row[i]) atomicExch(status, DEV_BAD_ID);
        if (i < m && (unsigned)col[i] >= (unsigned)n) atomicExch(status, DEV_BAD_ID);
    }
}

// Symmetry check on sorted rows: every (u,v) has (v,u).
template <typename RT>
__global__ void k_check_sym(const RT *__restrict__ row, const int *__restrict__ col, int n, int *flags)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += stride) {
        const RT b = row[u], e = row[u + 1];
        for (RT i = b; i < e; i++) {
            const int v = col[i];
            RT lo = row[v], hi = row[v + 1];
            while (lo < hi) {
                const RT mid = (lo + hi) >> 1;
                if (col[mid] < (int)u) lo = mid + 1; else hi = mid;
            }
            if (lo >= row[v + 1] || col[lo] != (int)u) {
                flags[1] = 1;
                break;
            }
        }
    }
}

template <typename RT>
__global__ void k_check_sorted(const RT *__restrict__ row, const int *__restrict__ col, int n, int *flags)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += stride) {
        const RT b = row[u], e = row[u + 1];
        for (RT i = b + 1; i < e; i++)
            if (col[i - 1] > col[i]) {
                flags[0] = 1;
                break;
            }
    }
}

// Hub-first order: each row's highest-degree neighbour (lowest id among
// ties) is swapped to the row's front, the neighbour a bottom-up step
// probes first.  One warp per row below HUB_CTA_ROW, one CTA above.
constexpr int HUB_CTA_ROW = 4096;

template <typename RT>
__device__ __forceinline__ unsigned long long hub_key(const RT *row, int v, int pos)
{
    const unsigned d = (unsigned)(row[v + 1] - row[v]);
    return ((unsigned long long)d << 32) | (unsigned)(0x7fffffff - pos);
}

template <typename RT>
__global__ void k_hub_first_warp(const RT *__restrict__ row, int n, int *col)
{
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        const RT b = row[r];
        const int d = (int)(row[r + 1] - b);
        if (d < 2 || d >= HUB_CTA_ROW) continue;
        unsigned long long best = 0;
        for (int i = lane_id(); i < d; i += 32) {
            const unsigned long long k = hub_key(row, col[b + i], i);
            best = k > best ? k : best;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(FULL, best, o);
            best = y > best ? y : best;
        }
        const int pos = 0x7fffffff - (int)(best & 0xffffffffu);
        __syncwarp();
        if (lane_id() == 0 && pos > 0) {
            const int t = col[b];
            col[b] = col[b + pos];
            col[b + pos] = t;
        }
    }
}

// Rows of HUB_GIANT_ROW entries or more: the whole grid splits each one.
constexpr int HUB_GIANT_ROW = 65536;

// Appends the rows of length in [lo, hi) to list (count in *cnt).
template <typename RT>
__global__ void k_rows_by_len(const RT *__restrict__ row, int n, int lo, int hi, int *list, unsigned *cnt)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const int64_t r = base + lane_id();
        bool in = false;
        if (r < n) {
            const int64_t d = (int64_t)(row[r + 1] - row[r]);
            in = d >= lo && d < hi;
        }
        const unsigned m = __ballot_sync(FULL, in);
        if (!m) continue;
        unsigned pos = 0;
        if (lane_id() == 0) pos = atomicAdd(cnt, (unsigned)__popc(m));
        pos = __shfl_sync(FULL, pos, 0);
        if (in) list[pos + __popc(m & lanemask_lt())] = (int)r;
    }
}

// One CTA per listed row (list[0, *cnt)).
template <typename RT>
__global__ void k_hub_first_cta(const RT *__restrict__ row, const int *__restrict__ list, const unsigned *cnt, int *col)
{
    __shared__ unsigned long long s_best[32];
    const int count = (int)*cnt;
    for (int li = blockIdx.x; li < count; li += gridDim.x) {
        const int r = list[li];
        const RT b = row[r];
        const int d = (int)(row[r + 1] - b);
        unsigned long long best = 0;
        for (int i = threadIdx.x; i < d; i += blockDim.x) {
            const unsigned long long k = hub_key(row, col[b + i], i);
            best = k > best ? k : best;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(FULL, best, o);
            best = y > best ? y : best;
        }
        if (lane_id() == 0) s_best[threadIdx.x >> 5] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (unsigned w = 1; w < (blockDim.x >> 5); w++) best = s_best[w] > best ? s_best[w] : best;
            const int pos = 0x7fffffff - (int)(best & 0xffffffffu);
            if (pos > 0) {
                const int t = col[b];
                col[b] = col[b + pos];
                col[b + pos] = t;
            }
        }
        __syncthreads();
    }
}

// The listed giant rows one after another, each split over the whole grid:
// every warp folds its entries' keys and takes the row's maximum with one
// atomicMax (best[g], zeroed by the caller); k_hub_giant_swap then moves it.
template <typename RT>
__global__ void k_hub_giant_max(const RT *__restrict__ row, const int *__restrict__ list, const unsigned *cnt,
                                const int *__restrict__ col, unsigned long long *best)
{
    const int count = (int)*cnt;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int g = 0; g < count; g++) {
        const int r = list[g];
        const RT b = row[r];
        const int d = (int)(row[r + 1] - b);
        unsigned long long mine = 0;
        for (int64_t i = tid; i < d; i += stride) {
            const unsigned long long k = hub_key(row, col[b + i], (int)i);
            mine = k > mine ? k : mine;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(FULL, mine, o);
            mine = y > mine ? y : mine;
        }
        if (lane_id() == 0 && mine) atomicMax(best + g, mine);
    }
}

template <typename RT>
__global__ void k_hub_giant_swap(const RT *__restrict__ row, const int *__restrict__ list, const unsigned *cnt,
                                 const unsigned long long *best, int *col)
{
    const int count = (int)*cnt;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < count; g += gridDim.x * blockDim.x) {
        const RT b = row[list[g]];
        const int pos = 0x7fffffff - (int)(best[g] & 0xffffffffu);
        if (best[g] && pos > 0) {
            const int t = col[b];
            col[b] = col[b + pos];
            col[b + pos] = t;
        }
    }
}

int grid_for(int64_t work, int threads, int cap = 152 * 16)
{
    int64_t g = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

struct Scratch {
    void *p = nullptr;
    ~Scratch() { if (p) cudaFree(p); }
};

template <typename RT>
int finalize_t(DeviceCsr &out, const RT *row, cudaStream_t st, std::string &err)
{
    int rc = GBFS_OK;
    struct Res { unsigned long long nonisolated; int maxdeg; unsigned nheavy; } h{};
    Res *d_res = nullptr;
    const int W = (out.n + 31) / 32;
    CK(cudaMalloc(&out.zmask, sizeof(unsigned) * (size_t)W));
    CK(cudaMalloc(&d_res, sizeof(Res)));
    CK(cudaMemsetAsync(d_res, 0, sizeof(Res), st));
    k_finalize<<<grid_for((int64_t)W * 32, 256), 256, 0, st>>>(row, out.n, out.zmask, &d_res->maxdeg,
                                                                &d_res->nonisolated);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&h, d_res, sizeof(Res), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    out.max_degree = h.maxdeg;
    out.nonisolated = (int64_t)h.nonisolated;
    {
        // heavy-row list (sized by a first count pass folded into k_heavy_list's atomic)
        CK(cudaMalloc(&out.heavy, sizeof(int) * (size_t)std::max<int64_t>(1, out.n)));
        k_heavy_list<<<grid_for(out.n, 256), 256, 0, st>>>(row, out.n, out.heavy, &d_res->nheavy);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(&h, d_res, sizeof(Res), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        out.nheavy = (int32_t)h.nheavy;
    }
done:
    if (d_res) cudaFree(d_res);
    return rc;
}

int finalize(DeviceCsr &out, cudaStream_t st, std::string &err)
{
    return out.wide ? finalize_t(out, (const long long *)out.row64, st, err)
                    : finalize_t(out, (const int *)out.row, st, err);
}

// Sort every row of (row, col) in place (no dedup).  Scratch is allocated
// and freed here.  Synchronises st.
template <typename RT>
int sort_rows_inplace(const RT *row, int *col, int32_t n, int64_t m, cudaStream_t st, std::string &err)
{
    int rc = GBFS_OK;
    int *ucnt = nullptr, *med = nullptr, *large = nullptr, *tmp2 = nullptr, *w4 = nullptr, *w16 = nullptr;
    unsigned *lcnt = nullptr;
    int key_bits = 1;
    const int thr = 256;
    CK(cudaMalloc(&ucnt, sizeof(int) * ((size_t)n + 1)));
    CK(cudaMalloc(&med, sizeof(int) * (size_t)n));
    CK(cudaMalloc(&large, sizeof(int) * (size_t)n));
    CK(cudaMalloc(&w4, sizeof(int) * (size_t)n));
    CK(cudaMalloc(&w16, sizeof(int) * (size_t)n));
    CK(cudaMalloc(&lcnt, 16));
    CK(cudaMalloc(&tmp2, sizeof(int) * (size_t)std::max<int64_t>(m, 1)));
    CK(cudaMemsetAsync(lcnt, 0, 16, st));
    k_bin<RT><<<grid_for(n, BIN_THREADS, 152 * 4), BIN_THREADS, 0, st>>>(row, n, med, large, w4, w16, lcnt);
    CK(cudaGetLastError());
    k_sort_small<RT><<<grid_for((int64_t)n * 32, thr), thr, 0, st>>>(row, n, col, 0, ucnt);
    CK(cudaGetLastError());
    k_sort_warp<4, RT><<<152 * 8, 256, 0, st>>>(row, w4, lcnt + 2, col, 0, ucnt);
    CK(cudaGetLastError());
    k_sort_warp<16, RT><<<152 * 8, 256, 0, st>>>(row, w16, lcnt + 3, col, 0, ucnt);
    CK(cudaGetLastError());
    k_sort_medium<RT><<<152 * 4, MED_THREADS, 0, st>>>(row, med, lcnt, col, 0, ucnt);
    CK(cudaGetLastError());
    while (key_bits < 31 && (1LL << key_bits) < (int64_t)n) key_bits++;
    k_sort_large<RT><<<152 * 2, LARGE_THREADS, 0, st>>>(row, large, lcnt, col, tmp2, key_bits, 0, ucnt);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
done:
    if (ucnt) cudaFree(ucnt);
    if (med) cudaFree(med);
    if (large) cudaFree(large);
    if (w4) cudaFree(w4);
    if (w16) cudaFree(w16);
    if (lcnt) cudaFree(lcnt);
    if (tmp2) cudaFree(tmp2);
    return rc;
}

// Hub-first order for every row of (row, col), m entries: one warp per row
// below HUB_CTA_ROW entries, one CTA per listed row up to HUB_GIANT_ROW,
// the whole grid per longer row (the few longest rows of a power-law
// graph would otherwise each hold one CTA for most of the pass).
// Synchronises st.
template <typename RT>
int hub_first_rows(const RT *row, int n, int64_t m, int *col, cudaStream_t st, std::string &err)
{
    int rc = GBFS_OK;
    int *lists = nullptr;
    unsigned *cnts = nullptr;
    unsigned long long *best = nullptr;
    unsigned h[2] = {0, 0};
    const int64_t cap_long = std::min<int64_t>(n, m / HUB_CTA_ROW + 1);
    const int64_t cap_giant = std::min<int64_t>(n, m / HUB_GIANT_ROW + 1);
    CK(cudaMalloc(&lists, sizeof(int) * (size_t)(cap_long + cap_giant)));
    CK(cudaMalloc(&cnts, 2 * sizeof(unsigned)));
    CK(cudaMemsetAsync(cnts, 0, 2 * sizeof(unsigned), st));
    k_hub_first_warp<RT><<<grid_for((int64_t)n * 32, 256), 256, 0, st>>>(row, n, col);
    CK(cudaGetLastError());
    k_rows_by_len<RT><<<grid_for(n, 256), 256, 0, st>>>(row, n, HUB_CTA_ROW, HUB_GIANT_ROW, lists, cnts);
    CK(cudaGetLastError());
    k_rows_by_len<RT><<<grid_for(n, 256), 256, 0, st>>>(row, n, HUB_GIANT_ROW, INT_MAX, lists + cap_long, cnts + 1);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h, cnts, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h[0]) {
        k_hub_first_cta<RT><<<152 * 2, 512, 0, st>>>(row, lists, cnts, col);
        CK(cudaGetLastError());
    }
    if (h[1]) {
        CK(cudaMalloc(&best, sizeof(unsigned long long) * h[1]));
        CK(cudaMemsetAsync(best, 0, sizeof(unsigned long long) * h[1], st));
        k_hub_giant_max<RT><<<152 * 4, 512, 0, st>>>(row, lists + cap_long, cnts + 1, col, best);
        CK(cudaGetLastError());
        k_hub_giant_swap<RT><<<1, 256, 0, st>>>(row, lists + cap_long, cnts + 1, best, col);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(st));
done:
    if (lists) cudaFree(lists);
    if (cnts) cudaFree(cnts);
    if (best) cudaFree(best);
    return rc;
}

}  // namespace

int csr_check_symmetric(const DeviceCsr &c, cudaStream_t st, bool &sym, std::string &err)
{
    int rc = GBFS_OK;
    int *flags = nullptr, *copy = nullptr;
    int h[2] = {0, 0};
    const int grid = grid_for(c.n, 256, 152 * 8);
    CK(cudaMalloc(&flags, 8));
    CK(cudaMemsetAsync(flags, 0, 8, st));
    if (c.wide) k_check_sorted<<<grid, 256, 0, st>>>((const long long *)c.row64, c.col, c.n, flags);
    else k_check_sorted<<<grid, 256, 0, st>>>((const int *)c.row, c.col, c.n, flags);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h, flags, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    {
        const int *col = c.col;
        if (h[0]) {  // unsorted rows (hub-first ones, for instance): check a sorted copy
            CK(cudaMalloc(&copy, sizeof(int) * (size_t)std::max<int64_t>(c.m, 1)));
            CK(cudaMemcpyAsync(copy, c.col, sizeof(int) * (size_t)c.m, cudaMemcpyDeviceToDevice, st));
            rc = c.wide ? sort_rows_inplace((const long long *)c.row64, copy, c.n, c.m, st, err)
                        : sort_rows_inplace((const int *)c.row, copy, c.n, c.m, st, err);
            if (rc) goto done;
            col = copy;
        }
        if (c.wide) k_check_sym<<<grid, 256, 0, st>>>((const long long *)c.row64, col, c.n, flags);
        else k_check_sym<<<grid, 256, 0, st>>>((const int *)c.row, col, c.n, flags);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h, flags, 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        sym = h[1] == 0;
    }
done:
    if (flags) cudaFree(flags);
    if (copy) cudaFree(copy);
    return rc;
}

int csr_hub_first(DeviceCsr &c, cudaStream_t st, std::string &err)
{
    int rc = GBFS_OK;
    rc = c.wide ? hub_first_rows((const long long *)c.row64, c.n, c.m, c.col, st, err)
                : hub_first_rows((const int *)c.row, c.n, c.m, c.col, st, err);
    if (rc) goto done;
    c.hub_rows = true;
done:
    return rc;
}

namespace {

__global__ void k_in_count(const int *__restrict__ col, int64_t m, int *indeg)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&indeg[col[i]], 1);
}

// first[v] / second[v]: row v's first / second entry, -1 past its end
// (second may be null).
template <typename RT>
__global__ void k_first(const RT *__restrict__ row, const int *__restrict__ col, int n, int *first, int *second)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const RT b = row[v];
        const int d = (int)(row[v + 1] - b);
        first[v] = d > 0 ? col[b] : -1;
        if (second) second[v] = d > 1 ? col[b + 1] : -1;
    }
}

// One warp per row u: every out-edge u -> v lands in v's in-row.
__global__ void k_in_scatter(const int *__restrict__ row, const int *__restrict__ col, int n, int *cursor, int *tcol)
{
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += warps)
        for (int i = row[u] + (int)lane_id(); i < row[u + 1]; i += 32) tcol[atomicAdd(&cursor[col[i]], 1)] = (int)u;
}

}  // namespace

int csr_build_transpose(DeviceCsr &c, cudaStream_t st, std::string &err)
{
    if (c.trow) return GBFS_OK;
    if (c.wide) {
        err = "no transpose of a graph with 64-bit row offsets (its searches stay top-down)";
        return GBFS_ERR_TOO_LARGE;
    }
    int rc = GBFS_OK;
    const int n = c.n;
    const int64_t m = c.m;
    int *indeg = nullptr, *cursor = nullptr, *trow = nullptr, *tcol = nullptr, *theavy = nullptr, *tfirst = nullptr;
    unsigned *d_nheavy = nullptr, h_nheavy = 0;
    void *scan_mem = nullptr;
    ScanScratch ss;
    const int64_t tiles = scan_tiles((int64_t)n + 1);
    CK(cudaMalloc(&indeg, sizeof(int) * ((size_t)n + 1)));
    CK(cudaMalloc(&trow, sizeof(int) * ((size_t)n + 1)));
    CK(cudaMalloc(&cursor, sizeof(int) * ((size_t)n + 1)));
    CK(cudaMalloc(&tcol, sizeof(int) * (size_t)std::max<int64_t>(m, 1)));
    CK(cudaMalloc(&theavy, sizeof(int) * (size_t)std::max(1, n)));
    CK(cudaMalloc(&tfirst, sizeof(int) * (size_t)std::max(1, n)));
    CK(cudaMalloc(&d_nheavy, sizeof(unsigned)));
    CK(cudaMemsetAsync(d_nheavy, 0, sizeof(unsigned), st));
    CK(cudaMalloc(&scan_mem, scan_scratch_bytes(tiles)));
    CK(cudaMemsetAsync(scan_mem, 0, scan_scratch_bytes(tiles), st));
    scan_scratch_carve(scan_mem, tiles, ss);
    CK(cudaMemsetAsync(indeg, 0, sizeof(int) * ((size_t)n + 1), st));
    if (m > 0) {
        k_in_count<<<grid_for(m, 256), 256, 0, st>>>(c.col, m, indeg);
        CK(cudaGetLastError());
    }
    CK(scan_exclusive_i32_i32(indeg, trow, n, trow + n, ss, st));
    CK(cudaMemcpyAsync(cursor, trow, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
    if (m > 0) {
        k_in_scatter<<<grid_for((int64_t)n * 32, 256), 256, 0, st>>>(c.row, c.col, n, cursor, tcol);
        CK(cudaGetLastError());
    }
    k_heavy_list<<<grid_for(n, 256), 256, 0, st>>>((const int *)trow, n, theavy, d_nheavy);
    CK(cudaGetLastError());
    // in-rows hub-first (the in-neighbour of highest in-degree, the likeliest
    // to be reached early, is probed first), then their first entries
    rc = hub_first_rows((const int *)trow, n, m, tcol, st, err);
    if (rc) goto done;
    k_first<<<grid_for(n, 256), 256, 0, st>>>((const int *)trow, (const int *)tcol, n, tfirst, (int *)nullptr);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&h_nheavy, d_nheavy, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    {
        unsigned h_scan_status[3] = {0, 0, 0};
        CK(cudaMemcpy(h_scan_status, ss.ctl, 12, cudaMemcpyDeviceToHost));
        if (h_scan_status[2] != 0) {
            err = "scan look-back timed out";
            rc = GBFS_ERR_TIMEOUT;
            goto done;
        }
    }
    c.trow = trow;
    c.tcol = tcol;
    c.theavy = theavy;
    c.ntheavy = (int32_t)h_nheavy;
    c.tfirst = tfirst;
    trow = tcol = theavy = tfirst = nullptr;
done:
    if (theavy) cudaFree(theavy);
    if (tfirst) cudaFree(tfirst);
    if (d_nheavy) cudaFree(d_nheavy);
    if (indeg) cudaFree(indeg);
    if (cursor) cudaFree(cursor);
    if (trow) cudaFree(trow);
    if (tcol) cudaFree(tcol);
    if (scan_mem) cudaFree(scan_mem);
    return rc;
}

int csr_build_first(DeviceCsr &c, cudaStream_t st, std::string &err)
{
    int rc = GBFS_OK;
    if (!c.first) CK(cudaMalloc(&c.first, sizeof(int) * (size_t)std::max(1, c.n)));
    // hub-first rows are probed at their first entry alone: no second array
    if (!c.hub_rows && !c.second) CK(cudaMalloc(&c.second, sizeof(int) * (size_t)std::max(1, c.n)));
    if (c.n > 0) {
        if (c.wide)
            k_first<<<grid_for(c.n, 256), 256, 0, st>>>((const long long *)c.row64, (const int *)c.col, c.n, c.first,
                                                        c.second);
        else
            k_first<<<grid_for(c.n, 256), 256, 0, st>>>((const int *)c.row, (const int *)c.col, c.n, c.first,
                                                        c.second);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(st));
done:
    return rc;
}

int64_t csr_device_bytes(const DeviceCsr &c)
{
    const int64_t n = c.n, m = c.m;
    int64_t b = (c.wide ? 8 : 4) * (n + 1) + 4 * m + 4 * ((n + 31) / 32) + 4 * n;  // row, col, zmask, heavy list
    if (c.first) b += 4 * n;
    if (c.second) b += 4 * n;
    if (c.pieces) b += 8 * (int64_t)c.npieces;
    if (c.trow) b += 4 * (n + 1 + m) + 4 * n;                    // trow, tcol, theavy
    if (c.tfirst) b += 4 * n;
    if (c.tpieces) b += 8 * (int64_t)c.ntpieces;
    return b;
}

void csr_free(DeviceCsr &c)
{
    if (c.trow) cudaFree(c.trow);
    if (c.tcol) cudaFree(c.tcol);
    if (c.theavy) cudaFree(c.theavy);
    if (c.tfirst) cudaFree(c.tfirst);
    if (c.first) cudaFree(c.first);
    if (c.second) cudaFree(c.second);
    if (c.tpieces) cudaFree(c.tpieces);
    if (c.heavy) cudaFree(c.heavy);
    if (c.pieces) cudaFree(c.pieces);
    if (c.row) cudaFree(c.row);
    if (c.row64) cudaFree(c.row64);
    if (c.col) cudaFree(c.col);
    if (c.zmask) cudaFree(c.zmask);
    c = DeviceCsr{};
}

namespace {

inline cudaError_t scan_rows(const int *in, int *out, int64_t n, ScanScratch &ss, cudaStream_t st)
{
    return scan_exclusive_i32_i32(in, out, n, out + n, ss, st);
}
inline cudaError_t scan_rows(const int *in, long long *out, int64_t n, ScanScratch &ss, cudaStream_t st)
{
    return scan_exclusive_i32_i64(in, out, n, out + n, ss, st);
}

// Steps 2-5 with row offsets of type RT (int, or long long for wide
// graphs): offsets from the degrees, scatter, per-row sort, dedup
// compaction.  md: edges before deduplication.  On success the offsets and
// columns move to row_out / col_out.
template <typename RT>
int build_rows(int32_t n, int64_t m, int64_t md, const int *d_src, const int *d_dst, unsigned flags,
               const int *deg, ScanScratch &ss, unsigned *lcnt, cudaStream_t st, RT *&row_out, int *&col_out,
               int64_t &m_out, std::string &err)
{
    int rc = GBFS_OK;
    const bool dedup = flags & GBFS_DEDUP;
    RT *row = nullptr, *cursor = nullptr, *row2 = nullptr;
    int *tmp = nullptr, *tmp2 = nullptr, *ucnt = nullptr, *med = nullptr, *large = nullptr, *w4 = nullptr,
        *w16 = nullptr, *col = nullptr;
    int key_bits = 1;
    const int thr = 256;
    CK(cudaMalloc(&row, sizeof(RT) * ((size_t)n + 1)));
    CK(scan_rows(deg, row, n, ss, st));
    CK(cudaMalloc(&cursor, sizeof(RT) * ((size_t)n + 1)));
    CK(cudaMemcpyAsync(cursor, row, sizeof(RT) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
    CK(cudaMalloc(&tmp, sizeof(int) * (size_t)std::max<int64_t>(md, 1)));
    if (m > 0) {
        k_scatter<RT><<<grid_for(m, thr), thr, 0, st>>>(d_src, d_dst, m, n, flags, cursor, tmp);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(st));
    cudaFree(cursor);
    cursor = nullptr;

    // Per-row sort (+ distinct count).
    CK(cudaMalloc(&ucnt, sizeof(int) * ((size_t)n + 1)));
    CK(cudaMalloc(&med, sizeof(int) * (size_t)n));
    CK(cudaMalloc(&large, sizeof(int) * (size_t)n));
    CK(cudaMalloc(&w4, sizeof(int) * (size_t)n));
    CK(cudaMalloc(&w16, sizeof(int) * (size_t)n));
    k_bin<RT><<<grid_for(n, BIN_THREADS, 152 * 4), BIN_THREADS, 0, st>>>(row, n, med, large, w4, w16, lcnt);
    CK(cudaGetLastError());
    k_sort_small<RT><<<grid_for((int64_t)n * 32, thr), thr, 0, st>>>(row, n, tmp, dedup, ucnt);
    CK(cudaGetLastError());
    k_sort_warp<4, RT><<<152 * 8, 256, 0, st>>>(row, w4, lcnt + 2, tmp, dedup, ucnt);
    CK(cudaGetLastError());
    k_sort_warp<16, RT><<<152 * 8, 256, 0, st>>>(row, w16, lcnt + 3, tmp, dedup, ucnt);
    CK(cudaGetLastError());
    k_sort_medium<RT><<<152 * 4, MED_THREADS, 0, st>>>(row, med, lcnt, tmp, dedup, ucnt);
    CK(cudaGetLastError());
    while (key_bits < 31 && (1LL << key_bits) < (int64_t)n) key_bits++;
    CK(cudaMalloc(&tmp2, sizeof(int) * (size_t)std::max<int64_t>(md, 1)));
    k_sort_large<RT><<<152 * 2, LARGE_THREADS, 0, st>>>(row, large, lcnt, tmp, tmp2, key_bits, dedup, ucnt);
    CK(cudaGetLastError());

    if (dedup) {
        RT h_m2 = 0;
        CK(cudaMalloc(&row2, sizeof(RT) * ((size_t)n + 1)));
        CK(scan_rows(ucnt, row2, n, ss, st));
        CK(cudaMemcpyAsync(&h_m2, row2 + n, sizeof(RT), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        cudaFree(tmp2);  // the sorts are done; room for the compacted columns
        tmp2 = nullptr;
        CK(cudaMalloc(&col, sizeof(int) * (size_t)std::max<int64_t>((int64_t)h_m2, 1)));
        k_compact<RT><<<grid_for((int64_t)n * 32, thr), thr, 0, st>>>(row, row2, n, tmp, col);
        CK(cudaGetLastError());
        k_compact_long<RT><<<152 * 2, 1024, 0, st>>>(row, row2, large, lcnt, tmp, col);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        cudaFree(row);
        row = row2;
        row2 = nullptr;
        m_out = (int64_t)h_m2;
    } else {
        CK(cudaStreamSynchronize(st));
        col = tmp;
        tmp = nullptr;
        m_out = md;
    }
    row_out = row;
    col_out = col;
    row = nullptr;
    col = nullptr;
done:
    if (row) cudaFree(row);
    if (row2) cudaFree(row2);
    if (cursor) cudaFree(cursor);
    if (col) cudaFree(col);
    if (tmp) cudaFree(tmp);
    if (tmp2) cudaFree(tmp2);
    if (ucnt) cudaFree(ucnt);
    if (med) cudaFree(med);
    if (large) cudaFree(large);
    if (w4) cudaFree(w4);
    if (w16) cudaFree(w16);
    return rc;
}

}  // namespace

int csr_build_from_edges(int32_t n, int64_t m, const int *d_src, const int *d_dst, unsigned flags,
                         cudaStream_t st, DeviceCsr &out, std::string &err)
{
    int rc = GBFS_OK;
    int *deg = nullptr;
    unsigned *lcnt = nullptr;
    int *status = nullptr;
    unsigned long long *total = nullptr;
    void *scan_mem = nullptr;
    ScanScratch ss;
    unsigned long long h_total = 0;
    int h_status = 0;
    const int thr = 256;
    out = DeviceCsr{};
    out.n = n;

    // Scratch for both scans (n+1 elements at most).
    const int64_t tiles = scan_tiles((int64_t)n + 1);
    CK(cudaMalloc(&scan_mem, scan_scratch_bytes(tiles)));
    CK(cudaMemsetAsync(scan_mem, 0, scan_scratch_bytes(tiles), st));
    scan_scratch_carve(scan_mem, tiles, ss);

    CK(cudaMalloc(&deg, sizeof(int) * ((size_t)n + 1)));
    CK(cudaMalloc(&status, 64));
    total = (unsigned long long *)(status + 2);
    lcnt = (unsigned *)(status + 4);
    CK(cudaMemsetAsync(deg, 0, sizeof(int) * ((size_t)n + 1), st));
    CK(cudaMemsetAsync(status, 0, 64, st));
    if (m > 0) {
        k_count<<<grid_for(m, thr), thr, 0, st>>>(d_src, d_dst, m, n, flags, deg, total, status);
        CK(cudaGetLastError());
    }
    CK(cudaMemcpyAsync(&h_total, total, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&h_status, status, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h_status == DEV_OVERFLOW) {
        err = "a vertex with 2^30 or more edges";
        rc = GBFS_ERR_TOO_LARGE;
        goto done;
    }
    if (h_status != DEV_OK) {
        err = "edge endpoint outside [0, n)";
        rc = GBFS_ERR_INVALID_ARG;
        goto done;
    }
    out.wide = (flags & GBFS_WIDE_ROWS) || h_total > (unsigned long long)INT32_MAX;
    if (out.wide)
        rc = build_rows<long long>(n, m, (int64_t)h_total, d_src, d_dst, flags, deg, ss, lcnt, st, out.row64,
                                   out.col, out.m, err);
    else
        rc = build_rows<int>(n, m, (int64_t)h_total, d_src, d_dst, flags, deg, ss, lcnt, st, out.row, out.col,
                             out.m, err);
    if (rc) goto done;
    {
        unsigned h_scan_status[3] = {0, 0, 0};
        CK(cudaMemcpyAsync(h_scan_status, ss.ctl, 12, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (h_scan_status[2] != 0) {
            err = "scan look-back timed out";
            rc = GBFS_ERR_TIMEOUT;
            goto done;
        }
    }
    rc = finalize(out, st, err);

done:
    if (deg) cudaFree(deg);
    if (status) cudaFree(status);
    if (scan_mem) cudaFree(scan_mem);
    if (rc != GBFS_OK) csr_free(out);
    return rc;
}

namespace {

template <typename RT>
int csr_adopt_t(int32_t n, int64_t m, RT *d_row, int *d_col, cudaStream_t st, DeviceCsr &out, std::string &err)
{
    int rc = GBFS_OK;
    int *status = nullptr;
    RT h[2] = {0, 0};
    int h_status = 0;
    CK(cudaMalloc(&status, sizeof(int)));
    CK(cudaMemsetAsync(status, 0, sizeof(int), st));
    k_validate_csr<RT><<<grid_for(std::max<int64_t>(m, n), 256), 256, 0, st>>>(d_row, d_col, n, m, status);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&h[0], d_row, sizeof(RT), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&h[1], d_row + n, sizeof(RT), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&h_status, status, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h[0] != 0 || (int64_t)h[1] != m || h_status != DEV_OK) {
        err = "CSR is not well formed (row_offset[0]==0, non-decreasing, row_offset[n]==m, "
              "col ids in [0, n))";
        rc = GBFS_ERR_INVALID_ARG;
        goto done;
    }
    rc = finalize(out, st, err);
done:
    if (status) cudaFree(status);
    if (rc != GBFS_OK) csr_free(out);
    return rc;
}

}  // namespace

int csr_adopt(int32_t n, int64_t m, int *d_row, int *d_col, cudaStream_t st, DeviceCsr &out,
              std::string &err)
{
    out = DeviceCsr{};
    out.n = n;
    out.m = m;
    out.row = d_row;
    out.col = d_col;
    return csr_adopt_t(n, m, d_row, d_col, st, out, err);
}

int csr_adopt64(int32_t n, int64_t m, long long *d_row, int *d_col, cudaStream_t st, DeviceCsr &out,
                std::string &err)
{
    out = DeviceCsr{};
    out.n = n;
    out.m = m;
    out.row64 = d_row;
    out.wide = true;
    out.col = d_col;
    return csr_adopt_t(n, m, d_row, d_col, st, out, err);
}

}  // namespace gbfs
