// scan.cu -- decoupled look-back exclusive scan (see scan.cuh).
#include "common.cuh"
#include "scan.cuh"

namespace gbfs {

namespace {

constexpr unsigned ST_AGG = 1, ST_INC = 2;
constexpr unsigned long long LOOKBACK_TIMEOUT_NS = 2000000000ULL;  // 2 s

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_exclusive(const Tin *__restrict__ in, Tout *__restrict__ out, int64_t n,
                 Tout *__restrict__ total_out, unsigned *flags, long long *agg,
                 long long *inc, unsigned *ctl, unsigned epoch, int64_t ntiles)
{
    __shared__ long long s_warp[SCAN_THREADS / 32];
    __shared__ long long s_prefix;
    __shared__ unsigned s_tile;

    if (threadIdx.x == 0) s_tile = atomicAdd(&ctl[0], 1u);
    __syncthreads();
    const int64_t tile = s_tile;
    const int64_t base = tile * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;

    long long v[SCAN_ITEMS];
    long long sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + k;
        v[k] = i < n ? (long long)in[i] : 0;
        sum += v[k];
    }
    // Block exclusive scan of the per-thread sums.
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long incl = warp_incl_scan(sum);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0;
        long long wi = warp_incl_scan(w);
        if (lane < SCAN_THREADS / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
        if (lane == SCAN_THREADS / 32 - 1) {
            // lane 7 holds the tile aggregate in wi
            long long tile_sum = wi;
            unsigned tag = epoch << 2;
            if (tile == 0) {
                inc[0] = tile_sum;
                __threadfence();
                st_release_gpu(&flags[0], tag | ST_INC);
                s_prefix = 0;
            } else {
                agg[tile] = tile_sum;
                __threadfence();
                st_release_gpu(&flags[tile], tag | ST_AGG);
                // Look back over predecessors until an inclusive prefix.
                long long prefix = 0;
                int64_t p = tile - 1;
                unsigned long long t0 = globaltimer_ns();
                unsigned spins = 0;
                bool failed = false;
                while (p >= 0) {
                    unsigned f = ld_acquire_gpu(&flags[p]);
                    if ((f >> 2) == (epoch & 0x3fffffffu) && (f & 3u) != 0) {
                        if ((f & 3u) == ST_INC) {
                            prefix += (long long)ld_relaxed_u64((const unsigned long long *)&inc[p]);
                            break;
                        }
                        prefix += (long long)ld_relaxed_u64((const unsigned long long *)&agg[p]);
                        p--;
                        continue;
                    }
                    if ((++spins & 31u) == 0 && globaltimer_ns() - t0 > LOOKBACK_TIMEOUT_NS) {
                        atomicExch(&ctl[2], (unsigned)DEV_TIMEOUT);
                        failed = true;
                        break;
                    }
                }
                if (failed) prefix = 0;
                inc[tile] = prefix + tile_sum;
                __threadfence();
                st_release_gpu(&flags[tile], tag | ST_INC);
                s_prefix = prefix;
            }
            if (tile == ntiles - 1 && total_out) *total_out = (Tout)(s_prefix + tile_sum);
        }
    }
    __syncthreads();
    long long run = s_prefix + s_warp[warp] + (incl - sum);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t i = base + k;
        if (i < n) out[i] = (Tout)run;
        run += v[k];
    }
    // Self-cleaning counters: the last tile to finish resets them.
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned done = atomicAdd(&ctl[1], 1u);
        if (done == (unsigned)(ntiles - 1)) {
            ctl[0] = 0;
            ctl[1] = 0;
            __threadfence();
        }
    }
}

template <typename Tin, typename Tout>
cudaError_t launch_scan(const Tin *in, Tout *out, int64_t n, Tout *total_out, ScanScratch &s,
                        cudaStream_t st)
{
    if (n <= 0) {
        if (total_out) return cudaMemsetAsync(total_out, 0, sizeof(Tout), st);
        return cudaSuccess;
    }
    int64_t ntiles = scan_tiles(n);
    if (ntiles > s.max_tiles || ntiles > 0x7fffffff) return cudaErrorInvalidValue;
    s.epoch = (s.epoch + 1) & 0x3fffffffu;
    if (s.epoch == 0) s.epoch = 1;
    k_scan_exclusive<Tin, Tout><<<(unsigned)ntiles, SCAN_THREADS, 0, st>>>(
        in, out, n, total_out, s.flags, s.agg, s.inc, s.ctl, s.epoch, ntiles);
    return cudaGetLastError();
}

}  // namespace

size_t scan_scratch_bytes(int64_t max_tiles)
{
    size_t t = (size_t)max_tiles;
    return 256 + ((t * 4 + 255) & ~size_t(255)) + 2 * ((t * 8 + 255) & ~size_t(255));
}

void scan_scratch_carve(void *mem, int64_t max_tiles, ScanScratch &s)
{
    char *p = (char *)mem;
    size_t t = (size_t)max_tiles;
    s.ctl = (unsigned *)p;
    p += 256;
    s.flags = (unsigned *)p;
    p += (t * 4 + 255) & ~size_t(255);
    s.agg = (long long *)p;
    p += (t * 8 + 255) & ~size_t(255);
    s.inc = (long long *)p;
    s.max_tiles = max_tiles;
}

cudaError_t scan_exclusive_i32_i32(const int *in, int *out, int64_t n, int *total_out,
                                   ScanScratch &s, cudaStream_t st)
{
    return launch_scan<int, int>(in, out, n, total_out, s, st);
}

cudaError_t scan_exclusive_i32_i64(const int *in, long long *out, int64_t n,
                                   long long *total_out, ScanScratch &s, cudaStream_t st)
{
    return launch_scan<int, long long>(in, out, n, total_out, s, st);
}

}  // namespace gbfs
