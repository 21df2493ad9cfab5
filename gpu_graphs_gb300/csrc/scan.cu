// scan.cu -- decoupled look-back exclusive scan (see scan.cuh).
#include "common.cuh"
#include "scan.cuh"

namespace gbfs {

namespace {

constexpr unsigned ST_AGG = 1, ST_INC = 2;
constexpr int LB_WARPS = 4;  // warps of the look-back: 32 * LB_WARPS predecessors per step

// Barrier 1 over the look-back warps only (threads 0 .. 32 * LB_WARPS - 1).
__device__ __forceinline__ void lb_sync()
{
    asm volatile("bar.sync 1, %0;" ::"n"(32 * LB_WARPS) : "memory");
}
constexpr unsigned long long LOOKBACK_TIMEOUT_NS = 2000000000ULL;  // 2 s

// Shared-memory index of tile element i with one pad word per 32 words, so
// the blocked accesses (thread t: elements t*SCAN_ITEMS ... ) spread over the
// banks; 8-byte elements are padded per 16.
template <typename T>
__device__ __forceinline__ int pad_index(int i)
{
    return sizeof(T) == 8 ? i + (i >> 4) : i + (i >> 5);
}

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(SCAN_THREADS, 1)
k_scan_exclusive(const Tin *__restrict__ in, Tout *__restrict__ out, int64_t n,
                 Tout *__restrict__ total_out, unsigned *flags, long long *agg,
                 long long *inc, unsigned *ctl, unsigned epoch, int64_t ntiles)
{
    // staging area for the tile (dynamic, scan_stage_bytes()): read and
    // written coalesced (striped), used blocked by the scan
    extern __shared__ __align__(16) int s_stage[];
    __shared__ long long s_warp[SCAN_THREADS / 32];
    __shared__ long long s_prefix, s_tile_sum;
    __shared__ unsigned s_tile;
    __shared__ unsigned s_okm[LB_WARPS], s_incm[LB_WARPS];
    __shared__ long long s_part[LB_WARPS];
    __shared__ bool s_abort;

    if (threadIdx.x == 0) s_tile = atomicAdd(&ctl[0], 1u);
    __syncthreads();
    const int64_t tile = s_tile;
    const int64_t tbase = tile * SCAN_TILE;

    Tin *s_in = reinterpret_cast<Tin *>(s_stage);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int j = k * SCAN_THREADS + threadIdx.x;
        const int64_t i = tbase + j;
        s_in[pad_index<Tin>(j)] = i < n ? in[i] : Tin(0);
    }
    __syncthreads();
    Tin v[SCAN_ITEMS];
    long long sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = s_in[pad_index<Tin>(threadIdx.x * SCAN_ITEMS + k)];
        sum += (long long)v[k];
    }
    // Block exclusive scan of the per-thread sums.
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long incl = warp_incl_scan(sum);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const long long w = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0;
        const long long wi = warp_incl_scan(w);
        if (lane < SCAN_THREADS / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
        const long long tile_sum = __shfl_sync(FULL, wi, SCAN_THREADS / 32 - 1);
        if (lane == 0) {
            s_tile_sum = tile_sum;
            if (tile == 0) {
                inc[0] = tile_sum;
                __threadfence();
                st_release_gpu(&flags[0], (epoch << 2) | ST_INC);
                s_prefix = 0;
                if (ntiles == 1 && total_out) *total_out = (Tout)tile_sum;
            } else {
                agg[tile] = tile_sum;
                __threadfence();
                st_release_gpu(&flags[tile], (epoch << 2) | ST_AGG);
            }
        }
    }
    __syncthreads();
    if (tile > 0 && warp < LB_WARPS) {
        // Look-back by LB_WARPS warps: thread t of them reads predecessor
        // p - t.  The window is usable once every predecessor up to the
        // nearest inclusive prefix has published; then the aggregates before
        // it and that prefix are summed, else all of the window's aggregates
        // are and it moves on.  Decisions come from shared memory, so the
        // warps take them together (named barrier 1 over LB_WARPS warps).
        const unsigned tag = epoch << 2;
        const int t = (int)threadIdx.x;  // 0 .. 32 * LB_WARPS - 1
        long long prefix = 0;
        int64_t p = tile - 1;
        const unsigned long long t0 = globaltimer_ns();
        unsigned spins = 0;
        for (;;) {
            const int64_t idx = p - (int64_t)t;
            unsigned f = tag | ST_INC;  // before tile 0: an inclusive prefix of 0
            if (idx >= 0) f = ld_relaxed_u32(&flags[idx]);
            const bool ok = (f >> 2) == (epoch & 0x3fffffffu) && (f & 3u) != 0;
            const unsigned okm = __ballot_sync(FULL, ok);
            const unsigned incm = __ballot_sync(FULL, ok && (f & 3u) == ST_INC);
            if (lane == 0) {
                s_okm[warp] = okm;
                s_incm[warp] = incm;
            }
            lb_sync();
            int fi = 32 * LB_WARPS;  // window position of the nearest inclusive prefix
            bool valid = true;
#pragma unroll
            for (int w2 = 0; w2 < LB_WARPS; w2++) {
                if (fi < 32 * LB_WARPS) break;
                const unsigned im = s_incm[w2], om = s_okm[w2];
                if (im) {
                    const int l = __ffs(im) - 1;
                    const unsigned need = l < 31 ? ((2u << l) - 1u) : FULL;
                    valid = valid && (om & need) == need;
                    fi = w2 * 32 + l;
                } else {
                    valid = valid && om == FULL;
                }
            }
            if (valid) {
                __threadfence();  // acquire: the values published with those flags
                long long val = 0;
                if (t <= fi && idx >= 0)
                    val = t == fi ? (long long)ld_relaxed_u64((const unsigned long long *)&inc[idx])
                                  : (long long)ld_relaxed_u64((const unsigned long long *)&agg[idx]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(FULL, val, o);
                if (lane == 0) s_part[warp] = val;
                lb_sync();
#pragma unroll
                for (int w2 = 0; w2 < LB_WARPS; w2++) prefix += s_part[w2];
                lb_sync();  // before the next window reuses the shared words
                if (fi < 32 * LB_WARPS) break;
                p -= 32 * LB_WARPS;
                continue;
            }
            if (t == 0) s_abort = (++spins & 31u) == 0 && globaltimer_ns() - t0 > LOOKBACK_TIMEOUT_NS;
            lb_sync();
            const bool abort = s_abort;
            lb_sync();
            if (abort) {
                if (t == 0) atomicExch(&ctl[2], (unsigned)DEV_TIMEOUT);
                prefix = 0;
                break;
            }
        }
        if (t == 0) {
            const long long tile_sum = s_tile_sum;
            inc[tile] = prefix + tile_sum;
            __threadfence();
            st_release_gpu(&flags[tile], tag | ST_INC);
            s_prefix = prefix;
            if (tile == ntiles - 1 && total_out) *total_out = (Tout)(prefix + tile_sum);
        }
    }
    __syncthreads();  // also: every thread has read its inputs from s_stage
    long long run = s_prefix + s_warp[warp] + (incl - sum);
    Tout *s_out = reinterpret_cast<Tout *>(s_stage);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        s_out[pad_index<Tout>(threadIdx.x * SCAN_ITEMS + k)] = (Tout)run;
        run += (long long)v[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int j = k * SCAN_THREADS + threadIdx.x;
        const int64_t i = tbase + j;
        if (i < n) out[i] = s_out[pad_index<Tout>(j)];
    }
}

constexpr size_t scan_stage_bytes() { return (size_t)(SCAN_TILE + SCAN_TILE / 16) * 8; }

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
    static LaunchSetup setup;  // per template instance
    int unused_sms = 0, unused_occ = 0;
    cudaError_t e = setup.get(unused_sms, unused_occ, [&](int, int &, int &) {
        return cudaFuncSetAttribute(k_scan_exclusive<Tin, Tout>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)scan_stage_bytes());
    });
    if (e != cudaSuccess) return e;
    // the tile ticket starts at zero (flags carry the call number instead)
    e = cudaMemsetAsync(s.ctl, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_scan_exclusive<Tin, Tout><<<(unsigned)ntiles, SCAN_THREADS, scan_stage_bytes(), st>>>(
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
