// scan.cu -- decoupled look-back exclusive scan (see scan.cuh).
#include <algorithm>

#include "common.cuh"
#include "scan.cuh"

namespace gbfs {

namespace {

constexpr unsigned long long ST_AGG = 1, ST_INC = 2;
constexpr unsigned long long LOOKBACK_TIMEOUT_NS = 2000000000ULL;  // 2 s
constexpr int SCAN_WARPS = SCAN_THREADS / 32;
constexpr int WARP_ELEMS = SCAN_TILE / SCAN_WARPS;  // consecutive elements of one warp
constexpr int VEC_ROUNDS = WARP_ELEMS / 128;        // 16-byte vectors per lane
static_assert(WARP_ELEMS % 128 == 0, "a warp's part is whole rounds of 32 lanes x 4 elements");

// One tile's published state: its aggregate or inclusive prefix and a
// status word (call number << 2 | ST_AGG / ST_INC) in one 16-byte word,
// written and read with single 16-byte accesses, so a reader sees a value
// together with the status it was published under (16-byte aligned vector
// accesses are single transactions on these GPUs) and a look-back step
// costs one round trip.
__device__ __forceinline__ void desc_store(ScanDesc *d, long long value, unsigned long long status)
{
    asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(d), "l"(value), "l"(status) : "memory");
}

__device__ __forceinline__ void desc_load(const ScanDesc *d, long long &value, unsigned long long &status)
{
    asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(value), "=l"(status) : "l"(d) : "memory");
}

// Four consecutive outputs e, e+a, e+a+b, e+a+b+c as one 16-byte store (two
// for 8-byte outputs).
__device__ __forceinline__ void store4(int *o, long long e, int4 x)
{
    const long long e1 = e + x.x, e2 = e1 + x.y, e3 = e2 + x.z;
    *reinterpret_cast<int4 *>(o) = make_int4((int)e, (int)e1, (int)e2, (int)e3);
}
__device__ __forceinline__ void store4(long long *o, long long e, int4 x)
{
    const long long e1 = e + x.x, e2 = e1 + x.y, e3 = e2 + x.z;
    reinterpret_cast<longlong2 *>(o)[0] = make_longlong2(e, e1);
    reinterpret_cast<longlong2 *>(o)[1] = make_longlong2(e2, e3);
}

// One CTA per tile of SCAN_TILE elements; tile = blockIdx.x.  Thread 0
// bulk-copies (TMA) the tile into shared memory; warp w owns the tile's
// w-th run of WARP_ELEMS consecutive elements, which its lanes read as
// 16-byte vectors interleaved by lane (vector l + 32 r of the run is lane
// l's r-th: conflict-free in shared memory, coalesced in global memory).
// The tile reduces, publishes its aggregate, looks back over its
// predecessors' published aggregates / inclusive prefixes (the whole CTA,
// SCAN_THREADS predecessors per step), publishes its inclusive prefix and
// writes its outputs from registers, vector by vector, with a running warp
// scan.  A tile waits only on tiles with smaller indices, which the
// hardware dispatches first (CTAs start in blockIdx order), so they are
// running or done; every wait is bounded all the same.  vec: in and out
// are 16-byte aligned (the host checks); then full tiles are bulk-loaded
// and stored as vectors, other tiles use scalar accesses in the same
// layout.  Several CTAs per SM (small shared memory, few registers) keep
// several tiles' loads in flight.
template <typename Tin, typename Tout>
__global__ void __launch_bounds__(SCAN_THREADS, SCAN_MIN_BLOCKS)
k_scan_exclusive(const Tin *__restrict__ in, Tout *__restrict__ out, int64_t n,
                 Tout *__restrict__ total_out, ScanDesc *desc, unsigned *ctl, unsigned epoch, int64_t ntiles,
                 int vec)
{
    static_assert(sizeof(Tin) == 4, "4-byte inputs");
    extern __shared__ __align__(128) int s_in[];  // SCAN_TILE inputs
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ long long s_warp[SCAN_WARPS];
    __shared__ long long s_prefix, s_tile_sum;
    __shared__ unsigned s_okm[SCAN_WARPS], s_incm[SCAN_WARPS];
    __shared__ long long s_part[SCAN_WARPS];
    __shared__ bool s_abort;

    const int t = (int)threadIdx.x;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t tile = blockIdx.x;
    const int64_t tbase = tile * SCAN_TILE;
    const bool full = tbase + SCAN_TILE <= n;
    const bool bulk = vec && full;
    const unsigned long long tag = (unsigned long long)epoch << 2;

    if (bulk) {
        if (t == 0) {
            mbar_init(&s_bar, 1);
            mbar_init_fence();
            mbar_arrive_expect_tx(&s_bar, (unsigned)(SCAN_TILE * sizeof(Tin)));
            bulk_load(s_in, in + tbase, (unsigned)(SCAN_TILE * sizeof(Tin)), &s_bar);
        }
        __syncthreads();  // the barrier is initialised before anyone waits on it
        const unsigned long long w0 = globaltimer_ns();
        unsigned spins = 0;
        bool landed;
        while (!(landed = mbar_try_wait(&s_bar, 0u))) {
            if ((++spins & 63u) == 0 && globaltimer_ns() - w0 > LOOKBACK_TIMEOUT_NS) break;
        }
        if (__syncthreads_or(!landed)) {
            // the copy did not land in time: report it, and let it land
            // (bounded) before this CTA's shared memory goes away
            if (t == 0) {
                atomicExch(&ctl[2], (unsigned)DEV_TIMEOUT);
                const unsigned long long w1 = globaltimer_ns();
                while (!mbar_try_wait(&s_bar, 0u) && globaltimer_ns() - w1 < LOOKBACK_TIMEOUT_NS) {
                }
            }
            return;
        }
    }

    // the warp's vectors: vector r of this lane starts at element
    // wbase + (32 r + lane) * 4 of the tile
    const int wbase = (int)warp * WARP_ELEMS;
    auto vec_at = [&](int r) -> int4 {
        const int e = wbase + (r * 32 + (int)lane) * 4;
        if (bulk) return *reinterpret_cast<const int4 *>(s_in + e);
        int4 x;
        const int64_t g = tbase + e;
        x.x = g < n ? in[g] : 0;
        x.y = g + 1 < n ? in[g + 1] : 0;
        x.z = g + 2 < n ? in[g + 2] : 0;
        x.w = g + 3 < n ? in[g + 3] : 0;
        return x;
    };

    // tile reduction: lane sums, warp sums, block exclusive scan of the warps
    long long lsum = 0;
#pragma unroll
    for (int r = 0; r < VEC_ROUNDS; r++) {
        const int4 x = vec_at(r);
        lsum += (long long)x.x + x.y + x.z + x.w;
    }
    const long long wsum = warp_sum(lsum);
    if (lane == 0) s_warp[warp] = wsum;
    __syncthreads();
    if (warp == 0) {
        const long long w = lane < SCAN_WARPS ? s_warp[lane] : 0;
        const long long wi = warp_incl_scan(w);
        if (lane < SCAN_WARPS) s_warp[lane] = wi - w;  // exclusive warp offsets
        const long long tile_sum = __shfl_sync(FULL, wi, SCAN_WARPS - 1);
        if (lane == 0) {
            s_tile_sum = tile_sum;
            if (tile == 0) {
                desc_store(&desc[0], tile_sum, tag | ST_INC);
                s_prefix = 0;
                if (ntiles == 1 && total_out) *total_out = (Tout)tile_sum;
            } else {
                desc_store(&desc[tile], tile_sum, tag | ST_AGG);
            }
        }
    }
    __syncthreads();
    if (tile > 0) {
        // Look-back by the whole CTA: thread t reads predecessor p - t.  The
        // window is usable once every predecessor up to the nearest inclusive
        // prefix has published; then the aggregates before it and that
        // prefix are summed, else all of the window's aggregates are and it
        // moves on.  Decisions come from shared memory, so all warps take
        // them together.
        constexpr int LB = SCAN_THREADS;  // predecessors per step
        long long prefix = 0;
        int64_t p = tile - 1;
        const unsigned long long t0 = globaltimer_ns();
        unsigned spins = 0;
        for (;;) {
            const int64_t idx = p - (int64_t)t;
            long long val = 0;
            unsigned long long f = tag | ST_INC;  // before tile 0: an inclusive prefix of 0
            if (idx >= 0) desc_load(&desc[idx], val, f);
            const bool ok = (f >> 2) == (unsigned long long)epoch && (f & 3u) != 0;
            const unsigned okm = __ballot_sync(FULL, ok);
            const unsigned incm = __ballot_sync(FULL, ok && (f & 3u) == ST_INC);
            if (lane == 0) {
                s_okm[warp] = okm;
                s_incm[warp] = incm;
            }
            __syncthreads();
            int fi = LB;  // window position of the nearest inclusive prefix
            bool valid = true;
#pragma unroll
            for (int w2 = 0; w2 < SCAN_WARPS; w2++) {
                if (fi < LB) break;
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
                const long long part = warp_sum((t <= fi && idx >= 0) ? val : 0ll);
                if (lane == 0) s_part[warp] = part;
                __syncthreads();
#pragma unroll
                for (int w2 = 0; w2 < SCAN_WARPS; w2++) prefix += s_part[w2];
                __syncthreads();  // before the next window reuses the shared words
                if (fi < LB) break;
                p -= LB;
                continue;
            }
            if (t == 0) s_abort = (++spins & 31u) == 0 && globaltimer_ns() - t0 > LOOKBACK_TIMEOUT_NS;
            __syncthreads();
            const bool abort = s_abort;
            __syncthreads();
            if (abort) {
                if (t == 0) atomicExch(&ctl[2], (unsigned)DEV_TIMEOUT);
                prefix = 0;
                break;
            }
        }
        if (t == 0) {
            const long long tile_sum = s_tile_sum;
            desc_store(&desc[tile], prefix + tile_sum, tag | ST_INC);
            s_prefix = prefix;
            if (tile == ntiles - 1 && total_out) *total_out = (Tout)(prefix + tile_sum);
        }
    }
    __syncthreads();

    // outputs, vector by vector, with a running scan over the warp's lanes
    long long run = s_prefix + s_warp[warp];
#pragma unroll
    for (int r = 0; r < VEC_ROUNDS; r++) {
        const int4 x = vec_at(r);
        const long long vs = (long long)x.x + x.y + x.z + x.w;
        const long long incl = warp_incl_scan(vs);
        const long long e = run + incl - vs;
        const int el = wbase + (r * 32 + (int)lane) * 4;
        if (bulk) {
            store4(out + tbase + el, e, x);
        } else {
            const int64_t g = tbase + el;
            const long long o[4] = {e, e + x.x, e + x.x + x.y, e + x.x + x.y + x.z};
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (g + k < n) out[g + k] = (Tout)o[k];
        }
        run += __shfl_sync(FULL, incl, 31);
    }
}

constexpr size_t scan_smem_bytes() { return (size_t)SCAN_TILE * 4; }

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
                                    (int)scan_smem_bytes());
    });
    if (e != cudaSuccess) return e;
    const int vec = ((uintptr_t)in % 16 == 0) && ((uintptr_t)out % 16 == 0);
    k_scan_exclusive<Tin, Tout><<<(unsigned)ntiles, SCAN_THREADS, scan_smem_bytes(), st>>>(
        in, out, n, total_out, s.desc, s.ctl, s.epoch, ntiles, vec);
    return cudaGetLastError();
}

}  // namespace

size_t scan_scratch_bytes(int64_t max_tiles)
{
    return 256 + (((size_t)max_tiles * sizeof(ScanDesc) + 255) & ~size_t(255));
}

void scan_scratch_carve(void *mem, int64_t max_tiles, ScanScratch &s)
{
    char *p = (char *)mem;
    s.ctl = (unsigned *)p;
    s.desc = (ScanDesc *)(p + 256);
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
