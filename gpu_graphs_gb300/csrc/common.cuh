// common.cuh -- shared device helpers of the gbfs engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbfs.h"

namespace gbfs {

constexpr unsigned FULL = 0xffffffffu;

// ---- warp helpers ---------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T x)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(FULL, x, o);
        if ((int)lane_id() >= o) x += y;
    }
    return x;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    return x;
}

// ---- memory-model helpers -------------------------------------------------
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ int ld_relaxed_i32(const int *p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Read-only, streamed once: skip L1 allocation.
__device__ __forceinline__ int4 ld_stream_v4(const int *p)
{
    int4 v;
    asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

__device__ __forceinline__ int ld_stream(const int *p)
{
    int v;
    asm volatile("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---- device status codes (written to a control block, read by the host) --
enum DevStatus : int {
    DEV_OK = 0,
    DEV_TIMEOUT = 1,   // a bounded wait ran out
    DEV_BAD_ID = 2,    // an input id outside [0, n)
};

// ---- bounded grid barrier ---------------------------------------------------
// Used only by cooperative launches (all CTAs co-resident), so every wait
// ends once the other CTAs arrive.  Each wait is still bounded by
// `timeout_ns` of %globaltimer: when it runs out the CTA records
// DEV_TIMEOUT in *status and returns false; a CTA that sees a non-zero
// status while waiting also returns false, so every CTA leaves the kernel
// shortly after the first one gives up.
struct GridBarrier {
    unsigned count;
    unsigned gen;
};

__device__ __forceinline__ bool grid_sync(GridBarrier *bar, int *status,
                                          unsigned long long timeout_ns)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned g = ld_acquire_gpu(&bar->gen);
        __threadfence();
        unsigned t = atomicAdd(&bar->count, 1u);
        if (t == gridDim.x - 1) {
            bar->count = 0;
            __threadfence();
            st_release_gpu(&bar->gen, g + 1);
        } else {
            unsigned long long t0 = globaltimer_ns();
            unsigned spins = 0;
            while (ld_acquire_gpu(&bar->gen) == g) {
                if ((++spins & 63u) == 0) {
                    if (ld_relaxed_i32(status) != DEV_OK) { ok = 0; break; }
                    if (globaltimer_ns() - t0 > timeout_ns) {
                        atomicCAS(status, DEV_OK, DEV_TIMEOUT);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        __threadfence();
        if (ok && ld_relaxed_i32(status) != DEV_OK) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace gbfs
