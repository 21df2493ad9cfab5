// common.cuh -- shared device helpers of the gbfs engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/gbfs.h"

namespace gbfs {

// Per-device facts a kernel's launcher computes on first use (its dynamic
// shared-memory attribute, SM count, CTAs per SM), safe when several host
// threads launch for the first time at once.
struct LaunchSetup {
    std::mutex mu;
    bool done[64] = {};
    cudaError_t err[64] = {};
    int sms[64] = {};
    int occ[64] = {};

    // f(sms, occ) fills the facts for the current device once; returns its error.
    template <typename F>
    cudaError_t get(int &sms_out, int &occ_out, F f)
    {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lk(mu);
        if (!done[dev]) {
            err[dev] = f(dev, sms[dev], occ[dev]);
            done[dev] = err[dev] == cudaSuccess;
            if (!done[dev]) return err[dev];
        }
        sms_out = sms[dev];
        occ_out = occ[dev];
        return cudaSuccess;
    }
};

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

// Fetch-add with acquire-release ordering at GPU scope: publishes this
// thread's earlier writes and, for the thread that sees the final count,
// makes everyone's published writes visible.
__device__ __forceinline__ unsigned atom_add_acq_rel_gpu(unsigned *p, unsigned v)
{
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_relaxed_i32(const int *p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// ---- mbarrier and bulk (TMA) copies, shared memory of this CTA ------------
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes initialised mbarriers visible to the async proxy (bulk copies).
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// One arrival that also expects `bytes` of bulk-copy transactions.
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// True once the phase with this parity has completed.
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global memory into this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Orders this CTA's earlier generic shared-memory accesses before later
// bulk copies into the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

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
    DEV_OVERFLOW = 3,  // a bounded on-chip queue would have overflowed
};

// ---- bounded grid barrier ---------------------------------------------------
// Used only by cooperative launches (all CTAs co-resident), so every wait
// ends once the other CTAs arrive.  Arrival is a one-way release reduction
// on a counter that only grows during a launch; CTA thread 0 then spins
// with acquire loads until the counter reaches epoch * gridDim.x (epoch =
// barriers passed so far, identical in every CTA).  Each wait is bounded by
// `timeout_ns` of %globaltimer: when it runs out the CTA records
// DEV_TIMEOUT in *status and returns false; a CTA that sees a non-zero
// status while waiting also returns false, so every CTA leaves the kernel
// shortly after the first one gives up.  grid_exit() (called once by every
// CTA at the end of a successful launch) lets the last CTA out reset the
// counters for the next launch.
struct GridBarrier {
    unsigned count;
    unsigned exit;
};

__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool grid_sync(GridBarrier *bar, int *status, unsigned long long timeout_ns,
                                          unsigned &epoch)
{
    __shared__ int s_ok;
    __syncthreads();
    ++epoch;
    if (threadIdx.x == 0) {
        const unsigned target = epoch * gridDim.x;
        red_release_add(&bar->count, 1u);
        int ok = 1;
        unsigned long long t0 = 0;
        unsigned spins = 0;
        while ((int)(ld_acquire_gpu(&bar->count) - target) < 0) {
            if ((++spins & 31u) == 0) {
                if (ld_relaxed_i32(status) != DEV_OK) {
                    ok = 0;
                    break;
                }
                const unsigned long long now = globaltimer_ns();
                if (t0 == 0) {
                    t0 = now;
                } else if (now - t0 > timeout_ns) {
                    atomicCAS(status, DEV_OK, DEV_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Count this CTA out; the last one resets the barrier for the next launch
// and, if t_exit is given, stamps %globaltimer there.
__device__ __forceinline__ void grid_exit(GridBarrier *bar, unsigned long long *t_exit = nullptr)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned old = atomicAdd(&bar->exit, 1u);
        if (old == gridDim.x - 1) {
            bar->count = 0;
            bar->exit = 0;
            if (t_exit) *t_exit = globaltimer_ns();
            __threadfence();
        }
    }
}

}  // namespace gbfs
