// selftest.cu -- exercises the bounded device-side wait without a fault.
//
// A two-CTA cooperative kernel in which CTA 1 returns without arriving at
// the grid barrier: CTA 0's wait (the same grid_sync every persistent kernel
// of the engine uses) must run out after timeout_ms, record DEV_TIMEOUT and
// return, leaving the CUDA context usable.  Nothing faults, traps or hangs.
#include "graph.cuh"

using namespace gbfs;

namespace {

struct Probe {
    GridBarrier bar;
    int status;
    int passed;  // CTAs that got past the barrier
};

__global__ void k_wait_probe(Probe *p, unsigned long long timeout_ns)
{
    unsigned epoch = 0;
    if (blockIdx.x == 1) return;  // never arrives: nothing will release CTA 0
    if (grid_sync(&p->bar, &p->status, timeout_ns, epoch) && threadIdx.x == 0) atomicAdd(&p->passed, 1);
}

}  // namespace

extern "C" int gbfs_selftest_wait_timeout(int32_t timeout_ms)
{
    if (timeout_ms < 1 || timeout_ms > 10000) return fail(GBFS_ERR_INVALID_ARG, "timeout_ms must be in [1, 10000]");
    Probe *d = nullptr;
    Probe h{};
    cudaError_t e = cudaMalloc(&d, sizeof(Probe));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    unsigned long long ns = (unsigned long long)timeout_ms * 1000000ull;
    void *args[] = {&d, &ns};
    e = cudaMemset(d, 0, sizeof(Probe));
    if (e == cudaSuccess) e = cudaLaunchCooperativeKernel((const void *)k_wait_probe, dim3(2), dim3(64), args, 0, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(Probe), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "wait probe");
    if (h.status == DEV_TIMEOUT && h.passed == 0) return fail(GBFS_ERR_TIMEOUT, "bounded wait ran out as expected");
    return fail(GBFS_ERR_CUDA, "bounded wait did not report a timeout");
}
