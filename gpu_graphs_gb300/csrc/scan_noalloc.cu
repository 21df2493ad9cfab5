// scan_noalloc.cu -- the exclusive scan with no allocation at call time.
//
// gbfs_exclusive_scan_i32 keeps its look-back scratch in a pool that grows
// with cudaMalloc.  Some callers cannot let a library allocate device
// memory while they run: a serving process that has carved all of HBM into
// its own pools up front and treats any further cudaMalloc as an error or a
// stall (cudaMalloc and cudaFree can synchronise the device), a real-time
// loop that must not take the driver's allocation locks, or code that owns
// the allocator and calls in from inside it.  This entry point runs the same
// decoupled look-back scan (scan.cu) with its scratch in a fixed array
// compiled into the library, so it calls no cudaMalloc, cudaFree or other
// allocating routine.
//
// The price: the array (NOALLOC_BYTES, under 1 MB) is held on every GPU
// that loads the library until the process exits, the input is limited to
// GBFS_SCAN_NOALLOC_MAX_N elements, and all calls share the array, so
// calls whose work overlaps on the GPU (other streams, other threads) race
// and must be serialised by the caller.  What must start at zero (the
// status word) is cleared by every call; the per-tile states carry a call
// number, so the previous call's contents are ignored.
#include <mutex>

#include "../../include/gbfs.h"
#include "graph.cuh"
#include "scan.cuh"

namespace {

constexpr int64_t NOALLOC_TILES = (GBFS_SCAN_NOALLOC_MAX_N + gbfs::SCAN_TILE - 1) / gbfs::SCAN_TILE;
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
// Same carving as gbfs::scan_scratch_bytes(NOALLOC_TILES).
constexpr size_t NOALLOC_BYTES = 256 + align256(NOALLOC_TILES * sizeof(gbfs::ScanDesc));

static __device__ __align__(256) unsigned char g_scan_scratch[NOALLOC_BYTES];

struct DeviceState {
    std::mutex mu;
    bool ready = false;
    gbfs::ScanScratch s;
};
DeviceState g_state[64];

}  // namespace

extern "C" int gbfs_exclusive_scan_i32_noalloc(const int32_t *d_in, int64_t *d_out, int64_t n, void *stream)
{
    using namespace gbfs;
    if (n < 0 || (n > 0 && (!d_in || !d_out))) return fail(GBFS_ERR_INVALID_ARG, "bad argument");
    if (n > GBFS_SCAN_NOALLOC_MAX_N)
        return fail(GBFS_ERR_TOO_LARGE, "n exceeds GBFS_SCAN_NOALLOC_MAX_N (" +
                                            std::to_string((long long)GBFS_SCAN_NOALLOC_MAX_N) +
                                            " elements), the size of the built-in scratch");
    if (n == 0) return GBFS_OK;
    if (!is_device_ptr(d_in) || !is_device_ptr(d_out))
        return fail(GBFS_ERR_INVALID_ARG, "d_in and d_out must be device pointers");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return fail(GBFS_ERR_INVALID_ARG, "device ordinal >= 64");
    DeviceState &ds = g_state[dev];
    std::lock_guard<std::mutex> lk(ds.mu);
    if (!ds.ready) {
        // Once per device, with that device current: the array's device
        // address (in host code its name is only a host-side stand-in).
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_scan_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scan scratch)");
        scan_scratch_carve(ptr, NOALLOC_TILES, ds.s);
        ds.s.epoch = 0;
        ds.ready = true;
    }
    cudaStream_t st = (cudaStream_t)stream;
    e = cudaMemsetAsync(ds.s.ctl, 0, 3 * sizeof(unsigned), st);
    if (e == cudaSuccess) e = scan_exclusive_i32_i64(d_in, (long long *)d_out, n, nullptr, ds.s, st);
    if (e != cudaSuccess) return cuda_fail(e, "scan launch");
    unsigned status = 0;
    e = cudaMemcpyAsync(&status, ds.s.ctl + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "scan");
    if (status != 0) return fail(GBFS_ERR_TIMEOUT, "scan look-back wait ran out");
    return GBFS_OK;
}
