// fe_scan_counts_noalloc: the row-pointer scan (counts -> CSR offsets) for callers
// that may not allocate device memory.
//
// Who needs it: code that receives all of its device memory from someone else's
// pool -- a framework's caching allocator, a service with a fixed memory budget, a
// plugin whose host application owns the GPU -- and code on a hot path where a
// cudaMalloc / cudaFree would add an implicit device-wide synchronisation.  Such a
// caller hands in its own input and output buffers; the only extra memory this
// scan needs, one int64 sum per tile of 2048 counts, lives in a fixed array
// compiled into the library instead of being allocated per call.
//
// Limits and rules:
// * at most kNoAllocMaxTiles tiles, i.e. n <= 67,108,864 counts; larger n is rejected
//   with FE_BAD_INPUT before any GPU work;
// * the array exists once per GPU that loads the library and stays allocated until
//   the process exits (256 KiB + 8 bytes);
// * every call shares it: calls whose kernels overlap on the GPU (other streams, other
//   threads) race and corrupt each other's offsets -- serialise them;
// * the first call on a device looks the array's device address up (a runtime API
//   call); make that first call before capturing any stream into a CUDA graph;
// * that address is cached for the life of the process: a cudaDeviceReset (or any
//   teardown of the device's primary context) invalidates it, and the entry point must
//   not be called again in that process afterwards;
// * offsets[n] = -1 flags a total beyond int32: the offsets past that point have
//   wrapped, so check offsets[n] before using any of them.
#include <mutex>

#include "fe_internal.h"
#include "fe_scan_kernels.cuh"

namespace fe {
namespace {

constexpr int64_t kNoAllocMaxTiles = 1 << 15;
constexpr int64_t kNoAllocMaxCounts = kNoAllocMaxTiles * kTile;
constexpr int kMaxDevices = 64;

// per-tile sums, then the grand total in the last used slot
static __device__ __align__(256) long long g_scan_scratch[kNoAllocMaxTiles + 1];

std::mutex g_mutex;
long long *g_scratch_addr[kMaxDevices] = {};

// Device address of g_scan_scratch on the current device, looked up once per device
// (in host code the symbol names a host-side stand-in, not device memory).
int scratch_address(long long **out) {
    int dev = 0;
    FE_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("fe_scan_counts_noalloc: device ordinal beyond the supported 64");
        return FE_BAD_INPUT;
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("fe_scan_counts_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return FE_CUDA_ERR;
        }
        g_scratch_addr[dev] = static_cast<long long *>(p);
    }
    *out = g_scratch_addr[dev];
    return FE_OK;
}

}  // namespace
}  // namespace fe

using namespace fe;

extern "C" int fe_scan_counts_noalloc(const int32_t *counts_dev, int32_t *offsets_dev, int64_t n,
                                      void *stream) {
    if (n < 0) {
        set_error("fe_scan_counts_noalloc: negative count");
        return FE_BAD_INPUT;
    }
    if (n > kNoAllocMaxCounts) {
        set_error("fe_scan_counts_noalloc: " + std::to_string(n) + " counts exceed the limit of " +
                  std::to_string(kNoAllocMaxCounts) + " that the library's fixed scratch array can scan");
        return FE_BAD_INPUT;
    }
    if (!offsets_dev || (n > 0 && !counts_dev)) {
        set_error("fe_scan_counts_noalloc: null buffer");
        return FE_BAD_INPUT;
    }
    long long *scratch = nullptr;
    FE_CHECK(scratch_address(&scratch));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int64_t nt = (n + kTile - 1) / kTile;
    if (nt < 1) nt = 1;
    if (n > 0) {
        tile_sums<<<(unsigned)nt, kScanThreads, 0, s>>>(counts_dev, n, scratch);
    } else {
        // no tile to sum: the single tile sum the next kernel reads must start at zero
        FE_CUDA(cudaMemsetAsync(scratch, 0, sizeof(long long), s));
    }
    FE_LAUNCH_CHECK();
    scan_tile_sums<<<1, kScanThreads, 0, s>>>(scratch, nt, offsets_dev, n, scratch + nt);
    FE_LAUNCH_CHECK();
    if (n > 0) {
        scan_apply<<<(unsigned)nt, kScanThreads, 0, s>>>(counts_dev, n, scratch, offsets_dev);
        FE_LAUNCH_CHECK();
    }
    return FE_OK;
}
