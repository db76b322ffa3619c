// Device-wide exclusive scan of int32 counts (CSR row pointers of the pattern build).
// Three passes over tiles of 2048 counts: tile sums, a single-block scan of the
// tile sums (int64, so an overflow of the int32 offsets is caught), and a tile-local
// scan plus tile offset.
#include "fe_internal.h"
#include "fe_scan_kernels.cuh"

namespace fe {

int exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n, int64_t *total,
                       DBuf<int64_t> &tmp, cudaStream_t s) {
    int64_t nt = (n + kTile - 1) / kTile;
    if (nt < 1) nt = 1;
    FE_CHECK(dalloc(tmp, (size_t)nt + 1));
    long long *sums = (long long *)tmp.p;
    long long *tot_dev = sums + nt;
    if (n > 0) {
        tile_sums<<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums);
        FE_LAUNCH_CHECK();
    } else {
        FE_CUDA(cudaMemsetAsync(sums, 0, sizeof(long long), s));
    }
    scan_tile_sums<<<1, kScanThreads, 0, s>>>(sums, nt, out, n, tot_dev);
    FE_LAUNCH_CHECK();
    if (n > 0) {
        scan_apply<<<(unsigned)nt, kScanThreads, 0, s>>>(in, n, sums, out);
        FE_LAUNCH_CHECK();
    }
    long long t = 0;
    FE_CUDA(cudaMemcpyAsync(&t, tot_dev, sizeof(long long), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    if (t > 0x7fffffffLL) {
        set_error("pattern too large: more than 2^31-1 entries");
        return FE_BAD_INPUT;
    }
    *total = t;
    return FE_OK;
}

}  // namespace fe
