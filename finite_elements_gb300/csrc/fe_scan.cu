// Device-wide exclusive scan of int32 counts (CSR row pointers of the pattern build).
// Three passes over tiles of 2048 counts: tile sums, a single-block scan of the
// tile sums (int64, so an overflow of the int32 offsets is caught), and a tile-local
// scan plus tile offset.
#include "fe_internal.h"

namespace fe {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kTile = kScanThreads * kScanItems;

__device__ __forceinline__ long long block_exclusive_scan(long long v, long long *total) {
    __shared__ long long warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        long long s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long u = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += u;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    long long base = warp > 0 ? warp_sums[warp - 1] : 0;
    if (total) *total = warp_sums[kScanThreads / 32 - 1];
    long long r = base + inc - v;
    __syncthreads();
    return r;
}

__global__ void tile_sums(const int32_t *__restrict__ in, int64_t n, long long *__restrict__ sums) {
    int64_t base = (int64_t)blockIdx.x * kTile;
    long long s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
    long long tot;
    block_exclusive_scan(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void scan_tile_sums(long long *sums, int64_t nt, int32_t *out, int64_t n,
                               long long *total_out) {
    long long carry = 0;
    for (int64_t base = 0; base < nt; base += kScanThreads) {
        int64_t i = base + threadIdx.x;
        long long v = i < nt ? sums[i] : 0;
        long long tot;
        long long ex = block_exclusive_scan(v, &tot);
        if (i < nt) sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        *total_out = carry;
        out[n] = carry > 0x7fffffffLL ? -1 : (int32_t)carry;
    }
}

__global__ void scan_apply(const int32_t *__restrict__ in, int64_t n,
                           const long long *__restrict__ sums, int32_t *__restrict__ out) {
    int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    long long s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    long long ex = block_exclusive_scan(s, nullptr) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int64_t i = base + k;
        if (i < n) out[i] = (int32_t)ex;
        ex += v[k];
    }
}

}  // namespace

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
