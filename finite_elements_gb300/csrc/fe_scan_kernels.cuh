// Exclusive-scan kernels over int32 counts (tiles of 2048 counts): tile sums, a
// single-block scan of the tile sums in int64, and the tile-local scan plus tile
// offset.  Included by the translation units that launch them.
#pragma once

#include <stdint.h>

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
}  // namespace fe
