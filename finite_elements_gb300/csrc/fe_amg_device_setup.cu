// Device setup of the smoothed-aggregation hierarchy: amg::setup_hierarchy
// (fe_amg_passes.cuh, the passes fe_amg_build_parallel_host runs on the host) on the
// device executor -- every pass one grid-stride kernel over its rows, int64 prefix
// sums on the device between the passes that size the next ones -- and the dense
// inverse of the coarsest matrix (at most 4096 DOFs) by block sweeps on the device.
#include <algorithm>
#include <mutex>
#include <cmath>
#include <functional>
#include <vector>

#include "fe_amg_dev.h"
#include "fe_amg_par.cuh"
#include "fe_grid_sync.cuh"

namespace fe {
namespace {

constexpr int kST = 256;                 // threads per block
constexpr int kScanPer = 8;              // elements per thread in the scans
constexpr int kScanTile = kST * kScanPer;

inline int grid_s(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kST - 1) / kST, 152 * 8)); }

#define FE_ROWS(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------- int64 exclusive scan

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v) {
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive prefix of v over the block's threads; *total = the block's sum
__device__ int64_t block_excl_scan(int64_t v, int64_t *total) {
    __shared__ int64_t warp_sum[kST / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t inc = warp_incl_scan(v);
    if (lane == 31) warp_sum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int64_t w = lane < kST / 32 ? warp_sum[lane] : 0;
        const int64_t wi = warp_incl_scan(w);
        if (lane < kST / 32) warp_sum[lane] = wi - w;   // exclusive prefix of the warp sums
        if (lane == kST / 32 - 1) *total = wi;
    }
    __syncthreads();
    const int64_t out = warp_sum[wid] + inc - v;
    __syncthreads();
    return out;
}

__global__ void ks_tile_sums(const int64_t *__restrict__ in, int64_t n, int64_t *__restrict__ part) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    int64_t v = 0;
    for (int k = 0; k < kScanPer; ++k)
        if (base + k < n) v += in[base + k];
    __shared__ int64_t tot;
    block_excl_scan(v, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// exclusive scan of the tile sums by one block, kST at a time with a carry; out[n] = total
__global__ void __launch_bounds__(kST) ks_scan_tiles(int64_t nt, int64_t *part, int64_t *out, int64_t n) {
    __shared__ int64_t chunk_total;
    int64_t carry = 0;
    for (int64_t c0 = 0; c0 < nt; c0 += blockDim.x) {
        const int64_t t = c0 + threadIdx.x;
        const int64_t v = t < nt ? part[t] : 0;
        const int64_t ex = block_excl_scan(v, &chunk_total);
        if (t < nt) part[t] = carry + ex;
        carry += chunk_total;
        __syncthreads();   // every thread has read chunk_total before the next chunk writes it
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void ks_tile_scan(const int64_t *__restrict__ in, int64_t n, const int64_t *__restrict__ part,
                             int64_t *__restrict__ out) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    int64_t local[kScanPer];
    int64_t v = 0;
    for (int k = 0; k < kScanPer; ++k) {
        local[k] = base + k < n ? in[base + k] : 0;
        v += local[k];
    }
    __shared__ int64_t tot;
    int64_t run = part[blockIdx.x] + block_excl_scan(v, &tot);
    for (int k = 0; k < kScanPer; ++k)
        if (base + k < n) out[base + k] = run, run += local[k];
}

// out[0..n] = exclusive prefix sums of in[0..n), out[n] the total (also returned)
int scan64(const int64_t *in, int64_t n, int64_t *out, int64_t *total, DBuf<int64_t> &tmp, const MgMem &mem) {
    const cudaStream_t s = mem.s;
    const int64_t nt = std::max<int64_t>(1, (n + kScanTile - 1) / kScanTile);
    FE_CHECK(palloc(mem, tmp, (size_t)nt));
    ks_tile_sums<<<(unsigned)nt, kST, 0, s>>>(in, n, tmp.p);
    ks_scan_tiles<<<1, kST, 0, s>>>(nt, tmp.p, out, n);
    ks_tile_scan<<<(unsigned)nt, kST, 0, s>>>(in, n, tmp.p, out);
    FE_LAUNCH_CHECK();
    int64_t *pin = reinterpret_cast<int64_t *>(mem.pinned);
    FE_CUDA(cudaMemcpyAsync(pin, out + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    *total = *pin;
    return FE_OK;
}

// ---------------------------------------------------------------- device executor

template <typename F>
__global__ void k_rows(int64_t n, F f) {
    FE_ROWS(i, n) f(i);
}

__device__ __forceinline__ double block_sum_d(double v) {
    __shared__ double sh[kST / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < kST / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;
}

__global__ void kd_dot(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *part) {
    double s = 0.0;
    FE_ROWS(i, n) s = fma(a[i], b[i], s);
    s = block_sum_d(s);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void kd_dot_final(int nb, const double *__restrict__ part, double *out) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[i];
    s = block_sum_d(s);
    if (threadIdx.x == 0) *out = s;
}

// y = D^-1 A x, or y = A x when dinv is null (FP64), with G lanes of a warp per block
// row (a strided share of its blocks each, then a shuffle sum): the products of the
// lmax estimates
template <int D, int G>
__global__ void __launch_bounds__(kST) kd_dinv_product(int64_t n, amg::PassDinvProduct f) {
    const int sub = threadIdx.x & (G - 1);
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
    const int64_t rows_padded = ((n + groups - 1) / groups) * groups;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; i < rows_padded; i += groups) {
        double acc[D];
#pragma unroll
        for (int a = 0; a < D; ++a) acc[a] = 0.0;
        if (i < n) {
            for (int64_t s = f.ptr[i] + sub; s < f.ptr[i + 1]; s += G) {
                const double *b = f.val + s * D * D;
                const double *xc = f.x + (int64_t)f.col[s] * D;
#pragma unroll
                for (int a = 0; a < D; ++a)
#pragma unroll
                    for (int k = 0; k < D; ++k) acc[a] = fma(b[a * D + k], xc[k], acc[a]);
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int a = 0; a < D; ++a) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], o);
        if (i < n && sub == 0)
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double v = 0.0;
                if (f.dinv) {
#pragma unroll
                    for (int k = 0; k < D; ++k) v = fma(f.dinv[i * D * D + a * D + k], acc[k], v);
                } else {
                    v = acc[a];
                }
                f.y[i * D + a] = v;
            }
    }
}

template <int D>
int launch_dinv_product(int64_t n, const amg::PassDinvProduct &f, cudaStream_t s) {
    const double mean = n > 0 ? (double)f.nnzb / (double)n : 0.0;
    const int G = mean < 4 ? 2 : mean < 10 ? 4 : mean < 24 ? 8 : 32;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n * G + kST - 1) / kST, 152 * 8));
    switch (G) {
        case 2: kd_dinv_product<D, 2><<<grid, kST, 0, s>>>(n, f); break;
        case 4: kd_dinv_product<D, 4><<<grid, kST, 0, s>>>(n, f); break;
        case 8: kd_dinv_product<D, 8><<<grid, kST, 0, s>>>(n, f); break;
        default: kd_dinv_product<D, 32><<<grid, kST, 0, s>>>(n, f); break;
    }
    FE_LAUNCH_CHECK();
    return FE_OK;
}

// ---------------------------------------------------------------- sparse products, a warp per row
// Rows of C = A B whose product lists are long (the Galerkin products and the coarser
// levels) get a warp each instead of a thread: the candidates are gathered into shared
// memory by the 32 lanes, bitonic-sorted there and compacted; after a stable counting
// sort of the product terms by output entry the values are summed term-parallel
// (kd_prod_vals_warp) or by the lane owning the entry, in the factors' order
// (kd_prod_vals_long, the thread-per-row order).  Rows beyond the shared-memory capacity
// fall back to the row operation of one lane.

constexpr int kPW = 2;          // warps per block of the warp-per-row product kernels
constexpr int kColCap = 4096;   // candidates a warp sorts in shared memory
constexpr int kTermCap = 1024;  // product terms (and output entries) a warp orders in shared memory

// ascending bitonic sort of a[0..m), m a power of two, by the lanes of a warp
__device__ void warp_bitonic(int32_t *a, int m) {
    const int lane = threadIdx.x & 31;
    for (int k = 2; k <= m; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < m; i += 32) {
                const int l = i ^ j;
                if (l > i) {
                    const int32_t x = a[i], y = a[l];
                    if ((x > y) == ((i & k) == 0)) a[i] = y, a[l] = x;
                }
            }
            __syncwarp();
        }
}

// The distinct candidates of a row: inserted into an open-addressing table in shared
// memory (linear probing on a multiplicative hash, atomicCAS; at most `size` probes, and
// the table never holds more values than it has slots), compacted, then bitonic-sorted
// -- only the distinct values, far fewer than the candidates on the coarse levels.
constexpr int32_t kEmpty = -1;

__device__ __forceinline__ void table_insert(int32_t *tab, int size, int32_t c) {
    uint32_t h = ((uint32_t)c * 2654435761u) & (uint32_t)(size - 1);
    for (int probe = 0; probe < size; ++probe) {
        const int32_t old = atomicCAS(&tab[h], kEmpty, c);
        if (old == kEmpty || old == c) return;
        h = (h + 1) & (uint32_t)(size - 1);
    }
}

__global__ void __launch_bounds__(kPW * 32) kd_prod_cols_warp(int64_t n, amg::PassProdCols f) {
    __shared__ int32_t sh[kPW][kColCap];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    int32_t *a = sh[wl];
    const int64_t W = (int64_t)gridDim.x * kPW;
    for (int64_t i = (int64_t)blockIdx.x * kPW + wl; i < n; i += W) {
        const int64_t bound = f.boff[i + 1] - f.boff[i];
        int32_t *out = f.cand + f.boff[i];
        if (bound > kColCap) continue;   // kd_prod_cols_long's row
        int size = 32;
        while (size < 2 * bound && size < kColCap) size <<= 1;
        for (int t = lane; t < size; t += 32) a[t] = kEmpty;
        __syncwarp();
        for (int64_t s = f.aptr[i]; s < f.aptr[i + 1]; ++s) {
            const int32_t c = f.acol[s];
            const int64_t t0 = f.bptr[c], len = f.bptr[c + 1] - t0;
            for (int64_t t = lane; t < len; t += 32) table_insert(a, size, f.bcol[t0 + t]);
        }
        __syncwarp();
        // compact the occupied slots to the front (each chunk read before it is written)
        int run = 0;
        for (int t0 = 0; t0 < size; t0 += 32) {
            const int32_t v = a[t0 + lane];
            const bool keep = v != kEmpty;
            const unsigned mask = __ballot_sync(0xffffffffu, keep);
            __syncwarp();
            if (keep) a[run + __popc(mask & ((1u << lane) - 1u))] = v;
            run += __popc(mask);
            __syncwarp();
        }
        int m = 1;
        while (m < run) m <<= 1;
        for (int t = run + lane; t < m; t += 32) a[t] = 0x7fffffff;
        __syncwarp();
        warp_bitonic(a, m);
        for (int t = lane; t < run; t += 32) out[t] = a[t];
        if (lane == 0) f.cnt[i] = run;
        __syncwarp();
    }
}

// Dynamic shared memory of kd_prod_vals_warp, per warp: the 32 block products of a
// chunk of terms (a row of 33 doubles per block entry, so that lanes reading different
// entries of the same term hit different banks), six arrays of kTermCap ints (term
// positions, order, A and B indices, counts, offsets) and the chunk's segment bounds and
// keys (33 + 33, padded to 80).
constexpr int kSegStride = 33, kSegInts = 80;
template <int RA, int CB>
constexpr int warp_vals_bs() { return RA && CB ? RA * CB : 36; }
template <int RA, int CB>
constexpr size_t warp_vals_smem() {
    return (size_t)kPW * ((size_t)warp_vals_bs<RA, CB>() * kSegStride * sizeof(double) +
                          (6 * (size_t)kTermCap + kSegInts) * sizeof(int32_t));
}

// C row i's values; RA x CA times CA x CB blocks (0: the sizes of f at run time)
template <int RA, int CA, int CB>
__global__ void __launch_bounds__(kPW * 32) kd_prod_vals_warp(int64_t n, amg::PassProdVals f) {
    extern __shared__ __align__(16) unsigned char s_warp_vals[];
    constexpr int BSM = warp_vals_bs<RA, CB>();
    const int ra = RA ? RA : f.ra, ca = CA ? CA : f.ca, cb = CB ? CB : f.cb;
    const int bs = ra * cb;
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    double *vbuf = reinterpret_cast<double *>(s_warp_vals) + (size_t)wl * BSM * kSegStride;
    int32_t *ib = reinterpret_cast<int32_t *>(s_warp_vals + (size_t)kPW * BSM * kSegStride * sizeof(double)) +
                  (size_t)wl * (6 * kTermCap + kSegInts);
    int32_t *pos = ib, *ord = ib + kTermCap, *ss = ib + 2 * kTermCap, *ts = ib + 3 * kTermCap;
    int32_t *cnt = ib + 4 * kTermCap, *off = ib + 5 * kTermCap, *sstart = ib + 6 * kTermCap, *skey = sstart + 40;
    const int64_t W = (int64_t)gridDim.x * kPW;
    for (int64_t i = (int64_t)blockIdx.x * kPW + wl; i < n; i += W) {
        const int64_t T = f.boff[i + 1] - f.boff[i];
        const int64_t c0 = f.cptr[i], lc = f.cptr[i + 1] - c0;
        if (T > kTermCap || lc > kTermCap) continue;   // kd_prod_vals_long's row
        // the terms in factor order, with their output entries
        for (int64_t p = lane; p < lc; p += 32) cnt[p] = 0;
        int64_t base = 0;
        for (int64_t s = f.aptr[i]; s < f.aptr[i + 1]; ++s) {
            const int32_t c = f.acol[s];
            const int64_t t0 = f.bptr[c], len = f.bptr[c + 1] - t0;
            for (int64_t t = lane; t < len; t += 32) {
                const int32_t bc = f.bcol[t0 + t];
                const int64_t p = (f.upper && bc < i) ? -1 : amg::find_sorted(f.ccol, c0, c0 + lc, bc);
                pos[base + t] = p < 0 ? -1 : (int32_t)(p - c0);
                ss[base + t] = (int32_t)s;
                ts[base + t] = (int32_t)(t0 + t);
            }
            base += len;
        }
        __syncwarp();
        for (int64_t t = lane; t < T; t += 32)
            if (pos[t] >= 0) atomicAdd(&cnt[pos[t]], 1);
        __syncwarp();
        // exclusive scan of the counts into off
        int carry = 0;
        for (int64_t p0 = 0; p0 < lc; p0 += 32) {
            const int64_t p = p0 + lane;
            const int v = p < lc ? cnt[p] : 0;
            int x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (p < lc) off[p] = carry + x - v;
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
        __syncwarp();
        // stable scatter of the term indices by output entry (off[p] ends at its range's end)
        for (int64_t t0 = 0; t0 < T; t0 += 32) {
            const int64_t t = t0 + lane;
            const int p = t < T ? pos[t] : -1;
            const int key = p >= 0 ? p : -1 - lane;   // lanes without a term match no one
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            if (p >= 0) ord[off[p] + __popc(peers & ((1u << lane) - 1u))] = (int32_t)t;
            __syncwarp();
            if (p >= 0 && lane == 31 - __clz(peers)) off[p] += __popc(peers);
            __syncwarp();
        }
        // the values, term-parallel: the terms ordered by output entry are taken 32 at a
        // time and a lane computes one term's block product into shared memory; the
        // chunk's terms of one entry are contiguous (a segment), and the lanes then take
        // (segment, block entry) pairs, each summing its segment's values in term order
        // and adding that partial to the output -- chunk after chunk, so the sums are
        // deterministic.  A lane summing whole entries alone left ~3 of 4 lanes idle (rows
        // have few entries of uneven length); a shuffle scan across the lanes cost 5 FP64
        // additions per block entry and chunk, more than the products of a 6 x 3 x 6 term,
        // where this costs about one per block entry and chunk
        for (int64_t p = lane; p < lc; p += 32) {
            if (f.upper && f.ccol[c0 + p] < i) continue;   // filled by the mirror pass
            double *o = f.cval + (c0 + p) * bs;
            for (int k = 0; k < bs; ++k) o[k] = 0.0;
        }
        __syncwarp();
        const int tv = lc > 0 ? off[lc - 1] : 0;   // the terms that reach an entry
        for (int q0 = 0; q0 < tv; q0 += 32) {
            const int q = q0 + lane;
            const bool valid = q < tv;   // the valid lanes are a prefix of the warp
            const int t = valid ? ord[q] : 0;
            const int key = valid ? pos[t] : -1;   // non-decreasing over the valid lanes
            double v[BSM];
            for (int k = 0; k < bs; ++k) v[k] = 0.0;
            if (valid)
                amg::block_mul_add(f.aval + (int64_t)ss[t] * ra * ca, f.bval + (int64_t)ts[t] * ca * cb, ra, ca, cb,
                                   v);
            for (int k = 0; k < bs; ++k) vbuf[k * kSegStride + lane] = v[k];
            // segment starts: the first valid lane of each key
            const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
            const bool start = valid && (lane == 0 || kprev != key);
            const unsigned starts = __ballot_sync(0xffffffffu, start);
            if (start) {
                const int r = __popc(starts & ((1u << lane) - 1u));
                sstart[r] = lane;
                skey[r] = key;
            }
            const int nseg = __popc(starts);   // >= 1: lane 0 is valid
            if (lane == 0) sstart[nseg] = tv - q0 < 32 ? tv - q0 : 32;
            __syncwarp();
            for (int j = lane; j < nseg * bs; j += 32) {
                const int sg = j / bs, k = j - sg * bs;
                double acc = 0.0;
                for (int x = sstart[sg]; x < sstart[sg + 1]; ++x) acc += vbuf[k * kSegStride + x];
                f.cval[(c0 + skey[sg]) * bs + k] += acc;
            }
            __syncwarp();
        }
    }
}

template <int RA, int CA, int CB>
__global__ void __launch_bounds__(kST) kd_prod_vals_thread(int64_t n, amg::PassProdVals f) {
    FE_ROWS(i, n)
    amg::row_product_values_t<RA, CA, CB>(f.aptr, f.acol, f.aval, f.ra, f.ca, f.bptr, f.bcol, f.bval, f.cb, f.cptr,
                                          f.ccol, f.cval, i, f.upper != 0);
}

// mean product terms per row at and above which the products take a warp per row
constexpr double kWarpRowMean = 48.0;

inline int warp_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kPW - 1) / kPW, 152 * 32)); }

// Rows beyond the short kernels' capacity: one warp per block and the buffers in dynamic
// shared memory, 16-bit where they fit -- up to kLongTerms candidates (product terms),
// kLongOut output entries and kLongA entries of the row of A; beyond that the row
// operation of one lane.
constexpr int kLongTerms = 8192, kLongOut = 2048, kLongA = 512;
constexpr size_t kLongColsSmem = kLongTerms * sizeof(int32_t);
constexpr size_t kLongValsSmem = 2 * kLongTerms * sizeof(int16_t) + 2 * kLongOut * sizeof(int32_t) +
                                 (kLongA + 1) * sizeof(int32_t);

// Rows past the short kernel's capacity: the candidates are streamed from global memory
// into a table of kLongTerms slots in dynamic shared memory (one warp per block), which
// only has to hold the distinct columns -- a few hundred on the coarse levels, however
// many candidates; a row with more distinct columns than slots (an insert that finds
// no slot) takes the row operation of one lane.
__device__ __forceinline__ bool table_insert_checked(int32_t *tab, int size, int32_t c) {
    uint32_t h = ((uint32_t)c * 2654435761u) & (uint32_t)(size - 1);
    for (int probe = 0; probe < size; ++probe) {
        const int32_t old = atomicCAS(&tab[h], kEmpty, c);
        if (old == kEmpty || old == c) return true;
        h = (h + 1) & (uint32_t)(size - 1);
    }
    return false;
}

__global__ void __launch_bounds__(32) kd_prod_cols_long(int64_t n, amg::PassProdCols f) {
    extern __shared__ int32_t a[];
    const int lane = threadIdx.x & 31;
    constexpr int size = kLongTerms;
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const int64_t bound = f.boff[i + 1] - f.boff[i];
        if (bound <= kColCap) continue;   // the short kernel's row
        int32_t *out = f.cand + f.boff[i];
        for (int t = lane; t < size; t += 32) a[t] = kEmpty;
        __syncwarp();
        bool ok = true;
        for (int64_t s = f.aptr[i]; s < f.aptr[i + 1] && ok; ++s) {
            const int32_t c = f.acol[s];
            const int64_t t0 = f.bptr[c], len = f.bptr[c + 1] - t0;
            bool mine = true;
            for (int64_t t = lane; t < len; t += 32) mine = table_insert_checked(a, size, f.bcol[t0 + t]) && mine;
            ok = __all_sync(0xffffffffu, mine);
        }
        __syncwarp();
        if (!ok) {
            if (lane == 0) f.cnt[i] = amg::row_product_columns(f.aptr, f.acol, f.bptr, f.bcol, i, out);
            __syncwarp();
            continue;
        }
        int run = 0;
        for (int t0 = 0; t0 < size; t0 += 32) {
            const int32_t v = a[t0 + lane];
            const bool keep = v != kEmpty;
            const unsigned mask = __ballot_sync(0xffffffffu, keep);
            __syncwarp();
            if (keep) a[run + __popc(mask & ((1u << lane) - 1u))] = v;
            run += __popc(mask);
            __syncwarp();
        }
        int m = 1;
        while (m < run) m <<= 1;
        for (int t = run + lane; t < m; t += 32) a[t] = 0x7fffffff;
        __syncwarp();
        warp_bitonic(a, m);
        for (int t = lane; t < run; t += 32) out[t] = a[t];
        if (lane == 0) f.cnt[i] = run;
        __syncwarp();
    }
}

template <int RA, int CA, int CB>
__global__ void __launch_bounds__(32) kd_prod_vals_long(int64_t n, amg::PassProdVals f) {
    extern __shared__ int32_t dsm[];
    int32_t *cnt = dsm, *off = cnt + kLongOut, *aoff = off + kLongOut;
    int16_t *pos = reinterpret_cast<int16_t *>(aoff + kLongA + 1), *ord = pos + kLongTerms;
    const int ra = RA ? RA : f.ra, ca = CA ? CA : f.ca, cb = CB ? CB : f.cb;
    const int bs = ra * cb;
    const int lane = threadIdx.x & 31;
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const int64_t T = f.boff[i + 1] - f.boff[i];
        const int64_t c0 = f.cptr[i], lc = f.cptr[i + 1] - c0;
        if (T <= kTermCap && lc <= kTermCap) continue;   // the short kernel's row
        const int64_t a0 = f.aptr[i], la = f.aptr[i + 1] - a0;
        if (T > kLongTerms || lc > kLongOut || la > kLongA) {
            // beyond the shared-memory buffers: each lane takes output entries and, for
            // each, finds its column in the B row of every entry of A's row (a binary
            // search), summing in A's order -- the order of the term-by-term sum
            for (int64_t p = lane; p < lc; p += 32) {
                const int32_t c = f.ccol[c0 + p];
                if (f.upper && c < i) continue;   // filled by the mirror pass
                double acc[RA && CB ? RA * CB : 36];
                for (int k = 0; k < bs; ++k) acc[k] = 0.0;
                for (int64_t q = 0; q < la; ++q) {
                    const int64_t j = f.acol[a0 + q];
                    const int64_t t = amg::find_sorted(f.bcol, f.bptr[j], f.bptr[j + 1], c);
                    if (t >= 0) amg::block_mul_add(f.aval + (a0 + q) * ra * ca, f.bval + t * ca * cb, ra, ca, cb, acc);
                }
                double *o = f.cval + (c0 + p) * bs;
                for (int k = 0; k < bs; ++k) o[k] = acc[k];
            }
            __syncwarp();
            continue;
        }
        // first term of each entry of A's row (a serial prefix over <= kLongA entries)
        if (lane == 0) {
            int32_t run = 0;
            for (int64_t q = 0; q < la; ++q) {
                aoff[q] = run;
                const int32_t c = f.acol[a0 + q];
                run += (int32_t)(f.bptr[c + 1] - f.bptr[c]);
            }
            aoff[la] = run;
        }
        for (int64_t p = lane; p < lc; p += 32) cnt[p] = 0;
        __syncwarp();
        for (int64_t q = 0; q < la; ++q) {
            const int32_t c = f.acol[a0 + q];
            const int64_t t0 = f.bptr[c], len = f.bptr[c + 1] - t0;
            for (int64_t t = lane; t < len; t += 32) {
                const int32_t bc = f.bcol[t0 + t];
                const int64_t p = (f.upper && bc < i) ? -1 : amg::find_sorted(f.ccol, c0, c0 + lc, bc);
                pos[aoff[q] + t] = p < 0 ? (int16_t)-1 : (int16_t)(p - c0);
            }
        }
        __syncwarp();
        for (int64_t t = lane; t < T; t += 32)
            if (pos[t] >= 0) atomicAdd(&cnt[pos[t]], 1);
        __syncwarp();
        int carry = 0;
        for (int64_t p0 = 0; p0 < lc; p0 += 32) {
            const int64_t p = p0 + lane;
            const int v = p < lc ? cnt[p] : 0;
            int x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (p < lc) off[p] = carry + x - v;
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
        __syncwarp();
        for (int64_t t0 = 0; t0 < T; t0 += 32) {
            const int64_t t = t0 + lane;
            const int p = t < T ? pos[t] : -1;
            const int key = p >= 0 ? p : -1 - lane;
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            if (p >= 0) ord[off[p] + __popc(peers & ((1u << lane) - 1u))] = (int16_t)t;
            __syncwarp();
            if (p >= 0 && lane == 31 - __clz(peers)) off[p] += __popc(peers);
            __syncwarp();
        }
        for (int64_t p = lane; p < lc; p += 32) {
            double acc[RA && CB ? RA * CB : 36];
            for (int k = 0; k < bs; ++k) acc[k] = 0.0;
            for (int q = off[p] - cnt[p]; q < off[p]; ++q) {
                const int t = ord[q];
                // the entry of A's row the term belongs to: the last q' with aoff[q'] <= t
                int lo = 0, hi = (int)la - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (aoff[mid] <= t) lo = mid;
                    else hi = mid - 1;
                }
                const int64_t sidx = a0 + lo;
                const int64_t tidx = f.bptr[f.acol[sidx]] + (t - aoff[lo]);
                const double *a = f.aval + sidx * ra * ca;
                const double *b = f.bval + tidx * ca * cb;
                amg::block_mul_add(a, b, ra, ca, cb, acc);
            }
            if (f.upper && f.ccol[c0 + p] < i) continue;   // filled by the mirror pass
            double *o = f.cval + (c0 + p) * bs;
            for (int k = 0; k < bs; ++k) o[k] = acc[k];
        }
        __syncwarp();
    }
}

template <int RA, int CA, int CB>
int launch_prod_vals(int64_t n, const amg::PassProdVals &f, cudaStream_t s) {
    constexpr size_t smem = warp_vals_smem<RA, CB>();
    static_assert(smem <= 227 * 1024, "shared memory of kd_prod_vals_warp");
    FE_CUDA(cudaFuncSetAttribute(kd_prod_vals_warp<RA, CA, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    kd_prod_vals_warp<RA, CA, CB><<<warp_grid(n), kPW * 32, smem, s>>>(n, f);
    FE_LAUNCH_CHECK();
    static_assert(kLongTerms <= 32767 && kLongOut <= 32767, "16-bit term and entry indices");
    FE_CUDA(cudaFuncSetAttribute(kd_prod_vals_long<RA, CA, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kLongValsSmem));
    kd_prod_vals_long<RA, CA, CB><<<(int)std::max<int64_t>(1, std::min<int64_t>(n, 152 * 16)), 32, kLongValsSmem, s>>>(
        n, f);
    FE_LAUNCH_CHECK();
    return FE_OK;
}


struct DevEx {
    MgMem mem;
    cudaStream_t s;
    DBuf<int64_t> scan_tmp;
    DBuf<double> part;
    SetupTrace *trace = nullptr;
    // level 0's operator is the handle's eliminated system: its plain products run on
    // the handle's FP64 SELL copy
    fe_handle_s *h = nullptr;
    const int64_t *sell_ptr = nullptr;
    explicit DevEx(const MgMem &m) : mem(m), s(m.s) {}
    void phase(int k) {
        if (trace) trace->mark(s, k);
    }
    ~DevEx() { pfree(mem, scan_tmp), pfree(mem, part); }
    template <class T>
    int alloc(DBuf<T> &b, size_t n) { return palloc(mem, b, n); }
    template <class T>
    void release(DBuf<T> &b) { pfree(mem, b); }
    template <class T>
    int copy(T *dst, const T *src, size_t n) {
        if (n) FE_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
        return FE_OK;
    }
    template <class T>
    int read(T *dst, const T *src, size_t n) {
        if (n) FE_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        return FE_OK;
    }
    template <class F>
    int rows(int64_t n, const F &f) {
        if (n <= 0) return FE_OK;
        k_rows<F><<<grid_s(n), kST, 0, s>>>(n, f);
        FE_LAUNCH_CHECK();
        return FE_OK;
    }
    // the lmax estimates' products: level 0's on the FP64 SELL copy, the others with
    // lanes per row (other block sizes row by row)
    int rows(int64_t n, const amg::PassDinvProduct &f) {
        if (n <= 0) return FE_OK;
        if (!f.dinv && h && f.ptr == sell_ptr) return spmv64(h, f.x, f.y);
        switch (f.d) {
            case 1: return launch_dinv_product<1>(n, f, s);
            case 2: return launch_dinv_product<2>(n, f, s);
            case 3: return launch_dinv_product<3>(n, f, s);
            case 6: return launch_dinv_product<6>(n, f, s);
            default:
                k_rows<amg::PassDinvProduct><<<grid_s(n), kST, 0, s>>>(n, f);
                FE_LAUNCH_CHECK();
                return FE_OK;
        }
    }
    // the sparse products: a warp per row where rows are long, else row by row
    int rows(int64_t n, const amg::PassProdCols &f) {
        if (n <= 0) return FE_OK;
        if ((double)f.total < kWarpRowMean * (double)n) {
            k_rows<amg::PassProdCols><<<grid_s(n), kST, 0, s>>>(n, f);
        } else {
            kd_prod_cols_warp<<<warp_grid(n), kPW * 32, 0, s>>>(n, f);
            FE_LAUNCH_CHECK();
            FE_CUDA(cudaFuncSetAttribute(kd_prod_cols_long, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kLongColsSmem));
            kd_prod_cols_long<<<(int)std::max<int64_t>(1, std::min<int64_t>(n, 152 * 16)), 32, kLongColsSmem, s>>>(
                n, f);
        }
        FE_LAUNCH_CHECK();
        return FE_OK;
    }
    // a thread per row where rows are short, else a warp per row; block sizes fixed at
    // compile time for the shapes of the hierarchies (A x P, R x AP and the coarse
    // levels' products): 1 x 1 (magnetostatics), 2D elasticity's 2 x 2 A with three
    // rigid-body modes, 3D elasticity's 3 x 3 A with six -- the accumulators then
    // stay in registers
    template <int RA, int CA, int CB>
    int prod_vals_shape(int64_t n, const amg::PassProdVals &f, bool thread) {
        if (!thread) return launch_prod_vals<RA, CA, CB>(n, f, s);
        kd_prod_vals_thread<RA, CA, CB><<<grid_s(n), kST, 0, s>>>(n, f);
        FE_LAUNCH_CHECK();
        return FE_OK;
    }
    int rows(int64_t n, const amg::PassProdVals &f) {
        if (n <= 0) return FE_OK;
        const bool thread = !f.boff || (double)f.total < kWarpRowMean * (double)n;
        const int ra = f.ra, ca = f.ca, cb = f.cb;
        if (ra == 1 && ca == 1 && cb == 1) return prod_vals_shape<1, 1, 1>(n, f, thread);
        if (ra == 2 && ca == 2 && cb == 3) return prod_vals_shape<2, 2, 3>(n, f, thread);
        if (ra == 3 && ca == 2 && cb == 3) return prod_vals_shape<3, 2, 3>(n, f, thread);
        if (ra == 3 && ca == 3 && cb == 3) return prod_vals_shape<3, 3, 3>(n, f, thread);
        if (ra == 3 && ca == 3 && cb == 6) return prod_vals_shape<3, 3, 6>(n, f, thread);
        if (ra == 6 && ca == 3 && cb == 6) return prod_vals_shape<6, 3, 6>(n, f, thread);
        if (ra == 6 && ca == 6 && cb == 6) return prod_vals_shape<6, 6, 6>(n, f, thread);
        if (!thread) return launch_prod_vals<0, 0, 0>(n, f, s);
        k_rows<amg::PassProdVals><<<grid_s(n), kST, 0, s>>>(n, f);
        FE_LAUNCH_CHECK();
        return FE_OK;
    }
    int scan(const int64_t *in, int64_t n, int64_t *out, int64_t *total) { return scan64(in, n, out, total, scan_tmp, mem); }
    // a . b into device memory, in stream order (deterministic two-stage sum)
    int dot_to(const double *a, const double *b, int64_t n, double *dst) {
        const int g = grid_s(n);
        FE_CHECK(palloc(mem, part, (size_t)g));
        kd_dot<<<g, kST, 0, s>>>(n, a, b, part.p);
        kd_dot_final<<<1, kST, 0, s>>>(g, part.p, dst);
        FE_LAUNCH_CHECK();
        return FE_OK;
    }
};

// ---------------------------------------------------------------- inputs of level 0

struct PassPtr64 {
    const int32_t *p32; int64_t *p64;
    FE_HD void operator()(int64_t i) const { p64[i] = p32[i]; }
};

// near-null space per node: rigid-body modes (d = 2: 3, d = 3: 6) or the constant (d = 1)
struct PassNullspace {
    int d, cdim, m; const double *xy; double *B;
    FE_HD void operator()(int64_t i) const {
        const double x = xy[i * cdim], y = xy[i * cdim + 1], z = cdim == 3 ? xy[i * cdim + 2] : 0.0;
        double *b = &B[i * d * m];
        for (int k = 0; k < d * m; ++k) b[k] = 0.0;
        if (d == 1) {
            b[0] = 1.0;
        } else if (d == 2) {
            b[0 * m + 0] = 1.0, b[1 * m + 1] = 1.0, b[0 * m + 2] = -y, b[1 * m + 2] = x;
        } else {
            for (int k = 0; k < 3; ++k) b[k * m + k] = 1.0;
            b[0 * m + 3] = -y, b[1 * m + 3] = x;
            b[1 * m + 4] = -z, b[2 * m + 4] = y;
            b[0 * m + 5] = z, b[2 * m + 5] = -x;
        }
    }
};

struct PassZeroRows {
    const int64_t *dof; int m; double *B;
    FE_HD void operator()(int64_t k) const {
        for (int j = 0; j < m; ++j) B[dof[k] * m + j] = 0.0;
    }
};

template <typename T>
int to_host(std::vector<T> &dst, const DBuf<T> &src, size_t n, cudaStream_t s) {
    dst.resize(n);
    if (n) FE_CUDA(cudaMemcpyAsync(dst.data(), src.p, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    return FE_OK;
}

int csr_to_host(const DevCsr &D, BlockCsr &H, cudaStream_t s) {
    H.n = D.n, H.rd = D.rd, H.cd = D.cd;
    FE_CHECK(to_host(H.ptr, D.ptr, (size_t)D.n + 1, s));
    FE_CHECK(to_host(H.col, D.col, (size_t)D.nnzb, s));
    FE_CHECK(to_host(H.val, D.val, (size_t)D.nnzb * D.rd * D.cd, s));
    return FE_OK;
}

// ---------------------------------------------------------------- coarsest inverse
// Dense inverse of the coarsest matrix (symmetric positive definite once 1e-12 of its
// largest diagonal entry is added, as the host version does) by the sweep operator
// (Goodnight, "A tutorial on the SWEEP operator", The American Statistician 33, 1979):
// sweeping pivot p of a symmetric M,
//   m_pp <- -1 / m_pp,  m_ip <- m_ip / m_pp,  m_pj <- m_pj / m_pp,
//   m_ij <- m_ij - m_ip m_pj / m_pp              (i, j != p),
// keeps M symmetric, and sweeping every pivot once leaves -M^-1.  Sweeping a block K of
// pivots at once, with T = -S^-1 of S = M_KK and C = M_:K,
//   M_KK <- T,  M_IK <- -C_I T,  M_IJ <- M_IJ + (C_I T) C_J^T       (I, J outside K),
// equals sweeping its pivots one by one, and turns the work into rank-kSweepB updates.
// Only the upper triangle is kept (element (i, j), i <= j, stands for both), which
// halves the FP64 arithmetic against Gauss-Jordan on the full matrix.

constexpr int kMaxCoarse = 4096;   // DOFs of the coarsest level (a 128 MB inverse)
constexpr int kSweepB = 32;        // pivots per block sweep, and the tile edge of the update

__global__ void kc_dense_fill(int64_t nb_rows, int cd, const int64_t *__restrict__ ptr,
                              const int32_t *__restrict__ col, const double *__restrict__ val, int64_t n,
                              double *__restrict__ M) {
    FE_ROWS(i, nb_rows)
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s)
        for (int a = 0; a < cd; ++a)
            for (int b = 0; b < cd; ++b) M[(i * cd + a) * n + (int64_t)col[s] * cd + b] = val[(s * cd + a) * cd + b];
}

// one block: the diagonal gets 1e-12 of its largest magnitude added
__global__ void kc_regularise(int64_t n, double *M) {
    __shared__ double sh[kST / 32];
    double m = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(M[i * n + i]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < kST / 32; ++w) t = fmax(t, sh[w]);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) M[i * n + i] += 1e-12 * t;
}

// the upper-triangle element standing for (i, j)
__device__ __forceinline__ int64_t upper(int64_t i, int64_t j, int64_t n) { return i <= j ? i * n + j : j * n + i; }

// All block sweeps in one cooperative launch, two grid barriers per block of pivots:
//  (a) every block computes T = -S^-1 of the pivot block in shared memory (the same
//      arithmetic in every block), by sweeping its pivots one by one;
//  (b) a warp per row i outside K: C_i = M_iK and W_i = C_i T into Cs / Ws (zero rows
//      for i in K), and the new column -W_i into M;
//  (c) after a barrier, the upper 32 x 32 tiles of M += W C^T (rows and columns in K
//      skipped), and M_KK <- T;
// then, after the last block, the full inverse -M from the upper triangle.  A pivot that
// is not positive (the matrix is not positive definite) stops every block at the same
// step (*singular = 1); the barriers are bounded (grid_sync_bounded).
__global__ void __launch_bounds__(kST) kc_sweep(int64_t n, double *M, double *Cs, double *Ws, unsigned *bar, int *err,
                                                int *singular) {
    constexpr int B = kSweepB;
    __shared__ double T[B][B + 1];
    __shared__ double sw[B][B + 1], sc[B][B + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t nt = (n + B - 1) / B;   // tiles per dimension
    const int64_t n_upper = nt * (nt + 1) / 2;
    for (int64_t k0 = 0; k0 < n; k0 += B) {
        const int bk = (int)(n - k0 < B ? n - k0 : B);
        // (a) T = -S^-1
        for (int e = threadIdx.x; e < B * B; e += blockDim.x) {
            const int a = e / B, b = e % B;
            T[a][b] = (a < bk && b < bk) ? __ldcg(M + upper(k0 + a, k0 + b, n)) : 0.0;
        }
        __syncthreads();
        for (int p = 0; p < bk; ++p) {
            const double d = T[p][p];
            if (!(d > 0.0) || !isfinite(d)) {
                if (blockIdx.x == 0 && threadIdx.x == 0) *singular = 1;
                return;
            }
            const double id = 1.0 / d;
            double v[B * B / kST];
            int q = 0;
            for (int e = threadIdx.x; e < bk * B; e += blockDim.x, ++q) {
                const int a = e / B, b = e % B;
                if (b >= bk) continue;
                if (a == p && b == p) v[q] = -id;
                else if (a == p) v[q] = T[p][b] * id;
                else if (b == p) v[q] = T[a][p] * id;
                else v[q] = T[a][b] - T[a][p] * T[p][b] * id;
            }
            __syncthreads();
            q = 0;
            for (int e = threadIdx.x; e < bk * B; e += blockDim.x, ++q) {
                const int b = e % B;
                if (b < bk) T[e / B][b] = v[q];
            }
            __syncthreads();
        }
        // exactly symmetric T: the upper triangle stands for both
        for (int e = threadIdx.x; e < B * B; e += blockDim.x) {
            const int a = e / B, b = e % B;
            if (a > b) T[a][b] = T[b][a];
        }
        __syncthreads();
        // (b) C and W = C T per row, and the new column -W (rows in K: zeros)
        const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
        for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; i < n; i += warps) {
            const bool in_k = i >= k0 && i < k0 + bk;
            const double c = (!in_k && lane < bk) ? __ldcg(M + upper(i, k0 + lane, n)) : 0.0;
            double w = 0.0;
            for (int a = 0; a < bk; ++a) w = fma(__shfl_sync(0xffffffffu, c, a), T[a][lane], w);
            Cs[i * B + lane] = c;
            Ws[i * B + lane] = w;
            if (!in_k && lane < bk) M[upper(i, k0 + lane, n)] = -w;
        }
        if (!grid_sync_bounded(bar, err)) return;
        // (c) the upper tiles: M_IJ += W_I C_J^T
        for (int64_t u = blockIdx.x; u < n_upper; u += gridDim.x) {
            int64_t I = 0, off = 0;
            while (off + (nt - I) <= u) off += nt - I, ++I;
            const int64_t J = I + (u - off);
            const int64_t i0 = I * B, j0 = J * B;
            // tiles that lie inside the pivot rows or columns have nothing to update
            const bool skip = (i0 >= k0 && i0 + B <= k0 + bk) || (j0 >= k0 && j0 + B <= k0 + bk);
            if (skip) continue;
            for (int e = threadIdx.x; e < B * B; e += blockDim.x) {
                const int r = e / B, a = e % B;
                sw[r][a] = i0 + r < n ? __ldcg(Ws + (i0 + r) * B + a) : 0.0;
                sc[r][a] = j0 + r < n ? __ldcg(Cs + (j0 + r) * B + a) : 0.0;
            }
            __syncthreads();
            const int64_t j = j0 + lane;
            double acc[B * B / kST];
#pragma unroll
            for (int q = 0; q < B * B / kST; ++q) acc[q] = 0.0;
            for (int a = 0; a < bk; ++a) {
                const double cv = sc[lane][a];
#pragma unroll
                for (int q = 0; q < B * B / kST; ++q) acc[q] = fma(sw[warp + q * (kST / 32)][a], cv, acc[q]);
            }
#pragma unroll
            for (int q = 0; q < B * B / kST; ++q) {
                const int64_t i = i0 + warp + q * (kST / 32);
                const bool in_k = (i >= k0 && i < k0 + bk) || (j >= k0 && j < k0 + bk);
                // coherent read: other blocks wrote this element (the new column, M_KK)
                if (i < n && j < n && j >= i && !in_k) M[i * n + j] = __ldcg(M + i * n + j) + acc[q];
            }
            __syncthreads();
        }
        if (blockIdx.x == 0)
            for (int e = threadIdx.x; e < bk * bk; e += blockDim.x) {
                const int a = e / bk, b = e % bk;
                if (a <= b) M[(k0 + a) * n + k0 + b] = T[a][b];
            }
        if (!grid_sync_bounded(bar, err)) return;
    }
    // the inverse: -M, the lower triangle from the upper one first
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x)
        for (int64_t j = threadIdx.x; j < i; j += blockDim.x) M[i * n + j] = -__ldcg(M + j * n + i);
    if (!grid_sync_bounded(bar, err)) return;
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x)
        for (int64_t j = i + threadIdx.x; j < n; j += blockDim.x) M[i * n + j] = -__ldcg(M + i * n + j);
}

int coarse_inverse_device(const DevCsr &C, DevAmg &G) {
    const cudaStream_t s = G.mem.s;
    const int64_t n = C.n * C.rd;
    if (n > kMaxCoarse) {
        set_error("multigrid setup: coarsest level too large for its dense solve");
        return FE_BAD_INPUT;
    }
    G.nc = n;
    FE_CHECK(palloc(G.mem, G.cinv, (size_t)std::max<int64_t>(n * n, 1)));
    if (n == 0) return FE_OK;
    DBuf<int> flag;      // [0] singular, [1] [2] the grid barrier, [3] its error word
    DBuf<double> cw;     // the C and W panels, n x kSweepB each
    struct Free {
        const MgMem &m;
        DBuf<int> &f;
        DBuf<double> &p;
        ~Free() { pfree(m, f), pfree(m, p); }
    } fr{G.mem, flag, cw};
    FE_CHECK(palloc(G.mem, flag, 4));
    FE_CHECK(palloc(G.mem, cw, (size_t)2 * n * kSweepB));
    FE_CUDA(cudaMemsetAsync(flag.p, 0, 4 * sizeof(int), s));
    FE_CUDA(cudaMemsetAsync(G.cinv.p, 0, (size_t)n * n * sizeof(double), s));
    kc_dense_fill<<<grid_s(C.n), kST, 0, s>>>(C.n, C.rd, C.ptr.p, C.col.p, C.val.p, n, G.cinv.p);
    kc_regularise<<<1, kST, 0, s>>>(n, G.cinv.p);
    FE_LAUNCH_CHECK();
    // the cooperative grid: at most two blocks per SM (measured 16 ms for the 1,941-DOF
    // coarsest level of the 4M-DOF system, 22.6 ms on four: more barrier arrivals, and
    // the 32 x 32 tiles of one update number about (n / 32)^2 / 2)
    int dev = 0, sms = 0, per_sm = 0;
    FE_CUDA(cudaGetDevice(&dev));
    FE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)kc_sweep, kST, 0));
    if (per_sm < 1) {
        set_error("multigrid setup: the coarsest inverse kernel does not fit on an SM");
        return FE_CUDA_ERR;
    }
    const int grid = sms * std::min(per_sm, 2);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kST);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FE_CUDA(cudaLaunchKernelEx(&cfg, kc_sweep, n, G.cinv.p, cw.p, cw.p + n * kSweepB, (unsigned *)(flag.p + 1),
                               flag.p + 3, flag.p));
    int host[4] = {0, 0, 0, 0};
    FE_CUDA(cudaMemcpyAsync(host, flag.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    if (host[3]) {
        set_error("multigrid setup: a grid barrier of the coarsest inverse timed out");
        return FE_CUDA_ERR;
    }
    if (host[0]) {
        set_error("multigrid setup: the coarsest matrix is not positive definite");
        return FE_BREAKDOWN;
    }
    return FE_OK;
}

}  // namespace

// One pool per device for the whole process, shared by the handles (a user who makes a
// handle per problem reuses the memory of the previous ones); fe_trim_memory_pools
// gives it back.
constexpr int kMaxDevices = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[kMaxDevices] = {};

int device_pool(cudaMemPool_t *out) {
    int dev = 0;
    FE_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("multigrid: device index out of range");
        return FE_BAD_INPUT;
    }
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        FE_CUDA(cudaMemPoolCreate(&pool, &props));
        uint64_t keep = ~0ull;
        if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
            cudaMemPoolDestroy(pool);
            set_error("multigrid: cannot set the memory pool's release threshold");
            return FE_CUDA_ERR;
        }
        g_pools[dev] = pool;
    }
    *out = g_pools[dev];
    return FE_OK;
}

int mg_memory(fe_handle_s *h, MgMem *out) {
    if (!h->mg_pool) FE_CHECK(device_pool(&h->mg_pool));
    if (!h->mg_pinned) FE_CUDA(cudaMallocHost((void **)&h->mg_pinned, 8 * sizeof(double)));
    out->s = h->stream;
    out->pool = h->mg_pool;
    out->pinned = h->mg_pinned;
    return FE_OK;
}

int amg_setup_device(fe_handle_s *h, double theta, int64_t coarse_dofs, DevAmg &G, SetupTrace *trace) {
    FE_CHECK(mg_memory(h, &G.mem));
    DevEx ex(G.mem);
    ex.trace = trace;
    ex.h = h;
    ex.phase(amg::kPhaseInput);
    const int D = h->dim;
    const int64_t n0 = h->n_nodes;
    const int m = D == 2 ? 3 : D == 3 ? 6 : 1;
    // level-0 operator (own copies, int64 row pointers) and near-null space, both
    // handed over to setup_hierarchy
    DevCsr A;
    DBuf<double> B;
    A.n = n0, A.rd = A.cd = D, A.nnzb = h->nnzb;
    int st = FE_OK;
    if ((st = palloc(G.mem, A.ptr, (size_t)n0 + 1)) ||
        (st = palloc(G.mem, A.col, (size_t)std::max<int64_t>(h->nnzb, 1))) ||
        (st = palloc(G.mem, A.val, (size_t)std::max<int64_t>(h->nnzb * D * D, 1))) ||
        (st = palloc(G.mem, B, (size_t)std::max<int64_t>(n0 * D * m, 1))) ||
        (st = ex.rows(n0 + 1, PassPtr64{h->blk_ptr.p, A.ptr.p})) ||
        (st = ex.copy(A.col.p, h->blk_col.p, (size_t)h->nnzb)) ||
        (st = ex.copy(A.val.p, h->aval.p, (size_t)(h->nnzb * D * D))) ||
        (st = ex.rows(n0, PassNullspace{D, h->cdim, m, h->coords.p, B.p})) ||
        (st = ex.rows(h->n_bc, PassZeroRows{h->bc_dof.p, m, B.p}))) {
        drelease(G.mem, A);
        pfree(G.mem, B);
        return st;
    }
    ex.sell_ptr = A.ptr.p;
    std::vector<amg::Level> levels;
    // level 0's D^-1: the node-block Jacobi inverse of the assembly
    st = amg::setup_hierarchy(ex, A, B, m, theta, coarse_dofs, levels, G.coarse, &G.mis_rounds, h->dinv.p);
    // the levels move into G (released with it, also after a failure)
    for (auto &l : levels) {
        DevLevel L;
        L.A = l.A, L.P = l.P, L.PT = l.PT, L.dinv = l.dinv, L.agg = l.agg, L.lmax = l.lmax;
        G.L.push_back(L);
    }
    FE_CHECK(st);
    // coarsest level: its dense inverse, on the device
    ex.phase(amg::kPhaseCoarse);
    return coarse_inverse_device(G.coarse, G);
}

int amg_download(const DevAmg &G, fe_amg_s *out, cudaStream_t s) {
    out->levels.resize(G.L.size());
    for (size_t l = 0; l < G.L.size(); ++l) {
        const DevLevel &D = G.L[l];
        AmgLevel &H = out->levels[l];
        FE_CHECK(csr_to_host(D.A, H.A, s));
        FE_CHECK(csr_to_host(D.P, H.P, s));
        FE_CHECK(csr_to_host(D.PT, H.PT, s));
        FE_CHECK(to_host(H.dinv, D.dinv, (size_t)D.A.n * D.A.rd * D.A.rd, s));
        FE_CHECK(to_host(H.agg, D.agg, (size_t)D.A.n, s));
        H.lmax = D.lmax;
    }
    FE_CHECK(csr_to_host(G.coarse, out->coarse, s));
    FE_CHECK(to_host(out->coarse_inv, G.cinv, (size_t)(G.nc * G.nc), s));
    FE_CUDA(cudaStreamSynchronize(s));
    return FE_OK;
}

}  // namespace fe

using namespace fe;

extern "C" int fe_trim_memory_pools(uint64_t keep_bytes) {
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    for (cudaMemPool_t p : g_pools)
        if (p && cudaMemPoolTrimTo(p, (size_t)keep_bytes) != cudaSuccess) {
            set_error("fe_trim_memory_pools: cudaMemPoolTrimTo failed");
            return FE_CUDA_ERR;
        }
    return FE_OK;
}

extern "C" int fe_amg_build_device(fe_handle h, double theta, int64_t coarse_dofs, fe_amg *out) {
    if (!h || !out) {
        set_error("fe_amg_build_device: bad arguments");
        return FE_BAD_INPUT;
    }
    *out = nullptr;
    if (!h->sys_ready) {
        set_error("fe_amg_build_device: the system is not assembled");
        return FE_NOT_READY;
    }
    DevAmg G;
    FE_CHECK(amg_setup_device(h, theta, coarse_dofs, G));
    fe_amg_s *a = new fe_amg_s();
    const int st = amg_download(G, a, h->stream);
    if (st != FE_OK) {
        fe_amg_destroy(a);
        return st;
    }
    *out = a;
    return FE_OK;
}
