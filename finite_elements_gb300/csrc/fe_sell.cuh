// Node-block vectors and the SELL-32 row product shared by the solver kernels
// (fe_solver.cu) and the batched persistent solver (fe_batch.cu).
//
// A node vector holds D values per node (D = 1, 2, 3 DOF per node), loaded and stored
// with one vector access for D = 2.  The SELL-32 copy of a node-block matrix keeps
// slices of 32 consecutive block rows; entry k of row 32 s + l sits at
// off[s] + 32 k + l, so each warp load of columns and blocks is one contiguous segment.
//
// Loads of node vectors come in two kinds.  The default (`ld`) lets the compiler use
// the read-only data path, which is valid in kernels that do not write the vector.
// A persistent kernel that writes a vector in one phase and gathers it in the next,
// after a grid barrier, must read it coherently: `ldc` loads through L2
// (ld.global.cg), and sell_row<..., COHERENT = true> gathers that way.
#pragma once

#include <stdint.h>

#include <type_traits>

namespace fe {
namespace {

// ---------------------------------------------------------------- node vectors

template <int D, typename T>
struct NodeVec {
    T v[D];
};

template <int D, typename T>
__device__ __forceinline__ NodeVec<D, T> ld(const T *__restrict__ a, int64_t r) {
    NodeVec<D, T> o;
    if constexpr (D == 2 && sizeof(T) == 8) {
        double2 t = reinterpret_cast<const double2 *>(a)[r];
        o.v[0] = t.x, o.v[1] = t.y;
    } else if constexpr (D == 2) {
        float2 t = reinterpret_cast<const float2 *>(a)[r];
        o.v[0] = t.x, o.v[1] = t.y;
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) o.v[k] = a[r * D + k];
    }
    return o;
}

template <int D, typename T>
__device__ __forceinline__ void st(T *__restrict__ a, int64_t r, const NodeVec<D, T> &o) {
    if constexpr (D == 2 && sizeof(T) == 8) {
        reinterpret_cast<double2 *>(a)[r] = make_double2(o.v[0], o.v[1]);
    } else if constexpr (D == 2) {
        reinterpret_cast<float2 *>(a)[r] = make_float2(o.v[0], o.v[1]);
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) a[r * D + k] = o.v[k];
    }
}

// Coherent load of node r (L2, bypassing the SM's L1 and the read-only path): for
// vectors that other blocks of the same launch wrote before a grid barrier.
template <int D, typename T>
__device__ __forceinline__ NodeVec<D, T> ldc(const T *a, int64_t r) {
    NodeVec<D, T> o;
    if constexpr (D == 2 && sizeof(T) == 8) {
        const double2 t = __ldcg(reinterpret_cast<const double2 *>(a) + r);
        o.v[0] = t.x, o.v[1] = t.y;
    } else if constexpr (D == 2) {
        const float2 t = __ldcg(reinterpret_cast<const float2 *>(a) + r);
        o.v[0] = t.x, o.v[1] = t.y;
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) o.v[k] = __ldcg(a + r * D + k);
    }
    return o;
}

// ld or ldc
template <int D, typename T, bool COHERENT>
__device__ __forceinline__ NodeVec<D, T> ldv(const T *a, int64_t r) {
    if constexpr (COHERENT) return ldc<D, T>(a, r);
    else return ld<D, T>(a, r);
}

// y = M^-1 x for one node (M^-1 stored row-major per node)
template <int D, typename T>
__device__ __forceinline__ NodeVec<D, T> apply_dinv(const T *__restrict__ dinv, int64_t r, const NodeVec<D, T> &x) {
    NodeVec<D, T> y;
    if constexpr (D == 2) {
        if constexpr (sizeof(T) == 8) {
            const double2 m0 = reinterpret_cast<const double2 *>(dinv)[2 * r];
            const double2 m1 = reinterpret_cast<const double2 *>(dinv)[2 * r + 1];
            y.v[0] = m0.x * x.v[0] + m0.y * x.v[1];
            y.v[1] = m1.x * x.v[0] + m1.y * x.v[1];
        } else {
            const float4 m = reinterpret_cast<const float4 *>(dinv)[r];
            y.v[0] = m.x * x.v[0] + m.y * x.v[1];
            y.v[1] = m.z * x.v[0] + m.w * x.v[1];
        }
    } else {
#pragma unroll
        for (int i = 0; i < D; ++i) {
            T acc = dinv[r * D * D + i * D] * x.v[0];
#pragma unroll
            for (int k = 1; k < D; ++k) acc += dinv[r * D * D + i * D + k] * x.v[k];
            y.v[i] = acc;
        }
    }
    return y;
}

// acc += B x for one D x D block, as a chain of fused multiply-adds into the
// accumulator: 2 D FMAs per block, the least work for the FP64 pipe that bounds the
// FP64 SpMV on this GPU.
template <int D, typename T>
__device__ __forceinline__ void block_mac(const T *__restrict__ blk, const NodeVec<D, T> &x, NodeVec<D, T> &acc) {
    if constexpr (D == 2) {
        if constexpr (sizeof(T) == 8) {
            const double2 b0 = __ldg(reinterpret_cast<const double2 *>(blk));
            const double2 b1 = __ldg(reinterpret_cast<const double2 *>(blk) + 1);
            acc.v[0] = fma(b0.x, x.v[0], acc.v[0]);
            acc.v[1] = fma(b1.x, x.v[0], acc.v[1]);
            acc.v[0] = fma(b0.y, x.v[1], acc.v[0]);
            acc.v[1] = fma(b1.y, x.v[1], acc.v[1]);
        } else {
            const float4 b = __ldg(reinterpret_cast<const float4 *>(blk));
            acc.v[0] = fmaf(b.x, x.v[0], acc.v[0]);
            acc.v[1] = fmaf(b.z, x.v[0], acc.v[1]);
            acc.v[0] = fmaf(b.y, x.v[1], acc.v[0]);
            acc.v[1] = fmaf(b.w, x.v[1], acc.v[1]);
        }
    } else {
        // column by column, as the D = 2 chains
#pragma unroll
        for (int b = 0; b < D; ++b)
#pragma unroll
            for (int a = 0; a < D; ++a) acc.v[a] = fma(__ldg(blk + a * D + b), x.v[b], acc.v[a]);
    }
}

struct Sell {
    const int32_t *off, *col;
    const int16_t *dcol;   // column offsets c - r when every one fits in 16 bits, else null
    int64_t n_slices;
    // FP32 copy, 2 DOF per node: the first keep bytes of the values are loaded with L2
    // priority evict_last and the rest (up to total) evict_first, so that a prefix of
    // the matrix stays in L2 from one Chebyshev step to the next; 0 = plain loads
    uint32_t keep = 0, total = 0;
};

// Loads of the FP32 2x2 blocks under the L2 policy of Sell::keep.
__device__ __forceinline__ uint64_t l2_keep_policy(const void *base, uint32_t keep, uint32_t total) {
    uint64_t pol;
    asm("createpolicy.range.global.L2::evict_last.L2::evict_first.b64 %0, [%1], %2, %3;"
                 : "=l"(pol)
                 : "l"(base), "r"(keep), "r"(total));
    return pol;
}

__device__ __forceinline__ float4 ld_block_hint(const float *p, uint64_t pol) {
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}

// Calls f(std::true_type) when an FP32 kernel can read the 16-bit column offsets,
// else f(std::false_type); FP64 kernels always read the int32 columns.
template <typename T, typename F>
void with_col16(const Sell &A, F f) {
    if constexpr (sizeof(T) == 4) {
        if (A.dcol) {
            f(std::true_type{});
            return;
        }
    }
    f(std::false_type{});
}

// Row r of A x from the SELL-32 copy: one lane per block row, one warp per slice of
// 32 rows, entry k of the slice at base + 32 k + lane, so each warp load of columns
// and blocks is one contiguous segment.  FP64: the diagonal block comes from diag and
// every entry multiplies x_c.  FP32 (difference form): an entry with column c != r
// multiplies x_c - x_r, an entry with column r (the row-sum entry, or padding with a
// zero block) multiplies x_r; there is no diagonal term.  Rows past the last node
// (padding of the final slice) gather their own padding row -- the solver's vectors
// are allocated for whole slices -- and their result is discarded.
// COHERENT: x is read with ldc (explicit ld.global.cg, see the header), for kernels
// that wrote x themselves earlier in the same launch.
template <int D, typename T, bool C16 = false, bool KEEP = false, bool COHERENT = false>
__device__ __forceinline__ NodeVec<D, T> sell_row(int64_t r, bool valid, const Sell &A, const T *__restrict__ val,
                                                  const T *__restrict__ diag, const T *__restrict__ x) {
    constexpr bool DIFF = sizeof(T) == 4;
    NodeVec<D, T> xr, acc;
#pragma unroll
    for (int a = 0; a < D; ++a) xr.v[a] = T(0), acc.v[a] = T(0);
    if (valid) {
        xr = ldv<D, T, COHERENT>(x, r);
        if constexpr (!DIFF) block_mac<D, T>(diag + r * D * D, xr, acc);
    }
    const int64_t sl = r >> 5;
    const int lane = (int)(r & 31);
    const int64_t base = A.off[sl];
    const int w = (A.off[sl + 1] - (int)base) >> 5;
    // KEEP (FP32, 2 DOF per node): the block loads carry the L2 policy of A.keep
    constexpr bool HINT = KEEP && D == 2 && sizeof(T) == 4;
    uint64_t pol = 0;
    if constexpr (HINT) pol = l2_keep_policy(val, A.keep, A.total);
    // FP32: four entries per trip, their column loads and then their gathers all in
    // flight before the first product (entries past w read the row itself and add
    // 0).  FP64 is bound by the FP64 FMA rate and runs one entry per trip.
    constexpr int U = sizeof(T) == 4 ? (D == 3 ? 2 : 4) : 1;
    for (int k = 0; k < w; k += U) {
        int c[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            c[u] = (k + u < w) ? (C16 ? (int)r + (int)__ldg(A.dcol + base + 32 * (int64_t)(k + u) + lane)
                                      : __ldg(A.col + base + 32 * (int64_t)(k + u) + lane))
                               : (int)r;
        NodeVec<D, T> xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = ldv<D, T, COHERENT>(x, c[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (k + u < w) {
                if (DIFF && c[u] != (int)r) {
#pragma unroll
                    for (int a = 0; a < D; ++a) xv[u].v[a] -= xr.v[a];
                }
                const T *blk = val + (base + 32 * (int64_t)(k + u) + lane) * D * D;
                if constexpr (HINT) {
                    const float4 b = ld_block_hint(blk, pol);
                    acc.v[0] = fmaf(b.x, xv[u].v[0], acc.v[0]);
                    acc.v[1] = fmaf(b.z, xv[u].v[0], acc.v[1]);
                    acc.v[0] = fmaf(b.y, xv[u].v[1], acc.v[0]);
                    acc.v[1] = fmaf(b.w, xv[u].v[1], acc.v[1]);
                } else {
                    block_mac<D, T>(blk, xv[u], acc);
                }
            }
        }
    }
    return acc;
}

}  // namespace
}  // namespace fe
