// Preconditioned conjugate gradients on the eliminated system, replacing
// scipy.sparse.linalg.spsolve in FiniteElementAnalysis.solve
// (finite_elements/analysis.py:816-830).
//
// * SpMV: node-block CSR (d x d blocks), G lanes per block row (G = 1, 2, 4, 8 chosen
//   by an autotuner), vector loads of blocks (32 B for 2x2 FP64) and of the node
//   vector (16 B), FP64 or FP32 values.
// * One PCG iteration is three kernels: q = A p with p.q, the fused update
//   x += alpha p, r -= alpha q, z = M^-1 r with r.z and r.r, and p = z + beta p.
//   Each reduction ends in the last block to finish (ticket counter), which sums the
//   per-block partials in a fixed order and takes the iteration's scalar decisions on
//   the device, so results are identical run to run and the host never waits inside
//   the loop.  Chunks of iterations are captured once in a CUDA graph and replayed.
// * Preconditioner: node-block Jacobi (inverse d x d diagonal blocks), optionally
//   followed by k-1 Chebyshev steps on D^-1 A; the Chebyshev interval comes from a
//   Lanczos estimate of the largest eigenvalue built from the first PCG coefficients.
// * Mixed precision: FP32 SpMV, preconditioner and Krylov vectors (r, p, q, z), with
//   FP64 kept for the solution update x += alpha p, the reduction trees and the
//   refinement step: whenever the FP32 recurrence residual has fallen by a factor 10,
//   the FP64 true residual b - A x replaces it and the iteration continues along the
//   same search direction (iterative refinement with reliable updates: the Krylov
//   space is not restarted).  x stays FP64 because its own rounding would leave a
//   residual of order eps32 * cond(A); GB300 runs FP64 FMAs at 1/59 of the FP32 rate,
//   so that one FMA per DOF is the only FP64 arithmetic of the iteration.
//   The FP32 SpMV uses the difference form y_r = sum_{m != r} A_rm (x_m - x_r) + S_r x_r,
//   S_r the block row sum (zero at interior nodes: K annihilates translations), so
//   FP32 rounding scales with the variation of x between neighbours instead of with
//   x itself; smooth error modes are no longer swamped by rounding.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

#include "fe_internal.h"
#include "fe_sell.cuh"

namespace fe {
namespace {

constexpr int kVecThreads = 256;

inline int vec_grid(int64_t n_nodes) { return grid_for(n_nodes, kVecThreads, 152 * 8); }

// At most one resident wave of a grid-stride kernel: the SMs times the blocks of
// kVecThreads that stay resident per SM for that kernel (its registers and shared
// memory decide), looked up once per kernel and device.  Used for the Chebyshev steps:
// the FP64 step keeps 5 blocks per SM resident, and its 1216-block grid (8 per SM) ran
// as 1.6 waves, 161 us against 157 us in one wave at the 4M-DOF workload.  The FP64
// PCG SpMV measured the other way (138 us with 1216 blocks, 142.5 us in one wave) and
// keeps the larger grid.
int wave_grid(const void *kernel, int grid) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> waves;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return grid;
    std::lock_guard<std::mutex> lock(mu);
    auto it = waves.find({dev, kernel});
    if (it == waves.end()) {
        // the first lookup may come while the stream is being captured into a graph: the
        // queries enqueue nothing, so this thread allows them for their duration
        cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
        cudaThreadExchangeStreamCaptureMode(&mode);
        int sms = 0, per_sm = 0;
        const bool ok = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
                        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kVecThreads, 0) ==
                            cudaSuccess;
        cudaThreadExchangeStreamCaptureMode(&mode);
        if (!ok || sms <= 0 || per_sm <= 0) return grid;
        it = waves.emplace(std::make_pair(dev, kernel), sms * per_sm).first;
    }
    return std::max(1, std::min(grid, it->second));
}

// ---------------------------------------------------------------- reductions

template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV]) {
    __shared__ double sh[NV][kVecThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sh[k][warp] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = lane < (int)(blockDim.x >> 5) ? sh[k][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            v[k] = s;
        }
    }
    __syncthreads();
}

// Block partial sums -> partials[k * gridDim.x + block]; the last block to arrive sums
// them in block order and returns true in every thread of that block, with the totals
// in thread 0's out[].
template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double *partials, unsigned int *ticket,
                                            double (&out)[NV]) {
    __shared__ bool is_last;
    block_reduce<NV>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (unsigned int i = threadIdx.x; i < gridDim.x; i += blockDim.x)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += __ldcg(partials + k * gridDim.x + i);
    block_reduce<NV>(acc);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = acc[k];
        *ticket = 0;
    }
    return true;
}

// ---------------------------------------------------------------- SpMV row kernel
// Row r of A x, with G lanes of the warp sharing the row.  Blocks are read with
// 16-byte loads; the node vector x is read as one 16-byte (FP64) or 8-byte (FP32)
// load per block column.  The sum over the G lanes is a shuffle reduction.
// FP32 values are stored in difference form (see the header): the diagonal slot holds
// the block row sum S_r and every other block multiplies x_m - x_r.
// Every lane of the warp calls this (the shuffles need all 32); a lane whose row is
// past the end passes valid = false and contributes nothing.
// With SROW (FP64 difference form) the diagonal block comes from srow[r] instead of
// the stored diagonal slot.
template <int D, typename T, int G, bool DIFF = (sizeof(T) == 4), bool SROW = false>
__device__ __forceinline__ NodeVec<D, T> row_product(int64_t r, bool valid, const int32_t *__restrict__ ptr,
                                                     const int32_t *__restrict__ col,
                                                     const T *__restrict__ val, const T *__restrict__ x,
                                                     int sub, const T *__restrict__ srow = nullptr) {
    NodeVec<D, T> acc, xr;
#pragma unroll
    for (int a = 0; a < D; ++a) acc.v[a] = T(0), xr.v[a] = T(0);
    const int k0 = valid ? ptr[r] : 0, k1 = valid ? ptr[r + 1] : 0;
    if (DIFF && valid) xr = ld<D, T>(x, r);
    for (int k = k0 + sub; k < k1; k += G) {
        const int c = __ldg(col + k);
        NodeVec<D, T> xv = ld<D, T>(x, c);
        if (DIFF && c != (int)r) {
#pragma unroll
            for (int a = 0; a < D; ++a) xv.v[a] -= xr.v[a];
        }
        const T *blk = (SROW && c == (int)r) ? srow + r * D * D : val + (int64_t)k * D * D;
        if constexpr (D == 2) {
            if constexpr (sizeof(T) == 8) {
                const double2 b0 = __ldg(reinterpret_cast<const double2 *>(blk));
                const double2 b1 = __ldg(reinterpret_cast<const double2 *>(blk) + 1);
                acc.v[0] += b0.x * xv.v[0] + b0.y * xv.v[1];
                acc.v[1] += b1.x * xv.v[0] + b1.y * xv.v[1];
            } else {
                const float4 b = __ldg(reinterpret_cast<const float4 *>(blk));
                acc.v[0] += b.x * xv.v[0] + b.y * xv.v[1];
                acc.v[1] += b.z * xv.v[0] + b.w * xv.v[1];
            }
        } else {
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
                for (int b = 0; b < D; ++b) acc.v[a] += __ldg(blk + a * D + b) * xv.v[b];
        }
    }
    if constexpr (G > 1) {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int a = 0; a < D; ++a) acc.v[a] += __shfl_xor_sync(0xffffffffu, acc.v[a], o);
    }
    return acc;
}

// Block rows handled by this thread's group of G lanes: row = global_thread / G,
// grid-stride.  Every thread runs the same number of trips (rows_padded is a
// multiple of the stride) so that the warp shuffles always see all 32 lanes.
#define FE_ROW_LOOP(G)                                                                      \
    const int sub = threadIdx.x & ((G)-1);                                                  \
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / (G);                         \
    const int64_t rows_padded = ((n_nodes + groups - 1) / groups) * groups;                 \
    for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / (G); row < rows_padded; row += groups)

// Resident blocks per SM the SELL kernels are compiled for: FP32 with 1 or 2 DOF per
// node 8 (32 registers, the 1216-block grid is one wave); FP64, and FP32 with 3 DOF
// per node (whose 3 x 3 blocks and 3-vectors do not fit 32 registers), 0, i.e.
// ptxas's default (for FP64 40-48 registers; a floor of 1 makes it spend ~120 and
// lose the occupancy, 5 makes the Chebyshev step spill).
template <int D, typename T>
constexpr int kSellBlocks = (sizeof(T) == 4 && D <= 3) ? 8 : 0;


// Rows of the SELL copy handled by this thread (grid-stride in whole warps, so a
// warp always covers one slice).
#define FE_SELL_LOOP                                                                     \
    const int64_t rows_padded = A.n_slices * 32;                                         \
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < rows_padded; \
         row += (int64_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------- kernels

// y = A x (timing)
template <int D, typename T, bool C16 = false>
__global__ void __launch_bounds__(kVecThreads, kSellBlocks<D, T>)
k_spmv(int64_t n_nodes, Sell A, const T *__restrict__ val, const T *__restrict__ diag, const T *__restrict__ dscale,
       const T *__restrict__ x, T *__restrict__ y) {
    FE_SELL_LOOP {
        const bool valid = row < n_nodes;
        NodeVec<D, T> v = sell_row<D, T, C16>(row, valid, A, val, diag, x);
        if (valid) {
            if (dscale) v = apply_dinv<D, T>(dscale, row, v);   // prescaled copy: A x = A_rr (D^-1 A x)
            st<D, T>(y, row, v);
        }
    }
}

// FP64 true residual r = b - A x of the eliminated system (x == nullptr: r = b),
// evaluated in the difference form with the double-double row sums, stored as OUT
// (double, or float for the mixed solver's residual replacement), and r.r in FP64.
template <int D, int G, typename OUT>
__global__ void __launch_bounds__(kVecThreads)
k_residual(int64_t n_nodes, const int32_t *__restrict__ ptr, const int32_t *__restrict__ col,
           const double *__restrict__ val, const double *__restrict__ srow, const double *__restrict__ b,
           const double *__restrict__ x, OUT *__restrict__ r, double *partials, unsigned int *ticket, double *out) {
    double lrr = 0.0;
    FE_ROW_LOOP(G) {
        const bool valid = row < n_nodes;
        NodeVec<D, double> v;
        if (x) {
            v = row_product<D, double, G, true, true>(row, valid, ptr, col, val, x, sub, srow);
        } else {
#pragma unroll
            for (int a = 0; a < D; ++a) v.v[a] = 0.0;
        }
        if (valid && sub == 0) {
            NodeVec<D, double> bv = ld<D, double>(b, row);
            NodeVec<D, OUT> o;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                bv.v[a] -= v.v[a];
                lrr += bv.v[a] * bv.v[a];
                o.v[a] = (OUT)bv.v[a];
            }
            st<D, OUT>(r, row, o);
        }
    }
    double loc[1] = {lrr}, tot[1];
    if (grid_reduce<1>(loc, partials, ticket, tot) && threadIdx.x == 0) *out = tot[0];
}

// q = A p and p.q; the last block sets alpha = r.z / p.q or stops the loop.
template <int D, typename T, bool C16 = false>
__global__ void __launch_bounds__(kVecThreads, kSellBlocks<D, T>)
k_pcg_spmv(int64_t n_nodes, Sell A, const T *__restrict__ val, const T *__restrict__ diag,
           const T *__restrict__ dscale, const T *__restrict__ p, T *__restrict__ q, double *partials,
           PcgScalars *sc) {
    if (sc->done) return;
    T lt = T(0);
    FE_SELL_LOOP {
        const bool valid = row < n_nodes;
        NodeVec<D, T> y = sell_row<D, T, C16>(row, valid, A, val, diag, p);
        if (valid) {
            if (dscale) y = apply_dinv<D, T>(dscale, row, y);   // prescaled copy: A p = A_rr (D^-1 A p)
            st<D, T>(q, row, y);
            NodeVec<D, T> pv = ld<D, T>(p, row);
#pragma unroll
            for (int a = 0; a < D; ++a) lt += pv.v[a] * y.v[a];
        }
    }
    double loc[1] = {(double)lt}, tot[1];
    if (grid_reduce<1>(loc, partials, &sc->ticket[0], tot) && threadIdx.x == 0) {
        double pq = tot[0];
        sc->pq = pq;
        if (!isfinite(pq)) {
            sc->status = FE_NONFINITE;
            sc->done = 1;
        } else if (!(pq > 0.0)) {
            sc->status = FE_BREAKDOWN;
            sc->done = 1;
        } else {
            sc->alpha = sc->rz / pq;
        }
    }
}

// Convergence test, iteration count and beta, once r.z (and r.r) of the new iterate
// are known.
__device__ __forceinline__ void finish_iteration(PcgScalars *sc, double rz_new) {
    int it = sc->iter;
    if (it < 64) sc->hist_alpha[it] = sc->alpha;
    sc->iter = it + 1;
    if (!isfinite(rz_new) || !isfinite(sc->rr)) {
        sc->status = FE_NONFINITE;
        sc->done = 1;
        return;
    }
    if (sc->rr <= sc->tol2 * sc->bb) {
        sc->status = FE_OK;
        sc->done = 1;
        return;
    }
    if (sc->iter >= sc->max_iter) {
        sc->status = FE_MAXITER;
        sc->done = 1;
        return;
    }
    if (!(rz_new > 0.0)) {
        sc->status = FE_BREAKDOWN;
        sc->done = 1;
        return;
    }
    sc->beta = rz_new / sc->rz;
    if (it < 64) sc->hist_beta[it] = sc->beta;
    sc->rz = rz_new;
}

// x += alpha p (x in FP64); r -= alpha q; then z = M^-1 r (Jacobi) or, with CHEB,
// the first Chebyshev term z_1 = M^-1 r / theta, and M^-1 r into rh when the
// Chebyshev steps run on the prescaled copy (rh non-null).  Reduces r.z and r.r.
template <int D, typename T, bool CHEB>
__global__ void __launch_bounds__(kVecThreads)
k_pcg_update(int64_t n_nodes, double *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
             const T *__restrict__ q, const T *__restrict__ dinv, T *__restrict__ z, T *__restrict__ rh,
             double *partials, PcgScalars *sc) {
    if (sc->done) return;
    const double alpha = sc->alpha;
    const T alpha_t = (T)alpha;
    const T inv_theta = CHEB ? (T)(1.0 / sc->cheb_theta) : T(1);
    T lrz = T(0), lrr = T(0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        NodeVec<D, double> xv = ld<D, double>(x, i);
        NodeVec<D, T> rv = ld<D, T>(r, i), pv = ld<D, T>(p, i), qv = ld<D, T>(q, i);
#pragma unroll
        for (int a = 0; a < D; ++a) {
            xv.v[a] += alpha * (double)pv.v[a];
            rv.v[a] -= alpha_t * qv.v[a];
        }
        st<D, double>(x, i, xv);
        st<D, T>(r, i, rv);
        NodeVec<D, T> zv = apply_dinv<D, T>(dinv, i, rv);
        if (CHEB) {
            if (rh) st<D, T>(rh, i, zv);
#pragma unroll
            for (int a = 0; a < D; ++a) zv.v[a] *= inv_theta;
        }
        st<D, T>(z, i, zv);
#pragma unroll
        for (int a = 0; a < D; ++a) {
            lrz += rv.v[a] * zv.v[a];
            lrr += rv.v[a] * rv.v[a];
        }
    }
    double loc[2] = {(double)lrz, (double)lrr}, tot[2];
    if (grid_reduce<2>(loc, partials, &sc->ticket[1], tot) && threadIdx.x == 0) {
        sc->rr = tot[1];
        if (CHEB) {
            // r.z comes from the last Chebyshev step; stop here already if r is small.
            if (!isfinite(tot[1])) {
                sc->status = FE_NONFINITE;
                sc->done = 1;
            } else if (tot[1] <= sc->tol2 * sc->bb) {
                sc->iter += 1;
                sc->status = FE_OK;
                sc->done = 1;
            }
        } else {
            finish_iteration(sc, tot[0]);
        }
    }
}

// One Chebyshev step on D^-1 A z = D^-1 r in three-term form:
//   z_{k+1} = z_k + c1 (z_k - z_{k-1}) + c2 D^-1 (r - A z_k),
// with z_0 = 0 (FIRST: step k = 1).  z_{k+1} is written over z_{k-1} in zprev_out:
// every thread reads and writes only its own rows there, while the gathers of the
// product read z_k.  FP64 (unscaled copy): rres = r, D^-1 applied with dinv.  FP32
// (prescaled copy, val = D^-1 A_rm, diag = D^-1 S_r): rres = D^-1 r and no dinv.
// MODE 0: at the start of a loop (no reduction, runs even when done is set);
// MODE 1: last step of an iteration (reduces rdot.z_{k+1} in FP64, finishes the
//         iteration; rdot is the recurrence's residual);
// MODE 2: intermediate step.
template <int D, typename T, typename RD, int MODE, bool FIRST, bool C16, bool KEEP = false>
__global__ void __launch_bounds__(kVecThreads, KEEP ? 6 : kSellBlocks<D, T>)   // FP32: 8 blocks per SM, one wave
k_cheb_step(int64_t n_nodes, Sell A, const T *__restrict__ val, const T *__restrict__ diag,
            const T *__restrict__ dinv, const T *__restrict__ rres, const T *__restrict__ z_in,
            T *__restrict__ zprev_out, double c1, double c2, double *partials, PcgScalars *sc,
            const RD *__restrict__ rdot) {
    constexpr bool PRE = sizeof(T) == 4;
    if (MODE != 0 && sc->done) return;
    const T c1t = (T)c1, c2t = (T)c2;
    double lrz = 0.0;
    FE_SELL_LOOP {
        const bool valid = row < n_nodes;
        NodeVec<D, T> az = sell_row<D, T, C16, KEEP>(row, valid, A, val, diag, z_in);
        if (valid) {
            NodeVec<D, T> rv = ld<D, T>(rres, row), zv = ld<D, T>(z_in, row), zp;
            if (FIRST) {
#pragma unroll
                for (int a = 0; a < D; ++a) zp.v[a] = T(0);
            } else {
                zp = ld<D, T>(zprev_out, row);
            }
            NodeVec<D, T> mr;
#pragma unroll
            for (int a = 0; a < D; ++a) mr.v[a] = rv.v[a] - az.v[a];
            if (!PRE) mr = apply_dinv<D, T>(dinv, row, mr);
#pragma unroll
            for (int a = 0; a < D; ++a) zv.v[a] += c1t * (zv.v[a] - zp.v[a]) + c2t * mr.v[a];
            st<D, T>(zprev_out, row, zv);
            if (MODE == 1) {
                const NodeVec<D, RD> rd = ld<D, RD>(rdot, row);
#pragma unroll
                for (int a = 0; a < D; ++a) lrz += (double)rd.v[a] * (double)zv.v[a];
            }
        }
    }
    if (MODE == 1) {
        double loc[1] = {lrz}, tot[1];
        if (grid_reduce<1>(loc, partials, &sc->ticket[2], tot) && threadIdx.x == 0) finish_iteration(sc, tot[0]);
    }
}

// p = z + beta p
template <int D, typename T>
__global__ void __launch_bounds__(kVecThreads)
k_pcg_direction(int64_t n_nodes, const T *__restrict__ z, T *__restrict__ p, PcgScalars *sc) {
    if (sc->done) return;
    const T beta = (T)sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        NodeVec<D, T> zv = ld<D, T>(z, i), pv = ld<D, T>(p, i);
#pragma unroll
        for (int a = 0; a < D; ++a) pv.v[a] = zv.v[a] + beta * pv.v[a];
        st<D, T>(p, i, pv);
    }
}

// Start of a loop, given r: z = M^-1 r (times 1/theta with CHEB: the first
// Chebyshev term z_1), and M^-1 r into rh for prescaled Chebyshev steps.
template <int D, typename T, bool CHEB>
__global__ void __launch_bounds__(kVecThreads)
k_start_precond(int64_t n_nodes, const T *__restrict__ r, const T *__restrict__ dinv, T *__restrict__ z,
                T *__restrict__ rh, double theta) {
    const T inv_theta = CHEB ? (T)(1.0 / theta) : T(1);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        NodeVec<D, T> zv = apply_dinv<D, T>(dinv, i, ld<D, T>(r, i));
        if (CHEB && rh) st<D, T>(rh, i, zv);
        if (CHEB) {
#pragma unroll
            for (int a = 0; a < D; ++a) zv.v[a] *= inv_theta;
        }
        st<D, T>(z, i, zv);
    }
}

// Start of a loop, after z: r.z and r.r, then p = z (fresh start) or, when the loop
// continues after a residual replacement, p = z + (r.z / r.z_previous) p so that the
// search direction is kept.  Stops at once if r is already below the tolerance.
template <int D, typename T, bool CONT>
__global__ void __launch_bounds__(kVecThreads)
k_start_finish(int64_t n_nodes, const T *__restrict__ r, const T *__restrict__ z, T *__restrict__ p,
               double *partials, PcgScalars *sc) {
    // reduction first (needed for beta), then the direction in a second sweep by the
    // same threads: r.z over the block partials is only known to the last block, so
    // with CONT the direction update reads beta from a kernel that runs after this one
    T lrz = T(0), lrr = T(0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        NodeVec<D, T> rv = ld<D, T>(r, i), zv = ld<D, T>(z, i);
        if (!CONT) st<D, T>(p, i, zv);
#pragma unroll
        for (int a = 0; a < D; ++a) {
            lrz += rv.v[a] * zv.v[a];
            lrr += rv.v[a] * rv.v[a];
        }
    }
    double loc[2] = {(double)lrz, (double)lrr}, tot[2];
    if (grid_reduce<2>(loc, partials, &sc->ticket[3], tot) && threadIdx.x == 0) {
        double rz_old = sc->rz;
        sc->rz = tot[0];
        sc->rr = tot[1];
        sc->beta = CONT && rz_old > 0.0 ? tot[0] / rz_old : 0.0;
        sc->iter = 0;
        sc->status = FE_OK;
        sc->done = 0;
        if (!isfinite(tot[0]) || !isfinite(tot[1])) {
            sc->status = FE_NONFINITE;
            sc->done = 1;
        } else if (tot[1] <= sc->tol2 * sc->bb) {
            sc->done = 1;
        } else if (!(tot[0] > 0.0)) {
            sc->status = FE_BREAKDOWN;
            sc->done = 1;
        } else if (sc->max_iter <= 0) {
            sc->status = FE_MAXITER;
            sc->done = 1;
        }
    }
}

// p = z + beta p after a residual replacement (beta set by k_start_finish<CONT>),
// run whether or not the loop is done so the direction stays consistent.
template <int D, typename T>
__global__ void __launch_bounds__(kVecThreads)
k_continue_direction(int64_t n_nodes, const T *__restrict__ z, T *__restrict__ p, const PcgScalars *sc) {
    const T beta = (T)sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        NodeVec<D, T> zv = ld<D, T>(z, i), pv = ld<D, T>(p, i);
#pragma unroll
        for (int a = 0; a < D; ++a) pv.v[a] = zv.v[a] + beta * pv.v[a];
        st<D, T>(p, i, pv);
    }
}

// ---- FP64 CG recurrence around an FP32 Chebyshev preconditioner (FE_PREC_MIXED_CG64):
// x, r, p, q in FP64 and q = A p on the FP64 copy; z and the Chebyshev iterates in
// FP32, fed with an FP32 copy of r.

// x += alpha p; r -= alpha q (FP64); rh = M^-1 (float) r; z = rh (/ theta with CHEB).
// Reduces r.z and r.r in FP64.
template <int D, bool CHEB>
__global__ void __launch_bounds__(kVecThreads)
k_mp_update(int64_t n_nodes, double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
            const double *__restrict__ q, const float *__restrict__ dinv, float *__restrict__ rh,
            float *__restrict__ z, double *partials, PcgScalars *sc) {
    if (sc->done) return;
    const double alpha = sc->alpha;
    const float inv_theta = CHEB ? (float)(1.0 / sc->cheb_theta) : 1.0f;
    double lrz = 0.0, lrr = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        NodeVec<D, double> xv = ld<D, double>(x, i), rv = ld<D, double>(r, i);
        const NodeVec<D, double> pv = ld<D, double>(p, i), qv = ld<D, double>(q, i);
        NodeVec<D, float> rf;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            xv.v[a] = fma(alpha, pv.v[a], xv.v[a]);
            rv.v[a] = fma(-alpha, qv.v[a], rv.v[a]);
            rf.v[a] = (float)rv.v[a];
        }
        st<D, double>(x, i, xv);
        st<D, double>(r, i, rv);
        NodeVec<D, float> zv = apply_dinv<D, float>(dinv, i, rf);
        if (CHEB) st<D, float>(rh, i, zv);
#pragma unroll
        for (int a = 0; a < D; ++a) {
            if (CHEB) zv.v[a] *= inv_theta;
            lrz += rv.v[a] * (double)zv.v[a];
            lrr += rv.v[a] * rv.v[a];
        }
        st<D, float>(z, i, zv);
    }
    double loc[2] = {lrz, lrr}, tot[2];
    if (grid_reduce<2>(loc, partials, &sc->ticket[1], tot) && threadIdx.x == 0) {
        sc->rr = tot[1];
        if (CHEB) {
            if (!isfinite(tot[1])) {
                sc->status = FE_NONFINITE;
                sc->done = 1;
            } else if (tot[1] <= sc->tol2 * sc->bb) {
                sc->iter += 1;
                sc->status = FE_OK;
                sc->done = 1;
            }
        } else {
            finish_iteration(sc, tot[0]);
        }
    }
}

// p = z + beta p with z in FP32, p in FP64.
template <int D>
__global__ void __launch_bounds__(kVecThreads)
k_mp_direction(int64_t n_nodes, const float *__restrict__ z, double *__restrict__ p, PcgScalars *sc) {
    if (sc->done) return;
    const double beta = sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        const NodeVec<D, float> zv = ld<D, float>(z, i);
        NodeVec<D, double> pv = ld<D, double>(p, i);
#pragma unroll
        for (int a = 0; a < D; ++a) pv.v[a] = fma(beta, pv.v[a], (double)zv.v[a]);
        st<D, double>(p, i, pv);
    }
}

// Start of a loop from the FP64 residual r: rh = M^-1 (float) r, z = rh (/ theta).
template <int D, bool CHEB>
__global__ void __launch_bounds__(kVecThreads)
k_mp_start_precond(int64_t n_nodes, const double *__restrict__ r, const float *__restrict__ dinv,
                   float *__restrict__ rh, float *__restrict__ z, double theta) {
    const float inv_theta = CHEB ? (float)(1.0 / theta) : 1.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        const NodeVec<D, double> rv = ld<D, double>(r, i);
        NodeVec<D, float> rf;
#pragma unroll
        for (int a = 0; a < D; ++a) rf.v[a] = (float)rv.v[a];
        NodeVec<D, float> zv = apply_dinv<D, float>(dinv, i, rf);
        if (CHEB) st<D, float>(rh, i, zv);
        if (CHEB) {
#pragma unroll
            for (int a = 0; a < D; ++a) zv.v[a] *= inv_theta;
        }
        st<D, float>(z, i, zv);
    }
}

// After z: p = (double) z, r.z and r.r in FP64, loop scalars reset (a fresh start).
template <int D>
__global__ void __launch_bounds__(kVecThreads)
k_mp_start_finish(int64_t n_nodes, const double *__restrict__ r, const float *__restrict__ z,
                  double *__restrict__ p, double *partials, PcgScalars *sc) {
    double lrz = 0.0, lrr = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        const NodeVec<D, double> rv = ld<D, double>(r, i);
        const NodeVec<D, float> zv = ld<D, float>(z, i);
        NodeVec<D, double> pv;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            pv.v[a] = (double)zv.v[a];
            lrz += rv.v[a] * pv.v[a];
            lrr += rv.v[a] * rv.v[a];
        }
        st<D, double>(p, i, pv);
    }
    double loc[2] = {lrz, lrr}, tot[2];
    if (grid_reduce<2>(loc, partials, &sc->ticket[3], tot) && threadIdx.x == 0) {
        sc->rz = tot[0];
        sc->rr = tot[1];
        sc->beta = 0.0;
        sc->iter = 0;
        sc->status = FE_OK;
        sc->done = 0;
        if (!isfinite(tot[0]) || !isfinite(tot[1])) {
            sc->status = FE_NONFINITE;
            sc->done = 1;
        } else if (tot[1] <= sc->tol2 * sc->bb) {
            sc->done = 1;
        } else if (!(tot[0] > 0.0)) {
            sc->status = FE_BREAKDOWN;
            sc->done = 1;
        } else if (sc->max_iter <= 0) {
            sc->status = FE_MAXITER;
            sc->done = 1;
        }
    }
}

// x[dof_k] = g_k on every constrained DOF.  The eliminated rows are identity rows
// decoupled from the free ones, so with this start their residual is exactly zero
// and node-block Jacobi keeps them exact for the whole solve.
__global__ void k_set_prescribed(int64_t n_bc, const int64_t *__restrict__ bc_dof,
                                 const double *__restrict__ bc_val, double *__restrict__ x) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_bc;
         k += (int64_t)gridDim.x * blockDim.x)
        x[bc_dof[k]] = bc_val[k];
}

// lambda_k = F[p_k] - (K u)[p_k], K the full (not eliminated) stiffness: the first
// block row of the reference's saddle system, K u + C^T lambda = F.
template <int D>
__global__ void k_multipliers(int64_t n_bc, const int64_t *__restrict__ bc_dof, const int32_t *__restrict__ ptr,
                              const int32_t *__restrict__ col, const double *__restrict__ kval,
                              const double *__restrict__ F, const double *__restrict__ u, double *__restrict__ lam) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_bc;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = bc_dof[k];
        int64_t r = p / D;
        int a = (int)(p - r * D);
        double acc = 0.0;
        for (int s = ptr[r]; s < ptr[r + 1]; ++s) {
            int m = col[s];
#pragma unroll
            for (int b = 0; b < D; ++b) acc += kval[(int64_t)s * D * D + a * D + b] * u[(int64_t)m * D + b];
        }
        lam[k] = F[p] - acc;
    }
}

// ---------------------------------------------------------------- host side

template <typename T>
struct Sys {
    Sell A;                                   // SELL-32 structure
    const T *sval = nullptr, *diag = nullptr;  // SELL values and diagonal blocks
    const T *val = nullptr, *dinv = nullptr;
    const T *dblk = nullptr;  // FP32: A_rr, scales a product with the prescaled copy back to A x
    double *x = nullptr;   // the solution, FP64 in both precisions
    T *r = nullptr, *p = nullptr, *q = nullptr, *z = nullptr, *zc = nullptr;
    T *rh = nullptr;       // right-hand side of the Chebyshev steps: r (FP64) or D^-1 r (FP32)
};

struct Cheb {
    int k = 1;                 // Chebyshev terms (1 = plain node-block Jacobi)
    double theta = 1, delta = 1;
    double c1[128], c2[128];   // coefficients of steps 1..k-1
};

Cheb make_cheb(int degree, double lmax, double ratio) {
    Cheb c;
    c.k = std::max(1, std::min(degree, 128));
    if (c.k <= 1 || !(lmax > 0)) {
        c.k = 1;
        return c;
    }
    double hi = lmax * 1.05, lo = hi / ratio;
    c.theta = 0.5 * (hi + lo);
    c.delta = 0.5 * (hi - lo);
    double sigma = c.theta / c.delta, rho = 1.0 / sigma;
    for (int s = 1; s < c.k; ++s) {
        double rn = 1.0 / (2.0 * sigma - rho);
        c.c1[s] = rn * rho;
        c.c2[s] = 2.0 * rn / c.delta;
        rho = rn;
    }
    return c;
}

template <int D, typename T>
Sys<T> make_sys(fe_handle_s *h) {
    Sys<T> s;
    SolverWork &w = h->w;
    s.x = w.x.p;
    s.A = Sell{h->sell_off.p, h->sell_col.p, h->sell_c16 ? h->sell_dcol.p : nullptr, h->n_slices};
    if constexpr (sizeof(T) == 4) {
        if (D == 2 && h->l2_keep > 0) {
            const uint64_t total = (uint64_t)h->sell_val32.n * sizeof(float);
            if (total <= 0xffffffffULL) {
                s.A.total = (uint32_t)total;
                s.A.keep = (uint32_t)std::min<uint64_t>(h->l2_keep, total);
            }
        }
    }
    if constexpr (sizeof(T) == 8) {
        s.sval = h->sell_val64.p, s.diag = h->diag64.p;
        s.val = h->aval.p, s.dinv = h->dinv.p;
        s.r = w.r.p, s.p = w.p.p, s.q = w.q.p, s.z = w.z.p, s.zc = w.t.p;
        s.rh = s.r;
    } else {
        s.sval = h->sell_val32.p, s.diag = h->diag32.p;
        s.val = h->aval32.p, s.dinv = h->dinv32.p, s.dblk = h->dblk32.p;
        s.r = w.r32.p, s.p = w.p32.p, s.q = w.q32.p, s.z = w.z32.p, s.zc = w.zc32.p;
        s.rh = w.rh32.p;
    }
    return s;
}

template <int D, typename T, typename RD, int MODE>
void launch_cheb_step(fe_handle_s *h, const Sys<T> &s, bool first, const T *zin, T *zout, double c1, double c2,
                      double *part, PcgScalars *sc, int grid, const RD *rdot) {
    with_col16<T>(s.A, [&](auto c16) {
        constexpr bool C = decltype(c16)::value;
        if constexpr (MODE == 2 && D == 2 && sizeof(T) == 4) {
            // intermediate steps with an L2-resident prefix of the matrix: 6 blocks per SM
            if (!first && s.A.keep > 0) {
                k_cheb_step<D, T, RD, MODE, false, C, true><<<std::min(grid, 152 * 6), kVecThreads, 0, h->stream>>>(
                    h->n_nodes, s.A, s.sval, s.diag, s.dinv, s.rh, zin, zout, c1, c2, part, sc, rdot);
                return;
            }
        }
        const auto kern = first ? k_cheb_step<D, T, RD, MODE, true, C> : k_cheb_step<D, T, RD, MODE, false, C>;
        kern<<<wave_grid((const void *)kern, grid), kVecThreads, 0, h->stream>>>(
            h->n_nodes, s.A, s.sval, s.diag, s.dinv, s.rh, zin, zout, c1, c2, part, sc, rdot);
    });
}

// Chebyshev steps 1..k-1 after z_1 is in s.z; z ping-pongs between s.z and s.zc
// (each step overwrites z_{k-1} with z_{k+1}); *z_final is the buffer holding z_k.
// rdot: the residual the last step dots with z (the recurrence's r).
template <int D, typename T, typename RD>
void enqueue_cheb_steps(fe_handle_s *h, const Sys<T> &s, const Cheb &cb, PcgScalars *sc, double *part, int grid,
                        bool start, T **z_final, cudaEvent_t *ev, const RD *rdot) {
    T *zin = s.z, *zout = s.zc;
    for (int k = 1; k < cb.k; ++k) {
        const bool last = (k == cb.k - 1), first = (k == 1);
        // the intermediate steps 2 .. k-2 (MODE 2, not FIRST) are timed as one run
        if (ev && k == 2 && !last) cudaEventRecordWithFlags(ev[2], h->stream, cudaEventRecordExternal);
        if (start)
            launch_cheb_step<D, T, RD, 0>(h, s, first, zin, zout, cb.c1[k], cb.c2[k], part, sc, grid, rdot);
        else if (last)
            launch_cheb_step<D, T, RD, 1>(h, s, first, zin, zout, cb.c1[k], cb.c2[k], part, sc, grid, rdot);
        else
            launch_cheb_step<D, T, RD, 2>(h, s, first, zin, zout, cb.c1[k], cb.c2[k], part, sc, grid, rdot);
        if (ev && k >= 2 && k == cb.k - 2) cudaEventRecordWithFlags(ev[3], h->stream, cudaEventRecordExternal);
        std::swap(zin, zout);
    }
    *z_final = zin;
}

inline int sell_grid(const fe_handle_s *h) { return grid_for(h->n_slices * 32, kVecThreads, 152 * 8); }


template <int D, typename T>
void enqueue_iteration(fe_handle_s *h, const Sys<T> &s, const Cheb &cb, PcgScalars *sc, double *part,
                       cudaEvent_t *ev = nullptr) {
    const int gv = vec_grid(h->n_nodes);
    const int gs = sell_grid(h);
    if (ev) cudaEventRecordWithFlags(ev[0], h->stream, cudaEventRecordExternal);
    with_col16<T>(s.A, [&](auto c16) {
        k_pcg_spmv<D, T, decltype(c16)::value><<<gs, kVecThreads, 0, h->stream>>>(h->n_nodes, s.A, s.sval, s.diag,
                                                                                   s.dblk, s.p, s.q, part, sc);
    });
    if (ev) cudaEventRecordWithFlags(ev[1], h->stream, cudaEventRecordExternal);
    T *zf = s.z;
    T *rh = s.rh != s.r ? s.rh : nullptr;
    if (cb.k > 1) {
        k_pcg_update<D, T, true><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.x, s.r, s.p, s.q, s.dinv, s.z,
                                                                    rh, part, sc);
        enqueue_cheb_steps<D, T, T>(h, s, cb, sc, part, gs, false, &zf, ev, s.r);
    } else {
        k_pcg_update<D, T, false><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.x, s.r, s.p, s.q, s.dinv, s.z,
                                                                     rh, part, sc);
    }
    k_pcg_direction<D, T><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, zf, s.p, sc);
}

// Start (or continue, CONT) a loop: s.r holds the residual of s.x.  z = P r, then
// p = z (start) or p = z + beta p (continue after a residual replacement).
template <int D, typename T, int G, bool CONT>
int enqueue_start(fe_handle_s *h, const Sys<T> &s, const Cheb &cb, PcgScalars *sc, double *part) {
    const int gv = vec_grid(h->n_nodes);
    const int gs = sell_grid(h);
    T *zf = s.z;
    T *rh = s.rh != s.r ? s.rh : nullptr;
    if (cb.k > 1) {
        k_start_precond<D, T, true><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.r, s.dinv, s.z, rh, cb.theta);
        enqueue_cheb_steps<D, T, T>(h, s, cb, sc, part, gs, true, &zf, nullptr, s.r);
    } else {
        k_start_precond<D, T, false><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.r, s.dinv, s.z, rh, 1.0);
    }
    k_start_finish<D, T, CONT><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.r, zf, s.p, part, sc);
    if (CONT) k_continue_direction<D, T><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, zf, s.p, sc);
    FE_LAUNCH_CHECK();
    h->launches += 2 + (cb.k - 1) + (CONT ? 1 : 0);
    return FE_OK;
}

// FP64 CG recurrence around the FP32 preconditioner: d holds x, r, p, q and the FP64
// SELL copy; f holds the prescaled FP32 SELL copy, dinv32, D^-1 r in FP32 (f.rh) and
// the Chebyshev iterates (f.z, f.zc).
struct SysMP {
    Sys<double> d;
    Sys<float> f;
};

template <int D>
void enqueue_iteration_mp(fe_handle_s *h, const SysMP &s, const Cheb &cb, PcgScalars *sc, double *part,
                          cudaEvent_t *ev = nullptr) {
    const int gv = vec_grid(h->n_nodes);
    const int gs = sell_grid(h);
    if (ev) cudaEventRecordWithFlags(ev[0], h->stream, cudaEventRecordExternal);
    k_pcg_spmv<D, double><<<gs, kVecThreads, 0, h->stream>>>(h->n_nodes, s.d.A, s.d.sval, s.d.diag, nullptr,
                                                               s.d.p, s.d.q, part, sc);
    if (ev) cudaEventRecordWithFlags(ev[1], h->stream, cudaEventRecordExternal);
    float *zf = s.f.z;
    if (cb.k > 1) {
        k_mp_update<D, true><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.d.x, s.d.r, s.d.p, s.d.q, s.f.dinv,
                                                                 s.f.rh, s.f.z, part, sc);
        enqueue_cheb_steps<D, float, double>(h, s.f, cb, sc, part, gs, false, &zf, ev, s.d.r);
    } else {
        k_mp_update<D, false><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.d.x, s.d.r, s.d.p, s.d.q, s.f.dinv,
                                                                  s.f.rh, s.f.z, part, sc);
    }
    k_mp_direction<D><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, zf, s.d.p, sc);
}

// Fresh start from the FP64 residual in s.d.r: z = P r (FP32), p = z.
template <int D>
int enqueue_start_mp(fe_handle_s *h, const SysMP &s, const Cheb &cb, PcgScalars *sc, double *part) {
    const int gv = vec_grid(h->n_nodes);
    const int gs = sell_grid(h);
    float *zf = s.f.z;
    if (cb.k > 1) {
        k_mp_start_precond<D, true><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.d.r, s.f.dinv, s.f.rh, s.f.z,
                                                                        cb.theta);
        enqueue_cheb_steps<D, float, double>(h, s.f, cb, sc, part, gs, true, &zf, nullptr, s.d.r);
    } else {
        k_mp_start_precond<D, false><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.d.r, s.f.dinv, s.f.rh, s.f.z,
                                                                         1.0);
    }
    k_mp_start_finish<D><<<gv, kVecThreads, 0, h->stream>>>(h->n_nodes, s.d.r, zf, s.d.p, part, sc);
    FE_LAUNCH_CHECK();
    h->launches += 2 + (cb.k - 1);
    return FE_OK;
}

// FP64 residual r = b - A x (x may be nullptr) written as OUT, r.r into *out.
template <int D, int G, typename OUT>
int residual(fe_handle_s *h, const double *x, OUT *r, double *out) {
    const int gs = vec_grid(h->n_nodes * G);
    PcgScalars *sc = h->w.sc.p;
    k_residual<D, G, OUT><<<gs, kVecThreads, 0, h->stream>>>(h->n_nodes, h->blk_ptr.p, h->blk_col.p, h->aval.p,
                                                             h->srow.p, h->b.p, x, r, h->w.partials.p,
                                                             &sc->ticket[4], out);
    FE_LAUNCH_CHECK();
    h->launches += 1;
    return FE_OK;
}

// Initial solution: x0 (host or device) or zero, with the prescribed values on the
// constrained DOFs.  Returns whether x is non-zero.
int init_solution(fe_handle_s *h, const fe_solve_opts *o, double *x) {
    if (o->x0)
        FE_CUDA(cudaMemcpyAsync(x, o->x0, h->n_dof * sizeof(double),
                                o->x0_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    else
        FE_CUDA(cudaMemsetAsync(x, 0, h->n_dof * sizeof(double), h->stream));
    if (h->n_bc > 0) {
        k_set_prescribed<<<grid_for(h->n_bc), kThreads, 0, h->stream>>>(h->n_bc, h->bc_dof.p, h->bc_val.p, x);
        FE_LAUNCH_CHECK();
        h->launches += 1;
    }
    return FE_OK;
}

int read_scalars(fe_handle_s *h);

// Starting point of a solve: x0 (or zero) with the prescribed values.  With
// FE_SOLVE_X0_IF_BETTER a given x0 is kept only when its FP64 true residual is below
// that of the zero start, so a poor warm start costs two residuals and nothing more.
template <int D, int G>
int start_point(fe_handle_s *h, const fe_solve_opts *o, double *x, int *x0_used) {
    if (h->x0_ready) {   // an asynchronous prediction of x0: wait for it here, not earlier
        FE_CUDA(cudaStreamWaitEvent(h->stream, h->x0_ready, 0));
        h->x0_ready = nullptr;
    }
    FE_CHECK(init_solution(h, o, x));
    *x0_used = o->x0 ? 1 : 0;
    if (!o->x0 || !(o->flags & FE_SOLVE_X0_IF_BETTER)) return FE_OK;
    PcgScalars *sc = h->w.sc.p;
    double *tmp = h->w.t.p;
    FE_CHECK((residual<D, G, double>(h, x, tmp, &sc->rr)));
    FE_CHECK(read_scalars(h));
    const double rr_x0 = h->w.sc_host->rr;
    fe_solve_opts zero = *o;
    zero.x0 = nullptr;
    FE_CHECK(init_solution(h, &zero, x));
    FE_CHECK((residual<D, G, double>(h, h->n_bc > 0 ? x : nullptr, tmp, &sc->rr)));
    FE_CHECK(read_scalars(h));
    if (h->w.sc_host->rr <= rr_x0) {
        *x0_used = 0;
        return FE_OK;
    }
    return init_solution(h, o, x);
}

int read_scalars(fe_handle_s *h) {
    FE_CUDA(cudaMemcpyAsync(h->w.sc_host, h->w.sc.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

// Progress watch of a running loop: the host sees r.r after every chunk; a running
// minimum that has not improved by 10% (in norm) for `window` iterations marks the
// loop as stalled and ends it at that chunk boundary (x, r, p stay consistent).
struct StallWatch {
    int window = 0;
    double best = INFINITY;
    int best_iter = 0;
    bool stalled = false;
};

// Run PCG iterations until the device says done, replaying a captured chunk of
// iterations (captured once per configuration and graph slot, reused across solves).
// enq(ev) enqueues one iteration, with event records when ev is non-null.
template <typename Enq>
int run_chunks(fe_handle_s *h, int slot, const void *key_ptr, int G, const Cheb &cb, int chunk, Enq enq,
               StallWatch *watch) {
    SolverWork &w = h->w;
    SolverWork::Key &kk = w.key[slot];
    const bool prof = w.prof && w.pev[0];
    bool same = w.graph[slot] && kk.k == cb.k && kk.G == G && kk.chunk == chunk && kk.x == key_ptr &&
                kk.theta == cb.theta && kk.delta == cb.delta && kk.prof == prof && kk.keep == h->l2_keep;
    if (!same) {
        if (w.graph[slot]) {
            cudaGraphExecDestroy(w.graph[slot]);
            w.graph[slot] = nullptr;
        }
        cudaGraph_t g;
        FE_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < chunk; ++i) enq((prof && i == 0) ? w.pev : nullptr);
        cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
        if (ce != cudaSuccess) {
            set_error(std::string("graph capture: ") + cudaGetErrorString(ce));
            return FE_CUDA_ERR;
        }
        ce = cudaGraphInstantiate(&w.graph[slot], g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            w.graph[slot] = nullptr;
            set_error(std::string("graph instantiate: ") + cudaGetErrorString(ce));
            return FE_CUDA_ERR;
        }
        kk.k = cb.k, kk.G = G, kk.chunk = chunk, kk.x = key_ptr, kk.theta = cb.theta, kk.delta = cb.delta;
        kk.prof = prof, kk.keep = h->l2_keep;
    }
    const int per_iter = 3 + (cb.k - 1);
    bool launched = false;
    int it_prev = 0;
    for (;;) {
        FE_CHECK(read_scalars(h));
        // the chunk's first iteration ran in full when a second one followed it
        if (prof && launched && w.sc_host->iter - it_prev >= 2) {
            float a = 0.f;
            if (cudaEventElapsedTime(&a, w.pev[0], w.pev[1]) == cudaSuccess)
                w.prof_ms[slot][1] += a, w.prof_n[slot][1] += 1;
            if (cb.k >= 4 && cudaEventElapsedTime(&a, w.pev[2], w.pev[3]) == cudaSuccess)
                w.prof_ms[slot][0] += a, w.prof_n[slot][0] += cb.k - 3;
        }
        if (w.sc_host->done) break;
        if (watch) {
            const double rr = w.sc_host->rr;
            const int it = w.sc_host->iter;
            if (rr < 0.81 * watch->best) {
                watch->best = rr;
                watch->best_iter = it;
            } else if (it - watch->best_iter > watch->window) {
                watch->stalled = true;
                break;
            }
        }
        it_prev = w.sc_host->iter;
        FE_CUDA(cudaGraphLaunch(w.graph[slot], h->stream));
        launched = true;
        h->launches += (int64_t)chunk * per_iter;
    }
    return FE_OK;
}

template <int D, typename T, int G>
int run_loop(fe_handle_s *h, const Sys<T> &s, const Cheb &cb, int chunk, StallWatch *watch = nullptr) {
    SolverWork &w = h->w;
    return run_chunks(
        h, sizeof(T) == 8 ? 0 : 1, s.p, G, cb, chunk,
        [&](cudaEvent_t *ev) { enqueue_iteration<D, T>(h, s, cb, w.sc.p, w.partials.p, ev); }, watch);
}

template <int D, int G>
int run_loop_mp(fe_handle_s *h, const SysMP &s, const Cheb &cb, int chunk) {
    SolverWork &w = h->w;
    return run_chunks(
        h, 2, s.d.p, G, cb, chunk,
        [&](cudaEvent_t *ev) { enqueue_iteration_mp<D>(h, s, cb, w.sc.p, w.partials.p, ev); }, nullptr);
}

template <typename F>
int dispatch_lanes(int lanes, F &&f) {
    switch (lanes) {
        case 1: return f(std::integral_constant<int, 1>{});
        case 2: return f(std::integral_constant<int, 2>{});
        case 4: return f(std::integral_constant<int, 4>{});
        default: return f(std::integral_constant<int, 8>{});
    }
}

int ensure_work(fe_handle_s *h, bool need64, bool need32) {
    SolverWork &w = h->w;
    // whole SELL slices: the padding rows of the last slice gather their own (unused)
    // entries
    size_t n = (size_t)std::max<int64_t>(std::max<int64_t>(h->n_dof, h->n_slices * 32 * h->dim), 1);
    FE_CHECK(dalloc(w.x, n));
    FE_CHECK(dalloc(w.r, n));
    FE_CHECK(dalloc(w.t, n));
    if (need64) {
        FE_CHECK(dalloc(w.z, n));
        FE_CHECK(dalloc(w.p, n));
        FE_CHECK(dalloc(w.q, n));
    }
    if (need32) {
        FE_CHECK(dalloc(w.r32, n));
        FE_CHECK(dalloc(w.z32, n));
        FE_CHECK(dalloc(w.p32, n));
        FE_CHECK(dalloc(w.q32, n));
        FE_CHECK(dalloc(w.zc32, n));
        FE_CHECK(dalloc(w.rh32, n));
    }
    FE_CHECK(dalloc(w.partials, (size_t)4 * 152 * 8 + 64));
    if (!w.sc.p) {
        FE_CHECK(dalloc(w.sc, 1));
        FE_CUDA(cudaMemsetAsync(w.sc.p, 0, sizeof(PcgScalars), h->stream));
    }
    if (!w.sc_host) FE_CUDA(cudaMallocHost((void **)&w.sc_host, sizeof(PcgScalars)));
    return FE_OK;
}

// Write the loop parameters (tolerance, cap, b.b, Chebyshev centre) to the device
// scalars; tickets and running values are left alone.
int set_params(fe_handle_s *h, double tol2, int max_iter, double bb, double theta) {
    PcgScalars *hs = h->w.sc_host, *ds = h->w.sc.p;
    hs->tol2 = tol2;
    hs->max_iter = max_iter;
    hs->bb = bb;
    hs->cheb_theta = theta;
    FE_CUDA(cudaMemcpyAsync(&ds->tol2, &hs->tol2, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    FE_CUDA(cudaMemcpyAsync(&ds->max_iter, &hs->max_iter, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    FE_CUDA(cudaMemcpyAsync(&ds->bb, &hs->bb, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    FE_CUDA(cudaMemcpyAsync(&ds->cheb_theta, &hs->cheb_theta, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    // the copies read the pinned mirror asynchronously: keep it stable until done
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

template <int D, typename T, int G>
int time_spmv_impl(fe_handle_s *h, int reps, double *ms) {
    Sys<T> s = make_sys<D, T>(h);
    T *x = s.p, *y = s.q;
    FE_CUDA(cudaMemsetAsync(x, 0, h->n_dof * sizeof(T), h->stream));
    const int gs = sell_grid(h);
    for (int i = 0; i < 2; ++i)
        with_col16<T>(s.A, [&](auto c16) {
            k_spmv<D, T, decltype(c16)::value><<<gs, kVecThreads, 0, h->stream>>>(h->n_nodes, s.A, s.sval, s.diag,
                                                                                   s.dblk, x, y);
        });
    FE_CUDA(cudaEventRecord(h->events[8], h->stream));
    for (int i = 0; i < reps; ++i)
        with_col16<T>(s.A, [&](auto c16) {
            k_spmv<D, T, decltype(c16)::value><<<gs, kVecThreads, 0, h->stream>>>(h->n_nodes, s.A, s.sval, s.diag,
                                                                                   s.dblk, x, y);
        });
    FE_CUDA(cudaEventRecord(h->events[9], h->stream));
    FE_LAUNCH_CHECK();
    FE_CUDA(cudaEventSynchronize(h->events[9]));
    float t = 0;
    FE_CUDA(cudaEventElapsedTime(&t, h->events[8], h->events[9]));
    *ms = (double)t / std::max(reps, 1);
    return FE_OK;
}

int time_spmv_any(fe_handle_s *h, int precision, int lanes, int reps, double *ms) {
    bool f32 = precision == FE_PREC_MIXED;
    FE_CHECK(ensure_work(h, !f32, f32));
    // 3 DOF per node: one instantiation, 2 lanes per block row in the BSR kernel
    if (h->dim == 3) return f32 ? time_spmv_impl<3, float, 2>(h, reps, ms) : time_spmv_impl<3, double, 2>(h, reps, ms);
    return dispatch_lanes(lanes, [&](auto g) {
        constexpr int G = decltype(g)::value;
        if (h->dim == 2) return f32 ? time_spmv_impl<2, float, G>(h, reps, ms) : time_spmv_impl<2, double, G>(h, reps, ms);
        return f32 ? time_spmv_impl<1, float, G>(h, reps, ms) : time_spmv_impl<1, double, G>(h, reps, ms);
    });
}

// Lanes per block row of the BSR true-residual kernel (the PCG SpMVs use the SELL
// copy, one lane per row).
int pick_lanes(fe_handle_s *h, int precision, int requested, int *out) {
    (void)h, (void)precision;
    *out = (requested == 1 || requested == 2 || requested == 4 || requested == 8) ? requested : 2;
    return FE_OK;
}

// Largest eigenvalue of D^-1 A from a short Jacobi-PCG probe on b (Lanczos matrix of
// the CG coefficients).  Leaves x, r, p, q, z of the system overwritten.
template <int D, typename T, int G>
int estimate_lmax(fe_handle_s *h, const Sys<T> &s, double bb, int chunk, double *lmax) {
    const int probe = 40;
    PcgScalars *sc = h->w.sc.p;
    FE_CUDA(cudaMemsetAsync(s.x, 0, h->n_dof * sizeof(double), h->stream));
    FE_CHECK(residual<D, G, T>(h, nullptr, s.r, &sc->rr));
    Cheb jac;
    FE_CHECK(set_params(h, 0.0, probe, bb, 1.0));
    FE_CHECK((enqueue_start<D, T, G, false>(h, s, jac, sc, h->w.partials.p)));
    FE_CHECK((run_loop<D, T, G>(h, s, jac, chunk)));
    int m = std::min(h->w.sc_host->iter, 64);
    if (m > 1) m -= 1;
    double lm = lanczos_lmax(h->w.sc_host->hist_alpha, h->w.sc_host->hist_beta, m);
    *lmax = lm > 0 ? lm : 2.0;
    return FE_OK;
}

// PCG with FP64 true residuals from the solution already in x (its true residual
// in r) until the FP64 true residual meets tol.  start() begins a Krylov space from
// r, loop() runs it.  When the recurrence reaches tol but the true residual does not
// (the recurrence drifts from b - A x by about eps * cond(A)), the Krylov space
// restarts from the true residual and runs until its recurrence has halved it; a
// restart that gains less than 2x marks the rounding floor, final with
// accept_stagnation.  Adds to *total and st->spmv.
template <int D, int G, typename Start, typename Loop>
int pcg_restarted(fe_handle_s *h, double *x, double *r, const Cheb &cb, double bb, double tol, int max_iter,
                  int max_restart, bool accept_stagnation, int *total, int *restarts, double *relres, int *status,
                  fe_solve_stats *st, Start start, Loop loop) {
    SolverWork &w = h->w;
    PcgScalars *sc = w.sc.p;
    double prev = 1e300, target = tol;
    *restarts = 0;
    for (;;) {
        FE_CHECK(set_params(h, target * target, max_iter - *total, bb, cb.theta));
        FE_CHECK(start());
        FE_CHECK(loop());
        const int it = w.sc_host->iter, stv = w.sc_host->status;
        *total += it;
        st->spmv += it * cb.k + (cb.k - 1);
        // true residual, which also seeds a restart
        FE_CHECK((residual<D, G, double>(h, x, r, &sc->rr)));
        st->spmv += 1;
        FE_CHECK(read_scalars(h));
        *relres = sqrt(w.sc_host->rr / bb);
        *status = stv;
        if (*relres <= tol) {
            *status = FE_OK;
            return FE_OK;
        }
        if (stv == FE_NONFINITE || stv == FE_BREAKDOWN) return FE_OK;
        if (*total >= max_iter) {
            *status = FE_MAXITER;
            return FE_OK;
        }
        if (*relres > 0.5 * prev || *restarts >= max_restart) {
            *status = accept_stagnation ? FE_OK : FE_MAXITER;
            return FE_OK;
        }
        prev = *relres;
        target = std::min(tol, 0.5 * *relres);
        ++*restarts;
    }
}

template <int D, int G>
int fp64_iterate(fe_handle_s *h, const Sys<double> &s, const Cheb &cb, int chunk, double bb, double tol,
                 int max_iter, int max_restart, bool accept_stagnation, int *total, int *restarts, double *relres,
                 int *status, fe_solve_stats *st) {
    SolverWork &w = h->w;
    return pcg_restarted<D, G>(
        h, s.x, s.r, cb, bb, tol, max_iter, max_restart, accept_stagnation, total, restarts, relres, status, st,
        [&]() { return enqueue_start<D, double, G, false>(h, s, cb, w.sc.p, w.partials.p); },
        [&]() { return run_loop<D, double, G>(h, s, cb, chunk); });
}

template <int D, int G>
int solve_fp64(fe_handle_s *h, const fe_solve_opts *o, fe_solve_stats *st) {
    SolverWork &w = h->w;
    Sys<double> s = make_sys<D, double>(h);
    const int chunk = o->chunk > 0 ? o->chunk : 16;
    const int max_iter = o->max_iter > 0 ? o->max_iter : 200000;
    const int max_restart = o->max_outer > 0 ? o->max_outer : 8;
    const double tol = o->tol > 0 ? o->tol : 1e-10;
    const bool accept_stagnation = (o->flags & FE_SOLVE_ACCEPT_STAGNATION) != 0;
    PcgScalars *sc = w.sc.p;
    FE_CHECK((residual<D, G, double>(h, nullptr, w.t.p, &sc->bb)));
    FE_CHECK(read_scalars(h));
    const double bb = w.sc_host->bb;
    st->bnorm = sqrt(bb);
    Cheb cb;
    if (o->cheb_degree >= 2) {
        if (!(w.lmax[0] > 0)) FE_CHECK((estimate_lmax<D, double, G>(h, s, bb, chunk, &w.lmax[0])));
        cb = make_cheb(o->cheb_degree, w.lmax[0], o->cheb_ratio > 0 ? o->cheb_ratio : 20.0);
    }
    if (bb == 0.0) {
        FE_CUDA(cudaMemsetAsync(s.x, 0, h->n_dof * sizeof(double), h->stream));
        st->relres = 0.0;
        st->status = FE_OK;
        return FE_OK;
    }
    int x0_used = 0;
    FE_CHECK((start_point<D, G>(h, o, s.x, &x0_used)));
    st->x0_used = x0_used;
    const bool nonzero = x0_used || h->n_bc > 0;
    FE_CHECK((residual<D, G, double>(h, nonzero ? s.x : nullptr, s.r, &sc->rr)));
    st->spmv += nonzero ? 1 : 0;
    int total = 0, restarts = 0, status = FE_OK;
    double relres = 0;
    FE_CHECK((fp64_iterate<D, G>(h, s, cb, chunk, bb, tol, max_iter, max_restart, accept_stagnation, &total, &restarts,
                                 &relres, &status, st)));
    st->iterations = total;
    st->outer = restarts;
    st->relres = relres;
    st->status = status;
    return FE_OK;
}

// FP64 CG recurrence with an FP32 Chebyshev preconditioner: x, r, p, q and the
// product q = A p are FP64 (one FP64 SpMV per iteration), the node-block Jacobi and
// the k - 1 Chebyshev SpMVs of the preconditioner run on the FP32 copy of A.  The
// preconditioner's rounding only makes it a slightly different SPD-like
// preconditioner; the FP64 recurrence keeps CG's convergence, which an FP32 product
// A p loses on ill-conditioned problems (its rounding in the smooth modes costs
// ~40% more iterations at 4M DOF).  The FP64 true residual decides convergence as in
// the plain solve.
template <int D, int G>
int solve_mp(fe_handle_s *h, const fe_solve_opts *o, fe_solve_stats *st) {
    SolverWork &w = h->w;
    SysMP s{make_sys<D, double>(h), make_sys<D, float>(h)};
    const int chunk = o->chunk > 0 ? o->chunk : 16;
    const int max_iter = o->max_iter > 0 ? o->max_iter : 200000;
    const int max_restart = o->max_outer > 0 ? o->max_outer : 8;
    const double tol = o->tol > 0 ? o->tol : 1e-8;
    const bool accept_stagnation = (o->flags & FE_SOLVE_ACCEPT_STAGNATION) != 0;
    PcgScalars *sc = w.sc.p;
    FE_CHECK((residual<D, G, double>(h, nullptr, w.t.p, &sc->bb)));
    FE_CHECK(read_scalars(h));
    const double bb = w.sc_host->bb;
    st->bnorm = sqrt(bb);
    Cheb cb;
    if (o->cheb_degree >= 2) {
        if (!(w.lmax[1] > 0)) FE_CHECK((estimate_lmax<D, float, G>(h, s.f, bb, chunk, &w.lmax[1])));
        cb = make_cheb(o->cheb_degree, w.lmax[1], o->cheb_ratio > 0 ? o->cheb_ratio : 20.0);
    }
    if (bb == 0.0) {
        FE_CUDA(cudaMemsetAsync(s.d.x, 0, h->n_dof * sizeof(double), h->stream));
        st->relres = 0.0;
        st->status = FE_OK;
        return FE_OK;
    }
    int x0_used = 0;
    FE_CHECK((start_point<D, G>(h, o, s.d.x, &x0_used)));
    st->x0_used = x0_used;
    const bool nonzero = x0_used || h->n_bc > 0;
    FE_CHECK((residual<D, G, double>(h, nonzero ? s.d.x : nullptr, s.d.r, &sc->rr)));
    st->spmv += nonzero ? 1 : 0;
    int total = 0, restarts = 0, status = FE_OK;
    double relres = 0;
    FE_CHECK((pcg_restarted<D, G>(
        h, s.d.x, s.d.r, cb, bb, tol, max_iter, max_restart, accept_stagnation, &total, &restarts, &relres, &status, st,
        [&]() { return enqueue_start_mp<D>(h, s, cb, w.sc.p, w.partials.p); },
        [&]() { return run_loop_mp<D, G>(h, s, cb, chunk); })));
    st->iterations = total;
    st->outer = restarts;
    st->relres = relres;
    st->status = status;
    return FE_OK;
}

// Mixed precision: one Krylov run in FP32 (difference-form SpMV, FP32 Jacobi /
// Chebyshev, FP32 r, p, q, z) accumulating the solution in FP64.  Each time the FP32
// residual has fallen by `delta` since the last refinement step, the FP64 true
// residual b - A x replaces it (refinement step) and the iteration continues with the
// same search direction.  The solve ends when the FP64 true residual meets tol.
//
// FP32 arithmetic has a floor: on strongly heterogeneous problems the FP32 operator
// cannot resolve the smooth, low-stiffness modes that remain near tol, and the FP32
// iteration stalls above it however often the residual is refreshed.  An FP32 run
// whose residual has not improved by 10% for max(2000, iterations so far)
// iterations (50000 for the first run of a Krylov space), or a refinement step that
// gains less than 2x, counts as stalled: the
// solve then continues with FP64 PCG from the FP64 solution reached so far, so the
// tolerance is met in any case.
template <int D, int G>
int solve_mixed(fe_handle_s *h, const fe_solve_opts *o, fe_solve_stats *st) {
    SolverWork &w = h->w;
    Sys<float> s = make_sys<D, float>(h);
    double *x64 = s.x;
    const int chunk = o->chunk > 0 ? o->chunk : 16;
    const int max_iter = o->max_iter > 0 ? o->max_iter : 400000;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 200;
    const double tol = o->tol > 0 ? o->tol : 1e-8;
    const double delta = o->inner_tol > 0 ? o->inner_tol : 0.1;
    PcgScalars *sc = w.sc.p;
    FE_CHECK((residual<D, G, double>(h, nullptr, w.t.p, &sc->bb)));
    FE_CHECK(read_scalars(h));
    const double bb = w.sc_host->bb;
    st->bnorm = sqrt(bb);
    Cheb cb;
    if (o->cheb_degree >= 2) {
        if (!(w.lmax[1] > 0)) FE_CHECK((estimate_lmax<D, float, G>(h, s, bb, chunk, &w.lmax[1])));
        cb = make_cheb(o->cheb_degree, w.lmax[1], o->cheb_ratio > 0 ? o->cheb_ratio : 20.0);
    }
    if (bb == 0.0) {
        FE_CUDA(cudaMemsetAsync(x64, 0, h->n_dof * sizeof(double), h->stream));
        st->relres = 0;
        st->status = FE_OK;
        return FE_OK;
    }
    int x0_used = 0;
    FE_CHECK((start_point<D, G>(h, o, x64, &x0_used)));
    st->x0_used = x0_used;
    const bool nonzero = x0_used || h->n_bc > 0;
    // r32 = b - A x64 (FP64 residual, stored in FP32)
    FE_CHECK((residual<D, G, float>(h, nonzero ? x64 : nullptr, s.r, &sc->rr)));
    FE_CHECK(read_scalars(h));
    double rr_true = w.sc_host->rr;
    st->spmv += nonzero ? 1 : 0;
    int total = 0, outer = 0, status = FE_OK;
    double relres = sqrt(rr_true / bb);
    bool first = true, stalled = false;
    const bool restart_each = (o->flags & FE_SOLVE_RESTART_EACH_STEP) != 0;
    const char *verbose_env = getenv("FE_VERBOSE");
    const bool verbose = verbose_env && verbose_env[0] == '1';
    while (relres > tol) {
        if (outer >= max_outer || total >= max_iter) {
            status = FE_MAXITER;
            break;
        }
        // the FP32 loop runs until its residual has fallen by delta (or to 0.5 tol)
        double target = std::max(delta * delta * rr_true, 0.25 * tol * tol * bb);
        FE_CHECK(set_params(h, target / bb, max_iter - total, bb, cb.theta));
        if (first)
            FE_CHECK((enqueue_start<D, float, G, false>(h, s, cb, sc, w.partials.p)));
        else
            FE_CHECK((enqueue_start<D, float, G, true>(h, s, cb, sc, w.partials.p)));
        // the 2-norm residual of a fresh Krylov space may rise for a long while
        // before it falls; continued runs fall steadily
        StallWatch watch;
        watch.window = first ? 50000 : std::max(2000, total);
        first = restart_each;
        FE_CHECK((run_loop<D, float, G>(h, s, cb, chunk, &watch)));
        const int it = w.sc_host->iter, stv = w.sc_host->status;
        const double rr_rec = w.sc_host->rr;
        total += it;
        st->spmv += it * cb.k + (cb.k - 1);
        ++outer;
        // refinement step: the FP64 true residual replaces the FP32 recurrence residual
        FE_CHECK((residual<D, G, float>(h, x64, s.r, &sc->rr)));
        st->spmv += 1;
        FE_CHECK(read_scalars(h));
        double rr_new = w.sc_host->rr;
        if (verbose)
            fprintf(stderr, "fe mixed step %d: %d it (status %d) fp32 residual %.3e -> true %.3e\n", outer, it, stv,
                    sqrt(rr_rec / bb), sqrt(rr_new / bb));
        if (!isfinite(rr_new)) {
            status = FE_NONFINITE;
            relres = rr_new;
            break;
        }
        relres = sqrt(rr_new / bb);
        if (relres <= tol) break;
        if (stv == FE_NONFINITE) {
            status = stv;
            break;
        }
        if (total >= max_iter) {
            status = FE_MAXITER;
            break;
        }
        if (watch.stalled || rr_new > 0.25 * rr_true) {
            stalled = true;
            break;
        }
        if (stv == FE_BREAKDOWN) {
            // lost positive definiteness in FP32: restart the Krylov space from the
            // true residual; give up if that makes no progress either
            if (it == 0) {
                status = stv;
                break;
            }
            first = true;
        }
        rr_true = rr_new;
    }
    st->fp64_iterations = 0;
    if (stalled) {
        // FP64 finish from the FP64 solution; the FP32 Chebyshev bounds describe the
        // same operator
        FE_CHECK(ensure_work(h, true, false));
        Sys<double> s64 = make_sys<D, double>(h);
        FE_CHECK((residual<D, G, double>(h, x64, s64.r, &sc->rr)));
        st->spmv += 1;
        const int before = total;
        int restarts = 0;
        FE_CHECK((fp64_iterate<D, G>(h, s64, cb, chunk, bb, tol, max_iter, 8,
                                     (o->flags & FE_SOLVE_ACCEPT_STAGNATION) != 0, &total, &restarts, &relres,
                                     &status, st)));
        st->fp64_iterations = total - before;
        if (verbose)
            fprintf(stderr, "fe mixed: FP32 stalled, FP64 finish %d it -> true %.3e (status %d)\n", total - before,
                    relres, status);
    }
    if (relres <= tol) status = FE_OK;
    st->iterations = total;
    st->outer = outer;
    st->relres = relres;
    st->status = status;
    return FE_OK;
}

}  // namespace

// The start of a solve (x = opts.x0 or 0, the prescribed values on constrained DOFs;
// with FE_SOLVE_X0_IF_BETTER the start whose FP64 residual is smaller), for solvers
// outside this file.
int solve_start_point(fe_handle_s *h, const fe_solve_opts *o, double *x, int *x0_used) {
    return with_dim(h->dim, [&](auto d) { return start_point<decltype(d)::value, 2>(h, o, x, x0_used); });
}

// Largest eigenvalue of the tridiagonal Lanczos matrix built from CG coefficients,
// by bisection on the Sturm sequence.
double lanczos_lmax(const double *alpha, const double *beta, int m) {
    if (m <= 0) return 0.0;
    std::vector<double> dg(m), off(m > 1 ? m - 1 : 1);
    for (int j = 0; j < m; ++j) {
        dg[j] = 1.0 / alpha[j] + (j > 0 ? beta[j - 1] / alpha[j - 1] : 0.0);
        if (j + 1 < m) off[j] = sqrt(std::max(beta[j], 0.0)) / alpha[j];
    }
    double hi = 0.0;
    for (int j = 0; j < m; ++j) {
        double rr = fabs(dg[j]) + (j > 0 ? fabs(off[j - 1]) : 0) + (j + 1 < m ? fabs(off[j]) : 0);
        hi = std::max(hi, rr);
    }
    double lo = 0.0;
    auto count_below = [&](double x) {
        int c = 0;
        double q = dg[0] - x;
        if (q < 0) ++c;
        for (int j = 1; j < m; ++j) {
            if (q == 0) q = 1e-300;
            q = dg[j] - x - off[j - 1] * off[j - 1] / q;
            if (q < 0) ++c;
        }
        return c;
    };
    for (int it = 0; it < 200; ++it) {
        double mid = 0.5 * (lo + hi);
        if (count_below(mid) < m) lo = mid;
        else hi = mid;
    }
    return hi;
}

// ---------------------------------------------------------------- entry points

int solve(fe_handle_s *h, const fe_solve_opts *o, fe_solve_stats *st) {
    if (!h->sys_ready && h->k_ready && h->f_ready) {
        // K and F are assembled but the system matrix was replaced (fe_modal)
        h->singular = false;
        FE_CHECK(apply_dirichlet(h));
        FE_CHECK(check_error_word(h, "fe_solve"));
    }
    if (!h->sys_ready) {
        set_error("fe_solve: the system is not assembled (call fe_assemble with K and F)");
        return FE_NOT_READY;
    }
    const bool mixed = o->precision == FE_PREC_MIXED, mp = o->precision == FE_PREC_MIXED_CG64;
    if (o->precision != FE_PREC_FP64 && !mixed && !mp) {
        set_error("fe_solve: unknown precision");
        return FE_BAD_INPUT;
    }
    FE_CHECK(ensure_work(h, !mixed, mixed || mp));
    if (h->singular) {
        // a node without stiffness: the system is singular; like scipy's spsolve the
        // result is NaN
        FE_CUDA(cudaMemsetAsync(h->w.x.p, 0xff, h->n_dof * sizeof(double), h->stream));
        FE_CHECK(dalloc(h->lambda, (size_t)std::max<int64_t>(h->n_bc, 1)));
        FE_CUDA(cudaMemsetAsync(h->lambda.p, 0xff, std::max<int64_t>(h->n_bc, 1) * sizeof(double), h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
        h->mu_host.assign((size_t)h->n_cont, NAN);
        st->status = FE_BREAKDOWN;
        st->relres = NAN;
        h->have_solution = true;
        return FE_OK;
    }
    // continuity conditions: the projected FP64 PCG, whatever the precision asked
    if (h->n_cont > 0) {
        if (h->x0_ready) {
            FE_CUDA(cudaStreamWaitEvent(h->stream, h->x0_ready, 0));
            h->x0_ready = nullptr;
        }
        return solve_continuity(h, o, st);
    }
    if (o->flags & FE_SOLVE_MULTIGRID) return solve_multigrid(h, o, st);
    int lanes = 2;
    FE_CHECK(pick_lanes(h, o->precision, o->lanes, &lanes));
    FE_CUDA(cudaEventRecord(h->events[6], h->stream));
    int rc = h->dim == 3
                 ? (mixed ? solve_mixed<3, 2>(h, o, st) : mp ? solve_mp<3, 2>(h, o, st) : solve_fp64<3, 2>(h, o, st))
                 : dispatch_lanes(lanes, [&](auto g) {
                       constexpr int G = decltype(g)::value;
                       if (h->dim == 2)
                           return mixed ? solve_mixed<2, G>(h, o, st)
                                        : mp ? solve_mp<2, G>(h, o, st) : solve_fp64<2, G>(h, o, st);
                       return mixed ? solve_mixed<1, G>(h, o, st) : mp ? solve_mp<1, G>(h, o, st)
                                                                         : solve_fp64<1, G>(h, o, st);
                   });
    FE_CHECK(rc);
    FE_CHECK(recover_multipliers(h));
    FE_CUDA(cudaEventRecord(h->events[7], h->stream));
    FE_CUDA(cudaEventSynchronize(h->events[7]));
    float ms = 0;
    FE_CUDA(cudaEventElapsedTime(&ms, h->events[6], h->events[7]));
    st->solve_ms = ms;
    st->assemble_ms = h->last_assemble_ms;
    h->have_solution = true;
    return FE_OK;
}

int recover_multipliers(fe_handle_s *h) {
    FE_CHECK(dalloc(h->lambda, (size_t)std::max<int64_t>(h->n_bc, 1)));
    if (h->n_bc == 0) return FE_OK;
    int g = grid_for(h->n_bc);
    FE_CHECK(with_dim(h->dim, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        k_multipliers<D><<<g, kThreads, 0, h->stream>>>(h->n_bc, h->bc_dof.p, h->blk_ptr.p, h->blk_col.p, h->kval.p,
                                                        h->F.p, h->w.x.p, h->lambda.p);
        return FE_OK;
    }));
    FE_LAUNCH_CHECK();
    h->launches += 1;
    return FE_OK;
}

int autotune_spmv(fe_handle_s *h, int precision, int *lanes, double *ms) {
    if (!h->sys_ready) {
        set_error("assemble first");
        return FE_NOT_READY;
    }
    *lanes = 1;   // SELL-32: one lane per block row, one warp per slice
    return time_spmv_any(h, precision, 1, 10, ms);
}

int time_spmv(fe_handle_s *h, int precision, int lanes, int reps, double *ms) {
    if (!h->sys_ready) {
        set_error("assemble first");
        return FE_NOT_READY;
    }
    return time_spmv_any(h, precision, lanes, reps, ms);
}

// y = A x with the FP64 SELL copy of the eliminated matrix (used by the warm-start
// network's loss).  Enqueued on the handle's stream.
int spmv64(fe_handle_s *h, const double *x, double *y) { return spmv64_on(h, x, y, h->stream); }

int spmv64_on(fe_handle_s *h, const double *x, double *y, cudaStream_t stream) {
    if (!h->sys_ready) {
        set_error("spmv64: the system is not assembled");
        return FE_NOT_READY;
    }
    Sell A{h->sell_off.p, h->sell_col.p, nullptr, h->n_slices};
    FE_CHECK(with_dim(h->dim, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        k_spmv<D, double><<<sell_grid(h), kVecThreads, 0, stream>>>(h->n_nodes, A, h->sell_val64.p, h->diag64.p,
                                                                     nullptr, x, y);
        return FE_OK;
    }));
    FE_LAUNCH_CHECK();
    h->launches += 1;
    return FE_OK;
}

// ---------------------------------------------------------------- multigrid level 0 on SELL
// The V-cycle's finest level is the eliminated system itself, so its smoothing and
// residual run on the handle's prescaled FP32 SELL copy (D^-1 A_rm, D^-1 S_r with the
// node-block Jacobi inverse D^-1) with the Chebyshev step kernel of the mixed solver.

namespace {

// rh = D^-1 r (r rounded to FP32) and z_1 = rh / theta: the first Chebyshev step from
// z_0 = 0, which needs no product
template <int D>
__global__ void __launch_bounds__(kVecThreads)
k_mg_level0_start(int64_t n_nodes, const double *__restrict__ r, const float *__restrict__ dinv,
                  float *__restrict__ rh, float *__restrict__ z1, float inv_theta) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_nodes;
         i += (int64_t)gridDim.x * blockDim.x) {
        const NodeVec<D, double> r64 = ld<D, double>(r, i);
        NodeVec<D, float> rv;
#pragma unroll
        for (int a = 0; a < D; ++a) rv.v[a] = (float)r64.v[a];
        NodeVec<D, float> zv = apply_dinv<D, float>(dinv, i, rv);
        st<D, float>(rh, i, zv);
#pragma unroll
        for (int a = 0; a < D; ++a) zv.v[a] *= inv_theta;
        st<D, float>(z1, i, zv);
    }
}

// t = r - A x = A_rr (D^-1 r - D^-1 A x), given rh = D^-1 r
template <int D, bool C16>
__global__ void __launch_bounds__(kVecThreads, kSellBlocks<D, float>)
k_mg_level0_residual(int64_t n_nodes, Sell A, const float *__restrict__ val, const float *__restrict__ diag,
                     const float *__restrict__ dblk, const float *__restrict__ rh, const float *__restrict__ x,
                     float *__restrict__ t) {
    FE_SELL_LOOP {
        const bool valid = row < n_nodes;
        const NodeVec<D, float> ax = sell_row<D, float, C16>(row, valid, A, val, diag, x);
        if (valid) {
            NodeVec<D, float> rv = ld<D, float>(rh, row);
#pragma unroll
            for (int a = 0; a < D; ++a) rv.v[a] -= ax.v[a];
            st<D, float>(t, row, apply_dinv<D, float>(dblk, row, rv));
        }
    }
}

}  // namespace

int mg_level0_start(fe_handle_s *h, const double *r, float *rh, float *z1, double inv_theta) {
    FE_CHECK(with_dim(h->dim, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        k_mg_level0_start<D><<<vec_grid(h->n_nodes), kVecThreads, 0, h->stream>>>(h->n_nodes, r, h->dinv32.p, rh, z1,
                                                                                  (float)inv_theta);
        return FE_OK;
    }));
    FE_LAUNCH_CHECK();
    h->launches += 1;
    return FE_OK;
}

int mg_level0_cheb(fe_handle_s *h, bool first, const float *rh, const float *zin, float *zout, double c1, double c2) {
    FE_CHECK(with_dim(h->dim, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        Sys<float> s = make_sys<D, float>(h);
        s.rh = const_cast<float *>(rh);
        launch_cheb_step<D, float, float, 0>(h, s, first, zin, zout, c1, c2, nullptr, nullptr, sell_grid(h),
                                             (const float *)nullptr);
        return FE_OK;
    }));
    FE_LAUNCH_CHECK();
    h->launches += 1;
    return FE_OK;
}

int mg_level0_residual(fe_handle_s *h, const float *rh, const float *x, float *t) {
    FE_CHECK(with_dim(h->dim, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        const Sys<float> s = make_sys<D, float>(h);
        with_col16<float>(s.A, [&](auto c16) {
            k_mg_level0_residual<D, decltype(c16)::value><<<sell_grid(h), kVecThreads, 0, h->stream>>>(
                h->n_nodes, s.A, s.sval, s.diag, s.dblk, rh, x, t);
        });
        return FE_OK;
    }));
    FE_LAUNCH_CHECK();
    h->launches += 1;
    return FE_OK;
}

int profile_kernels(fe_handle_s *h, int enable) {
    SolverWork &w = h->w;
    if (enable && !w.pev[0])
        for (int i = 0; i < 4; ++i) FE_CUDA(cudaEventCreate(&w.pev[i]));
    w.prof = enable != 0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 2; ++b) w.prof_ms[a][b] = 0.0, w.prof_n[a][b] = 0;
    for (int a = 0; a < 3; ++a) w.mg_ms[a] = 0.0, w.mg_n[a] = 0;
    for (double &t : w.mg_phase_ms) t = 0.0;
    return FE_OK;
}

void release_solver(fe_handle_s *h) {
    SolverWork &w = h->w;
    for (int i = 0; i < 4; ++i)
        if (w.pev[i]) cudaEventDestroy(w.pev[i]), w.pev[i] = nullptr;
    w.prof = false;
    for (int i = 0; i < 3; ++i)
        if (w.graph[i]) cudaGraphExecDestroy(w.graph[i]), w.graph[i] = nullptr;
    dfree(w.x), dfree(w.r), dfree(w.z), dfree(w.p), dfree(w.q), dfree(w.t);
    dfree(w.r32), dfree(w.z32), dfree(w.p32), dfree(w.q32), dfree(w.zc32), dfree(w.rh32);
    dfree(w.partials), dfree(w.sc);
    if (w.sc_host) cudaFreeHost(w.sc_host), w.sc_host = nullptr;
}

}  // namespace fe
