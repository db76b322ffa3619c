// Batched solve of many independent elasticity instances of uneven size: one persistent
// kernel per chunk of iterations, captured in a CUDA graph.
//
// The instances are assembled together as one block-diagonal system: their meshes are
// concatenated into one handle (disjoint node ranges), so the element kernels, the
// pattern build, the reduction, the Dirichlet elimination and the SELL copies of
// fe_assemble are built once for all of them.  The batched solve is the library's
// mixed-precision PCG (FE_PREC_MIXED_CG64) run per instance: FP64 CG recurrence (x, r,
// p, q, and q = A p on the FP64 SELL copy), node-block Jacobi + Chebyshev
// preconditioner in FP32 on the prescaled FP32 copy, with per-instance step sizes,
// Chebyshev intervals and convergence.
//
// * One cooperative kernel runs a chunk of iterations for every instance.  Its phases
//   (SpMV, step sizes, update, Chebyshev steps, convergence, direction) are separated
//   by grid barriers whose waits are bounded: a barrier that waits too long sets an
//   error word, every block then leaves the kernel and the host reports the error.  The
//   chunk is captured once as a one-node CUDA graph and replayed until every instance
//   is done.
// * Work items are runs of consecutive SELL slices (32 node rows each); a warp owns an
//   item and keeps the same items in every phase, so a row's own values never cross
//   threads.  Items whose instances have all converged are skipped.
// * Reductions are deterministic: each (slice, instance) pair owns one partial-sum slot,
//   written by the warp that owns the slice; one warp per instance sums its slots in a
//   fixed order.  Results are identical run to run.
// * Each instance gets its own Chebyshev interval [lmax_i / ratio, 1.05 lmax_i]; lmax_i
//   comes from the Lanczos matrix of the first CG coefficients of a short Jacobi-PCG
//   probe run by the same kernel.
// * fe_batch_autotune picks the blocks per SM and the slices per work item on the live
//   system.
#include <math.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fe_internal.h"
#include "fe_grid_sync.cuh"
#include "fe_sell.cuh"

namespace fe {
namespace {

constexpr int kBT = 256;                       // threads per block
constexpr int kWarps = kBT / 32;
constexpr int kMaxTerms = 128;                 // Chebyshev terms per preconditioner application
constexpr int kHist = 64;                      // CG coefficients kept per instance for the Lanczos estimate
constexpr int kProbe = 40;                     // iterations of the Jacobi-PCG probe

struct BatchArgs {
    int64_t n_nodes = 0, n_slices = 0, n_slots = 0;
    int n_inst = 0;
    Sell A64, A32;                             // SELL structure; A32 may carry 16-bit column offsets
    const double *val64 = nullptr, *diag64 = nullptr;
    const float *val32 = nullptr, *diag32 = nullptr, *dinv32 = nullptr;
    const double *b = nullptr;                 // right-hand side of the eliminated union system
    const int32_t *inst = nullptr;             // instance of each node row
    const int64_t *slot_off = nullptr;         // [n_inst + 1] first partial-sum slot of each instance
    const int64_t *first_slice = nullptr;      // [n_inst] first slice of each instance
    double *x = nullptr, *r = nullptr, *p = nullptr, *q = nullptr;
    float *rh = nullptr, *z = nullptr, *zc = nullptr;
    double *part = nullptr;                    // [3][n_slots]
    // per instance
    double *rz = nullptr, *rr = nullptr, *bb = nullptr, *alpha = nullptr, *beta = nullptr;
    int *done = nullptr, *iter = nullptr, *status = nullptr;
    double *hist_a = nullptr, *hist_b = nullptr;   // [n_inst][kHist]
    const float *c1 = nullptr, *c2 = nullptr;       // [terms - 1][n_inst]
    const float *inv_theta = nullptr;               // [n_inst]
    int terms = 1;                             // 1: node-block Jacobi; k: Jacobi + k - 1 Chebyshev steps
    int slices_per_item = 1;
    double tol2 = 0.0;
    int max_iter = 0;
    unsigned *bar = nullptr;                   // [0] arrivals, [1] generation
    int *active = nullptr;                     // instances not done
    int *err = nullptr;                        // 1: a grid barrier gave up
};

__device__ __forceinline__ int ld_volatile(const int *p) { return *(const volatile int *)p; }

// The grid barrier between phases (fe_grid_sync.cuh): false once any block has given up
// waiting, and the caller then leaves the kernel.
__device__ __forceinline__ bool grid_barrier(const BatchArgs &a) { return grid_sync_bounded(a.bar, a.err); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Slots of slice s: for every instance j the slice touches, the warp's sum of v over
// the lanes whose rows belong to j goes to slot slot_off[j] + (s - first_slice[j]) of
// part[k].  Every lane of the warp calls this.
__device__ __forceinline__ void slice_partial(const BatchArgs &a, int k, int64_t s, int i_first, int i_last, int i,
                                              double v) {
    const int lane = threadIdx.x & 31;
    for (int j = i_first; j <= i_last; ++j) {
        const double t = warp_sum(i == j ? v : 0.0);
        if (lane == 0) a.part[k * a.n_slots + a.slot_off[j] + (s - a.first_slice[j])] = t;
    }
}

// Sum of instance i's slots of part[k]: per lane in slot order, then a fixed shuffle
// tree; the same value in every lane.
__device__ __forceinline__ double instance_sum(const BatchArgs &a, int k, int i) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int64_t t = a.slot_off[i] + lane; t < a.slot_off[i + 1]; t += 32) s += __ldcg(a.part + k * a.n_slots + t);
    return warp_sum(s);
}

// This warp's slices (runs of slices_per_item consecutive slices, the same runs in every
// phase): f(slice, row, valid, instance, on, i_first, i_last) for each slice whose
// instances are not all done; on = the row exists and its instance is not done.
template <typename F>
__device__ __forceinline__ void for_slices(const BatchArgs &a, F f) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * kWarps;
    const int64_t S = a.slices_per_item;
    for (int64_t item = gw; item * S < a.n_slices; item += nw) {
        const int64_t s1 = min(a.n_slices, (item + 1) * S);
        for (int64_t s = item * S; s < s1; ++s) {
            const int64_t r0 = s * 32, rl = min(a.n_nodes - 1, r0 + 31);
            const int i_first = a.inst[r0], i_last = a.inst[rl];
            bool any = false;
            for (int j = i_first; j <= i_last; ++j) any |= ld_volatile(a.done + j) == 0;
            if (!any) continue;
            const int64_t row = r0 + lane;
            const bool valid = row < a.n_nodes;
            const int i = valid ? a.inst[row] : i_last;
            const bool on = valid && ld_volatile(a.done + i) == 0;
            f(s, row, valid, i, on, i_first, i_last);
        }
    }
}

// Preconditioner start for the rows of active instances: rh = D^-1 (float) r and
// z = rh / theta_i (Jacobi: z = rh); r.r into part[1] and, for Jacobi, r.z into part[2].
// START: first r = b - A x (and b.b into part[0] when want_bb).
template <bool START>
__device__ __forceinline__ void precond_start_phase(const BatchArgs &a, bool want_bb) {
    for_slices(a, [&](int64_t s, int64_t row, bool valid, int i, bool on, int i_first, int i_last) {
        NodeVec<2, double> ax;
        if (START) ax = sell_row<2, double, false, false, true>(row, valid, a.A64, a.val64, a.diag64, a.x);
        double rr = 0.0, rz = 0.0, bbv = 0.0;
        if (on) {
            NodeVec<2, double> rv;
            if (START) {
                const NodeVec<2, double> bv = ld<2, double>(a.b, row);
                rv.v[0] = bv.v[0] - ax.v[0], rv.v[1] = bv.v[1] - ax.v[1];
                st<2, double>(a.r, row, rv);
                bbv = bv.v[0] * bv.v[0] + bv.v[1] * bv.v[1];
            } else {
                rv = ldc<2, double>(a.r, row);
            }
            NodeVec<2, float> rf;
            rf.v[0] = (float)rv.v[0], rf.v[1] = (float)rv.v[1];
            NodeVec<2, float> zv = apply_dinv<2, float>(a.dinv32, row, rf);
            if (a.terms > 1) {
                st<2, float>(a.rh, row, zv);
                const float it = a.inv_theta[i];
                zv.v[0] *= it, zv.v[1] *= it;
            }
            st<2, float>(a.z, row, zv);
            rr = rv.v[0] * rv.v[0] + rv.v[1] * rv.v[1];
            rz = rv.v[0] * (double)zv.v[0] + rv.v[1] * (double)zv.v[1];
        }
        if (START && want_bb) slice_partial(a, 0, s, i_first, i_last, i, bbv);
        slice_partial(a, 1, s, i_first, i_last, i, rr);
        if (a.terms == 1) slice_partial(a, 2, s, i_first, i_last, i, rz);
    });
}

// One Chebyshev step on the prescaled FP32 copy for the rows of active instances:
//   zout = zin + c1 (zin - zout) + c2 (rh - D^-1 A zin)    (first: zout = zin + c2 (...)),
// with instance i's coefficients of this step (the three-term form of the single
// solve); on the last step r.zout into part[2] (r the FP64 recurrence residual).
template <bool C16>
__device__ __forceinline__ void cheb_phase(const BatchArgs &a, int step, const float *zin, float *zout, bool first,
                                           bool last) {
    for_slices(a, [&](int64_t s, int64_t row, bool valid, int i, bool on, int i_first, int i_last) {
        const NodeVec<2, float> az = sell_row<2, float, C16, false, true>(row, valid, a.A32, a.val32, a.diag32, zin);
        double rz = 0.0;
        if (on) {
            const int64_t ci = (int64_t)(step - 1) * a.n_inst + i;
            const float c1 = a.c1[ci], c2 = a.c2[ci];
            const NodeVec<2, float> rv = ldc<2, float>(a.rh, row);
            NodeVec<2, float> zv = ldc<2, float>(zin, row), zp;
            zp.v[0] = zp.v[1] = 0.0f;
            if (!first) zp = ldc<2, float>(zout, row);
#pragma unroll
            for (int d = 0; d < 2; ++d) zv.v[d] += c1 * (zv.v[d] - zp.v[d]) + c2 * (rv.v[d] - az.v[d]);
            st<2, float>(zout, row, zv);
            if (last) {
                const NodeVec<2, double> r64 = ldc<2, double>(a.r, row);
                rz = r64.v[0] * (double)zv.v[0] + r64.v[1] * (double)zv.v[1];
            }
        }
        if (last) slice_partial(a, 2, s, i_first, i_last, i, rz);
    });
}

// The Chebyshev steps after precond_start_phase, each behind a grid barrier.  Returns
// the buffer holding the preconditioned residual, or nullptr when a barrier gave up.
template <bool C16>
__device__ __forceinline__ float *chebyshev_phases(const BatchArgs &a) {
    float *zin = a.z, *zout = a.zc;
    for (int k = 1; k < a.terms; ++k) {
        if (!grid_barrier(a)) return nullptr;
        cheb_phase<C16>(a, k, zin, zout, k == 1, k == a.terms - 1);
        float *t = zin;
        zin = zout;
        zout = t;
    }
    return zin;
}

// Ends instance i (lane 0 of its warp) with status st.
__device__ __forceinline__ void finish_instance(const BatchArgs &a, int64_t i, int st) {
    a.status[i] = st;
    a.done[i] = 1;
    atomicSub(a.active, 1);
}

// The batched PCG.  start != 0: a (re)start of the instances not done -- r = b - A x,
// the preconditioner, p = z, r.z, r.r (and b.b with want_bb) -- before the iterations;
// then up to `iters` iterations.  Instances leave when their recurrence residual meets
// tol (FE_OK), at the iteration cap (FE_MAXITER) or on a breakdown.
template <bool C16>
__global__ void __launch_bounds__(kBT, 2)
kb_pcg(BatchArgs a, int start, int want_bb, int iters) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * kWarps;
    if (start) {
        precond_start_phase<true>(a, want_bb != 0);
        float *zf = chebyshev_phases<C16>(a);
        if (!zf || !grid_barrier(a)) return;
        for (int64_t i = gw; i < a.n_inst; i += nw) {
            if (ld_volatile(a.done + i)) continue;
            const double bbs = want_bb ? instance_sum(a, 0, (int)i) : __ldcg(a.bb + i);
            const double rr = instance_sum(a, 1, (int)i), rz = instance_sum(a, 2, (int)i);
            if (lane == 0) {
                if (want_bb) a.bb[i] = bbs;
                a.rr[i] = rr, a.rz[i] = rz;
                if (!isfinite(rr) || !isfinite(rz)) finish_instance(a, i, FE_NONFINITE);
                else if (rr <= a.tol2 * bbs) finish_instance(a, i, FE_OK);
                else if (!(rz > 0.0)) finish_instance(a, i, FE_BREAKDOWN);
                else if (__ldcg(a.iter + i) >= a.max_iter) finish_instance(a, i, FE_MAXITER);
            }
        }
        if (!grid_barrier(a)) return;
        for_slices(a, [&](int64_t, int64_t row, bool, int, bool on, int, int) {
            if (on) {
                const NodeVec<2, float> zv = ldc<2, float>(zf, row);
                st<2, double>(a.p, row, NodeVec<2, double>{{(double)zv.v[0], (double)zv.v[1]}});
            }
        });
        if (!grid_barrier(a)) return;
    }
    for (int it = 0; it < iters; ++it) {
        // written before the last barrier: every block reads the same count
        if (ld_volatile(a.active) <= 0) return;
        // q = A p (FP64) and p.q
        for_slices(a, [&](int64_t s, int64_t row, bool valid, int i, bool on, int i_first, int i_last) {
            const NodeVec<2, double> y = sell_row<2, double, false, false, true>(row, valid, a.A64, a.val64, a.diag64,
                                                                                 a.p);
            double pq = 0.0;
            if (on) {
                st<2, double>(a.q, row, y);
                const NodeVec<2, double> pv = ldc<2, double>(a.p, row);
                pq = pv.v[0] * y.v[0] + pv.v[1] * y.v[1];
            }
            slice_partial(a, 0, s, i_first, i_last, i, pq);
        });
        if (!grid_barrier(a)) return;
        // alpha_i = r.z / p.q
        for (int64_t i = gw; i < a.n_inst; i += nw) {
            if (ld_volatile(a.done + i)) continue;
            const double pq = instance_sum(a, 0, (int)i);
            if (lane == 0) {
                if (!isfinite(pq)) finish_instance(a, i, FE_NONFINITE);
                else if (!(pq > 0.0)) finish_instance(a, i, FE_BREAKDOWN);
                else a.alpha[i] = __ldcg(a.rz + i) / pq;
            }
        }
        if (!grid_barrier(a)) return;
        // x += alpha p, r -= alpha q (FP64)
        for_slices(a, [&](int64_t, int64_t row, bool, int i, bool on, int, int) {
            if (on) {
                const double al = __ldcg(a.alpha + i);
                NodeVec<2, double> xv = ldc<2, double>(a.x, row), rv = ldc<2, double>(a.r, row);
                const NodeVec<2, double> pv = ldc<2, double>(a.p, row), qv = ldc<2, double>(a.q, row);
#pragma unroll
                for (int d = 0; d < 2; ++d) {
                    xv.v[d] = fma(al, pv.v[d], xv.v[d]);
                    rv.v[d] = fma(-al, qv.v[d], rv.v[d]);
                }
                st<2, double>(a.x, row, xv);
                st<2, double>(a.r, row, rv);
            }
        });
        // z = M^-1 r (the same rows, the same thread: no barrier needed before it)
        precond_start_phase<false>(a, false);
        float *zf = chebyshev_phases<C16>(a);
        if (!zf || !grid_barrier(a)) return;
        // convergence and beta per instance
        for (int64_t i = gw; i < a.n_inst; i += nw) {
            if (ld_volatile(a.done + i)) continue;
            const double rr = instance_sum(a, 1, (int)i), rzn = instance_sum(a, 2, (int)i);
            if (lane == 0) {
                const int k = __ldcg(a.iter + i);
                if (k < kHist) a.hist_a[i * kHist + k] = __ldcg(a.alpha + i);
                a.iter[i] = k + 1;
                a.rr[i] = rr;
                if (!isfinite(rzn) || !isfinite(rr)) {
                    finish_instance(a, i, FE_NONFINITE);
                } else if (rr <= a.tol2 * __ldcg(a.bb + i)) {
                    finish_instance(a, i, FE_OK);
                } else if (k + 1 >= a.max_iter) {
                    finish_instance(a, i, FE_MAXITER);
                } else if (!(rzn > 0.0)) {
                    finish_instance(a, i, FE_BREAKDOWN);
                } else {
                    const double be = rzn / __ldcg(a.rz + i);
                    if (k < kHist) a.hist_b[i * kHist + k] = be;
                    a.beta[i] = be;
                    a.rz[i] = rzn;
                }
            }
        }
        if (!grid_barrier(a)) return;
        // p = z + beta p
        for_slices(a, [&](int64_t, int64_t row, bool, int i, bool on, int, int) {
            if (on) {
                const double be = __ldcg(a.beta + i);
                const NodeVec<2, float> zv = ldc<2, float>(zf, row);
                NodeVec<2, double> pv = ldc<2, double>(a.p, row);
                pv.v[0] = fma(be, pv.v[0], (double)zv.v[0]);
                pv.v[1] = fma(be, pv.v[1], (double)zv.v[1]);
                st<2, double>(a.p, row, pv);
            }
        });
        if (!grid_barrier(a)) return;
    }
}

// ||b - A x||^2 per (slice, instance) slot of part[0] (FP64, every instance); a warp per
// slice, grid-stride.
__global__ void __launch_bounds__(kBT)
kb_true_residual(BatchArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * kWarps;
    for (int64_t s = gw; s < a.n_slices; s += nw) {
        const int64_t r0 = s * 32, rl = min(a.n_nodes - 1, r0 + 31);
        const int i_first = a.inst[r0], i_last = a.inst[rl];
        const int64_t row = r0 + lane;
        const bool valid = row < a.n_nodes;
        const int i = valid ? a.inst[row] : i_last;
        const NodeVec<2, double> ax = sell_row<2, double>(row, valid, a.A64, a.val64, a.diag64, a.x);
        double v = 0.0;
        if (valid) {
            const NodeVec<2, double> bv = ld<2, double>(a.b, row);
            const double e0 = bv.v[0] - ax.v[0], e1 = bv.v[1] - ax.v[1];
            v = e0 * e0 + e1 * e1;
        }
        slice_partial(a, 0, s, i_first, i_last, i, v);
    }
}

// out[i] = the sum of instance i's slots of part[0]; a warp per instance
__global__ void __launch_bounds__(kBT)
kb_instance_sums(BatchArgs a, double *out) {
    const int64_t gw = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * kWarps;
    for (int64_t i = gw; i < a.n_inst; i += nw) {
        const double s = instance_sum(a, 0, (int)i);
        if ((threadIdx.x & 31) == 0) out[i] = s;
    }
}

__global__ void kb_inst_of_node(int n_inst, const int64_t *__restrict__ node_ptr, int32_t *__restrict__ inst) {
    for (int i = blockIdx.x; i < n_inst; i += gridDim.x)
        for (int64_t r = node_ptr[i] + threadIdx.x; r < node_ptr[i + 1]; r += blockDim.x) inst[r] = i;
}

__global__ void kb_set_prescribed(int64_t n_bc, const int64_t *__restrict__ bc_dof, const double *__restrict__ bc_val,
                                  double *__restrict__ x) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_bc; k += (int64_t)gridDim.x * blockDim.x)
        x[bc_dof[k]] = bc_val[k];
}

}  // namespace
}  // namespace fe

struct fe_batch_s {
    fe_handle_s *h = nullptr;
    int n_inst = 0;
    std::vector<int64_t> node_ptr_host;
    fe::DBuf<int64_t> node_ptr, slot_off, first_slice;
    fe::DBuf<int32_t> inst;
    int64_t n_slots = 0;
    fe::DBuf<double> x, r, p, q, part, dscal, hist, res;
    fe::DBuf<float> rh, z, zc, cheb;
    fe::DBuf<int> iscal, err;
    fe::DBuf<unsigned> bar;
    int *host_flags = nullptr;       // pinned: [0] active, [1] error word
    // tiles: resident blocks per SM (0 = as many as fit) and slices per work item
    int blocks_per_sm = 0;
    int slices_per_item = 4;
    // preconditioner: Chebyshev terms (1 = node-block Jacobi) over [lmax_i / ratio, 1.05 lmax_i]
    int cheb_degree = 16;
    double cheb_ratio = 1e4;
    std::vector<double> lmax;        // per instance, for system generation lmax_gen
    uint64_t lmax_gen = 0;
    int coef_terms = 0;              // what the coefficient table holds
    double coef_ratio = 0.0;
    uint64_t coef_gen = 0;
    cudaGraphExec_t graph = nullptr;
    bool graph_unsupported = false;  // the runtime refused to capture the cooperative launch
    struct Key {
        int grid = -1, spi = -1, terms = -1, c16 = -1, chunk = -1, max_iter = -1;
        double tol2 = -1.0;
        const void *v64 = nullptr, *v32 = nullptr;
    } key;
    // the last fe_batch_solve: replays of the captured chunk, persistent-kernel launches
    int last_graph_launches = 0, last_kernel_launches = 0;
};

namespace fe {
namespace {

int64_t slices_of(const fe_handle_s *h) { return h->n_slices; }

BatchArgs batch_args(fe_batch_s *b) {
    fe_handle_s *h = b->h;
    const int n = b->n_inst;
    BatchArgs a;
    a.n_nodes = h->n_nodes, a.n_slices = slices_of(h), a.n_slots = b->n_slots, a.n_inst = n;
    a.A64 = Sell{h->sell_off.p, h->sell_col.p, nullptr, h->n_slices};
    a.A32 = Sell{h->sell_off.p, h->sell_col.p, h->sell_c16 ? h->sell_dcol.p : nullptr, h->n_slices};
    a.val64 = h->sell_val64.p, a.diag64 = h->diag64.p;
    a.val32 = h->sell_val32.p, a.diag32 = h->diag32.p, a.dinv32 = h->dinv32.p;
    a.b = h->b.p;
    a.inst = b->inst.p, a.slot_off = b->slot_off.p, a.first_slice = b->first_slice.p;
    a.x = b->x.p, a.r = b->r.p, a.p = b->p.p, a.q = b->q.p;
    a.rh = b->rh.p, a.z = b->z.p, a.zc = b->zc.p;
    a.part = b->part.p;
    double *d = b->dscal.p;
    a.rz = d, a.rr = d + n, a.bb = d + 2 * n, a.alpha = d + 3 * n, a.beta = d + 4 * n;
    int *k = b->iscal.p;
    a.done = k, a.iter = k + n, a.status = k + 2 * n, a.active = k + 3 * n;
    a.hist_a = b->hist.p, a.hist_b = b->hist.p + (int64_t)n * kHist;
    a.inv_theta = b->cheb.p;
    a.c1 = b->cheb.p + n;
    a.c2 = b->cheb.p + n + (int64_t)(kMaxTerms - 1) * n;
    a.slices_per_item = b->slices_per_item;
    a.bar = b->bar.p, a.err = b->err.p;
    return a;
}

template <bool C16>
const void *pcg_kernel() {
    return (const void *)kb_pcg<C16>;
}

// Cooperative grid of the persistent kernel: SMs x resident blocks per SM (capped by
// blocks_per_sm when set).
int pcg_grid(fe_batch_s *b, int *grid) {
    const void *k = b->h->sell_c16 ? pcg_kernel<true>() : pcg_kernel<false>();
    int dev = 0, sms = 0, per_sm = 0;
    FE_CUDA(cudaGetDevice(&dev));
    FE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBT, 0));
    if (per_sm < 1) {
        set_error("fe_batch_solve: the batched kernel does not fit on an SM");
        return FE_CUDA_ERR;
    }
    const int bps = b->blocks_per_sm > 0 ? std::min(b->blocks_per_sm, per_sm) : per_sm;
    *grid = sms * bps;
    return FE_OK;
}

// One cooperative launch of kb_pcg on the handle's stream.
int launch_pcg(fe_batch_s *b, const BatchArgs &a, int grid, int start, int want_bb, int iters) {
    fe_handle_s *h = b->h;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (h->sell_c16)
        FE_CUDA(cudaLaunchKernelEx(&cfg, kb_pcg<true>, a, start, want_bb, iters));
    else
        FE_CUDA(cudaLaunchKernelEx(&cfg, kb_pcg<false>, a, start, want_bb, iters));
    h->launches += 1;
    return FE_OK;
}

// Reads the active count and the barrier error word (synchronises the stream).
int read_flags(fe_batch_s *b, int *active) {
    fe_handle_s *h = b->h;
    const int n = b->n_inst;
    FE_CUDA(cudaMemcpyAsync(b->host_flags, b->iscal.p + 3 * n, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaMemcpyAsync(b->host_flags + 1, b->err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    if (b->host_flags[1]) {
        set_error("batched solve: a grid barrier of the persistent kernel timed out");
        return FE_CUDA_ERR;
    }
    *active = b->host_flags[0];
    return FE_OK;
}

// Fresh state: x = the prescribed values (0 elsewhere), every instance active, counters
// and histories cleared.
int reset_state(fe_batch_s *b) {
    fe_handle_s *h = b->h;
    cudaStream_t s = h->stream;
    const int n = b->n_inst;
    FE_CUDA(cudaMemsetAsync(b->x.p, 0, b->x.n * sizeof(double), s));
    if (h->n_bc > 0) {
        kb_set_prescribed<<<grid_for(h->n_bc), kThreads, 0, s>>>(h->n_bc, h->bc_dof.p, h->bc_val.p, b->x.p);
        FE_LAUNCH_CHECK();
        h->launches += 1;
    }
    FE_CUDA(cudaMemsetAsync(b->dscal.p, 0, b->dscal.n * sizeof(double), s));
    FE_CUDA(cudaMemsetAsync(b->hist.p, 0, b->hist.n * sizeof(double), s));
    FE_CUDA(cudaMemsetAsync(b->iscal.p, 0, 3 * n * sizeof(int), s));
    FE_CUDA(cudaMemcpyAsync(b->iscal.p + 3 * n, &b->n_inst, sizeof(int), cudaMemcpyHostToDevice, s));
    FE_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(int), s));
    FE_CUDA(cudaMemsetAsync(b->bar.p, 0, 2 * sizeof(unsigned), s));
    return FE_OK;
}

// Runs the batched PCG with `terms` preconditioner terms from the current state: a
// start launch, then chunks of `chunk` iterations from the captured graph until every
// instance is done.  *graph_launches counts the replays.
int run_pcg(fe_batch_s *b, int terms, double tol, int max_iter, bool first_start, bool use_graph, int chunk,
            int *graph_launches) {
    fe_handle_s *h = b->h;
    int grid = 0;
    FE_CHECK(pcg_grid(b, &grid));
    BatchArgs a = batch_args(b);
    a.terms = terms, a.tol2 = tol * tol, a.max_iter = max_iter;
    FE_CHECK(launch_pcg(b, a, grid, 1, first_start ? 1 : 0, chunk));
    b->last_kernel_launches += 1;
    int active = 0;
    FE_CHECK(read_flags(b, &active));
    if (graph_launches) *graph_launches = 0;
    if (active <= 0) return FE_OK;
    fe_batch_s::Key key;
    key.grid = grid, key.spi = b->slices_per_item, key.terms = terms, key.c16 = h->sell_c16 ? 1 : 0;
    key.chunk = chunk, key.max_iter = max_iter, key.tol2 = a.tol2, key.v64 = a.val64, key.v32 = a.val32;
    const bool same = b->graph && key.grid == b->key.grid && key.spi == b->key.spi && key.terms == b->key.terms &&
                      key.c16 == b->key.c16 && key.chunk == b->key.chunk && key.max_iter == b->key.max_iter &&
                      key.tol2 == b->key.tol2 && key.v64 == b->key.v64 && key.v32 == b->key.v32;
    use_graph = use_graph && !b->graph_unsupported;
    if (use_graph && !same) {
        if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
        cudaGraph_t g = nullptr;
        FE_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = launch_pcg(b, a, grid, 0, 0, chunk);
        cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
        h->launches -= 1;   // captured, not run
        if (ce == cudaSuccess && rc == FE_OK) {
            ce = cudaGraphInstantiate(&b->graph, g, 0);
            if (ce != cudaSuccess) b->graph = nullptr;
        }
        if (g) cudaGraphDestroy(g);
        if (rc != FE_OK || ce != cudaSuccess) {
            // a runtime that does not capture cooperative launches: launch the chunks
            // directly from here on (the same kernel, one launch per chunk)
            cudaGetLastError();
            b->graph_unsupported = true;
            use_graph = false;
        } else {
            b->key = key;
        }
    }
    while (active > 0) {
        if (use_graph) {
            FE_CUDA(cudaGraphLaunch(b->graph, h->stream));
            h->launches += 1;
            b->last_graph_launches += 1;
        } else {
            FE_CHECK(launch_pcg(b, a, grid, 0, 0, chunk));
        }
        b->last_kernel_launches += 1;
        if (graph_launches) ++*graph_launches;
        FE_CHECK(read_flags(b, &active));
    }
    return FE_OK;
}

// Per-instance largest eigenvalue of D^-1 A_i (Lanczos matrix of the CG coefficients of
// a short Jacobi-PCG probe), computed once per assembled system.
int ensure_lmax(fe_batch_s *b) {
    fe_handle_s *h = b->h;
    if (b->lmax_gen == h->sys_generation && (int)b->lmax.size() == b->n_inst) return FE_OK;
    const int n = b->n_inst;
    FE_CHECK(reset_state(b));
    FE_CHECK(run_pcg(b, 1, 0.0, kProbe + 1, true, false, kProbe + 1, nullptr));
    std::vector<double> hist((size_t)2 * n * kHist);
    std::vector<int> iters(n);
    FE_CUDA(cudaMemcpyAsync(hist.data(), b->hist.p, hist.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaMemcpyAsync(iters.data(), b->iscal.p + n, n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    b->lmax.assign(n, 2.0);
    for (int i = 0; i < n; ++i) {
        int m = std::min(iters[i], kHist);
        if (m > 1) m -= 1;
        const double lm = lanczos_lmax(&hist[(size_t)i * kHist], &hist[(size_t)n * kHist + (size_t)i * kHist], m);
        if (lm > 0 && std::isfinite(lm)) b->lmax[i] = lm;
    }
    b->lmax_gen = h->sys_generation;
    return FE_OK;
}

// Per-instance Chebyshev coefficients of `terms` terms over [lmax_i / ratio, 1.05 lmax_i]
// (the single solve's three-term recurrence) into the device table.
int ensure_coefficients(fe_batch_s *b, int terms) {
    fe_handle_s *h = b->h;
    if (b->coef_terms == terms && b->coef_ratio == b->cheb_ratio && b->coef_gen == b->lmax_gen) return FE_OK;
    const int n = b->n_inst;
    std::vector<float> tab(b->cheb.n, 0.0f);
    for (int i = 0; i < n; ++i) {
        const double hi = 1.05 * b->lmax[i], lo = hi / b->cheb_ratio;
        const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
        tab[i] = (float)(1.0 / theta);
        double rho = 1.0 / sigma;
        for (int s = 1; s < terms; ++s) {
            const double rn = 1.0 / (2.0 * sigma - rho);
            tab[n + (size_t)(s - 1) * n + i] = (float)(rn * rho);
            tab[n + (size_t)(kMaxTerms - 1) * n + (size_t)(s - 1) * n + i] = (float)(2.0 * rn / delta);
            rho = rn;
        }
    }
    FE_CUDA(cudaMemcpyAsync(b->cheb.p, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    b->coef_terms = terms, b->coef_ratio = b->cheb_ratio, b->coef_gen = b->lmax_gen;
    return FE_OK;
}

// Per-instance ||b - A x||^2 into b->res (deterministic).
int true_residuals(fe_batch_s *b) {
    fe_handle_s *h = b->h;
    BatchArgs a = batch_args(b);
    const int g = grid_for(a.n_slices * 32, kBT, 152 * 8);
    kb_true_residual<<<g, kBT, 0, h->stream>>>(a);
    kb_instance_sums<<<grid_for((int64_t)b->n_inst * 32, kBT, 152 * 8), kBT, 0, h->stream>>>(a, b->res.p);
    FE_LAUNCH_CHECK();
    h->launches += 2;
    return FE_OK;
}

}  // namespace
}  // namespace fe

using namespace fe;

extern "C" {

int fe_batch_create(fe_handle h, int32_t n_instances, const int64_t *node_ptr_host, fe_batch *out) {
    if (!h || !out || n_instances <= 0 || !node_ptr_host) {
        set_error("fe_batch_create: bad arguments");
        return FE_BAD_INPUT;
    }
    if (h->kind != FE_KIND_ELASTIC_TRI) {
        set_error("fe_batch_create: batched solves are for elasticity meshes");
        return FE_BAD_INPUT;
    }
    if (node_ptr_host[0] != 0 || node_ptr_host[n_instances] != h->n_nodes) {
        set_error("fe_batch_create: node_ptr must run from 0 to the handle's node count");
        return FE_BAD_INPUT;
    }
    for (int i = 0; i < n_instances; ++i)
        if (node_ptr_host[i + 1] <= node_ptr_host[i]) {
            set_error("fe_batch_create: every instance needs at least one node, in increasing order");
            return FE_BAD_INPUT;
        }
    fe_batch_s *b = new fe_batch_s();
    b->h = h;
    b->n_inst = n_instances;
    b->node_ptr_host.assign(node_ptr_host, node_ptr_host + n_instances + 1);
    // partial-sum slots: one per (slice, instance) pair, instance by instance
    std::vector<int64_t> slot_off(n_instances + 1), first_slice(n_instances);
    slot_off[0] = 0;
    for (int i = 0; i < n_instances; ++i) {
        const int64_t f = node_ptr_host[i] / 32, l = (node_ptr_host[i + 1] - 1) / 32;
        first_slice[i] = f;
        slot_off[i + 1] = slot_off[i] + (l - f + 1);
    }
    b->n_slots = slot_off[n_instances];
    // vectors cover whole slices: the SELL rows past the last node gather their own row
    const int64_t rows = (int64_t)((h->n_nodes + 31) / 32) * 32;
    const size_t nv = (size_t)std::max<int64_t>(rows * 2, 2);
    const int n = n_instances;
    int st = dalloc(b->node_ptr, (size_t)n + 1);
    if (!st) st = dalloc(b->slot_off, (size_t)n + 1);
    if (!st) st = dalloc(b->first_slice, (size_t)n);
    if (!st) st = dalloc(b->inst, (size_t)std::max<int64_t>(rows, 1));
    if (!st) st = dalloc(b->x, nv);
    if (!st) st = dalloc(b->r, nv);
    if (!st) st = dalloc(b->p, nv);
    if (!st) st = dalloc(b->q, nv);
    if (!st) st = dalloc(b->rh, nv);
    if (!st) st = dalloc(b->z, nv);
    if (!st) st = dalloc(b->zc, nv);
    if (!st) st = dalloc(b->part, (size_t)3 * std::max<int64_t>(b->n_slots, 1));
    if (!st) st = dalloc(b->dscal, (size_t)5 * n);
    if (!st) st = dalloc(b->hist, (size_t)2 * n * kHist);
    if (!st) st = dalloc(b->res, (size_t)n);
    if (!st) st = dalloc(b->cheb, (size_t)n + (size_t)2 * (kMaxTerms - 1) * n);
    if (!st) st = dalloc(b->iscal, (size_t)3 * n + 1);
    if (!st) st = dalloc(b->err, 1);
    if (!st) st = dalloc(b->bar, 2);
    if (!st && cudaMallocHost((void **)&b->host_flags, 2 * sizeof(int)) != cudaSuccess) {
        set_error("fe_batch_create: pinned host flags");
        st = FE_CUDA_ERR;
    }
    if (st) {
        fe_batch_destroy(b);
        return st;
    }
    cudaStream_t s = h->stream;
    bool ok = cudaMemcpyAsync(b->node_ptr.p, node_ptr_host, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s) ==
                  cudaSuccess &&
              cudaMemcpyAsync(b->slot_off.p, slot_off.data(), (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s) ==
                  cudaSuccess &&
              cudaMemcpyAsync(b->first_slice.p, first_slice.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, s) ==
                  cudaSuccess &&
              cudaMemsetAsync(b->inst.p, 0, b->inst.n * sizeof(int32_t), s) == cudaSuccess &&
              cudaMemsetAsync(b->x.p, 0, nv * sizeof(double), s) == cudaSuccess &&
              cudaMemsetAsync(b->p.p, 0, nv * sizeof(double), s) == cudaSuccess &&
              cudaMemsetAsync(b->z.p, 0, nv * sizeof(float), s) == cudaSuccess &&
              cudaMemsetAsync(b->zc.p, 0, nv * sizeof(float), s) == cudaSuccess;
    if (ok) {
        kb_inst_of_node<<<std::min(n, 152 * 8), 256, 0, s>>>(n, b->node_ptr.p, b->inst.p);
        ok = cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
    }
    if (!ok) {
        fe_batch_destroy(b);
        set_error("fe_batch_create: device set-up failed");
        return FE_CUDA_ERR;
    }
    h->launches += 1;
    *out = b;
    return FE_OK;
}

int fe_batch_destroy(fe_batch b) {
    if (!b) return FE_OK;
    if (b->h && b->h->stream) cudaStreamSynchronize(b->h->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    dfree(b->node_ptr), dfree(b->slot_off), dfree(b->first_slice), dfree(b->inst);
    dfree(b->x), dfree(b->r), dfree(b->p), dfree(b->q), dfree(b->rh), dfree(b->z), dfree(b->zc);
    dfree(b->part), dfree(b->dscal), dfree(b->hist), dfree(b->res), dfree(b->cheb);
    dfree(b->iscal), dfree(b->err), dfree(b->bar);
    if (b->host_flags) cudaFreeHost(b->host_flags);
    delete b;
    return FE_OK;
}

int fe_batch_set_tiles(fe_batch b, int32_t blocks_per_sm, int64_t slices_per_item) {
    if (!b || blocks_per_sm < 0 || blocks_per_sm > 32 || slices_per_item < 1 || slices_per_item > 64) {
        set_error("fe_batch_set_tiles: blocks per SM in 0..32 (0 = as many as fit) and 1..64 slices per item");
        return FE_BAD_INPUT;
    }
    b->blocks_per_sm = blocks_per_sm;
    b->slices_per_item = (int)slices_per_item;
    return FE_OK;
}

int fe_batch_set_preconditioner(fe_batch b, int32_t cheb_degree, double cheb_ratio) {
    if (!b || cheb_degree < 1 || cheb_degree > kMaxTerms || !(cheb_ratio > 1.0)) {
        set_error("fe_batch_set_preconditioner: degree 1..128 (1 = node-block Jacobi) and a ratio above 1");
        return FE_BAD_INPUT;
    }
    b->cheb_degree = cheb_degree;
    b->cheb_ratio = cheb_ratio;
    return FE_OK;
}

int fe_batch_solve(fe_batch b, double tol, int32_t max_iter, int32_t *iterations_host, int32_t *status_host,
                   double *relres_host, double *x_host, double *ms_out) {
    if (!b) {
        set_error("fe_batch_solve: null batch");
        return FE_BAD_INPUT;
    }
    fe_handle_s *h = b->h;
    if (!h->sys_ready) {
        set_error("fe_batch_solve: assemble the union handle first");
        return FE_NOT_READY;
    }
    if (h->singular) {
        set_error("fe_batch_solve: a node without stiffness makes an instance singular");
        return FE_BREAKDOWN;
    }
    const int chunk = 32;
    if (tol <= 0) tol = 1e-8;
    if (max_iter <= 0) max_iter = 200000;
    const int n = b->n_inst;
    FE_CUDA(cudaEventRecord(h->events[6], h->stream));
    const int terms = b->cheb_degree;
    if (terms > 1) {
        FE_CHECK(ensure_lmax(b));
        FE_CHECK(ensure_coefficients(b, terms));
    }
    FE_CHECK(reset_state(b));
    b->last_graph_launches = b->last_kernel_launches = 0;
    int launches = 0;
    FE_CHECK(run_pcg(b, terms, tol, max_iter, true, true, chunk, &launches));
    // instances whose FP64 true residual missed tol restart from it (the recurrence
    // residual drifts from b - A x by about eps cond(A)), at most four times
    std::vector<double> rr(n), bb(n);
    std::vector<int> stv(n), done(n);
    for (int round = 0;; ++round) {
        FE_CHECK(true_residuals(b));
        FE_CUDA(cudaMemcpyAsync(rr.data(), b->res.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaMemcpyAsync(bb.data(), b->dscal.p + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaMemcpyAsync(stv.data(), b->iscal.p + 2 * n, n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
        int again = 0;
        for (int i = 0; i < n; ++i) {
            done[i] = 1;
            if (stv[i] == FE_OK && rr[i] > tol * tol * bb[i]) done[i] = 0, ++again;
        }
        if (again == 0 || round >= 4) break;
        FE_CUDA(cudaMemcpyAsync(b->iscal.p, done.data(), n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
        FE_CUDA(cudaMemcpyAsync(b->iscal.p + 3 * n, &again, sizeof(int), cudaMemcpyHostToDevice, h->stream));
        FE_CHECK(run_pcg(b, terms, tol, max_iter, false, true, chunk, &launches));
    }
    FE_CUDA(cudaEventRecord(h->events[7], h->stream));
    FE_CUDA(cudaEventSynchronize(h->events[7]));
    float ms = 0;
    FE_CUDA(cudaEventElapsedTime(&ms, h->events[6], h->events[7]));
    if (ms_out) *ms_out = ms;
    if (relres_host)
        for (int i = 0; i < n; ++i) relres_host[i] = bb[i] > 0 ? sqrt(rr[i] / bb[i]) : 0.0;
    if (iterations_host)
        FE_CUDA(cudaMemcpyAsync(iterations_host, b->iscal.p + n, n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (status_host)
        FE_CUDA(cudaMemcpyAsync(status_host, b->iscal.p + 2 * n, n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (x_host) FE_CUDA(cudaMemcpyAsync(x_host, b->x.p, h->n_dof * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

int fe_batch_last_run(fe_batch b, int32_t *graph_launches, int32_t *kernel_launches, int32_t *uses_graph,
                      int32_t *grid) {
    if (!b) {
        set_error("fe_batch_last_run: null batch");
        return FE_BAD_INPUT;
    }
    if (graph_launches) *graph_launches = b->last_graph_launches;
    if (kernel_launches) *kernel_launches = b->last_kernel_launches;
    if (uses_graph) *uses_graph = b->graph_unsupported ? 0 : 1;
    if (grid) FE_CHECK(pcg_grid(b, grid));
    return FE_OK;
}

// Autotuner: time a chunk of batched iterations (from a fresh start, the current
// preconditioner) for each (blocks per SM, slices per work item) candidate on the live
// system and keep the fastest.
int fe_batch_autotune(fe_batch b, int32_t *blocks_per_sm_out, int64_t *slices_per_item_out,
                      double *us_per_iter_out) {
    if (!b) {
        set_error("fe_batch_autotune: null batch");
        return FE_BAD_INPUT;
    }
    fe_handle_s *h = b->h;
    if (!h->sys_ready) {
        set_error("fe_batch_autotune: assemble first");
        return FE_NOT_READY;
    }
    const int terms = b->cheb_degree;
    if (terms > 1) {
        FE_CHECK(ensure_lmax(b));
        FE_CHECK(ensure_coefficients(b, terms));
    }
    int per_sm = 0;
    {
        const void *k = h->sell_c16 ? pcg_kernel<true>() : pcg_kernel<false>();
        FE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBT, 0));
    }
    const int bps_c[3] = {1, 2, per_sm};
    const int spi_c[4] = {1, 2, 4, 8};
    const int iters = 8;
    double best = 1e300;
    int bb_best = 0, sb_best = 4;
    for (int bi = 0; bi < 3; ++bi) {
        if (bps_c[bi] > per_sm || (bi == 2 && per_sm <= 2)) continue;
        for (int si = 0; si < 4; ++si) {
            b->blocks_per_sm = bps_c[bi];
            b->slices_per_item = spi_c[si];
            FE_CHECK(reset_state(b));
            int grid = 0;
            FE_CHECK(pcg_grid(b, &grid));
            BatchArgs a = batch_args(b);
            a.terms = terms, a.tol2 = 0.0, a.max_iter = 1 << 30;
            FE_CHECK(launch_pcg(b, a, grid, 1, 1, 0));   // the start alone
            FE_CUDA(cudaEventRecord(h->events[8], h->stream));
            FE_CHECK(launch_pcg(b, a, grid, 0, 0, iters));
            FE_CUDA(cudaEventRecord(h->events[9], h->stream));
            int active = 0;
            FE_CHECK(read_flags(b, &active));
            float ms = 0;
            FE_CUDA(cudaEventElapsedTime(&ms, h->events[8], h->events[9]));
            const double us = ms * 1e3 / iters;
            if (us < best) best = us, bb_best = bps_c[bi], sb_best = spi_c[si];
        }
    }
    b->blocks_per_sm = bb_best;
    b->slices_per_item = sb_best;
    if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
    if (blocks_per_sm_out) *blocks_per_sm_out = bb_best;
    if (slices_per_item_out) *slices_per_item_out = sb_best;
    if (us_per_iter_out) *us_per_iter_out = best;
    return FE_OK;
}

}  // extern "C"
