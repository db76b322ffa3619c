// Batched solve of many independent instances of uneven size in one set of launches.
//
// The instances are assembled together as one block-diagonal system: their meshes are
// concatenated into one handle (disjoint node ranges), so the element kernels, the
// pattern build, the reduction and the Dirichlet elimination of fe_assemble run once
// for all of them.  The batched PCG (FP64, node-block Jacobi) then runs each phase of
// an iteration for every instance in one launch:
// * kernels are persistent: a grid sized to the machine walks contiguous chunks of R
//   block rows (R and the lanes per row G chosen by fe_batch_autotune);
// * dot products are segmented by instance: per chunk, a shared-memory FP64 sum per
//   instance the chunk touches, then one global atomic per (chunk, instance);
// * alpha, beta and the convergence test are per instance; a chunk whose instances
//   have all converged is skipped;
// * chunks of iterations are captured once in a CUDA graph and replayed until every
//   instance is done (or hits the iteration cap).
#include <math.h>

#include <algorithm>
#include <vector>

#include "fe_internal.h"

namespace fe {
namespace {

constexpr int kBT = 256;
constexpr int kMaxLocal = 64;   // instances one chunk may touch through shared memory

struct BatchState {
    // per instance
    double *rz, *pq, *rr, *rz_new, *bb, *alpha, *beta;
    int *done, *iter, *status;
    int *active;   // number of instances not done (device counter)
};

__device__ __forceinline__ void seg_add(double *sh, int local, double v, double *global_acc, int inst) {
    if (local < kMaxLocal) atomicAdd(&sh[local], v);
    else atomicAdd(&global_acc[inst], v);
}

// Warp-aggregated segmented add; every lane of the warp calls it.  Lanes with
// on = false contribute nothing.  When every contributing lane belongs to the same
// instance (the usual case: a warp covers consecutive rows), the warp sums by
// shuffles and one lane adds; otherwise each contributing lane adds itself.
__device__ __forceinline__ void seg_add_warp(double *sh, int local, double v, double *global_acc, int inst,
                                             bool on) {
    const unsigned any = __ballot_sync(0xffffffffu, on);
    if (!any) return;
    const int leader = __ffs(any) - 1;
    const int l0 = __shfl_sync(0xffffffffu, local, leader);
    const bool same = __all_sync(0xffffffffu, !on || local == l0);
    if (same) {
        double t = on ? v : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if ((int)(threadIdx.x & 31) == leader) seg_add(sh, local, t, global_acc, inst);
    } else if (on) {
        seg_add(sh, local, v, global_acc, inst);
    }
}

// Row loop of one chunk: rows [c0, c1) processed in steps of kBT / G rows.
#define FE_CHUNK_LOOP(G)                                                                  \
    const int sub = threadIdx.x & ((G)-1);                                                \
    for (int64_t base = c0; base < c1; base += kBT / (G))

template <int G>
__device__ __forceinline__ double2 bsr_row(int64_t r, bool valid, const int32_t *__restrict__ ptr,
                                           const int32_t *__restrict__ col, const double *__restrict__ val,
                                           const double *__restrict__ x, int sub) {
    double a0 = 0.0, a1 = 0.0;
    const int k0 = valid ? ptr[r] : 0, k1 = valid ? ptr[r + 1] : 0;
    for (int k = k0 + sub; k < k1; k += G) {
        const int c = __ldg(col + k);
        const double2 xv = reinterpret_cast<const double2 *>(x)[c];
        const double2 b0 = __ldg(reinterpret_cast<const double2 *>(val) + 2 * (int64_t)k);
        const double2 b1 = __ldg(reinterpret_cast<const double2 *>(val) + 2 * (int64_t)k + 1);
        // one FMA chain per output row: 4 FP64 FMAs per block (the FP64 pipe bounds this)
        a0 = fma(b0.x, xv.x, a0);
        a1 = fma(b1.x, xv.x, a1);
        a0 = fma(b0.y, xv.y, a0);
        a1 = fma(b1.y, xv.y, a1);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    }
    return make_double2(a0, a1);
}

// Chunk bookkeeping shared by the kernels: rows [c0, c1), first instance i0; the chunk
// is skipped when every instance it touches is done.
__device__ __forceinline__ bool chunk_active(int64_t c0, int64_t c1, const int32_t *__restrict__ inst,
                                             const int *__restrict__ done) {
    const int i0 = inst[c0], i1 = inst[c1 - 1];
    for (int i = i0; i <= i1; ++i)
        if (!done[i]) return true;
    return false;
}

// q = A p, pq_i += p.q   (phase 1)
template <int G>
__global__ void __launch_bounds__(kBT)
kb_spmv(int64_t n_nodes, int64_t R, const int32_t *__restrict__ inst, const int32_t *__restrict__ ptr,
        const int32_t *__restrict__ col, const double *__restrict__ val, const double *__restrict__ p,
        double *__restrict__ q, BatchState S) {
    __shared__ double sh[kMaxLocal];
    const int64_t n_chunks = (n_nodes + R - 1) / R;
    for (int64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
        const int64_t c0 = ch * R, c1 = min(n_nodes, c0 + R);
        if (!chunk_active(c0, c1, inst, S.done)) continue;
        const int i0 = inst[c0];
        for (int j = threadIdx.x; j < kMaxLocal; j += kBT) sh[j] = 0.0;
        __syncthreads();
        FE_CHUNK_LOOP(G) {
            const int64_t r = base + threadIdx.x / G;
            const bool in = r < c1;
            const int ir = in ? inst[r] : i0;
            const bool valid = in && !S.done[ir];
            double2 y = bsr_row<G>(r, valid, ptr, col, val, p, sub);
            const bool on = valid && sub == 0;
            double pq = 0.0;
            if (on) {
                reinterpret_cast<double2 *>(q)[r] = y;
                const double2 pv = reinterpret_cast<const double2 *>(p)[r];
                pq = pv.x * y.x + pv.y * y.y;
            }
            seg_add_warp(sh, ir - i0, pq, S.pq, ir, on);
        }
        __syncthreads();
        const int nl = min(inst[c1 - 1] - i0 + 1, kMaxLocal);
        for (int j = threadIdx.x; j < nl; j += kBT)
            if (sh[j] != 0.0) atomicAdd(&S.pq[i0 + j], sh[j]);
        __syncthreads();
    }
}

// per instance: alpha = rz / pq (phase 2)
__global__ void kb_alpha(int n, BatchState S) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (S.done[i]) continue;
        const double pq = S.pq[i];
        S.pq[i] = 0.0;
        S.rz_new[i] = 0.0;
        S.rr[i] = 0.0;
        if (!isfinite(pq)) {
            S.status[i] = FE_NONFINITE, S.done[i] = 1;
            atomicSub(S.active, 1);
        } else if (!(pq > 0.0)) {
            S.status[i] = FE_BREAKDOWN, S.done[i] = 1;
            atomicSub(S.active, 1);
        } else {
            S.alpha[i] = S.rz[i] / pq;
        }
    }
}

// x += alpha p, r -= alpha q, z = M^-1 r, rz_new_i, rr_i (phase 3)
__global__ void __launch_bounds__(kBT)
kb_update(int64_t n_nodes, int64_t R, const int32_t *__restrict__ inst, double *__restrict__ x,
          double *__restrict__ r_, const double *__restrict__ p, const double *__restrict__ q,
          const double *__restrict__ dinv, double *__restrict__ z, BatchState S) {
    __shared__ double sh[2][kMaxLocal];
    const int64_t n_chunks = (n_nodes + R - 1) / R;
    for (int64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
        const int64_t c0 = ch * R, c1 = min(n_nodes, c0 + R);
        if (!chunk_active(c0, c1, inst, S.done)) continue;
        const int i0 = inst[c0];
        for (int j = threadIdx.x; j < 2 * kMaxLocal; j += kBT) sh[j / kMaxLocal][j % kMaxLocal] = 0.0;
        __syncthreads();
        for (int64_t base = c0; base < c1; base += kBT) {
            const int64_t r = base + threadIdx.x;
            const int ir = r < c1 ? inst[r] : i0;
            const bool on = r < c1 && !S.done[ir];
            double rz = 0.0, rr = 0.0;
            if (on) {
                const double a = S.alpha[ir];
                double2 xv = reinterpret_cast<double2 *>(x)[r], rv = reinterpret_cast<double2 *>(r_)[r];
                const double2 pv = reinterpret_cast<const double2 *>(p)[r];
                const double2 qv = reinterpret_cast<const double2 *>(q)[r];
                xv.x += a * pv.x, xv.y += a * pv.y;
                rv.x -= a * qv.x, rv.y -= a * qv.y;
                reinterpret_cast<double2 *>(x)[r] = xv;
                reinterpret_cast<double2 *>(r_)[r] = rv;
                const double2 m0 = reinterpret_cast<const double2 *>(dinv)[2 * r];
                const double2 m1 = reinterpret_cast<const double2 *>(dinv)[2 * r + 1];
                const double2 zv = make_double2(m0.x * rv.x + m0.y * rv.y, m1.x * rv.x + m1.y * rv.y);
                reinterpret_cast<double2 *>(z)[r] = zv;
                rz = rv.x * zv.x + rv.y * zv.y;
                rr = rv.x * rv.x + rv.y * rv.y;
            }
            seg_add_warp(sh[0], ir - i0, rz, S.rz_new, ir, on);
            seg_add_warp(sh[1], ir - i0, rr, S.rr, ir, on);
        }
        __syncthreads();
        const int nl = min(inst[c1 - 1] - i0 + 1, kMaxLocal);
        for (int j = threadIdx.x; j < nl; j += kBT) {
            if (sh[0][j] != 0.0) atomicAdd(&S.rz_new[i0 + j], sh[0][j]);
            if (sh[1][j] != 0.0) atomicAdd(&S.rr[i0 + j], sh[1][j]);
        }
        __syncthreads();
    }
}

// per instance: convergence, beta (phase 4)
__global__ void kb_beta(int n, double tol2, int max_iter, BatchState S) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (S.done[i]) continue;
        S.iter[i] += 1;
        const double rzn = S.rz_new[i], rr = S.rr[i];
        int finished = 0;
        if (!isfinite(rzn) || !isfinite(rr)) S.status[i] = FE_NONFINITE, finished = 1;
        else if (rr <= tol2 * S.bb[i]) S.status[i] = FE_OK, finished = 1;
        else if (S.iter[i] >= max_iter) S.status[i] = FE_MAXITER, finished = 1;
        else if (!(rzn > 0.0)) S.status[i] = FE_BREAKDOWN, finished = 1;
        if (finished) {
            S.done[i] = 1;
            atomicSub(S.active, 1);
        } else {
            S.beta[i] = rzn / S.rz[i];
            S.rz[i] = rzn;
        }
    }
}

// p = z + beta p (phase 5)
__global__ void __launch_bounds__(kBT)
kb_direction(int64_t n_nodes, const int32_t *__restrict__ inst, const double *__restrict__ z, double *__restrict__ p,
             BatchState S) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_nodes;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int ir = inst[r];
        if (S.done[ir]) continue;
        const double b = S.beta[ir];
        const double2 zv = reinterpret_cast<const double2 *>(z)[r];
        double2 pv = reinterpret_cast<double2 *>(p)[r];
        pv.x = zv.x + b * pv.x, pv.y = zv.y + b * pv.y;
        reinterpret_cast<double2 *>(p)[r] = pv;
    }
}

// Start: x = g on constrained DOFs (0 elsewhere), r = b - A x, z = M^-1 r, p = z,
// per-instance rz, rr and bb (= b.b).  Not chunk-skipped.
template <int G>
__global__ void __launch_bounds__(kBT)
kb_start(int64_t n_nodes, int64_t R, const int32_t *__restrict__ inst, const int32_t *__restrict__ ptr,
         const int32_t *__restrict__ col, const double *__restrict__ val, const double *__restrict__ b,
         const double *__restrict__ x, double *__restrict__ r_, const double *__restrict__ dinv,
         double *__restrict__ z, double *__restrict__ p, BatchState S) {
    __shared__ double sh[3][kMaxLocal];
    const int64_t n_chunks = (n_nodes + R - 1) / R;
    for (int64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
        const int64_t c0 = ch * R, c1 = min(n_nodes, c0 + R);
        const int i0 = inst[c0];
        for (int j = threadIdx.x; j < 3 * kMaxLocal; j += kBT) sh[j / kMaxLocal][j % kMaxLocal] = 0.0;
        __syncthreads();
        FE_CHUNK_LOOP(G) {
            const int64_t r = base + threadIdx.x / G;
            const bool valid = r < c1;
            double2 ax = bsr_row<G>(r, valid, ptr, col, val, x, sub);
            const bool on = valid && sub == 0;
            const int ir = valid ? inst[r] : i0;
            double rz = 0.0, rr = 0.0, bbv = 0.0;
            if (on) {
                const double2 bv = reinterpret_cast<const double2 *>(b)[r];
                const double2 rv = make_double2(bv.x - ax.x, bv.y - ax.y);
                reinterpret_cast<double2 *>(r_)[r] = rv;
                const double2 m0 = reinterpret_cast<const double2 *>(dinv)[2 * r];
                const double2 m1 = reinterpret_cast<const double2 *>(dinv)[2 * r + 1];
                const double2 zv = make_double2(m0.x * rv.x + m0.y * rv.y, m1.x * rv.x + m1.y * rv.y);
                reinterpret_cast<double2 *>(z)[r] = zv;
                reinterpret_cast<double2 *>(p)[r] = zv;
                rz = rv.x * zv.x + rv.y * zv.y;
                rr = rv.x * rv.x + rv.y * rv.y;
                bbv = bv.x * bv.x + bv.y * bv.y;
            }
            seg_add_warp(sh[0], ir - i0, rz, S.rz, ir, on);
            seg_add_warp(sh[1], ir - i0, rr, S.rr, ir, on);
            seg_add_warp(sh[2], ir - i0, bbv, S.bb, ir, on);
        }
        __syncthreads();
        const int nl = min(inst[c1 - 1] - i0 + 1, kMaxLocal);
        for (int j = threadIdx.x; j < nl; j += kBT) {
            if (sh[0][j] != 0.0) atomicAdd(&S.rz[i0 + j], sh[0][j]);
            if (sh[1][j] != 0.0) atomicAdd(&S.rr[i0 + j], sh[1][j]);
            if (sh[2][j] != 0.0) atomicAdd(&S.bb[i0 + j], sh[2][j]);
        }
        __syncthreads();
    }
}

// after the start: instances already converged (or with b = 0) are done
__global__ void kb_start_check(int n, double tol2, BatchState S) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        S.iter[i] = 0;
        S.status[i] = FE_OK;
        S.done[i] = 0;
        S.pq[i] = 0.0;
        if (S.rr[i] <= tol2 * S.bb[i]) {
            S.done[i] = 1;
            atomicSub(S.active, 1);
        }
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

// per-instance true residual ||b - A x||^2 (FP64) for the final report.  The row loop
// runs the same number of trips in every lane (rows past the end contribute 0), so the
// warp shuffles always see all 32 lanes; one atomic per warp when its rows share an
// instance.
__global__ void __launch_bounds__(kBT)
kb_true_residual(int64_t n_nodes, const int32_t *__restrict__ inst, const int32_t *__restrict__ ptr,
                 const int32_t *__restrict__ col, const double *__restrict__ val, const double *__restrict__ b,
                 const double *__restrict__ x, double *__restrict__ acc) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t rows_padded = ((n_nodes + stride - 1) / stride) * stride;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows_padded; r += stride) {
        const bool in = r < n_nodes;
        double v = 0.0;
        int key = -1;
        if (in) {
            double a0 = 0, a1 = 0;
            for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
                const int c = col[k];
                const double x0 = x[2 * (int64_t)c], x1 = x[2 * (int64_t)c + 1];
                a0 = fma(val[4 * (int64_t)k], x0, a0);
                a1 = fma(val[4 * (int64_t)k + 2], x0, a1);
                a0 = fma(val[4 * (int64_t)k + 1], x1, a0);
                a1 = fma(val[4 * (int64_t)k + 3], x1, a1);
            }
            const double e0 = b[2 * r] - a0, e1 = b[2 * r + 1] - a1;
            v = e0 * e0 + e1 * e1;
            key = inst[r];
        }
        const int k0 = __shfl_sync(0xffffffffu, key, 0);
        if (__all_sync(0xffffffffu, !in || key == k0)) {
            double t = v;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if ((threadIdx.x & 31) == 0 && k0 >= 0) atomicAdd(&acc[k0], t);
        } else if (in) {
            atomicAdd(&acc[key], v);
        }
    }
}

}  // namespace
}  // namespace fe

struct fe_batch_s {
    fe_handle_s *h = nullptr;
    int n_inst = 0;
    fe::DBuf<int64_t> node_ptr;
    fe::DBuf<int32_t> inst;
    fe::DBuf<double> x, r, p, q, z, scal, res;
    fe::DBuf<int> iscal;
    int *active_host = nullptr;
    int lanes = 2;
    int64_t rows_per_chunk = 1024;
    cudaGraphExec_t graph = nullptr;
    int graph_key[3] = {0, 0, 0};
    double graph_tol = -1.0;      // tolerance and cap baked into the captured kernels
    int graph_max_iter = -1;
    std::vector<int64_t> node_ptr_host;
};

namespace fe {
namespace {

BatchState state(fe_batch_s *b) {
    const int n = b->n_inst;
    BatchState S;
    double *d = b->scal.p;
    S.rz = d, S.pq = d + n, S.rr = d + 2 * n, S.rz_new = d + 3 * n, S.bb = d + 4 * n, S.alpha = d + 5 * n,
    S.beta = d + 6 * n;
    int *k = b->iscal.p;
    S.done = k, S.iter = k + n, S.status = k + 2 * n, S.active = k + 3 * n;
    return S;
}

inline int chunk_grid(const fe_batch_s *b) {
    int64_t nc = (b->h->n_nodes + b->rows_per_chunk - 1) / b->rows_per_chunk;
    return (int)std::max<int64_t>(1, std::min<int64_t>(nc, 152 * 8));
}

template <int G>
void enqueue_iteration(fe_batch_s *b, double tol2, int max_iter) {
    fe_handle_s *h = b->h;
    BatchState S = state(b);
    const int gc = chunk_grid(b), gi = grid_for(b->n_inst), gn = grid_for(h->n_nodes, kBT, 152 * 8);
    kb_spmv<G><<<gc, kBT, 0, h->stream>>>(h->n_nodes, b->rows_per_chunk, b->inst.p, h->blk_ptr.p, h->blk_col.p,
                                          h->aval.p, b->p.p, b->q.p, S);
    kb_alpha<<<gi, kThreads, 0, h->stream>>>(b->n_inst, S);
    kb_update<<<gc, kBT, 0, h->stream>>>(h->n_nodes, b->rows_per_chunk, b->inst.p, b->x.p, b->r.p, b->p.p, b->q.p,
                                         h->dinv.p, b->z.p, S);
    kb_beta<<<gi, kThreads, 0, h->stream>>>(b->n_inst, tol2, max_iter, S);
    kb_direction<<<gn, kBT, 0, h->stream>>>(h->n_nodes, b->inst.p, b->z.p, b->p.p, S);
}

template <int G>
int run(fe_batch_s *b, double tol, int max_iter, int chunk, int *graph_launches) {
    fe_handle_s *h = b->h;
    const int n = b->n_inst;
    const int64_t nd = h->n_dof;
    BatchState S = state(b);
    const double tol2 = tol * tol;
    cudaStream_t s = h->stream;
    FE_CUDA(cudaMemsetAsync(b->scal.p, 0, 7 * n * sizeof(double), s));
    FE_CUDA(cudaMemsetAsync(b->iscal.p, 0, (3 * n + 1) * sizeof(int), s));
    FE_CUDA(cudaMemcpyAsync(S.active, &b->n_inst, sizeof(int), cudaMemcpyHostToDevice, s));
    FE_CUDA(cudaMemsetAsync(b->x.p, 0, nd * sizeof(double), s));
    if (h->n_bc > 0)
        kb_set_prescribed<<<grid_for(h->n_bc), kThreads, 0, s>>>(h->n_bc, h->bc_dof.p, h->bc_val.p, b->x.p);
    kb_start<G><<<chunk_grid(b), kBT, 0, s>>>(h->n_nodes, b->rows_per_chunk, b->inst.p, h->blk_ptr.p, h->blk_col.p,
                                              h->aval.p, h->b.p, b->x.p, b->r.p, h->dinv.p, b->z.p, b->p.p, S);
    kb_start_check<<<grid_for(n), kThreads, 0, s>>>(n, tol2, S);
    FE_LAUNCH_CHECK();
    h->launches += 2 + (h->n_bc > 0 ? 1 : 0);
    const int key[3] = {G, (int)b->rows_per_chunk, chunk};
    if (!b->graph || key[0] != b->graph_key[0] || key[1] != b->graph_key[1] || key[2] != b->graph_key[2]) {
        if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
        cudaGraph_t g;
        FE_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < chunk; ++i) enqueue_iteration<G>(b, tol2, max_iter);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (ce != cudaSuccess) {
            set_error(std::string("batch graph capture: ") + cudaGetErrorString(ce));
            return FE_CUDA_ERR;
        }
        ce = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            b->graph = nullptr;
            set_error(std::string("batch graph instantiate: ") + cudaGetErrorString(ce));
            return FE_CUDA_ERR;
        }
        for (int i = 0; i < 3; ++i) b->graph_key[i] = key[i];
    }
    // the tolerance and cap are baked into the captured kernels' arguments: recapture
    // when they change
    *graph_launches = 0;
    for (;;) {
        FE_CUDA(cudaMemcpyAsync(b->active_host, S.active, sizeof(int), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        if (*b->active_host <= 0) break;
        FE_CUDA(cudaGraphLaunch(b->graph, s));
        h->launches += 5LL * chunk;
        ++*graph_launches;
    }
    return FE_OK;
}

template <typename F>
int dispatch(int lanes, F &&f) {
    switch (lanes) {
        case 1: return f(std::integral_constant<int, 1>{});
        case 4: return f(std::integral_constant<int, 4>{});
        default: return f(std::integral_constant<int, 2>{});
    }
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
    const size_t nd = (size_t)std::max<int64_t>(h->n_dof, 1);
    int st = dalloc(b->node_ptr, (size_t)n_instances + 1);
    if (!st) st = dalloc(b->inst, (size_t)std::max<int64_t>(h->n_nodes, 1));
    if (!st) st = dalloc(b->x, nd);
    if (!st) st = dalloc(b->r, nd);
    if (!st) st = dalloc(b->p, nd);
    if (!st) st = dalloc(b->q, nd);
    if (!st) st = dalloc(b->z, nd);
    if (!st) st = dalloc(b->scal, (size_t)7 * n_instances);
    if (!st) st = dalloc(b->res, (size_t)n_instances);
    if (!st) st = dalloc(b->iscal, (size_t)3 * n_instances + 1);
    if (!st && cudaMallocHost((void **)&b->active_host, sizeof(int)) != cudaSuccess) st = FE_CUDA_ERR;
    if (st) {
        fe_batch_destroy(b);
        return st;
    }
    if (cudaMemcpy(b->node_ptr.p, node_ptr_host, (n_instances + 1) * sizeof(int64_t), cudaMemcpyHostToDevice) !=
        cudaSuccess) {
        fe_batch_destroy(b);
        set_error("fe_batch_create: copy failed");
        return FE_CUDA_ERR;
    }
    kb_inst_of_node<<<std::min(n_instances, 152 * 8), 256, 0, h->stream>>>(n_instances, b->node_ptr.p, b->inst.p);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(h->stream) != cudaSuccess) {
        fe_batch_destroy(b);
        set_error("fe_batch_create: instance map kernel failed");
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
    dfree(b->node_ptr), dfree(b->inst), dfree(b->x), dfree(b->r), dfree(b->p), dfree(b->q), dfree(b->z);
    dfree(b->scal), dfree(b->res), dfree(b->iscal);
    if (b->active_host) cudaFreeHost(b->active_host);
    delete b;
    return FE_OK;
}

int fe_batch_set_tiles(fe_batch b, int32_t lanes, int64_t rows_per_chunk) {
    if (!b || (lanes != 1 && lanes != 2 && lanes != 4) || rows_per_chunk < 32) {
        set_error("fe_batch_set_tiles: lanes 1, 2 or 4 and at least 32 rows per chunk");
        return FE_BAD_INPUT;
    }
    b->lanes = lanes;
    b->rows_per_chunk = rows_per_chunk;
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
    // tol and max_iter are kernel arguments inside the captured graph
    if (tol != b->graph_tol || max_iter != b->graph_max_iter) {
        if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
        b->graph_tol = tol, b->graph_max_iter = max_iter;
    }
    FE_CUDA(cudaEventRecord(h->events[6], h->stream));
    int launches = 0;
    FE_CHECK(dispatch(b->lanes, [&](auto g) { return run<decltype(g)::value>(b, tol, max_iter, chunk, &launches); }));
    FE_CUDA(cudaEventRecord(h->events[7], h->stream));
    FE_CUDA(cudaEventSynchronize(h->events[7]));
    float ms = 0;
    FE_CUDA(cudaEventElapsedTime(&ms, h->events[6], h->events[7]));
    if (ms_out) *ms_out = ms;
    const int n = b->n_inst;
    BatchState S = state(b);
    if (relres_host) {
        FE_CUDA(cudaMemsetAsync(b->res.p, 0, n * sizeof(double), h->stream));
        kb_true_residual<<<grid_for(h->n_nodes, kBT, 152 * 8), kBT, 0, h->stream>>>(
            h->n_nodes, b->inst.p, h->blk_ptr.p, h->blk_col.p, h->aval.p, h->b.p, b->x.p, b->res.p);
        FE_LAUNCH_CHECK();
        h->launches += 1;
        std::vector<double> rr(n), bb(n);
        FE_CUDA(cudaMemcpyAsync(rr.data(), b->res.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaMemcpyAsync(bb.data(), S.bb, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
        for (int i = 0; i < n; ++i) relres_host[i] = bb[i] > 0 ? sqrt(rr[i] / bb[i]) : 0.0;
    }
    if (iterations_host)
        FE_CUDA(cudaMemcpyAsync(iterations_host, S.iter, n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (status_host)
        FE_CUDA(cudaMemcpyAsync(status_host, S.status, n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (x_host) FE_CUDA(cudaMemcpyAsync(x_host, b->x.p, h->n_dof * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

// Autotuner: time a few batched iterations for every (lanes, rows per chunk) pair on
// the batch's own matrix and keep the fastest.
int fe_batch_autotune(fe_batch b, int32_t *lanes_out, int64_t *rows_out, double *us_per_iter_out) {
    if (!b) {
        set_error("fe_batch_autotune: null batch");
        return FE_BAD_INPUT;
    }
    fe_handle_s *h = b->h;
    if (!h->sys_ready) {
        set_error("fe_batch_autotune: assemble first");
        return FE_NOT_READY;
    }
    const int lanes_c[3] = {1, 2, 4};
    const int64_t rows_c[4] = {256, 1024, 4096, 16384};
    double best = 1e300;
    int bl = 2;
    int64_t br = 1024;
    const int iters = 20;
    for (int li = 0; li < 3; ++li)
        for (int ri = 0; ri < 4; ++ri) {
            b->lanes = lanes_c[li];
            b->rows_per_chunk = rows_c[ri];
            BatchState S = state(b);
            // a fresh start so every instance is active, then timed iterations
            int rc = dispatch(b->lanes, [&](auto g) {
                constexpr int G = decltype(g)::value;
                cudaStream_t s = h->stream;
                FE_CUDA(cudaMemsetAsync(b->scal.p, 0, 7 * b->n_inst * sizeof(double), s));
                FE_CUDA(cudaMemsetAsync(b->iscal.p, 0, (3 * b->n_inst + 1) * sizeof(int), s));
                FE_CUDA(cudaMemsetAsync(b->x.p, 0, h->n_dof * sizeof(double), s));
                kb_start<G><<<chunk_grid(b), kBT, 0, s>>>(h->n_nodes, b->rows_per_chunk, b->inst.p, h->blk_ptr.p,
                                                          h->blk_col.p, h->aval.p, h->b.p, b->x.p, b->r.p, h->dinv.p,
                                                          b->z.p, b->p.p, S);
                FE_CUDA(cudaEventRecord(h->events[8], s));
                for (int k = 0; k < iters; ++k) enqueue_iteration<G>(b, 0.0, 1 << 30);
                FE_CUDA(cudaEventRecord(h->events[9], s));
                FE_LAUNCH_CHECK();
                FE_CUDA(cudaEventSynchronize(h->events[9]));
                h->launches += 1 + 5LL * iters;
                return FE_OK;
            });
            FE_CHECK(rc);
            float ms = 0;
            FE_CUDA(cudaEventElapsedTime(&ms, h->events[8], h->events[9]));
            double us = ms * 1e3 / iters;
            if (us < best) best = us, bl = lanes_c[li], br = rows_c[ri];
        }
    b->lanes = bl;
    b->rows_per_chunk = br;
    if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
    if (lanes_out) *lanes_out = bl;
    if (rows_out) *rows_out = br;
    if (us_per_iter_out) *us_per_iter_out = best;
    return FE_OK;
}

}  // extern "C"
