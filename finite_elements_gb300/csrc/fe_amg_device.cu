// Multigrid-preconditioned PCG on the device: the smoothed-aggregation hierarchy of
// the eliminated system (set up on the device, fe_amg_device_setup.cu) and a V-cycle
// whose kernels are loops of the row operations of fe_amg_rows.cuh -- the operations
// the host cycle fe_amg_vcycle_host runs serially.  The PCG recurrence, its SpMV and
// the true residual are FP64; the V-cycle runs in FP32 on FP32 copies of the levels
// (a CPU emulation of the cycle in FP32 gave the FP64 cycle's PCG iteration counts).
//
// WORK IN PROGRESS: not yet run on a GPU.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "fe_amg_dev.h"
#include "fe_amg_cycle.cuh"
#include "fe_amg_rows.cuh"
#include "fe_internal.h"

namespace fe {
namespace {

constexpr int kAT = 256;
inline int grid_a(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kAT - 1) / kAT, 152 * 8)); }

// the executor of the shared FP32 cycle (fe_amg_cycle.cuh): one grid-stride kernel per pass
template <typename F>
__global__ void ka_rows(int64_t n, F f) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        f(i);
}

// t = r - A x in FP64 (the true residual of the PCG)
struct PassResidual64 {
    const int64_t *ptr; const int32_t *col; const double *val; int d; const double *r; const double *x; double *t;
    FE_HD void operator()(int64_t i) const { amg::row_residual(ptr, col, val, d, r, x, t, i); }
};

struct CycleEx {
    fe_handle_s *h;
    template <class F>
    int rows(int64_t n, const F &f) {
        if (n <= 0) return FE_OK;
        ka_rows<F><<<grid_a(n), kAT, 0, h->stream>>>(n, f);
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return FE_OK;
    }
    template <class T>
    int copy(T *dst, const T *src, size_t n) {
        if (n) FE_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, h->stream));
        return FE_OK;
    }
    template <class T>
    int fill_zero(T *p, size_t n) {
        if (n) FE_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), h->stream));
        return FE_OK;
    }
};

// q = A p with the level-0 matrix (block rows of size d)
__global__ void ka_spmv(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                        const double *__restrict__ val, int d, const double *__restrict__ p, double *__restrict__ q) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double out[6];
        amg::row_product(ptr, col, val, d, d, p, i, out);
        for (int k = 0; k < d; ++k) q[i * d + k] = out[k];
    }
}

// deterministic dot products: per-block partials, then one block in block order
__device__ __forceinline__ double block_sum_a(double v) {
    __shared__ double sh[kAT / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < kAT / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;
}

__global__ void ka_dot(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *part) {
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i], b[i], s);
    s = block_sum_a(s);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void ka_dot_final(int nb, const double *__restrict__ part, double *out) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[i];
    s = block_sum_a(s);
    if (threadIdx.x == 0) *out = s;
}

// x += alpha p, r -= alpha q
__global__ void ka_update(int64_t n, double alpha, const double *__restrict__ p, const double *__restrict__ q,
                          double *__restrict__ x, double *__restrict__ r) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fma(alpha, p[i], x[i]);
        r[i] = fma(-alpha, q[i], r[i]);
    }
}

// p = z + beta p
__global__ void ka_direction(int64_t n, double beta, const double *__restrict__ z, double *__restrict__ p) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fma(beta, p[i], z[i]);
}

// FP32 copies of a level's values and its cycle vectors
int prepare_cycle(fe_handle_s *h, DevLevel &L) {
    const int d = L.A.rd, m = L.P.cd;
    const int64_t na = L.A.nnzb * d * d, np = L.P.nnzb * d * m, nt = L.PT.nnzb * m * d, ndi = L.A.n * d * d;
    FE_CHECK(dalloc(L.a32, (size_t)std::max<int64_t>(na, 1)));
    FE_CHECK(dalloc(L.p32, (size_t)std::max<int64_t>(np, 1)));
    FE_CHECK(dalloc(L.pt32, (size_t)std::max<int64_t>(nt, 1)));
    FE_CHECK(dalloc(L.dinv32, (size_t)std::max<int64_t>(ndi, 1)));
    CycleEx ex{h};
    FE_CHECK(ex.rows(na, amg::PassToF32{L.A.val.p, L.a32.p}));
    FE_CHECK(ex.rows(np, amg::PassToF32{L.P.val.p, L.p32.p}));
    FE_CHECK(ex.rows(nt, amg::PassToF32{L.PT.val.p, L.pt32.p}));
    FE_CHECK(ex.rows(ndi, amg::PassToF32{L.dinv.p, L.dinv32.p}));
    const size_t v = (size_t)std::max<int64_t>(L.A.n * d, 1);
    FE_CHECK(dalloc(L.r, v));
    FE_CHECK(dalloc(L.x, v));
    FE_CHECK(dalloc(L.t, v));
    FE_CHECK(dalloc(L.dir, v));
    FE_CHECK(dalloc(L.zn, v));
    return FE_OK;
}

}  // namespace

// PCG on the eliminated system preconditioned by one FP32 V-cycle (k = 3 Chebyshev steps
// per smoothing), FP64 recurrence, from x = 0 (opts.x0 is not used); the hierarchy is
// set up on the device from the system matrix and the rigid-body (elasticity) or
// constant (magnetostatics) modes, with the rows of the constrained DOFs zeroed.
int solve_multigrid(fe_handle_s *h, const fe_solve_opts *o, fe_solve_stats *st) {
    cudaStream_t s = h->stream;
    const int D = h->dim;
    const int64_t n = h->n_nodes, nd = h->n_dof;
    FE_CUDA(cudaEventRecord(h->events[6], s));
    // the hierarchy, set up on the device, and the cycle's vectors
    DevAmg G;
    FE_CHECK(amg_setup_device(h, 0.08, 400, G));
    for (auto &L : G.L) FE_CHECK(prepare_cycle(h, L));
    FE_CHECK(dalloc(G.rc, (size_t)std::max<int64_t>(G.nc, 1)));
    FE_CHECK(dalloc(G.xc, (size_t)std::max<int64_t>(G.nc, 1)));
    if (G.L.empty()) {
        set_error("fe_solve: the multigrid hierarchy has a single level (use the other preconditioners)");
        return FE_BAD_INPUT;
    }
    // PCG: level 0's r and x hold the V-cycle's input and output
    DevLevel &L0 = G.L[0];
    DBuf<double> r, p, q, z, part, sc;
    struct Free {
        DBuf<double> *b[6];
        ~Free() {
            for (auto *x : b) dfree(*x);
        }
    } fg{{&r, &p, &q, &z, &part, &sc}};
    const int gn = grid_a(nd);
    FE_CHECK(dalloc(h->w.x, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(dalloc(r, (size_t)nd));
    FE_CHECK(dalloc(p, (size_t)nd));
    FE_CHECK(dalloc(q, (size_t)nd));
    FE_CHECK(dalloc(z, (size_t)nd));
    FE_CHECK(dalloc(part, (size_t)gn));
    FE_CHECK(dalloc(sc, 4));
    double *x = h->w.x.p;
    auto dot = [&](const double *a, const double *b, double *out) -> int {
        ka_dot<<<gn, kAT, 0, s>>>(nd, a, b, part.p);
        ka_dot_final<<<1, kAT, 0, s>>>(gn, part.p, out);
        FE_LAUNCH_CHECK();
        h->launches += 2;
        return FE_OK;
    };
    // the levels as the shared cycle sees them
    std::vector<amg::CycleLevel> views(G.L.size());
    for (size_t l = 0; l < G.L.size(); ++l) {
        const DevLevel &D = G.L[l];
        amg::CycleLevel &V = views[l];
        V.n = D.A.n, V.d = D.A.rd, V.m = D.P.cd, V.lmax = D.lmax, V.nc = D.PT.n;
        V.aptr = D.A.ptr.p, V.acol = D.A.col.p, V.a = D.a32.p, V.dinv = D.dinv32.p;
        V.pptr = D.P.ptr.p, V.pcol = D.P.col.p, V.p = D.p32.p;
        V.tptr = D.PT.ptr.p, V.tcol = D.PT.col.p, V.pt = D.pt32.p;
        V.r = D.r.p, V.x = D.x.p, V.t = D.t.p, V.dir = D.dir.p, V.zn = D.zn.p;
    }
    amg::CycleCoarse coarse;
    coarse.n = G.nc, coarse.inv = G.cinv.p, coarse.r = G.rc.p, coarse.x = G.xc.p;
    CycleEx cex{h};
    auto enqueue_cycle = [&]() -> int {   // z = M^-1 r: the FP32 V-cycle on r rounded to FP32
        return amg::precondition(cex, views, coarse, 3, r.p, z.p);
    };
    // the cycle's fixed sequence of launches (about ten per level) captured once as a
    // CUDA graph, launched once per PCG iteration
    cudaGraphExec_t cycle = nullptr;
    struct GraphFree {
        cudaGraphExec_t *g;
        ~GraphFree() {
            if (*g) cudaGraphExecDestroy(*g);
        }
    } gf{&cycle};
    int64_t per_cycle = 0;
    {
        const int64_t l0 = h->launches;
        cudaGraph_t g = nullptr;
        FE_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_cycle();
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (rc != FE_OK) {
            if (ce == cudaSuccess && g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) {
            set_error(std::string("multigrid cycle capture: ") + cudaGetErrorString(ce));
            return FE_CUDA_ERR;
        }
        ce = cudaGraphInstantiate(&cycle, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            cycle = nullptr;
            set_error(std::string("multigrid cycle instantiate: ") + cudaGetErrorString(ce));
            return FE_CUDA_ERR;
        }
        per_cycle = h->launches - l0;
        h->launches = l0;
    }
    auto precond = [&]() -> int {
        FE_CUDA(cudaGraphLaunch(cycle, s));
        h->launches += per_cycle;
        return FE_OK;
    };
    FE_CUDA(cudaMemsetAsync(x, 0, nd * sizeof(double), s));
    FE_CUDA(cudaMemcpyAsync(r.p, h->b.p, nd * sizeof(double), cudaMemcpyDeviceToDevice, s));
    FE_CHECK(precond());
    FE_CUDA(cudaMemcpyAsync(p.p, z.p, nd * sizeof(double), cudaMemcpyDeviceToDevice, s));
    FE_CHECK(dot(r.p, z.p, sc.p));
    FE_CHECK(dot(r.p, r.p, sc.p + 1));
    double host[4];
    FE_CUDA(cudaMemcpyAsync(host, sc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    double rz = host[0];
    const double bb = host[1];
    const double tol = o->tol > 0 ? o->tol : 1e-10;
    const int max_iter = o->max_iter > 0 ? o->max_iter : 10000;
    int it = 0, status = bb > 0.0 ? FE_MAXITER : FE_OK;
    double rr = bb;
    while (status == FE_MAXITER && it < max_iter) {
        ka_spmv<<<grid_a(n), kAT, 0, s>>>(n, L0.A.ptr.p, L0.A.col.p, L0.A.val.p, D, p.p, q.p);
        FE_LAUNCH_CHECK();
        FE_CHECK(dot(p.p, q.p, sc.p + 2));
        FE_CUDA(cudaMemcpyAsync(host + 2, sc.p + 2, sizeof(double), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        if (!(host[2] > 0.0) || !std::isfinite(host[2])) {
            status = std::isfinite(host[2]) ? FE_BREAKDOWN : FE_NONFINITE;
            break;
        }
        const double alpha = rz / host[2];
        ka_update<<<gn, kAT, 0, s>>>(nd, alpha, p.p, q.p, x, r.p);
        FE_LAUNCH_CHECK();
        h->launches += 2;
        ++it;
        FE_CHECK(dot(r.p, r.p, sc.p + 1));
        FE_CHECK(precond());
        FE_CHECK(dot(r.p, z.p, sc.p));
        FE_CUDA(cudaMemcpyAsync(host, sc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        rr = host[1];
        if (!std::isfinite(rr) || !std::isfinite(host[0])) {
            status = FE_NONFINITE;
            break;
        }
        if (rr <= tol * tol * bb) {
            status = FE_OK;
            break;
        }
        const double beta = host[0] / rz;
        rz = host[0];
        ka_direction<<<gn, kAT, 0, s>>>(nd, beta, z.p, p.p);
        FE_LAUNCH_CHECK();
        h->launches += 1;
    }
    // true residual b - A x in FP64
    FE_CHECK(cex.rows(n, PassResidual64{L0.A.ptr.p, L0.A.col.p, L0.A.val.p, D, h->b.p, x, q.p}));
    FE_CHECK(dot(q.p, q.p, sc.p + 3));
    FE_CUDA(cudaMemcpyAsync(host + 3, sc.p + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    rr = host[3];
    st->iterations = it;
    st->spmv = it + 1;
    st->outer = 0;
    st->fp64_iterations = 0;
    st->x0_used = 0;
    st->bnorm = std::sqrt(bb);
    st->relres = bb > 0.0 ? std::sqrt(std::max(rr, 0.0) / bb) : 0.0;
    st->status = status;
    FE_CHECK(recover_multipliers(h));
    FE_CUDA(cudaEventRecord(h->events[7], s));
    FE_CUDA(cudaEventSynchronize(h->events[7]));
    float ms = 0;
    FE_CUDA(cudaEventElapsedTime(&ms, h->events[6], h->events[7]));
    st->solve_ms = ms;
    st->assemble_ms = h->last_assemble_ms;
    h->have_solution = true;
    return FE_OK;
}

}  // namespace fe
