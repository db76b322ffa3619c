// Multigrid-preconditioned PCG on the device: the smoothed-aggregation hierarchy of
// the eliminated system (set up on the device, fe_amg_device_setup.cu) and a V-cycle
// and the PCG around its FP32 V-cycle, both written once over an executor
// (fe_amg_cycle.cuh; fe_amg_pcg_host runs the same sequence on the host).  The PCG
// recurrence, its SpMV and the true residual are FP64; the V-cycle runs in FP32 on FP32
// copies of the levels and is captured once per solve as a CUDA graph.
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

struct CycleEx {
    fe_handle_s *h;
    DBuf<double> part, sc;
    ~CycleEx() { dfree(part), dfree(sc); }
    int dot(const double *a, const double *b, int64_t n, double *out) {
        const int g = grid_a(n);
        FE_CHECK(dalloc(part, (size_t)g));
        FE_CHECK(dalloc(sc, 1));
        ka_dot<<<g, kAT, 0, h->stream>>>(n, a, b, part.p);
        ka_dot_final<<<1, kAT, 0, h->stream>>>(g, part.p, sc.p);
        FE_LAUNCH_CHECK();
        h->launches += 2;
        FE_CUDA(cudaMemcpyAsync(out, sc.p, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
        return FE_OK;
    }
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
    // PCG vectors; the solution goes to the handle's x
    DevLevel &L0 = G.L[0];
    DBuf<double> r, p, q, z;
    struct Free {
        DBuf<double> *b[4];
        ~Free() {
            for (auto *x : b) dfree(*x);
        }
    } fg{{&r, &p, &q, &z}};
    FE_CHECK(dalloc(h->w.x, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(dalloc(r, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(dalloc(p, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(dalloc(q, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(dalloc(z, (size_t)std::max<int64_t>(nd, 1)));
    // the levels as the shared cycle sees them
    std::vector<amg::CycleLevel> views(G.L.size());
    for (size_t l = 0; l < G.L.size(); ++l) {
        const DevLevel &Dl = G.L[l];
        amg::CycleLevel &V = views[l];
        V.n = Dl.A.n, V.d = Dl.A.rd, V.m = Dl.P.cd, V.lmax = Dl.lmax, V.nc = Dl.PT.n;
        V.aptr = Dl.A.ptr.p, V.acol = Dl.A.col.p, V.a = Dl.a32.p, V.dinv = Dl.dinv32.p;
        V.pptr = Dl.P.ptr.p, V.pcol = Dl.P.col.p, V.p = Dl.p32.p;
        V.tptr = Dl.PT.ptr.p, V.tcol = Dl.PT.col.p, V.pt = Dl.pt32.p;
        V.r = Dl.r.p, V.x = Dl.x.p, V.t = Dl.t.p, V.dir = Dl.dir.p, V.zn = Dl.zn.p;
    }
    amg::CycleCoarse coarse;
    coarse.n = G.nc, coarse.inv = G.cinv.p, coarse.r = G.rc.p, coarse.x = G.xc.p;
    CycleEx cex{h};
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
        const int rc = amg::precondition(cex, views, coarse, 3, r.p, z.p);
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
    const double tol = o->tol > 0 ? o->tol : 1e-10;
    const int max_iter = o->max_iter > 0 ? o->max_iter : 10000;
    int it = 0, status = FE_OK;
    double relres = 0.0;
    const amg::PcgVectors v{h->w.x.p, r.p, p.p, q.p, z.p};
    FE_CHECK(amg::pcg(cex, n, D, L0.A.ptr.p, L0.A.col.p, L0.A.val.p, h->b.p, v, precond, tol, max_iter, &it,
                      &relres, &status));
    double bb = 0.0;
    FE_CHECK(cex.dot(h->b.p, h->b.p, nd, &bb));
    st->iterations = it;
    st->spmv = it + 1;
    st->outer = 0;
    st->fp64_iterations = 0;
    st->x0_used = 0;
    st->bnorm = std::sqrt(bb);
    st->relres = relres;
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
