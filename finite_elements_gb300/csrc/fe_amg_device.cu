// Multigrid-preconditioned PCG on the device: the smoothed-aggregation hierarchy of
// the eliminated system (set up on the device, fe_amg_device_setup.cu) and a V-cycle
// and the PCG around its FP32 V-cycle, both written once over an executor
// (fe_amg_cycle.cuh; fe_amg_pcg_host runs the same sequence on the host).  The PCG
// recurrence, its SpMV and the true residual are FP64; the V-cycle runs in FP32 on FP32
// copies of the levels and is captured once per solve as a CUDA graph.
#include <algorithm>
#include <cmath>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "fe_amg_dev.h"
#include "fe_amg_cycle.cuh"
#include "fe_amg_rows.cuh"
#include "fe_internal.h"

namespace fe {
static_assert(amg::kSetupPhases == FE_MG_PHASES, "setup phases of fe_profile_read_multigrid_phases");
static_assert(amg::kSetupPhases <= 16, "SolverWork::mg_phase_ms");
namespace {

constexpr int kAT = 256;
// Chebyshev smoothing steps per smoothing: on level 0 and on the coarser levels
constexpr int kSmooth0 = 3, kSmoothCoarse = 2;
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

// ---------------------------------------------------------------- cycle passes, G lanes per row
// The V-cycle's block-row passes with G lanes of a warp sharing a block row (a strided
// share of its blocks each, then a shuffle sum): coalesced block loads where one thread
// per row reads its row's blocks alone.  RD x CD are the block sizes, G is chosen per
// matrix from its mean row length.

#define FE_LANE_ROWS(G, n)                                                                 \
    const int sub = threadIdx.x & ((G)-1);                                                 \
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / (G);                        \
    const int64_t rows_padded = (((n) + groups - 1) / groups) * groups;                    \
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / (G); i < rows_padded; i += groups)

// acc = (B x)_i over the blocks of row i, summed over the G lanes (every lane of the warp
// calls this; lanes of rows past the end pass valid = false)
template <int RD, int CD, int G>
__device__ __forceinline__ void lanes_product(const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                              const float *__restrict__ val, const float *__restrict__ x, int64_t i,
                                              bool valid, int sub, float (&acc)[RD]) {
#pragma unroll
    for (int a = 0; a < RD; ++a) acc[a] = 0.0f;
    if (valid) {
        const int64_t s1 = ptr[i + 1];
        for (int64_t s = ptr[i] + sub; s < s1; s += G) {
            const float *b = val + s * RD * CD;
            const float *xc = x + (int64_t)__ldg(col + s) * CD;
            float xv[CD];
#pragma unroll
            for (int k = 0; k < CD; ++k) xv[k] = xc[k];
#pragma unroll
            for (int a = 0; a < RD; ++a)
#pragma unroll
                for (int k = 0; k < CD; ++k) acc[a] = fmaf(__ldg(b + a * CD + k), xv[k], acc[a]);
        }
    }
    if constexpr (G > 1) {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int a = 0; a < RD; ++a) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], o);
    }
}

template <int D, int G>
__global__ void __launch_bounds__(kAT) ka_cheb(int64_t n, amg::PassCheb f) {
    FE_LANE_ROWS(G, n) {
        const bool valid = i < n;
        float az[D];
        // the first step from zero: A z_in = 0 without reading the matrix
        lanes_product<D, D, G>(f.ptr, f.col, f.val, f.zin, i, valid && !f.zero, sub, az);
        if (valid && sub == 0) {
            float t[D];
#pragma unroll
            for (int k = 0; k < D; ++k) t[k] = f.r[i * D + k] - az[k];
#pragma unroll
            for (int p = 0; p < D; ++p) {
                float res = 0.0f;
#pragma unroll
                for (int k = 0; k < D; ++k) res += f.dinv[i * D * D + p * D + k] * t[k];
                const float dn = f.first ? f.b * res : f.a * f.dir[i * D + p] + f.b * res;
                f.dir[i * D + p] = dn;
                f.zout[i * D + p] = f.zin[i * D + p] + dn;
            }
        }
    }
}

template <int D, int G>
__global__ void __launch_bounds__(kAT) ka_residual(int64_t n, amg::PassResidual32 f) {
    FE_LANE_ROWS(G, n) {
        const bool valid = i < n;
        float ax[D];
        lanes_product<D, D, G>(f.ptr, f.col, f.val, f.x, i, valid, sub, ax);
        if (valid && sub == 0)
#pragma unroll
            for (int k = 0; k < D; ++k) f.t[i * D + k] = f.r[i * D + k] - ax[k];
    }
}

// rows of P^T (aggregates): M x D blocks
template <int M, int D, int G>
__global__ void __launch_bounds__(kAT) ka_restrict(int64_t n, amg::PassRestrict32 f) {
    FE_LANE_ROWS(G, n) {
        const bool valid = i < n;
        float o[M];
        lanes_product<M, D, G>(f.ptr, f.col, f.val, f.t, i, valid, sub, o);
        if (valid && sub == 0)
#pragma unroll
            for (int k = 0; k < M; ++k) f.rc[i * M + k] = o[k];
    }
}

// rows of P: D x M blocks
template <int D, int M, int G>
__global__ void __launch_bounds__(kAT) ka_prolong(int64_t n, amg::PassProlong32 f) {
    FE_LANE_ROWS(G, n) {
        const bool valid = i < n;
        float px[D];
        lanes_product<D, M, G>(f.ptr, f.col, f.val, f.xc, i, valid, sub, px);
        if (valid && sub == 0)
#pragma unroll
            for (int k = 0; k < D; ++k) f.x[i * D + k] += px[k];
    }
}

// x = inv r on the coarsest level: a warp per row, FP64 sums
__global__ void __launch_bounds__(kAT) ka_dense(amg::PassDense f) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < f.n; i += warps) {
        double acc = 0.0;
        for (int64_t j = lane; j < f.n; j += 32) acc = fma(f.inv[i * f.n + j], (double)f.r[j], acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) f.x[i] = (float)acc;
    }
}

// lanes per block row for a mean of `mean` blocks per row
inline int lanes_for(double mean) { return mean < 4 ? 2 : mean < 10 ? 4 : mean < 24 ? 8 : 32; }

template <typename F>
int with_lanes(int G, F f) {
    switch (G) {
        case 2: return f(std::integral_constant<int, 2>{});
        case 4: return f(std::integral_constant<int, 4>{});
        case 8: return f(std::integral_constant<int, 8>{});
        default: return f(std::integral_constant<int, 32>{});
    }
}

// Calls f(integral_constant RD, integral_constant CD) for the block shapes of the
// hierarchies: 1 x 1 (magnetostatics), 2 x 2 / 2 x 3 / 3 x 2 / 3 x 3 (plane elasticity),
// 3 x 3 / 3 x 6 / 6 x 3 / 6 x 6 (tetrahedra).
template <typename F>
int with_shape(int rd, int cd, F f) {
    using std::integral_constant;
    if (rd == 1 && cd == 1) return f(integral_constant<int, 1>{}, integral_constant<int, 1>{});
    if (rd == 2 && cd == 2) return f(integral_constant<int, 2>{}, integral_constant<int, 2>{});
    if (rd == 2 && cd == 3) return f(integral_constant<int, 2>{}, integral_constant<int, 3>{});
    if (rd == 3 && cd == 2) return f(integral_constant<int, 3>{}, integral_constant<int, 2>{});
    if (rd == 3 && cd == 3) return f(integral_constant<int, 3>{}, integral_constant<int, 3>{});
    if (rd == 3 && cd == 6) return f(integral_constant<int, 3>{}, integral_constant<int, 6>{});
    if (rd == 6 && cd == 3) return f(integral_constant<int, 6>{}, integral_constant<int, 3>{});
    if (rd == 6 && cd == 6) return f(integral_constant<int, 6>{}, integral_constant<int, 6>{});
    set_error("multigrid cycle: unsupported block shape");
    return FE_BAD_INPUT;
}

inline int grid_lanes(int64_t n, int G) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n * G + kAT - 1) / kAT, 152 * 8));
}

struct CycleEx {
    fe_handle_s *h;
    MgMem mem;
    DBuf<double> part, sc;
    // row pointer of the level-0 operator, whose FP64 products run on the handle's SELL copy
    const int64_t *sell_ptr = nullptr;
    // lanes per row of each matrix the cycle multiplies, keyed by its row pointer
    std::vector<std::pair<const int64_t *, int>> lanes;
    cudaEvent_t *marks = nullptr;   // events of the timing marks while profiling
    void mark(int k) {
        if (marks) cudaEventRecordWithFlags(marks[k], h->stream, cudaEventRecordExternal);
    }
    ~CycleEx() { pfree(mem, part), pfree(mem, sc); }
    int lanes_of(const int64_t *ptr) const {
        for (const auto &p : lanes)
            if (p.first == ptr) return p.second;
        return 32;
    }
    int rows(int64_t n, const amg::PassCheb &f) {
        if (n <= 0) return FE_OK;
        const int G = lanes_of(f.ptr);
        FE_CHECK(with_shape(f.d, f.d, [&](auto r, auto c) {
            constexpr int D = decltype(r)::value;
            if constexpr (D != decltype(c)::value) {
                return (int)FE_BAD_INPUT;
            } else {
                return with_lanes(G, [&](auto g) {
                    ka_cheb<D, decltype(g)::value><<<grid_lanes(n, G), kAT, 0, h->stream>>>(n, f);
                    return (int)FE_OK;
                });
            }
        }));
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return FE_OK;
    }
    int rows(int64_t n, const amg::PassResidual32 &f) {
        if (n <= 0) return FE_OK;
        const int G = lanes_of(f.ptr);
        FE_CHECK(with_shape(f.d, f.d, [&](auto r, auto c) {
            constexpr int D = decltype(r)::value;
            if constexpr (D != decltype(c)::value) {
                return (int)FE_BAD_INPUT;
            } else {
                return with_lanes(G, [&](auto g) {
                    ka_residual<D, decltype(g)::value><<<grid_lanes(n, G), kAT, 0, h->stream>>>(n, f);
                    return (int)FE_OK;
                });
            }
        }));
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return FE_OK;
    }
    int rows(int64_t n, const amg::PassRestrict32 &f) {
        if (n <= 0) return FE_OK;
        const int G = lanes_of(f.ptr);
        FE_CHECK(with_shape(f.m, f.d, [&](auto r, auto c) {
            return with_lanes(G, [&](auto g) {
                ka_restrict<decltype(r)::value, decltype(c)::value, decltype(g)::value>
                    <<<grid_lanes(n, G), kAT, 0, h->stream>>>(n, f);
                return (int)FE_OK;
            });
        }));
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return FE_OK;
    }
    int rows(int64_t n, const amg::PassProlong32 &f) {
        if (n <= 0) return FE_OK;
        const int G = lanes_of(f.ptr);
        FE_CHECK(with_shape(f.d, f.m, [&](auto r, auto c) {
            return with_lanes(G, [&](auto g) {
                ka_prolong<decltype(r)::value, decltype(c)::value, decltype(g)::value>
                    <<<grid_lanes(n, G), kAT, 0, h->stream>>>(n, f);
                return (int)FE_OK;
            });
        }));
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return FE_OK;
    }
    int rows(int64_t n, const amg::PassSpmv64 &f) {
        if (n <= 0) return FE_OK;
        if (sell_ptr && f.ptr == sell_ptr) return spmv64(h, f.p, f.q);
        ka_rows<amg::PassSpmv64><<<grid_a(n), kAT, 0, h->stream>>>(n, f);
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return FE_OK;
    }
    int rows(int64_t n, const amg::PassDense &f) {
        if (n <= 0) return FE_OK;
        ka_dense<<<grid_lanes(n, 32), kAT, 0, h->stream>>>(f);
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return FE_OK;
    }
    int dot(const double *a, const double *b, int64_t n, double *out) {
        const int g = grid_a(n);
        FE_CHECK(palloc(mem, part, (size_t)g));
        FE_CHECK(palloc(mem, sc, 1));
        ka_dot<<<g, kAT, 0, h->stream>>>(n, a, b, part.p);
        ka_dot_final<<<1, kAT, 0, h->stream>>>(g, part.p, sc.p);
        FE_LAUNCH_CHECK();
        h->launches += 2;
        FE_CUDA(cudaMemcpyAsync(mem.pinned, sc.p, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
        *out = mem.pinned[0];
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

// FP32 copies of a level's values and its cycle vectors (with_a: of A and D^-1 too;
// level 0 smooths on the handle's SELL copy instead)
int prepare_cycle(fe_handle_s *h, const MgMem &mem, DevLevel &L, bool with_a) {
    const int d = L.A.rd, m = L.P.cd;
    const int64_t na = with_a ? L.A.nnzb * d * d : 0, np = L.P.nnzb * d * m, nt = L.PT.nnzb * m * d,
                  ndi = with_a ? L.A.n * d * d : 0;
    FE_CHECK(palloc(mem, L.a32, (size_t)std::max<int64_t>(na, 1)));
    FE_CHECK(palloc(mem, L.p32, (size_t)std::max<int64_t>(np, 1)));
    FE_CHECK(palloc(mem, L.pt32, (size_t)std::max<int64_t>(nt, 1)));
    FE_CHECK(palloc(mem, L.dinv32, (size_t)std::max<int64_t>(ndi, 1)));
    CycleEx ex{h, mem};
    FE_CHECK(ex.rows(na, amg::PassToF32{L.A.val.p, L.a32.p}));
    FE_CHECK(ex.rows(np, amg::PassToF32{L.P.val.p, L.p32.p}));
    FE_CHECK(ex.rows(nt, amg::PassToF32{L.PT.val.p, L.pt32.p}));
    FE_CHECK(ex.rows(ndi, amg::PassToF32{L.dinv.p, L.dinv32.p}));
    const size_t v = (size_t)std::max<int64_t>(L.A.n * d, 1);
    FE_CHECK(palloc(mem, L.r, v));
    FE_CHECK(palloc(mem, L.x, v));
    FE_CHECK(palloc(mem, L.t, v));
    FE_CHECK(palloc(mem, L.dir, v));
    FE_CHECK(palloc(mem, L.zn, v));
    return FE_OK;
}

// Chebyshev(k) smoothing of level 0 on the SELL copy, over the interval of the shared
// cycle ([1.05 lmax / 30, 1.05 lmax]): from zero (z_1 = D^-1 r / theta needs no product;
// start) or from the iterate in *cur (then the first step is a full one).  The iterates
// ping-pong between *cur and *other; on return *cur holds the last.
int level0_chebyshev(fe_handle_s *h, const amg::CycleLevel &L, const double *r64, int k, bool from_zero,
                     float **cur, float **other, CycleEx &ex) {
    const double hi = 1.05 * L.lmax, lo = hi / 30.0;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    double rho = 1.0 / sigma;
    if (from_zero) {
        FE_CHECK(mg_level0_start(h, r64, L.r, *cur, 1.0 / theta));
        ex.mark(0);
    } else {
        FE_CHECK(mg_level0_cheb(h, true, L.r, *cur, *other, 0.0, 1.0 / theta));
        std::swap(*cur, *other);
    }
    for (int st = 1; st < k; ++st) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        const double a = rn * rho, b = 2.0 * rn / delta;
        rho = rn;
        // from zero, the second step's old iterate is z_0 = 0 (first)
        FE_CHECK(mg_level0_cheb(h, from_zero && st == 1, L.r, *cur, *other, a, b));
        std::swap(*cur, *other);
    }
    if (from_zero) ex.mark(1);
    return FE_OK;
}

// z = M^-1 r: the shared FP32 V-cycle below level 0, level 0 on the SELL copy (its
// right-hand side D^-1 r in L0.r, iterates in L0.x / L0.zn)
int precondition_sell(CycleEx &ex, const std::vector<amg::CycleLevel> &levels, const amg::CycleCoarse &C, int k,
                      int kc, const double *r, double *z) {
    fe_handle_s *h = ex.h;
    const amg::CycleLevel &L = levels[0];
    float *rc = levels.size() > 1 ? levels[1].r : C.r;
    float *xc = levels.size() > 1 ? levels[1].x : C.x;
    ex.mark(2);
    float *cur = L.x, *other = L.zn;
    FE_CHECK(level0_chebyshev(h, L, r, k, true, &cur, &other, ex));
    FE_CHECK(mg_level0_residual(h, L.r, cur, L.t));
    FE_CHECK(ex.rows(L.nc, amg::PassRestrict32{L.tptr, L.tcol, L.pt, L.m, L.d, L.t, rc}));
    FE_CHECK(amg::vcycle(ex, levels, C, 1, kc));
    FE_CHECK(ex.rows(L.n, amg::PassProlong32{L.pptr, L.pcol, L.p, L.d, L.m, xc, cur}));
    FE_CHECK(level0_chebyshev(h, L, r, k, false, &cur, &other, ex));
    FE_CHECK(ex.rows(L.n * L.d, amg::PassToF64{cur, z}));
    ex.mark(3);
    return FE_OK;
}

// z = M^-1 r when the hierarchy has no level (a system of at most a few thousand DOFs):
// the coarsest level is the system itself and its dense inverse the preconditioner
int precondition_dense(CycleEx &ex, const amg::CycleCoarse &C, const double *r, double *z) {
    ex.mark(2);
    ex.mark(0);
    FE_CHECK(ex.rows(C.n, amg::PassToF32{r, C.r}));
    FE_CHECK(ex.rows(C.n, amg::PassDense{C.n, C.inv, C.r, C.x}));
    FE_CHECK(ex.rows(C.n, amg::PassToF64{C.x, z}));
    ex.mark(1);
    ex.mark(3);
    return FE_OK;
}

}  // namespace

// PCG on the eliminated system preconditioned by one FP32 V-cycle (Chebyshev smoothing:
// kSmooth0 steps on level 0, kSmoothCoarse below), FP64 recurrence, from x = 0 or from
// opts.x0 (with FE_SOLVE_X0_IF_BETTER only when it beats the zero start); the hierarchy is
// set up on the device from the system matrix and the rigid-body (elasticity) or
// constant (magnetostatics) modes, with the rows of the constrained DOFs zeroed.
int solve_multigrid(fe_handle_s *h, const fe_solve_opts *o, fe_solve_stats *st) {
    cudaStream_t s = h->stream;
    const int D = h->dim;
    const int64_t n = h->n_nodes, nd = h->n_dof;
    FE_CUDA(cudaEventRecord(h->events[6], s));
    // the hierarchy, set up on the device, and the cycle's vectors
    const bool prof = h->w.prof && h->w.pev[0];
    DevAmg G;
    // down to at most 1500 DOFs (an eighth of small systems).  Below ~650 nodes the
    // aggregates of the plane-strain family stop shrinking while the coarse operators
    // fill in (4M DOF: 647 -> 365 -> 321 -> 217 nodes, rows of 100-200 blocks), so a
    // smaller coarsest level costs a level of long products: at 4M DOF the 1095-DOF
    // coarsest level (6 ms for its inverse, about 4 ms more of products) and the
    // 1941-DOF one (16 ms) measured the same solve time
    SetupTrace trace;
    FE_CHECK(amg_setup_device(h, 0.08, std::min<int64_t>(1500, std::max<int64_t>(100, nd / 8)), G,
                              prof ? &trace : nullptr));
    if (prof) trace.mark(s, amg::kPhaseCycle);
    for (size_t l = 0; l < G.L.size(); ++l) FE_CHECK(prepare_cycle(h, G.mem, G.L[l], l > 0));
    FE_CHECK(palloc(G.mem, G.rc, (size_t)std::max<int64_t>(G.nc, 1)));
    FE_CHECK(palloc(G.mem, G.xc, (size_t)std::max<int64_t>(G.nc, 1)));
    // the system's operator: level 0, or the coarsest level when there is no other
    const DevCsr &A0 = G.L.empty() ? G.coarse : G.L[0].A;
    // PCG vectors; the solution goes to the handle's x
    DBuf<double> r, p, q, z;
    struct Free {
        const MgMem &m;
        DBuf<double> *b[4];
        ~Free() {
            for (auto *x : b) pfree(m, *x);
        }
    } fg{G.mem, {&r, &p, &q, &z}};
    FE_CHECK(dalloc(h->w.x, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(palloc(G.mem, r, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(palloc(G.mem, p, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(palloc(G.mem, q, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(palloc(G.mem, z, (size_t)std::max<int64_t>(nd, 1)));
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
    CycleEx cex{h, G.mem};
    cex.sell_ptr = A0.ptr.p;
    if (prof) cex.marks = h->w.pev;
    for (const DevLevel &Dl : G.L) {
        const double n_rows = (double)std::max<int64_t>(Dl.A.n, 1), n_aggr = (double)std::max<int64_t>(Dl.PT.n, 1);
        cex.lanes.push_back({Dl.A.ptr.p, lanes_for((double)Dl.A.nnzb / n_rows)});
        cex.lanes.push_back({Dl.P.ptr.p, lanes_for((double)Dl.P.nnzb / n_rows)});
        cex.lanes.push_back({Dl.PT.ptr.p, lanes_for((double)Dl.PT.nnzb / n_aggr)});
    }
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
        const int rc = G.L.empty() ? precondition_dense(cex, coarse, r.p, z.p)
                                   : precondition_sell(cex, views, coarse, kSmooth0, kSmoothCoarse, r.p, z.p);
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
    if (prof) {
        // the setup: from the solve's start to here, and per phase
        trace.mark(s, amg::kSetupPhases);
        FE_CHECK(trace.collect(h->w.mg_phase_ms, 16));
        FE_CUDA(cudaEventRecord(h->events[7], s));
        FE_CUDA(cudaEventSynchronize(h->events[7]));
        float a = 0.f;
        FE_CUDA(cudaEventElapsedTime(&a, h->events[6], h->events[7]));
        h->w.mg_ms[1] += a, h->w.mg_n[1] += 1;
    }
    const int64_t smooth_launches = kSmooth0 - 1;   // SELL Chebyshev steps of level 0's pre-smoothing
    auto precond = [&]() -> int {
        FE_CUDA(cudaGraphLaunch(cycle, s));
        h->launches += per_cycle;
        if (prof) {
            FE_CUDA(cudaEventSynchronize(h->w.pev[3]));
            float a = 0.f, c = 0.f;
            if (cudaEventElapsedTime(&a, h->w.pev[0], h->w.pev[1]) == cudaSuccess)
                h->w.mg_ms[0] += a, h->w.mg_n[0] += smooth_launches;
            if (cudaEventElapsedTime(&c, h->w.pev[2], h->w.pev[3]) == cudaSuccess)
                h->w.mg_ms[2] += c, h->w.mg_n[2] += 1;
        }
        return FE_OK;
    };
    const double tol = o->tol > 0 ? o->tol : 1e-10;
    const int max_iter = o->max_iter > 0 ? o->max_iter : 10000;
    const int max_restart = o->max_outer > 0 ? o->max_outer : 4;
    int status = FE_OK, total = 0, restarts = 0, x0_used = 0;
    double relres = 0.0;
    // the start: the prescribed values on constrained DOFs, and opts.x0 where given (with
    // FE_SOLVE_X0_IF_BETTER only when its FP64 residual beats the zero start)
    FE_CHECK(solve_start_point(h, o, h->w.x.p, &x0_used));
    const amg::PcgVectors v{h->w.x.p, r.p, p.p, q.p, z.p};
    // PCG from x; when the recurrence met tol but the FP64 true residual did not (the
    // recurrence drifts from b - A x by about eps cond(A)), restart from the true residual;
    // a restart that gains less than 2x marks the rounding floor (FE_OK with
    // FE_SOLVE_ACCEPT_STAGNATION, else FE_MAXITER), as in the other solvers
    double prev = INFINITY;
    bool stagnated = false;
    for (;;) {
        int it = 0;
        FE_CHECK(amg::pcg(cex, n, D, A0.ptr.p, A0.col.p, A0.val.p, h->b.p, v, precond, tol,
                          max_iter - total, &it, &relres, &status, true));
        total += it;
        if (status != FE_OK || relres <= tol || restarts >= max_restart || total >= max_iter) break;
        if (relres > 0.5 * prev) {
            stagnated = true;
            break;
        }
        prev = relres;
        ++restarts;
    }
    if (status == FE_OK && relres > tol && !(stagnated && (o->flags & FE_SOLVE_ACCEPT_STAGNATION)))
        status = FE_MAXITER;
    double bb = 0.0;
    FE_CHECK(cex.dot(h->b.p, h->b.p, nd, &bb));
    st->iterations = total;
    st->spmv = total + 1 + restarts;
    st->outer = restarts;
    st->fp64_iterations = 0;
    st->x0_used = x0_used;
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
