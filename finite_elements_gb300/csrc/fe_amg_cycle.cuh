// The FP32 V-cycle of the multigrid preconditioner written once over an executor (see
// fe_amg_passes.cuh): the device runs it inside the PCG (fe_amg_device.cu, captured as
// a CUDA graph), the host runs the same sequence (fe_amg_vcycle_host_f32) so that the
// CPU tests check the cycle's wiring -- buffers per level, the Chebyshev ping-pong, the
// transfers and the coarsest solve -- against the FP64 host cycle.
//
// An executor provides, beside what fe_amg_passes.cuh lists:
//   template <class T> int fill_zero(T *p, size_t n);
//   void mark(int k);   // timing marks: 0 / 1 around level 0's pre-smoothing, 2 / 3 around
//                       // the whole cycle (the device records events; the host ignores them)
#pragma once

#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

#include "fe_amg_rows.cuh"
#include "fe_internal.h"

namespace fe {
namespace amg {

// One level as the cycle sees it: pattern arrays, FP32 values, FP32 vectors (n d each).
struct CycleLevel {
    int64_t n = 0;                 // block rows
    int d = 0, m = 0;              // block size, coarse block size (columns of P)
    double lmax = 0.0;
    const int64_t *aptr = nullptr; const int32_t *acol = nullptr; const float *a = nullptr;
    const float *dinv = nullptr;
    const int64_t *pptr = nullptr; const int32_t *pcol = nullptr; const float *p = nullptr;
    int64_t nc = 0;                // rows of P^T (aggregates)
    const int64_t *tptr = nullptr; const int32_t *tcol = nullptr; const float *pt = nullptr;
    float *r = nullptr, *x = nullptr, *t = nullptr, *dir = nullptr, *zn = nullptr;
};

// The coarsest level: dense FP64 inverse, FP32 vectors.
struct CycleCoarse {
    int64_t n = 0;                 // DOFs
    const double *inv = nullptr;
    float *r = nullptr, *x = nullptr;
};

// zero: z_in is zero (the first step from zero), so A z_in = 0; an executor may skip the
// product (the row operation computes it, exactly 0)
struct PassCheb {
    const int64_t *ptr; const int32_t *col; const float *val; const float *dinv; int d; const float *r;
    const float *zin; float *dir; float *zout; float a; float b; int first;
    int zero = 0;
    FE_HD void operator()(int64_t i) const { row_chebyshev(ptr, col, val, dinv, d, r, zin, dir, zout, a, b, first != 0, i); }
};

struct PassResidual32 {
    const int64_t *ptr; const int32_t *col; const float *val; int d; const float *r; const float *x; float *t;
    FE_HD void operator()(int64_t i) const { row_residual(ptr, col, val, d, r, x, t, i); }
};

struct PassRestrict32 {
    const int64_t *ptr; const int32_t *col; const float *val; int m; int d; const float *t; float *rc;
    FE_HD void operator()(int64_t I) const { row_restrict(ptr, col, val, m, d, t, rc, I); }
};

struct PassProlong32 {
    const int64_t *ptr; const int32_t *col; const float *val; int d; int m; const float *xc; float *x;
    FE_HD void operator()(int64_t i) const { row_prolong_add(ptr, col, val, d, m, xc, x, i); }
};

// x = inv r (dense, FP64 inverse and sums, FP32 vectors)
struct PassDense {
    int64_t n; const double *inv; const float *r; float *x;
    FE_HD void operator()(int64_t i) const {
        double acc = 0.0;
        for (int64_t j = 0; j < n; ++j) acc += inv[i * n + j] * (double)r[j];
        x[i] = (float)acc;
    }
};

struct PassToF32 {
    const double *in; float *out;
    FE_HD void operator()(int64_t i) const { out[i] = (float)in[i]; }
};

struct PassToF64 {
    const float *in; double *out;
    FE_HD void operator()(int64_t i) const { out[i] = (double)in[i]; }
};

// k Chebyshev steps on D^-1 A z = D^-1 r over [1.05 lmax / 30, 1.05 lmax] into L.x, from
// zero or from L.x (from_x0); steps alternate between L.x and L.zn.
template <class Ex>
int chebyshev_cycle(Ex &ex, const CycleLevel &L, int k, bool from_x0) {
    const int64_t nd = L.n * L.d;
    const double hi = 1.05 * L.lmax, lo = hi / 30.0;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    if (!from_x0) FE_CHECK(ex.fill_zero(L.x, (size_t)nd));
    float *cur = L.x, *nxt = L.zn;
    double rho = 1.0 / sigma;
    PassCheb first{L.aptr, L.acol, L.a, L.dinv, L.d, L.r, cur, L.dir, nxt, 0.0f, (float)(1.0 / theta), 1};
    first.zero = from_x0 ? 0 : 1;
    FE_CHECK(ex.rows(L.n, first));
    std::swap(cur, nxt);
    for (int st = 1; st < k; ++st) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        const double a = rn * rho, b = 2.0 * rn / delta;
        rho = rn;
        FE_CHECK(ex.rows(L.n, PassCheb{L.aptr, L.acol, L.a, L.dinv, L.d, L.r, cur, L.dir, nxt, (float)a, (float)b, 0}));
        std::swap(cur, nxt);
    }
    if (cur != L.x) FE_CHECK(ex.copy(L.x, cur, (size_t)nd));
    return FE_OK;
}

// V-cycle from level l: levels[l].r -> levels[l].x (the coarsest: C.r -> C.x)
template <class Ex>
int vcycle(Ex &ex, const std::vector<CycleLevel> &levels, const CycleCoarse &C, size_t l, int k) {
    if (l == levels.size()) return ex.rows(C.n, PassDense{C.n, C.inv, C.r, C.x});
    const CycleLevel &L = levels[l];
    float *rc = l + 1 < levels.size() ? levels[l + 1].r : C.r;
    float *xc = l + 1 < levels.size() ? levels[l + 1].x : C.x;
    if (l == 0) ex.mark(0);
    FE_CHECK(chebyshev_cycle(ex, L, k, false));
    if (l == 0) ex.mark(1);
    FE_CHECK(ex.rows(L.n, PassResidual32{L.aptr, L.acol, L.a, L.d, L.r, L.x, L.t}));
    FE_CHECK(ex.rows(L.nc, PassRestrict32{L.tptr, L.tcol, L.pt, L.m, L.d, L.t, rc}));
    FE_CHECK(vcycle(ex, levels, C, l + 1, k));
    FE_CHECK(ex.rows(L.n, PassProlong32{L.pptr, L.pcol, L.p, L.d, L.m, xc, L.x}));
    return chebyshev_cycle(ex, L, k, true);
}

// z = M^-1 r in FP64 through the FP32 cycle: r rounded to FP32 into level 0, z widened
template <class Ex>
int precondition(Ex &ex, const std::vector<CycleLevel> &levels, const CycleCoarse &C, int k, const double *r,
                 double *z) {
    const CycleLevel &L0 = levels[0];
    const int64_t nd = L0.n * L0.d;
    ex.mark(2);
    FE_CHECK(ex.rows(nd, PassToF32{r, L0.r}));
    FE_CHECK(vcycle(ex, levels, C, 0, k));
    FE_CHECK(ex.rows(nd, PassToF64{L0.x, z}));
    ex.mark(3);
    return FE_OK;
}

}  // namespace amg
}  // namespace fe

namespace fe {
namespace amg {

// ------------------------------------------------------------------ the PCG around the cycle

struct PassSpmv64 {
    const int64_t *ptr; const int32_t *col; const double *val; int d; const double *p; double *q;
    FE_HD void operator()(int64_t i) const {
        double out[6];
        row_product(ptr, col, val, d, d, p, i, out);
        for (int k = 0; k < d; ++k) q[i * d + k] = out[k];
    }
};

// x += alpha p, r -= alpha q
struct PassUpdate {
    double alpha; const double *p; const double *q; double *x; double *r;
    FE_HD void operator()(int64_t i) const {
        x[i] = fma(alpha, p[i], x[i]);
        r[i] = fma(-alpha, q[i], r[i]);
    }
};

// p = z + beta p
struct PassDirection {
    double beta; const double *z; double *p;
    FE_HD void operator()(int64_t i) const { p[i] = fma(beta, p[i], z[i]); }
};

struct PassResidual64 {
    const int64_t *ptr; const int32_t *col; const double *val; int d; const double *r; const double *x; double *t;
    FE_HD void operator()(int64_t i) const { row_residual(ptr, col, val, d, r, x, t, i); }
};

// Work vectors of the PCG, n d doubles each.
struct PcgVectors {
    double *x, *r, *p, *q, *z;
};

// PCG on A x = b with z = precond() (reading v.r, writing v.z), to ||r|| <= tol ||b||
// on the recurrence; relres is the true residual recomputed in FP64.  From x = 0, or
// with from_x from the x already in v.x (r = b - A x).  status: FE_OK, FE_MAXITER,
// FE_BREAKDOWN (p.Ap <= 0) or FE_NONFINITE.
template <class Ex, class Precond>
int pcg(Ex &ex, int64_t n, int d, const int64_t *ptr, const int32_t *col, const double *val, const double *b,
        const PcgVectors &v, Precond precond, double tol, int max_iter, int *iters, double *relres, int *status,
        bool from_x = false) {
    const int64_t nd = n * d;
    if (from_x) {
        FE_CHECK(ex.rows(n, PassResidual64{ptr, col, val, d, b, v.x, v.r}));
    } else {
        FE_CHECK(ex.fill_zero(v.x, (size_t)nd));
        FE_CHECK(ex.copy(v.r, b, (size_t)nd));
    }
    double rz = 0.0, bb = 0.0, rr0 = 0.0;
    FE_CHECK(ex.dot(b, b, nd, &bb));
    FE_CHECK(ex.dot(v.r, v.r, nd, &rr0));
    int it = 0, st = (bb > 0.0 && rr0 > tol * tol * bb) ? FE_MAXITER : FE_OK;
    if (st == FE_MAXITER) {
        FE_CHECK(precond());
        FE_CHECK(ex.copy(v.p, v.z, (size_t)nd));
        FE_CHECK(ex.dot(v.r, v.z, nd, &rz));
    }
    while (st == FE_MAXITER && it < max_iter) {
        FE_CHECK(ex.rows(n, PassSpmv64{ptr, col, val, d, v.p, v.q}));
        double pq = 0.0;
        FE_CHECK(ex.dot(v.p, v.q, nd, &pq));
        if (!(pq > 0.0) || !std::isfinite(pq)) {
            st = std::isfinite(pq) ? FE_BREAKDOWN : FE_NONFINITE;
            break;
        }
        FE_CHECK(ex.rows(nd, PassUpdate{rz / pq, v.p, v.q, v.x, v.r}));
        ++it;
        double rr = 0.0, rzn = 0.0;
        FE_CHECK(ex.dot(v.r, v.r, nd, &rr));
        if (!std::isfinite(rr)) {
            st = FE_NONFINITE;
            break;
        }
        if (rr <= tol * tol * bb) {
            st = FE_OK;
            break;
        }
        FE_CHECK(precond());
        FE_CHECK(ex.dot(v.r, v.z, nd, &rzn));
        if (!std::isfinite(rzn)) {
            st = FE_NONFINITE;
            break;
        }
        FE_CHECK(ex.rows(nd, PassDirection{rzn / rz, v.z, v.p}));
        rz = rzn;
    }
    FE_CHECK(ex.rows(n, PassResidual64{ptr, col, val, d, b, v.x, v.q}));
    double tr = 0.0;
    FE_CHECK(ex.dot(v.q, v.q, nd, &tr));
    *iters = it;
    *relres = bb > 0.0 ? std::sqrt(std::max(tr, 0.0) / bb) : 0.0;
    *status = st;
    return FE_OK;
}

}  // namespace amg
}  // namespace fe
