// The parallel smoothed-aggregation setup written once for two executors: the device
// (fe_amg_device_setup.cu: each pass a grid-stride kernel over its rows, int64 scans
// on the device) and the host (fe_amg_setup.cu: the same passes over row chunks on
// host threads).  Every pass is a functor over one row (or one aggregate) built on the
// row operations of fe_amg_par.cuh; the sequence of passes, the buffer sizes and the
// scans that size them are this file's, shared by both, so the host run (checked on
// the CPU against the model) exercises the device's bookkeeping too.
//
// An executor Ex provides:
//   template <class T> int alloc(DBuf<T> &b, size_t n);  template <class T> void release(DBuf<T> &b);
//   template <class T> int copy(T *dst, const T *src, size_t n);       // same memory space
//   template <class T> int read(T *host_dst, const T *src, size_t n);  // to the host, synchronous
//   template <class F> int rows(int64_t n, const F &f);                // f(i) for i < n, any order
//   int scan(const int64_t *in, int64_t n, int64_t *out, int64_t *total);   // exclusive, out[n] = total
//   int dot(const double *a, const double *b, int64_t n, double *out);      // host value
//   int dot_to(const double *a, const double *b, int64_t n, double *dst);   // into executor
//                                                                           // memory, no wait
//   void phase(int k);   // setup phase k (SetupPhase) starts here (timed by the device
//                        // executor when profiling, ignored by the host one)
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

#include "fe_amg.h"
#include "fe_amg_par.cuh"
#include "fe_internal.h"

namespace fe {
namespace amg {

// Phases of the setup, per level in this order, then the coarsest inverse and the
// cycle's preparation (FP32 copies, capture); kPhaseInput is level 0's own copy of the
// operator and its near-null space.
enum SetupPhase : int {
    kPhaseInput = 0,
    kPhaseDiag,          // D^-1 and the Lanczos estimate of lmax
    kPhaseAggregate,     // strength, the distance-2 independent set, the joins
    kPhaseTentative,     // member lists and the QR of every aggregate
    kPhaseProlongator,   // A P_t and the damped-Jacobi smoothing
    kPhaseAP,            // A P
    kPhaseRestriction,   // P^T: structure and values
    kPhaseGalerkin,      // P^T (A P)
    kPhaseCoarse,        // dense inverse of the coarsest level
    kPhaseCycle,         // FP32 copies, cycle vectors, graph capture
    kSetupPhases
};

// ------------------------------------------------------------------ storage

struct Csr {
    int64_t n = 0;
    int rd = 0, cd = 0;
    int64_t nnzb = 0;
    DBuf<int64_t> ptr;   // n + 1
    DBuf<int32_t> col;
    DBuf<double> val;    // nnzb row-major rd x cd blocks
};

struct Level {
    Csr A, P, PT;
    DBuf<double> dinv;
    DBuf<int32_t> agg;
    double lmax = 0.0;
};

template <class Ex>
void release(Ex &ex, Csr &c) {
    ex.release(c.ptr), ex.release(c.col), ex.release(c.val);
    c.nnzb = 0;
}

template <class Ex>
void release(Ex &ex, Level &l) {
    release(ex, l.A), release(ex, l.P), release(ex, l.PT);
    ex.release(l.dinv), ex.release(l.agg);
}

// ------------------------------------------------------------------ passes

struct PassDinv {
    const int64_t *ptr; const int32_t *col; const double *val; int d; double *dinv;
    FE_HD void operator()(int64_t i) const {
        double *o = &dinv[i * d * d];
        for (int k = 0; k < d * d; ++k) o[k] = 0.0;
        for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s)
            if (col[s] == i) sym_pinv(&val[s * d * d], d, o);
    }
};

// the start vector of the eigenvalue estimate, 1 + (i mod 7) / 7
struct PassPowerStart {
    double *x;
    FE_HD void operator()(int64_t i) const { x[i] = 1.0 + (double)(i % 7) / 7.0; }
};

// y = D^-1 A x (y = A x when dinv is null); nnzb: the matrix's block count (a device
// executor sizes its lanes per row with it)
struct PassDinvProduct {
    const int64_t *ptr; const int32_t *col; const double *val; const double *dinv; int d; const double *x; double *y;
    int64_t nnzb;
    FE_HD void operator()(int64_t i) const { row_dinv_product(ptr, col, val, dinv, d, x, i, y); }
};

// z_i = D_i^-1 r_i
struct PassJacobi {
    const double *dinv; int d; const double *r; double *z;
    FE_HD void operator()(int64_t i) const {
        for (int a = 0; a < d; ++a) {
            double v = 0.0;
            for (int k = 0; k < d; ++k) v += dinv[i * d * d + a * d + k] * r[i * d + k];
            z[i * d + a] = v;
        }
    }
};

// r_i -= alpha q_i, then z_i = D_i^-1 r_i
struct PassCgStep {
    double alpha; const double *q; const double *dinv; int d; double *r; double *z;
    FE_HD void operator()(int64_t i) const {
        for (int a = 0; a < d; ++a) r[i * d + a] -= alpha * q[i * d + a];
        PassJacobi{dinv, d, r, z}(i);
    }
};



struct PassBlockNorms {
    const int64_t *ptr; const int32_t *col; const double *val; int d; double *nrm; double *dg;
    FE_HD void operator()(int64_t i) const { row_block_norms(ptr, col, val, d, i, nrm, dg); }
};

struct PassStrength {
    const int64_t *ptr; const int32_t *col; const double *nrm; const double *dg; double theta; uint8_t *strong;
    FE_HD void operator()(int64_t i) const { row_strength(ptr, col, nrm, dg, theta, i, strong); }
};

struct PassStateInit {
    uint32_t *state;
    FE_HD void operator()(int64_t i) const { state[i] = kUndecided; }
};

struct PassMisKey {
    const uint32_t *state; uint64_t *key;
    FE_HD void operator()(int64_t i) const { key[i] = mis_key(state[i], i); }
};

struct PassMaxKey {
    const int64_t *ptr; const int32_t *col; const uint8_t *strong; const uint64_t *in; uint64_t *out;
    FE_HD void operator()(int64_t i) const { row_max_key(ptr, col, strong, in, i, out); }
};

// decides node i; flag[i] = 1 while it stays undecided
struct PassMisDecide {
    const uint64_t *m2; uint32_t *state; int64_t *flag;
    FE_HD void operator()(int64_t i) const { flag[i] = mis_decide(m2, i, state); }
};

struct PassRootFlags {
    const uint32_t *state; int64_t *flag;
    FE_HD void operator()(int64_t i) const { flag[i] = state[i] == kIn ? 1 : 0; }
};

struct PassRoots {
    const uint32_t *state; const int64_t *off; int32_t *rank; int32_t *roots;
    FE_HD void operator()(int64_t i) const {
        if (state[i] == kIn) {
            rank[i] = (int32_t)off[i];
            roots[off[i]] = (int32_t)i;
        } else {
            rank[i] = -1;
        }
    }
};

struct PassJoinRoot {
    const int64_t *ptr; const int32_t *col; const uint8_t *strong; const double *nrm; const uint32_t *state;
    const int32_t *rank; int32_t *agg1;
    FE_HD void operator()(int64_t i) const { row_join_root(ptr, col, strong, nrm, state, rank, i, agg1); }
};

// flag[i] = 1 for a node left without an aggregate
struct PassJoinNeighbour {
    const int64_t *ptr; const int32_t *col; const uint8_t *strong; const double *nrm; const int32_t *agg1;
    int32_t *agg; int64_t *flag;
    FE_HD void operator()(int64_t i) const {
        row_join_neighbour(ptr, col, strong, nrm, agg1, i, agg);
        flag[i] = agg[i] < 0 ? 1 : 0;
    }
};

// Member lists by a counting sort of the nodes on their aggregates: counts, offsets
// (a scan), then every node into its aggregate's row through an atomic cursor, then
// each row sorted, so that the lists come out in node order whatever the order of the
// atomics.
struct PassZeroI64 {
    int64_t *p;
    FE_HD void operator()(int64_t i) const { p[i] = 0; }
};

struct PassMemberCount {
    const int32_t *agg; int64_t *cnt;
    FE_HD void operator()(int64_t i) const { atomic_add_i64(&cnt[agg[i]], 1); }
};

struct PassMemberScatter {
    const int32_t *agg; const int64_t *mptr; int64_t *cursor; int32_t *mem;
    FE_HD void operator()(int64_t i) const {
        const int64_t c = agg[i];
        mem[mptr[c] + atomic_add_i64(&cursor[c], 1)] = (int32_t)i;
    }
};

struct PassSortRows {
    const int64_t *ptr; int32_t *col;
    FE_HD void operator()(int64_t r) const { heap_sort(col + ptr[r], ptr[r + 1] - ptr[r]); }
};

// packed rows: dst[off[r] ..] = src[boff[r] ..], off[r+1] - off[r] entries
struct PassPackRows {
    const int64_t *boff; const int64_t *off; const int32_t *src; int32_t *dst;
    FE_HD void operator()(int64_t r) const {
        const int64_t len = off[r + 1] - off[r];
        for (int64_t k = 0; k < len; ++k) dst[off[r] + k] = src[boff[r] + k];
    }
};

struct PassIota {
    int64_t *p;
    FE_HD void operator()(int64_t i) const { p[i] = i; }
};

struct PassQr {
    const int64_t *mptr; const int32_t *mem; int d; int m; double *pt; double *Bc;
    FE_HD void operator()(int64_t c) const { aggregate_qr(mem + mptr[c], mptr[c + 1] - mptr[c], d, m, pt, Bc + c * m * m); }
};

struct PassProdBound {
    const int64_t *aptr; const int32_t *acol; const int64_t *bptr; int64_t *bound;
    FE_HD void operator()(int64_t i) const { bound[i] = row_product_bound(aptr, acol, bptr, i); }
};

// total: the bounds' sum (set by distinct_rows); a device executor picks a warp per
// row when rows are long
struct PassProdCols {
    const int64_t *aptr; const int32_t *acol; const int64_t *bptr; const int32_t *bcol; const int64_t *boff;
    int32_t *cand; int64_t *cnt;
    int64_t total = 0;
    FE_HD void operator()(int64_t i) const { cnt[i] = row_product_columns(aptr, acol, bptr, bcol, i, cand + boff[i]); }
};

// boff / total: the row offsets and the sum of the rows' product counts (PassProdBound),
// for a device executor that gives long rows a warp each
// upper: the product is symmetric; only the entries on and above the diagonal are
// computed (PassMirrorLower fills the others)
struct PassProdVals {
    const int64_t *aptr; const int32_t *acol; const double *aval; int ra; int ca; const int64_t *bptr;
    const int32_t *bcol; const double *bval; int cb; const int64_t *cptr; const int32_t *ccol; double *cval;
    const int64_t *boff = nullptr;
    int64_t total = 0;
    int upper = 0;
    FE_HD void operator()(int64_t i) const {
        row_product_values(aptr, acol, aval, ra, ca, bptr, bcol, bval, cb, cptr, ccol, cval, i, upper != 0);
    }
};

struct PassMirrorLower {
    const int64_t *ptr; const int32_t *col; double *val; int m;
    FE_HD void operator()(int64_t i) const { row_mirror_lower(ptr, col, val, m, i); }
};

struct PassSmooth {
    const int64_t *pptr; const int32_t *pcol; double *pval; const double *dinv; const double *ptent;
    const int32_t *agg; int d; int m; double w;
    FE_HD void operator()(int64_t i) const { row_smooth_prolongator(pptr, pcol, pval, dinv, ptent, agg, d, m, w, i); }
};

struct PassRestrVals {
    const int64_t *rptr; const int32_t *rcol; double *rval; const int64_t *pptr; const int32_t *pcol;
    const double *pval; int d; int m;
    FE_HD void operator()(int64_t c) const { row_restriction_values(rptr, rcol, rval, pptr, pcol, pval, d, m, c); }
};

// ------------------------------------------------------------------ orchestration

template <class Ex>
struct Work {
    DBuf<int64_t> bound, boff, cnt, flag;
    DBuf<int32_t> cand;
    Ex &ex;
    explicit Work(Ex &e) : ex(e) {}
    ~Work() { ex.release(bound), ex.release(boff), ex.release(cnt), ex.release(flag), ex.release(cand); }
};

// Rows whose entries are sorted distinct candidates: bound pass, scan, candidate pass
// (count per row), scan into C.ptr, pack into C.col.
template <class Ex, class Bound, class Cols>
int distinct_rows(Ex &ex, int64_t n, Bound bound, Cols cols, Csr &C, Work<Ex> &W, int64_t *total_out = nullptr) {
    FE_CHECK(ex.alloc(W.bound, (size_t)std::max<int64_t>(n, 1)));
    FE_CHECK(ex.alloc(W.boff, (size_t)n + 1));
    FE_CHECK(ex.alloc(W.cnt, (size_t)std::max<int64_t>(n, 1)));
    bound.bound = W.bound.p;
    FE_CHECK(ex.rows(n, bound));
    int64_t total = 0;
    FE_CHECK(ex.scan(W.bound.p, n, W.boff.p, &total));
    FE_CHECK(ex.alloc(W.cand, (size_t)std::max<int64_t>(total, 1)));
    cols.boff = W.boff.p, cols.cand = W.cand.p, cols.cnt = W.cnt.p, cols.total = total;
    if (total_out) *total_out = total;
    FE_CHECK(ex.rows(n, cols));
    FE_CHECK(ex.alloc(C.ptr, (size_t)n + 1));
    int64_t nnzb = 0;
    FE_CHECK(ex.scan(W.cnt.p, n, C.ptr.p, &nnzb));
    C.nnzb = nnzb;
    FE_CHECK(ex.alloc(C.col, (size_t)std::max<int64_t>(nnzb, 1)));
    FE_CHECK(ex.rows(n, PassPackRows{W.boff.p, C.ptr.p, W.cand.p, C.col.p}));
    return FE_OK;
}

// C = A B (symmetric: C is known to be symmetric, so its upper entries are computed
// and the lower ones copied from them)
template <class Ex>
int product(Ex &ex, const Csr &A, const Csr &B, Csr &C, Work<Ex> &W, bool symmetric = false) {
    C.n = A.n, C.rd = A.rd, C.cd = B.cd;
    int64_t total = 0;
    FE_CHECK(distinct_rows(ex, A.n, PassProdBound{A.ptr.p, A.col.p, B.ptr.p, nullptr},
                           PassProdCols{A.ptr.p, A.col.p, B.ptr.p, B.col.p, nullptr, nullptr, nullptr}, C, W, &total));
    FE_CHECK(ex.alloc(C.val, (size_t)std::max<int64_t>(C.nnzb * C.rd * C.cd, 1)));
    PassProdVals vals{A.ptr.p, A.col.p, A.val.p, A.rd, A.cd, B.ptr.p, B.col.p, B.val.p, B.cd,
                      C.ptr.p, C.col.p, C.val.p};
    vals.boff = W.boff.p, vals.total = total, vals.upper = symmetric ? 1 : 0;
    FE_CHECK(ex.rows(A.n, vals));
    if (symmetric) FE_CHECK(ex.rows(A.n, PassMirrorLower{C.ptr.p, C.col.p, C.val.p, C.rd}));
    return FE_OK;
}

// Largest eigenvalue of D^-1 A from the Lanczos matrix of kLanczosSteps iterations of
// CG on A x = b preconditioned by D^-1, b_i = 1 + (i mod 7) / 7: the CG coefficients
// alpha_j, beta_j give the tridiagonal matrix (diagonal 1/alpha_j + beta_{j-1} /
// alpha_{j-1}, off-diagonal sqrt(beta_j) / alpha_j; Saad, Iterative Methods for Sparse
// Linear Systems, 6.7.3), whose largest eigenvalue lanczos_lmax finds.  Its Ritz value
// approaches lmax from below far faster than power iteration does.
constexpr int kLanczosSteps = 10;

// The Lanczos estimate's scalars, in executor memory so that the CG steps run without
// a read to the host: rz, rz0, p.q, r.z of the new residual, a stop flag, the steps done,
// then alpha_j and beta_j.
enum : int { kLzRz = 0, kLzRz0, kLzPq, kLzRzn, kLzStop, kLzM, kLzAlpha, kLzBeta = kLzAlpha + kLanczosSteps,
             kLzSize = kLzBeta + kLanczosSteps };

struct PassLanczosInit {
    double *S;
    FE_HD void operator()(int64_t) const {
        S[kLzRz0] = S[kLzRz];
        S[kLzStop] = S[kLzRz] > 0.0 ? 0.0 : 1.0;
        S[kLzM] = 0.0;
    }
};

// alpha_j = r.z / p.q; a product that is not positive stops the estimate
struct PassLanczosAlpha {
    double *S; int j;
    FE_HD void operator()(int64_t) const {
        if (S[kLzStop] != 0.0) return;
        const double pq = S[kLzPq];
        if (!(pq > 0.0) || !isfinite(pq)) {
            S[kLzStop] = 1.0;
            return;
        }
        S[kLzAlpha + j] = S[kLzRz] / pq;
    }
};

// r_i -= alpha_j q_i, then z_i = D_i^-1 r_i
struct PassLanczosStep {
    const double *S; int j; const double *q; const double *dinv; int d; double *r; double *z;
    FE_HD void operator()(int64_t i) const {
        if (S[kLzStop] != 0.0) return;
        PassCgStep{S[kLzAlpha + j], q, dinv, d, r, z}(i);
    }
};

// beta_j = r.z (new) / r.z; the estimate stops once the Krylov space is exhausted
struct PassLanczosBeta {
    double *S; int j;
    FE_HD void operator()(int64_t) const {
        if (S[kLzStop] != 0.0) return;
        const double rzn = S[kLzRzn];
        S[kLzBeta + j] = rzn / S[kLzRz];
        S[kLzM] = (double)(j + 1);
        S[kLzRz] = rzn;
        if (!(rzn > 1e-28 * S[kLzRz0])) S[kLzStop] = 1.0;
    }
};

struct PassLanczosDirection {
    const double *S; int j; const double *z; double *p;
    FE_HD void operator()(int64_t i) const {
        if (S[kLzStop] != 0.0) return;
        p[i] = z[i] + S[kLzBeta + j] * p[i];
    }
};

template <class Ex>
int lmax_of(Ex &ex, const Csr &A, const double *dinv, double *lmax) {
    const int d = A.rd;
    const int64_t nd = A.n * d;
    DBuf<double> r, z, p, q, S;
    struct Free {
        Ex &ex;
        DBuf<double> &r, &z, &p, &q, &S;
        ~Free() { ex.release(r), ex.release(z), ex.release(p), ex.release(q), ex.release(S); }
    } fr{ex, r, z, p, q, S};
    const size_t v = (size_t)std::max<int64_t>(nd, 1);
    FE_CHECK(ex.alloc(r, v));
    FE_CHECK(ex.alloc(z, v));
    FE_CHECK(ex.alloc(p, v));
    FE_CHECK(ex.alloc(q, v));
    FE_CHECK(ex.alloc(S, (size_t)kLzSize));
    FE_CHECK(ex.rows(nd, PassPowerStart{r.p}));
    FE_CHECK(ex.rows(A.n, PassJacobi{dinv, d, r.p, z.p}));
    FE_CHECK(ex.copy(p.p, z.p, (size_t)nd));
    FE_CHECK(ex.dot_to(r.p, z.p, nd, S.p + kLzRz));
    FE_CHECK(ex.rows(1, PassLanczosInit{S.p}));
    const PassDinvProduct prod{A.ptr.p, A.col.p, A.val.p, nullptr, d, p.p, q.p, A.nnzb};
    for (int j = 0; j < kLanczosSteps; ++j) {
        FE_CHECK(ex.rows(A.n, prod));
        FE_CHECK(ex.dot_to(p.p, q.p, nd, S.p + kLzPq));
        FE_CHECK(ex.rows(1, PassLanczosAlpha{S.p, j}));
        FE_CHECK(ex.rows(A.n, PassLanczosStep{S.p, j, q.p, dinv, d, r.p, z.p}));
        FE_CHECK(ex.dot_to(r.p, z.p, nd, S.p + kLzRzn));
        FE_CHECK(ex.rows(1, PassLanczosBeta{S.p, j}));
        if (j + 1 < kLanczosSteps) FE_CHECK(ex.rows(nd, PassLanczosDirection{S.p, j, z.p, p.p}));
    }
    double hs[kLzSize];
    FE_CHECK(ex.read(hs, S.p, (size_t)kLzSize));
    const int m = (int)hs[kLzM];
    *lmax = m > 0 ? lanczos_lmax(hs + kLzAlpha, hs + kLzBeta, m) : 0.0;
    if (!std::isfinite(*lmax) || !(*lmax > 0.0)) {
        set_error("multigrid setup: the largest eigenvalue estimate is not positive");
        return FE_BREAKDOWN;
    }
    return FE_OK;
}

// The hierarchy of A (consumed) with near-null space B (n d x m, consumed): levels down
// to at most coarse_dofs DOFs (or 12 levels); the coarsest operator in `coarse`.
// dinv0: level 0's block-diagonal inverse when the caller has it already.
template <class Ex>
int setup_hierarchy(Ex &ex, Csr A, DBuf<double> B, int m, double theta, int64_t coarse_dofs, std::vector<Level> &levels,
                    Csr &coarse, int *mis_rounds, const double *dinv0 = nullptr) {
    const int kMaxRounds = 256;
    DBuf<double> Bc, nrm, dg;
    DBuf<uint8_t> strong;
    DBuf<uint32_t> state;
    DBuf<uint64_t> key, m1, m2;
    DBuf<int32_t> rank, roots, agg1;
    DBuf<int64_t> roff;
    Work<Ex> W(ex);
    struct Free {
        Ex &ex;
        Csr &A;
        DBuf<double> &B, &Bc, &nrm, &dg;
        DBuf<uint8_t> &strong;
        DBuf<uint32_t> &state;
        DBuf<uint64_t> &key, &m1, &m2;
        DBuf<int32_t> &rank, &roots, &agg1;
        DBuf<int64_t> &roff;
        ~Free() {
            release(ex, A);
            ex.release(B), ex.release(Bc), ex.release(nrm), ex.release(dg), ex.release(strong), ex.release(state);
            ex.release(key), ex.release(m1), ex.release(m2), ex.release(rank), ex.release(roots), ex.release(agg1);
            ex.release(roff);
        }
    } fr{ex, A, B, Bc, nrm, dg, strong, state, key, m1, m2, rank, roots, agg1, roff};
    *mis_rounds = 0;
    while (A.n * A.rd > coarse_dofs && levels.size() < 12) {
        Level L;
        Csr Mem, Pt, AP, Ac;   // member lists, tentative prolongator, A P, Galerkin product
        struct LevelFree {
            Ex &ex;
            Level &L;
            Csr &Mem, &Pt, &AP, &Ac;
            ~LevelFree() { release(ex, L), release(ex, Mem), release(ex, Pt), release(ex, AP), release(ex, Ac); }
        } lf{ex, L, Mem, Pt, AP, Ac};
        const int dd = A.rd;
        const int64_t n = A.n;
        ex.phase(kPhaseDiag);
        FE_CHECK(ex.alloc(L.dinv, (size_t)std::max<int64_t>(n * dd * dd, 1)));
        if (levels.empty() && dinv0)
            FE_CHECK(ex.copy(L.dinv.p, dinv0, (size_t)(n * dd * dd)));
        else
            FE_CHECK(ex.rows(n, PassDinv{A.ptr.p, A.col.p, A.val.p, dd, L.dinv.p}));
        FE_CHECK(lmax_of(ex, A, L.dinv.p, &L.lmax));
        // strength and the distance-2 independent set
        ex.phase(kPhaseAggregate);
        FE_CHECK(ex.alloc(nrm, (size_t)std::max<int64_t>(A.nnzb, 1)));
        FE_CHECK(ex.alloc(strong, (size_t)std::max<int64_t>(A.nnzb, 1)));
        FE_CHECK(ex.alloc(dg, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.rows(n, PassBlockNorms{A.ptr.p, A.col.p, A.val.p, dd, nrm.p, dg.p}));
        FE_CHECK(ex.rows(n, PassStrength{A.ptr.p, A.col.p, nrm.p, dg.p, theta, strong.p}));
        FE_CHECK(ex.alloc(state, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.alloc(key, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.alloc(m1, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.alloc(m2, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.alloc(W.flag, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.alloc(roff, (size_t)n + 1));
        FE_CHECK(ex.rows(n, PassStateInit{state.p}));
        for (int round = 1;; ++round) {
            if (round > kMaxRounds) {
                set_error("multigrid setup: the independent set did not settle");
                return FE_BREAKDOWN;
            }
            FE_CHECK(ex.rows(n, PassMisKey{state.p, key.p}));
            FE_CHECK(ex.rows(n, PassMaxKey{A.ptr.p, A.col.p, strong.p, key.p, m1.p}));
            FE_CHECK(ex.rows(n, PassMaxKey{A.ptr.p, A.col.p, strong.p, m1.p, m2.p}));
            FE_CHECK(ex.rows(n, PassMisDecide{m2.p, state.p, W.flag.p}));
            int64_t undecided = 0;
            FE_CHECK(ex.scan(W.flag.p, n, roff.p, &undecided));
            ++*mis_rounds;
            if (undecided == 0) break;
        }
        // roots in node order, then the two joins
        FE_CHECK(ex.rows(n, PassRootFlags{state.p, W.flag.p}));
        int64_t na = 0;
        FE_CHECK(ex.scan(W.flag.p, n, roff.p, &na));
        if (na == 0) {
            set_error("multigrid setup: no aggregate root");
            return FE_BREAKDOWN;
        }
        FE_CHECK(ex.alloc(rank, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.alloc(roots, (size_t)na));
        FE_CHECK(ex.alloc(agg1, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.alloc(L.agg, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.rows(n, PassRoots{state.p, roff.p, rank.p, roots.p}));
        FE_CHECK(ex.rows(n, PassJoinRoot{A.ptr.p, A.col.p, strong.p, nrm.p, state.p, rank.p, agg1.p}));
        FE_CHECK(ex.rows(n, PassJoinNeighbour{A.ptr.p, A.col.p, strong.p, nrm.p, agg1.p, L.agg.p, W.flag.p}));
        int64_t left = 0;
        FE_CHECK(ex.scan(W.flag.p, n, roff.p, &left));
        if (left != 0) {
            set_error("multigrid setup: a node was left without an aggregate");
            return FE_BREAKDOWN;
        }
        // members of every aggregate in node order (rows = aggregates, no values)
        ex.phase(kPhaseTentative);
        Mem.n = na;
        FE_CHECK(ex.alloc(W.cnt, (size_t)na));
        FE_CHECK(ex.rows(na, PassZeroI64{W.cnt.p}));
        FE_CHECK(ex.rows(n, PassMemberCount{L.agg.p, W.cnt.p}));
        FE_CHECK(ex.alloc(Mem.ptr, (size_t)na + 1));
        FE_CHECK(ex.scan(W.cnt.p, na, Mem.ptr.p, &Mem.nnzb));
        FE_CHECK(ex.alloc(Mem.col, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.rows(na, PassZeroI64{W.cnt.p}));
        if (Mem.nnzb == n) {
            FE_CHECK(ex.rows(n, PassMemberScatter{L.agg.p, Mem.ptr.p, W.cnt.p, Mem.col.p}));
            FE_CHECK(ex.rows(na, PassSortRows{Mem.ptr.p, Mem.col.p}));
        }
        if (Mem.nnzb != n) {
            set_error("multigrid setup: aggregate members do not cover the nodes");
            return FE_BREAKDOWN;
        }
        // tentative prolongator: B's rows, one QR per aggregate in place
        Pt.n = n, Pt.rd = dd, Pt.cd = m, Pt.nnzb = n;
        FE_CHECK(ex.alloc(Pt.ptr, (size_t)n + 1));
        FE_CHECK(ex.alloc(Pt.col, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(ex.alloc(Pt.val, (size_t)std::max<int64_t>(n * dd * m, 1)));
        FE_CHECK(ex.rows(n + 1, PassIota{Pt.ptr.p}));
        FE_CHECK(ex.copy(Pt.col.p, L.agg.p, (size_t)n));
        FE_CHECK(ex.copy(Pt.val.p, B.p, (size_t)(n * dd * m)));
        FE_CHECK(ex.alloc(Bc, (size_t)std::max<int64_t>(na * m * m, 1)));
        FE_CHECK(ex.rows(na, PassQr{Mem.ptr.p, Mem.col.p, dd, m, Pt.val.p, Bc.p}));
        // P = P_t - w D^-1 A P_t
        ex.phase(kPhaseProlongator);
        FE_CHECK(product(ex, A, Pt, L.P, W));
        const double w = 4.0 / (3.0 * L.lmax);
        FE_CHECK(ex.rows(n, PassSmooth{L.P.ptr.p, L.P.col.p, L.P.val.p, L.dinv.p, Pt.val.p, L.agg.p, dd, m, w}));
        // restriction P^T and Galerkin product P^T (A P)
        ex.phase(kPhaseAP);
        FE_CHECK(product(ex, A, L.P, AP, W));
        ex.phase(kPhaseRestriction);
        L.PT.n = na, L.PT.rd = m, L.PT.cd = dd;
        // the pattern of P^T: the columns of (member lists) x A, as a product's
        FE_CHECK(distinct_rows(ex, na, PassProdBound{Mem.ptr.p, Mem.col.p, A.ptr.p, nullptr},
                               PassProdCols{Mem.ptr.p, Mem.col.p, A.ptr.p, A.col.p, nullptr, nullptr, nullptr}, L.PT,
                               W));
        FE_CHECK(ex.alloc(L.PT.val, (size_t)std::max<int64_t>(L.PT.nnzb * m * dd, 1)));
        FE_CHECK(ex.rows(na, PassRestrVals{L.PT.ptr.p, L.PT.col.p, L.PT.val.p, L.P.ptr.p, L.P.col.p, L.P.val.p, dd, m}));
        ex.phase(kPhaseGalerkin);
        FE_CHECK(product(ex, L.PT, AP, Ac, W, true));
        // the level keeps A; the next level starts from A_c and the coarse near-null space
        L.A = A;
        A = Ac;
        Ac = Csr();
        std::swap(B, Bc);
        levels.push_back(L);
        L = Level();
    }
    coarse = A;
    A = Csr();
    return FE_OK;
}

}  // namespace amg
}  // namespace fe
