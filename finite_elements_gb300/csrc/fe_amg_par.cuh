// Row operations of the parallel smoothed-aggregation setup, shared by the host executor
// (fe_amg_setup.cu, fe_amg_build_parallel_host) and the device setup: every function
// computes one row (or one aggregate) from arrays that the pass does not write, so a
// pass is a loop over rows in any order and its result does not depend on the order.
//
//   strength      block 1-norms ||A_ij||_1 >= theta sqrt(||A_ii||_1 ||A_jj||_1)
//   aggregation   distance-2 maximal independent set of the strong graph (Bell, Dalton
//                 and Olson, "Exposing fine-grained parallelism in algebraic multigrid
//                 methods", SIAM J. Sci. Comput. 34, 2012): rounds in which an undecided
//                 node enters the set when its (state, hash, index) key is the largest
//                 within two strong hops; then every node joins the strongest root next
//                 to it, and the rest the strongest neighbour that joined
//   prolongator   one thin QR of the near-null-space rows per aggregate (modified
//                 Gram-Schmidt, diag(R) >= 0), smoothed by P = P_t - w D^-1 A P_t
//   products      row-wise sparse products: candidate columns, heap sort, unique, then
//                 the values accumulated in the order of the factors' entries
#pragma once

#include <math.h>
#include <stdint.h>

#include "fe_amg_rows.cuh"

namespace fe {
namespace amg {

// ------------------------------------------------------------------ small helpers

// Integer hash "lowbias32" (C. Wellons, hash-prospector, public domain): the random
// priority of a node in the independent-set rounds.
FE_HD uint32_t node_hash(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

// Independent-set states, ordered so that a member of the set dominates every key.
constexpr uint32_t kOut = 0, kUndecided = 1, kIn = 2;

FE_HD uint64_t mis_key(uint32_t state, int64_t i) {
    return ((uint64_t)state << 62) | ((uint64_t)(node_hash((uint32_t)i) >> 2) << 32) | (uint64_t)(uint32_t)i;
}

// In-place heap sort of a[0..n), ascending.
FE_HD void heap_sort(int32_t *a, int64_t n) {
    auto sift = [&](int64_t root, int64_t end) {
        while (true) {
            int64_t c = 2 * root + 1;
            if (c >= end) return;
            if (c + 1 < end && a[c + 1] > a[c]) ++c;
            if (a[root] >= a[c]) return;
            const int32_t t = a[root];
            a[root] = a[c];
            a[c] = t;
            root = c;
        }
    };
    for (int64_t s = n / 2 - 1; s >= 0; --s) sift(s, n);
    for (int64_t e = n - 1; e > 0; --e) {
        const int32_t t = a[0];
        a[0] = a[e];
        a[e] = t;
        sift(0, e);
    }
}

// Atomic add on an int64 counter, on the device and on the host executor's threads;
// returns the old value.
FE_HD int64_t atomic_add_i64(int64_t *p, int64_t v) {
#ifdef __CUDA_ARCH__
    return (int64_t)atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
#else
    return __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
#endif
}

// Sort a[0..n) and drop repeats; returns the number of distinct values.
FE_HD int64_t sort_unique(int32_t *a, int64_t n) {
    if (n <= 1) return n;
    heap_sort(a, n);
    int64_t u = 1;
    for (int64_t k = 1; k < n; ++k)
        if (a[k] != a[u - 1]) a[u++] = a[k];
    return u;
}

// Position of value v in the sorted a[lo..hi), or -1.
FE_HD int64_t find_sorted(const int32_t *a, int64_t lo, int64_t hi, int32_t v) {
    const int64_t end = hi;
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return (lo < end && a[lo] == v) ? lo : -1;
}

// ------------------------------------------------------------------ block inverses

// Inverse of a symmetric D x D block: by Cholesky when it is positive definite (every
// pivot above 1e-12 of the largest diagonal entry), else the pseudo-inverse by cyclic
// Jacobi, V diag(1/l) V^T over the eigenvalues above 1e-12 of the largest in magnitude.  The sweeps stop once the
// off-diagonal part is below 1e-30 of the block's squared Frobenius norm (rounding
// level; Jacobi converges quadratically, a few sweeps), or after 60.  D is a template
// argument so that the block and its eigenvectors stay in registers.
template <int D>
FE_HD void sym_pinv_n(const double *a, double *out) {
    // positive definite blocks (nearly all of them): the inverse by Cholesky, when every
    // pivot is above 1e-12 of the largest diagonal entry; the Jacobi pseudo-inverse below
    // otherwise (blocks of dropped near-null-space columns are singular)
    {
        double dmax = 0.0;
        for (int i = 0; i < D; ++i) dmax = fabs(a[i * D + i]) > dmax ? fabs(a[i * D + i]) : dmax;
        double L[D * D];
        bool ok = dmax > 0.0;
        for (int j = 0; j < D && ok; ++j) {
            double s = a[j * D + j];
            for (int k = 0; k < j; ++k) s -= L[j * D + k] * L[j * D + k];
            if (!(s > 1e-12 * dmax)) {
                ok = false;
                break;
            }
            const double l = sqrt(s);
            L[j * D + j] = l;
            for (int i = j + 1; i < D; ++i) {
                double t = a[i * D + j];
                for (int k = 0; k < j; ++k) t -= L[i * D + k] * L[j * D + k];
                L[i * D + j] = t / l;
            }
        }
        if (ok) {
            // W = L^-1 (lower), then out = W^T W
            double W[D * D];
            for (int i = 0; i < D * D; ++i) W[i] = 0.0;
            for (int c = 0; c < D; ++c) {
                W[c * D + c] = 1.0 / L[c * D + c];
                for (int i = c + 1; i < D; ++i) {
                    double t = 0.0;
                    for (int k = c; k < i; ++k) t += L[i * D + k] * W[k * D + c];
                    W[i * D + c] = -t / L[i * D + i];
                }
            }
            for (int i = 0; i < D; ++i)
                for (int j = 0; j < D; ++j) {
                    double t = 0.0;
                    for (int k = (i > j ? i : j); k < D; ++k) t += W[k * D + i] * W[k * D + j];
                    out[i * D + j] = t;
                }
            return;
        }
    }
    double A[D * D], V[D * D];
    double fro = 0.0;
    for (int i = 0; i < D * D; ++i) A[i] = a[i], fro += a[i] * a[i];
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) V[i * D + j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < D; ++p)
            for (int q = p + 1; q < D; ++q) off += A[p * D + q] * A[p * D + q];
        if (off <= 1e-30 * fro) break;
        for (int p = 0; p < D; ++p)
            for (int q = p + 1; q < D; ++q) {
                const double apq = A[p * D + q];
                if (apq == 0.0) continue;
                const double th = (A[q * D + q] - A[p * D + p]) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < D; ++k) {
                    const double akp = A[k * D + p], akq = A[k * D + q];
                    A[k * D + p] = c * akp - s * akq;
                    A[k * D + q] = s * akp + c * akq;
                }
                for (int k = 0; k < D; ++k) {
                    const double apk = A[p * D + k], aqk = A[q * D + k];
                    A[p * D + k] = c * apk - s * aqk;
                    A[q * D + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < D; ++k) {
                    const double vkp = V[k * D + p], vkq = V[k * D + q];
                    V[k * D + p] = c * vkp - s * vkq;
                    V[k * D + q] = s * vkp + c * vkq;
                }
            }
    }
    double lmax = 0.0;
    for (int i = 0; i < D; ++i) lmax = fabs(A[i * D + i]) > lmax ? fabs(A[i * D + i]) : lmax;
    for (int i = 0; i < D * D; ++i) out[i] = 0.0;
    for (int k = 0; k < D; ++k) {
        const double l = A[k * D + k];
        if (fabs(l) <= 1e-12 * lmax || l == 0.0) continue;
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j) out[i * D + j] += V[i * D + k] * V[j * D + k] / l;
    }
}

// the same for the block sizes of the hierarchies (1, 2, 3, 6); other sizes get zeros
FE_HD void sym_pinv(const double *a, int d, double *out) {
    switch (d) {
        case 1: sym_pinv_n<1>(a, out); return;
        case 2: sym_pinv_n<2>(a, out); return;
        case 3: sym_pinv_n<3>(a, out); return;
        case 4: sym_pinv_n<4>(a, out); return;
        case 5: sym_pinv_n<5>(a, out); return;
        case 6: sym_pinv_n<6>(a, out); return;
        default:
            for (int i = 0; i < d * d; ++i) out[i] = 0.0;
    }
}

// y_i = D_i^-1 (A x)_i (d x d blocks); y = A x when dinv is null
FE_HD void row_dinv_product(const int64_t *ptr, const int32_t *col, const double *val, const double *dinv, int d,
                            const double *x, int64_t i, double *y) {
    double acc[6];
    row_product(ptr, col, val, d, d, x, i, acc);
    if (!dinv) {   // y = A x
        for (int a = 0; a < d; ++a) y[i * d + a] = acc[a];
        return;
    }
    for (int a = 0; a < d; ++a) {
        double v = 0.0;
        for (int k = 0; k < d; ++k) v += dinv[i * d * d + a * d + k] * acc[k];
        y[i * d + a] = v;
    }
}

// ------------------------------------------------------------------ strength

// ||A_s||_1 (sum of absolute entries) of every block slot of row i; dg[i] = that of the
// diagonal block.
FE_HD void row_block_norms(const int64_t *ptr, const int32_t *col, const double *val, int d, int64_t i,
                           double *nrm, double *dg) {
    double diag = 0.0;
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s) {
        double t = 0.0;
        for (int k = 0; k < d * d; ++k) t += fabs(val[s * d * d + k]);
        nrm[s] = t;
        if (col[s] == i) diag = t;
    }
    dg[i] = diag;
}

// strong[s] = 1 for the off-diagonal slots of row i that pass the strength test
FE_HD void row_strength(const int64_t *ptr, const int32_t *col, const double *nrm, const double *dg, double theta,
                        int64_t i, uint8_t *strong) {
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s) {
        const int64_t j = col[s];
        strong[s] = (j != i && nrm[s] >= theta * sqrt(dg[i] * dg[j])) ? 1 : 0;
    }
}

// ------------------------------------------------------------------ independent set

// out[i] = the largest of in[i] and in[j] over the strong neighbours j of i
FE_HD void row_max_key(const int64_t *ptr, const int32_t *col, const uint8_t *strong, const uint64_t *in, int64_t i,
                       uint64_t *out) {
    uint64_t m = in[i];
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s)
        if (strong[s] && in[col[s]] > m) m = in[col[s]];
    out[i] = m;
}

// One round's decision for node i from m2 = the largest key within two strong hops:
// its own key -> in the set; a set member's key -> out; else undecided.  Returns 1 if
// i is still undecided.
FE_HD int mis_decide(const uint64_t *m2, int64_t i, uint32_t *state) {
    if (state[i] != kUndecided) return 0;
    const uint64_t own = mis_key(kUndecided, i);
    if (m2[i] == own) {
        state[i] = kIn;
        return 0;
    }
    if ((m2[i] >> 62) == kIn) {
        state[i] = kOut;
        return 0;
    }
    return 1;
}

// ------------------------------------------------------------------ aggregates

// First join: a root keeps its own aggregate; another node joins the root among its
// strong neighbours with the largest block norm (ties: the smaller index), or stays -1.
FE_HD void row_join_root(const int64_t *ptr, const int32_t *col, const uint8_t *strong, const double *nrm,
                         const uint32_t *state, const int32_t *root_rank, int64_t i, int32_t *agg) {
    if (state[i] == kIn) {
        agg[i] = root_rank[i];
        return;
    }
    int32_t best = -1;
    int64_t bj = -1;
    double bn = -1.0;
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s) {
        const int64_t j = col[s];
        if (!strong[s] || state[j] != kIn) continue;
        if (nrm[s] > bn || (nrm[s] == bn && j < bj)) bn = nrm[s], bj = j, best = root_rank[j];
    }
    agg[i] = best;
}

// Second join: a node left out joins the aggregate of its strong neighbour, assigned in
// the first join, with the largest block norm (ties: the smaller index).
FE_HD void row_join_neighbour(const int64_t *ptr, const int32_t *col, const uint8_t *strong, const double *nrm,
                              const int32_t *agg1, int64_t i, int32_t *agg2) {
    if (agg1[i] >= 0) {
        agg2[i] = agg1[i];
        return;
    }
    int32_t best = -1;
    int64_t bj = -1;
    double bn = -1.0;
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s) {
        const int64_t j = col[s];
        if (!strong[s] || agg1[j] < 0) continue;
        if (nrm[s] > bn || (nrm[s] == bn && j < bj)) bn = nrm[s], bj = j, best = agg1[j];
    }
    agg2[i] = best;
}

// Thin QR of the aggregate's near-null-space rows, in place: on entry pt[(i d + a) m + b]
// holds B of member i (rows a < d, columns b < m), on exit the orthonormal factor Q
// (columns whose remainder falls below 1e-12 of their norm set to zero); R (m x m,
// diag >= 0) is the aggregate's coarse near-null-space block.
FE_HD void aggregate_qr(const int32_t *members, int64_t cnt, int d, int m, double *pt, double *R) {
    for (int k = 0; k < m * m; ++k) R[k] = 0.0;
    for (int j = 0; j < m; ++j) {
        double n0 = 0.0;
        for (int64_t t = 0; t < cnt; ++t)
            for (int a = 0; a < d; ++a) {
                const double v = pt[((int64_t)members[t] * d + a) * m + j];
                n0 += v * v;
            }
        n0 = sqrt(n0);
        for (int q = 0; q < j; ++q) {
            double dot = 0.0;
            for (int64_t t = 0; t < cnt; ++t)
                for (int a = 0; a < d; ++a) {
                    const double *row = &pt[((int64_t)members[t] * d + a) * m];
                    dot += row[q] * row[j];
                }
            R[q * m + j] = dot;
            for (int64_t t = 0; t < cnt; ++t)
                for (int a = 0; a < d; ++a) {
                    double *row = &pt[((int64_t)members[t] * d + a) * m];
                    row[j] -= dot * row[q];
                }
        }
        double nv = 0.0;
        for (int64_t t = 0; t < cnt; ++t)
            for (int a = 0; a < d; ++a) {
                const double v = pt[((int64_t)members[t] * d + a) * m + j];
                nv += v * v;
            }
        nv = sqrt(nv);
        const bool keep = nv > 0.0 && nv > 1e-12 * (n0 > 1e-300 ? n0 : 1e-300);
        if (keep) R[j * m + j] = nv;
        for (int64_t t = 0; t < cnt; ++t)
            for (int a = 0; a < d; ++a) {
                double *v = &pt[((int64_t)members[t] * d + a) * m + j];
                *v = keep ? *v / nv : 0.0;
            }
    }
}

// ------------------------------------------------------------------ sparse products

// Number of block products of row i of C = A B (an upper bound on the row's length).
FE_HD int64_t row_product_bound(const int64_t *aptr, const int32_t *acol, const int64_t *bptr, int64_t i) {
    int64_t b = 0;
    for (int64_t s = aptr[i]; s < aptr[i + 1]; ++s) b += bptr[acol[s] + 1] - bptr[acol[s]];
    return b;
}

// The distinct columns of row i of C = A B, sorted, in cand[] (row_product_bound
// entries); returns their count.
// Rows of A with at most kMergeA entries merge the sorted B rows they select (one cursor
// each) instead of gathering and sorting: row_product_columns and row_product_values.
constexpr int kMergeA = 16;

FE_HD int64_t row_product_columns(const int64_t *aptr, const int32_t *acol, const int64_t *bptr, const int32_t *bcol,
                                  int64_t i, int32_t *cand) {
    const int64_t a0 = aptr[i], la = aptr[i + 1] - a0;
    if (la <= kMergeA) {
        int64_t cur[kMergeA], end[kMergeA];
        for (int64_t q = 0; q < la; ++q) {
            const int64_t j = acol[a0 + q];
            cur[q] = bptr[j], end[q] = bptr[j + 1];
        }
        int64_t n = 0;
        for (;;) {
            int32_t m = 0;
            bool any = false;
            for (int64_t q = 0; q < la; ++q)
                if (cur[q] < end[q] && (!any || bcol[cur[q]] < m)) m = bcol[cur[q]], any = true;
            if (!any) return n;
            cand[n++] = m;
            for (int64_t q = 0; q < la; ++q)
                if (cur[q] < end[q] && bcol[cur[q]] == m) ++cur[q];
        }
    }
    int64_t n = 0;
    for (int64_t s = a0; s < a0 + la; ++s)
        for (int64_t t = bptr[acol[s]]; t < bptr[acol[s] + 1]; ++t) cand[n++] = bcol[t];
    return sort_unique(cand, n);
}

// Values of row i of C = A B on its sorted columns ccol[cptr[i] .. cptr[i+1]): each
// block product (ra x ca times ca x cb) added in the order of A's and then B's entries.
// o += a b for an ra x ca block a and a ca x cb block b, every product fused into the
// accumulator (ca FP64 FMAs per entry of o, no separate additions: these products are
// bound by the FP64 rate).  The device's warp-per-row products use the same sequence.
FE_HD void block_mul_add(const double *a, const double *b, int ra, int ca, int cb, double *o) {
    for (int x = 0; x < ra; ++x)
        for (int z = 0; z < cb; ++z) {
            double acc = o[x * cb + z];
            for (int y = 0; y < ca; ++y) acc = fma(a[x * ca + y], b[y * cb + z], acc);
            o[x * cb + z] = acc;
        }
}

// Row i of C = A B (upper: only the entries whose block column is at least i, for a
// product known to be symmetric; the others are left for PassMirrorLower).  C's row is
// the union of the B rows that A's row selects, all sorted, so the entries are produced
// in column order by a merge: one cursor per entry of A's row into its B row, and each
// entry summed in registers over A's entries in order (the order of a term-by-term
// accumulation, without a search or a read-modify-write per term).  RA, CA, CB: the
// block sizes when known at compile time (0: ra, ca, cb).  Rows of more than kMergeA
// entries of A take the term-by-term path.

template <int RA, int CA, int CB>
FE_HD void row_product_values_t(const int64_t *aptr, const int32_t *acol, const double *aval, int ra_, int ca_,
                                const int64_t *bptr, const int32_t *bcol, const double *bval, int cb_,
                                const int64_t *cptr, const int32_t *ccol, double *cval, int64_t i, bool upper) {
    const int ra = RA ? RA : ra_, ca = CA ? CA : ca_, cb = CB ? CB : cb_;
    const int bs = ra * cb;
    const int64_t a0 = aptr[i], la = aptr[i + 1] - a0;
    if (la <= kMergeA) {
        int64_t cur[kMergeA], end[kMergeA];
        for (int64_t q = 0; q < la; ++q) {
            const int64_t j = acol[a0 + q];
            cur[q] = bptr[j], end[q] = bptr[j + 1];
        }
        for (int64_t p = cptr[i]; p < cptr[i + 1]; ++p) {
            const int32_t c = ccol[p];
            if (upper && c < i) continue;   // filled by the mirror pass; cursors move on below
            double acc[RA && CB ? RA * CB : 36];
            for (int k = 0; k < bs; ++k) acc[k] = 0.0;
            for (int64_t q = 0; q < la; ++q) {
                int64_t t = cur[q];
                while (t < end[q] && bcol[t] < c) ++t;
                if (t < end[q] && bcol[t] == c) {
                    block_mul_add(&aval[(a0 + q) * ra * ca], &bval[t * ca * cb], ra, ca, cb, acc);
                    ++t;
                }
                cur[q] = t;
            }
            double *o = &cval[p * bs];
            for (int k = 0; k < bs; ++k) o[k] = acc[k];
        }
        return;
    }
    for (int64_t k = cptr[i] * bs; k < cptr[i + 1] * bs; ++k) cval[k] = 0.0;
    for (int64_t s = a0; s < a0 + la; ++s) {
        const double *a = &aval[s * ra * ca];
        const int64_t j = acol[s];
        for (int64_t t = bptr[j]; t < bptr[j + 1]; ++t) {
            if (upper && bcol[t] < i) continue;
            const int64_t p = find_sorted(ccol, cptr[i], cptr[i + 1], bcol[t]);
            if (p < 0) continue;   // cannot happen: the columns come from these products
            block_mul_add(a, &bval[t * ca * cb], ra, ca, cb, &cval[p * bs]);
        }
    }
}

FE_HD void row_product_values(const int64_t *aptr, const int32_t *acol, const double *aval, int ra, int ca,
                              const int64_t *bptr, const int32_t *bcol, const double *bval, int cb,
                              const int64_t *cptr, const int32_t *ccol, double *cval, int64_t i,
                              bool upper = false) {
    row_product_values_t<0, 0, 0>(aptr, acol, aval, ra, ca, bptr, bcol, bval, cb, cptr, ccol, cval, i, upper);
}

// The lower entries of a symmetric product row: block (i, j), j < i, is the transpose
// of block (j, i).
FE_HD void row_mirror_lower(const int64_t *ptr, const int32_t *col, double *val, int m, int64_t i) {
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s) {
        const int64_t j = col[s];
        if (j >= i) break;   // columns are sorted
        const int64_t q = find_sorted(col, ptr[j], ptr[j + 1], i);
        if (q < 0) continue;   // cannot happen: the pattern of a symmetric product is symmetric
        for (int x = 0; x < m; ++x)
            for (int z = 0; z < m; ++z) val[s * m * m + x * m + z] = val[q * m * m + z * m + x];
    }
}

// Smoothing of row i of the prolongator, in place on the row of A P_t:
// P_i = P_t,i - w D_i^-1 (A P_t)_i, with P_t,i (d x m) on the column agg[i].
FE_HD void row_smooth_prolongator(const int64_t *pptr, const int32_t *pcol, double *pval, const double *dinv,
                                  const double *ptent, const int32_t *agg, int d, int m, double w, int64_t i) {
    const int bs = d * m;
    const double *di = &dinv[i * d * d];
    for (int64_t s = pptr[i]; s < pptr[i + 1]; ++s) {
        double t[36];
        double *v = &pval[s * bs];
        for (int x = 0; x < d; ++x)
            for (int z = 0; z < m; ++z) {
                double acc = 0.0;
                for (int y = 0; y < d; ++y) acc += di[x * d + y] * v[y * m + z];
                t[x * m + z] = -w * acc;
            }
        if (pcol[s] == agg[i])
            for (int r = 0; r < bs; ++r) t[r] += ptent[i * bs + r];
        for (int r = 0; r < bs; ++r) v[r] = t[r];
    }
}

// Rows of the restriction P^T: row c holds the nodes i whose prolongator row has the
// column c, i.e. (A's pattern being symmetric) the neighbours of c's members -- the
// columns of the product (member lists) x A, found with the product passes.

// Values of row c of P^T: the transposed block (m x d) of P at (i, c) for every column i.
FE_HD void row_restriction_values(const int64_t *rptr, const int32_t *rcol, double *rval, const int64_t *pptr,
                                  const int32_t *pcol, const double *pval, int d, int m, int64_t c) {
    for (int64_t s = rptr[c]; s < rptr[c + 1]; ++s) {
        const int64_t i = rcol[s];
        const int64_t p = find_sorted(pcol, pptr[i], pptr[i + 1], (int32_t)c);
        double *o = &rval[s * m * d];
        if (p < 0) {
            for (int k = 0; k < m * d; ++k) o[k] = 0.0;
            continue;
        }
        const double *b = &pval[p * d * m];
        for (int x = 0; x < d; ++x)
            for (int z = 0; z < m; ++z) o[z * d + x] = b[x * m + z];
    }
}

}  // namespace amg
}  // namespace fe
