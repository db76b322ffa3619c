// Setup of a smoothed-aggregation multigrid hierarchy (Vanek, Mandel and Brezina,
// Computing 56, 1996) on the host, from the node-block CSR of the eliminated system
// matrix: the stage before a device V-cycle preconditioner.
//
// Per level, with d x d blocks and a near-null space B (n d x m, the rigid-body modes
// on the fine level):
//   strength      block (i, j), i != j, is strong when sum|A_ij| >= theta sqrt(sum|A_ii| sum|A_jj|)
//   aggregation   in node order, a node whose strong neighbours are all free starts an
//                 aggregate with them; the nodes left join the aggregate of their first
//                 aggregated strong neighbour (in column order), else form a singleton
//   P_tent        per aggregate, the thin QR of B on its DOFs (modified Gram-Schmidt,
//                 non-negative diag(R), dropped columns kept as zeros); R is the
//                 coarse near-null space
//   P             (I - 4/(3 lmax) D^-1 A) P_tent, D^-1 the block-diagonal
//                 pseudo-inverse, lmax of D^-1 A from 10 CG-Lanczos steps from
//                 b_i = 1 + (i mod 7) / 7
//   A_c           P^T A P, m x m blocks
// down to at most `coarse_dofs` DOFs (or 12 levels).  Host code only: no device call.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "fe_amg.h"
#include "fe_amg_dev.h"
#include "fe_amg_par.cuh"
#include "fe_amg_cycle.cuh"
#include "fe_amg_passes.cuh"
#include "fe_amg_rows.cuh"
#include "fe_internal.h"

namespace fe {
namespace {

// Work split into a fixed number of chunks (independent of the thread count, so that
// chunked sums and concatenations are the same on every machine), run on up to
// hardware_concurrency threads.
constexpr int kChunks = 64;

template <typename F>
void parallel_chunks(int64_t n, F f) {
    const int nt = std::max(1, std::min<int>(kChunks, (int)std::thread::hardware_concurrency()));
    auto run = [&](int t) {
        for (int c = t; c < kChunks; c += nt) {
            const int64_t lo = n * c / kChunks, hi = n * (c + 1) / kChunks;
            f(lo, hi, c);
        }
    };
    if (nt == 1 || n < 4096) {
        run(0);
        if (nt > 1)
            for (int t = 1; t < nt; ++t) run(t);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(run, t);
    run(0);
    for (auto &x : th) x.join();
}

std::vector<double> block_diag_pinv(const BlockCsr &A) {
    const int d = A.rd;
    std::vector<double> dinv((size_t)A.n * d * d, 0.0);
    parallel_chunks(A.n, [&](int64_t lo, int64_t hi, int) {
        for (int64_t i = lo; i < hi; ++i)
            for (int64_t s = A.ptr[i]; s < A.ptr[i + 1]; ++s)
                if (A.col[s] == i) amg::sym_pinv(&A.val[(size_t)s * d * d], d, &dinv[(size_t)i * d * d]);
    });
    return dinv;
}

// Largest eigenvalue of D^-1 A: the Lanczos matrix of amg::kLanczosSteps CG iterations
// on A x = b preconditioned by D^-1, b_i = 1 + (i mod 7) / 7 (the sequence of
// amg::lmax_of); sums are taken per chunk and added in chunk order.
double lmax_lanczos(const BlockCsr &A, const std::vector<double> &dinv) {
    const int d = A.rd;
    const int64_t n = A.n, nd = n * d;
    std::vector<double> r((size_t)nd), z((size_t)nd), p((size_t)nd), q((size_t)nd);
    for (int64_t i = 0; i < nd; ++i) r[i] = 1.0 + (double)(i % 7) / 7.0;
    auto jacobi = [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) amg::PassJacobi{dinv.data(), d, r.data(), z.data()}(i);
    };
    auto dot = [&](const std::vector<double> &a, const std::vector<double> &b) {
        double part[kChunks];
        parallel_chunks(nd, [&](int64_t lo, int64_t hi, int c) {
            double t = 0.0;
            for (int64_t k = lo; k < hi; ++k) t += a[k] * b[k];
            part[c] = t;
        });
        double t = 0.0;
        for (int c = 0; c < kChunks; ++c) t += part[c];
        return t;
    };
    parallel_chunks(n, [&](int64_t lo, int64_t hi, int) { jacobi(lo, hi); });
    p = z;
    double rz = dot(r, z);
    const double rz0 = rz;
    double alpha[amg::kLanczosSteps], beta[amg::kLanczosSteps];
    int m = 0;
    for (int j = 0; j < amg::kLanczosSteps && rz > 0.0; ++j) {
        parallel_chunks(n, [&](int64_t lo, int64_t hi, int) {
            for (int64_t i = lo; i < hi; ++i)
                amg::row_dinv_product(A.ptr.data(), A.col.data(), A.val.data(), nullptr, d, p.data(), i, q.data());
        });
        const double pq = dot(p, q);
        if (!(pq > 0.0) || !std::isfinite(pq)) break;
        const double a = rz / pq;
        alpha[m] = a;
        parallel_chunks(n, [&](int64_t lo, int64_t hi, int) {
            for (int64_t i = lo; i < hi; ++i)
                amg::PassCgStep{a, q.data(), dinv.data(), d, r.data(), z.data()}(i);
        });
        const double rzn = dot(r, z);
        beta[m] = rzn / rz;
        ++m;
        rz = rzn;
        if (!(rzn > 1e-28 * rz0)) break;
        const double b = beta[m - 1];
        parallel_chunks(nd, [&](int64_t lo, int64_t hi, int) {
            for (int64_t k = lo; k < hi; ++k) p[k] = z[k] + b * p[k];
        });
    }
    return m > 0 ? lanczos_lmax(alpha, beta, m) : 0.0;
}

std::vector<int32_t> aggregate(const BlockCsr &A, double theta, int32_t *n_agg) {
    const int d = A.rd;
    const int64_t n = A.n;
    std::vector<double> nrm((size_t)A.nnzb()), dg((size_t)n, 0.0);
    for (int64_t s = 0; s < A.nnzb(); ++s) {
        double t = 0.0;
        for (int k = 0; k < d * d; ++k) t += std::fabs(A.val[(size_t)s * d * d + k]);
        nrm[s] = t;
    }
    for (int64_t i = 0; i < n; ++i)
        for (int64_t s = A.ptr[i]; s < A.ptr[i + 1]; ++s)
            if (A.col[s] == i) dg[i] = nrm[s];
    std::vector<int64_t> sptr((size_t)n + 1, 0);
    std::vector<int32_t> scol;
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t s = A.ptr[i]; s < A.ptr[i + 1]; ++s) {
            const int64_t j = A.col[s];
            if (j != i && nrm[s] >= theta * std::sqrt(dg[i] * dg[j])) scol.push_back((int32_t)j);
        }
        sptr[i + 1] = (int64_t)scol.size();
    }
    std::vector<int32_t> agg((size_t)n, -1);
    int32_t na = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        bool free_all = true;
        for (int64_t s = sptr[i]; s < sptr[i + 1] && free_all; ++s) free_all = agg[scol[s]] < 0;
        if (!free_all) continue;
        agg[i] = na;
        for (int64_t s = sptr[i]; s < sptr[i + 1]; ++s) agg[scol[s]] = na;
        ++na;
    }
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        int32_t a = -1;
        for (int64_t s = sptr[i]; s < sptr[i + 1] && a < 0; ++s)
            if (agg[scol[s]] >= 0) a = agg[scol[s]];
        agg[i] = a >= 0 ? a : na++;
    }
    *n_agg = na;
    return agg;
}

// Thin QR by modified Gram-Schmidt (k x m, column-major in Q), diag(R) >= 0, columns
// whose remainder is below 1e-12 of their norm dropped to zero.
void qr_mgs(const std::vector<double> &X, int k, int m, std::vector<double> &Q, double *R) {
    Q.assign((size_t)k * m, 0.0);
    for (int i = 0; i < m * m; ++i) R[i] = 0.0;
    std::vector<double> v((size_t)k);
    for (int j = 0; j < m; ++j) {
        double n0 = 0.0;
        for (int r = 0; r < k; ++r) v[r] = X[(size_t)r * m + j], n0 += v[r] * v[r];
        n0 = std::sqrt(n0);
        for (int i = 0; i < j; ++i) {
            double dot = 0.0;
            for (int r = 0; r < k; ++r) dot += Q[(size_t)i * k + r] * v[r];
            R[i * m + j] = dot;
            for (int r = 0; r < k; ++r) v[r] -= dot * Q[(size_t)i * k + r];
        }
        double nv = 0.0;
        for (int r = 0; r < k; ++r) nv += v[r] * v[r];
        nv = std::sqrt(nv);
        if (nv > 0.0 && nv > 1e-12 * std::max(n0, 1e-300)) {
            R[j * m + j] = nv;
            for (int r = 0; r < k; ++r) Q[(size_t)j * k + r] = v[r] / nv;
        }
    }
}

// C = A B for block CSR (A: ra x ca blocks, B: ca x cb blocks); columns sorted.  Rows
// are computed per chunk into chunk-local buffers, then concatenated in order.
BlockCsr spgemm(const BlockCsr &A, const BlockCsr &B, int64_t n_cols) {
    BlockCsr C;
    C.n = A.n, C.rd = A.rd, C.cd = B.cd;
    C.ptr.assign((size_t)A.n + 1, 0);
    const int ra = A.rd, ca = A.cd, cb = B.cd, bs = ra * cb;
    struct Part {
        std::vector<int32_t> col;
        std::vector<double> val;
        std::vector<int64_t> len;
    };
    std::vector<Part> parts(kChunks);
    parallel_chunks(A.n, [&](int64_t lo, int64_t hi, int c) {
        Part &pt = parts[c];
        std::vector<int64_t> slot((size_t)n_cols, -1);
        std::vector<int32_t> cols;
        std::vector<double> vals;
        std::vector<int> order;
        for (int64_t i = lo; i < hi; ++i) {
            cols.clear(), vals.clear();
            for (int64_t s = A.ptr[i]; s < A.ptr[i + 1]; ++s) {
                const int64_t j = A.col[s];
                const double *a = &A.val[(size_t)s * ra * ca];
                for (int64_t t = B.ptr[j]; t < B.ptr[j + 1]; ++t) {
                    const int32_t cc = B.col[t];
                    const double *b = &B.val[(size_t)t * ca * cb];
                    if (slot[cc] < 0) {
                        slot[cc] = (int64_t)cols.size();
                        cols.push_back(cc);
                        vals.resize(vals.size() + bs, 0.0);
                    }
                    double *o = &vals[(size_t)slot[cc] * bs];
                    for (int x = 0; x < ra; ++x)
                        for (int z = 0; z < cb; ++z) {
                            double acc = 0.0;
                            for (int y = 0; y < ca; ++y) acc += a[x * ca + y] * b[y * cb + z];
                            o[x * cb + z] += acc;
                        }
                }
            }
            order.resize(cols.size());
            for (size_t k = 0; k < order.size(); ++k) order[k] = (int)k;
            for (size_t k = 1; k < order.size(); ++k) {   // insertion sort: rows are short
                const int v = order[k];
                size_t m = k;
                while (m > 0 && cols[order[m - 1]] > cols[v]) order[m] = order[m - 1], --m;
                order[m] = v;
            }
            for (int k : order) {
                pt.col.push_back(cols[k]);
                pt.val.insert(pt.val.end(), vals.begin() + (size_t)k * bs, vals.begin() + (size_t)(k + 1) * bs);
                slot[cols[k]] = -1;
            }
            pt.len.push_back((int64_t)cols.size());
        }
    });
    int64_t row = 0;
    for (int c = 0; c < kChunks; ++c) {
        for (int64_t l : parts[c].len) C.ptr[row + 1] = C.ptr[row] + l, ++row;
        C.col.insert(C.col.end(), parts[c].col.begin(), parts[c].col.end());
        C.val.insert(C.val.end(), parts[c].val.begin(), parts[c].val.end());
    }
    return C;
}

// Block transpose: (n x n_cols blocks of rd x cd) -> (n_cols x n blocks of cd x rd)
BlockCsr transpose(const BlockCsr &A, int64_t n_cols) {
    BlockCsr T;
    T.n = n_cols, T.rd = A.cd, T.cd = A.rd;
    T.ptr.assign((size_t)n_cols + 1, 0);
    for (int32_t c : A.col) ++T.ptr[(size_t)c + 1];
    for (int64_t i = 0; i < n_cols; ++i) T.ptr[i + 1] += T.ptr[i];
    T.col.resize(A.col.size());
    T.val.resize(A.val.size());
    std::vector<int64_t> fill(T.ptr.begin(), T.ptr.end() - 1);
    const int bs = A.rd * A.cd;
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t s = A.ptr[i]; s < A.ptr[i + 1]; ++s) {
            const int64_t o = fill[A.col[s]]++;
            T.col[o] = (int32_t)i;
            for (int x = 0; x < A.rd; ++x)
                for (int z = 0; z < A.cd; ++z) T.val[(size_t)o * bs + z * A.rd + x] = A.val[(size_t)s * bs + x * A.cd + z];
        }
    return T;
}

// Dense inverse of a small matrix (row-major, n x n) by Gauss-Jordan with partial
// pivoting; false when a pivot vanishes.
bool dense_inverse(std::vector<double> a, int n, std::vector<double> &inv) {
    inv.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) inv[(size_t)i * n + i] = 1.0;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(a[(size_t)r * n + c]) > std::fabs(a[(size_t)p * n + c])) p = r;
        if (a[(size_t)p * n + c] == 0.0) return false;
        if (p != c)
            for (int k = 0; k < n; ++k) {
                std::swap(a[(size_t)p * n + k], a[(size_t)c * n + k]);
                std::swap(inv[(size_t)p * n + k], inv[(size_t)c * n + k]);
            }
        const double piv = a[(size_t)c * n + c];
        for (int k = 0; k < n; ++k) a[(size_t)c * n + k] /= piv, inv[(size_t)c * n + k] /= piv;
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = a[(size_t)r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                a[(size_t)r * n + k] -= f * a[(size_t)c * n + k];
                inv[(size_t)r * n + k] -= f * inv[(size_t)c * n + k];
            }
        }
    }
    return true;
}

}  // namespace
}  // namespace fe



namespace fe {

// Dense inverse of the coarsest matrix, shifted by 1e-12 of its largest diagonal entry
// (zero rows of rank-deficient aggregates).
int coarse_inverse_of(const BlockCsr &C, std::vector<double> &inv, const char *who) {
    const int64_t n = C.n * C.rd;
    if (n > 4096) {
        set_error(std::string(who) + ": coarsest level too large for its dense solve");
        return FE_BAD_INPUT;
    }
    std::vector<double> dense((size_t)n * n, 0.0);
    double dmax = 0.0;
    const int cd = C.rd;
    for (int64_t i = 0; i < C.n; ++i)
        for (int64_t s = C.ptr[i]; s < C.ptr[i + 1]; ++s)
            for (int a = 0; a < cd; ++a)
                for (int b = 0; b < cd; ++b) {
                    const double v = C.val[(size_t)s * cd * cd + a * cd + b];
                    dense[(size_t)(i * cd + a) * n + (int64_t)C.col[s] * cd + b] += v;
                }
    for (int64_t i = 0; i < n; ++i) dmax = std::max(dmax, std::fabs(dense[(size_t)i * n + i]));
    for (int64_t i = 0; i < n; ++i) dense[(size_t)i * n + i] += 1e-12 * dmax;
    if (n > 0 && !dense_inverse(dense, (int)n, inv)) {
        set_error(std::string(who) + ": singular coarsest matrix");
        return FE_BREAKDOWN;
    }
    return FE_OK;
}

}  // namespace fe

namespace fe {
namespace {

// k Chebyshev steps on D^-1 A z = D^-1 r over [1.05 lmax / 30, 1.05 lmax], from x0 (or
// zero): z_1 = x0 + D^-1 (r - A x0) / theta, then the three-term updates.
void chebyshev_host(const AmgLevel &L, int k, const std::vector<double> &r, std::vector<double> &z, bool from_x0) {
    const BlockCsr &A = L.A;
    const int d = A.rd;
    const int64_t n = A.n;
    const double hi = 1.05 * L.lmax, lo = hi / 30.0;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    if (!from_x0) z.assign((size_t)n * d, 0.0);
    std::vector<double> dir((size_t)n * d, 0.0), zn((size_t)n * d);
    double rho = 1.0 / sigma;
    for (int64_t i = 0; i < n; ++i)
        amg::row_chebyshev(A.ptr.data(), A.col.data(), A.val.data(), L.dinv.data(), d, r.data(), z.data(),
                           dir.data(), zn.data(), 0.0, 1.0 / theta, true, i);
    z.swap(zn);
    for (int s = 1; s < k; ++s) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        const double a = rn * rho, b = 2.0 * rn / delta;
        rho = rn;
        for (int64_t i = 0; i < n; ++i)
            amg::row_chebyshev(A.ptr.data(), A.col.data(), A.val.data(), L.dinv.data(), d, r.data(), z.data(),
                               dir.data(), zn.data(), a, b, false, i);
        z.swap(zn);
    }
}

void vcycle_host(const fe_amg_s *h, size_t l, int k, const std::vector<double> &r, std::vector<double> &x) {
    if (l == h->levels.size()) {
        const int64_t n = (int64_t)r.size();
        x.assign((size_t)n, 0.0);
        for (int64_t i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int64_t j = 0; j < n; ++j) acc += h->coarse_inv[(size_t)i * n + j] * r[j];
            x[i] = acc;
        }
        return;
    }
    const AmgLevel &L = h->levels[l];
    const BlockCsr &A = L.A;
    const int d = A.rd, m = L.P.cd;
    chebyshev_host(L, k, r, x, false);
    std::vector<double> t((size_t)A.n * d), rc((size_t)L.PT.n * m), xc;
    for (int64_t i = 0; i < A.n; ++i)
        amg::row_residual(A.ptr.data(), A.col.data(), A.val.data(), d, r.data(), x.data(), t.data(), i);
    for (int64_t I = 0; I < L.PT.n; ++I)
        amg::row_restrict(L.PT.ptr.data(), L.PT.col.data(), L.PT.val.data(), m, d, t.data(), rc.data(), I);
    vcycle_host(h, l + 1, k, rc, xc);
    for (int64_t i = 0; i < A.n; ++i)
        amg::row_prolong_add(L.P.ptr.data(), L.P.col.data(), L.P.val.data(), d, m, xc.data(), x.data(), i);
    chebyshev_host(L, k, r, x, true);
}


// Dense inverse of the coarsest matrix of h.
int coarse_inverse(fe_amg_s *h, const char *who) { return coarse_inverse_of(h->coarse, h->coarse_inv, who); }

// ---------------------------------------------------------------- parallel setup (host)
// amg::setup_hierarchy (fe_amg_passes.cuh), the device setup's sequence of passes, on
// a host executor: passes over row chunks on host threads, serial scans, dot products
// summed per chunk in chunk order.

struct HostEx {
    void mark(int) {}    // the device cycle's timing marks: nothing to time here
    void phase(int) {}   // nor the setup's phases
    template <class T>
    int alloc(DBuf<T> &b, size_t n) {
        if (b.p && b.n >= n) return FE_OK;
        std::free(b.p);
        b.p = (T *)std::malloc(std::max<size_t>(n, 1) * sizeof(T));
        b.n = b.p ? n : 0;
        if (!b.p) {
            set_error("multigrid setup: out of host memory");
            return FE_BAD_INPUT;
        }
        return FE_OK;
    }
    template <class T>
    void release(DBuf<T> &b) {
        std::free(b.p);
        b.p = nullptr;
        b.n = 0;
    }
    template <class T>
    int copy(T *dst, const T *src, size_t n) {
        if (n) std::memcpy(dst, src, n * sizeof(T));
        return FE_OK;
    }
    template <class T>
    int read(T *dst, const T *src, size_t n) {
        return copy(dst, src, n);
    }
    template <class T>
    int fill_zero(T *p, size_t n) {
        if (n) std::memset(p, 0, n * sizeof(T));
        return FE_OK;
    }
    template <class F>
    int rows(int64_t n, const F &f) {
        parallel_chunks(n, [&](int64_t lo, int64_t hi, int) {
            for (int64_t i = lo; i < hi; ++i) f(i);
        });
        return FE_OK;
    }
    int scan(const int64_t *in, int64_t n, int64_t *out, int64_t *total) {
        int64_t run = 0;
        for (int64_t i = 0; i < n; ++i) {
            const int64_t v = in[i];
            out[i] = run;
            run += v;
        }
        out[n] = run;
        *total = run;
        return FE_OK;
    }
    int dot_to(const double *a, const double *b, int64_t n, double *dst) { return dot(a, b, n, dst); }
    int dot(const double *a, const double *b, int64_t n, double *out) {
        double part[kChunks];
        for (int c = 0; c < kChunks; ++c) part[c] = 0.0;
        parallel_chunks(n, [&](int64_t lo, int64_t hi, int c) {
            double t = 0.0;
            for (int64_t i = lo; i < hi; ++i) t += a[i] * b[i];
            part[c] = t;
        });
        double t = 0.0;
        for (int c = 0; c < kChunks; ++c) t += part[c];
        *out = t;
        return FE_OK;
    }
};

BlockCsr to_block_csr(const amg::Csr &c) {
    BlockCsr H;
    H.n = c.n, H.rd = c.rd, H.cd = c.cd;
    H.ptr.assign(c.ptr.p, c.ptr.p + c.n + 1);
    H.col.assign(c.col.p, c.col.p + c.nnzb);
    H.val.assign(c.val.p, c.val.p + c.nnzb * c.rd * c.cd);
    return H;
}

// The hierarchy by the parallel passes on the host.  Returns FE_OK or a failure status.
int build_parallel(fe_amg_s *h, int64_t n, int d, const int64_t *ptr, const int32_t *col, const double *vals,
                   const double *nullspace, int m, double theta, int64_t coarse_dofs) {
    HostEx ex;
    amg::Csr A;
    DBuf<double> B;
    A.n = n, A.rd = A.cd = d, A.nnzb = ptr[n];
    int st = FE_OK;
    if ((st = ex.alloc(A.ptr, (size_t)n + 1)) || (st = ex.alloc(A.col, (size_t)std::max<int64_t>(A.nnzb, 1))) ||
        (st = ex.alloc(A.val, (size_t)std::max<int64_t>(A.nnzb * d * d, 1))) ||
        (st = ex.alloc(B, (size_t)std::max<int64_t>(n * d * m, 1)))) {
        amg::release(ex, A);
        ex.release(B);
        return st;
    }
    ex.copy(A.ptr.p, ptr, (size_t)n + 1);
    ex.copy(A.col.p, col, (size_t)A.nnzb);
    ex.copy(A.val.p, vals, (size_t)(A.nnzb * d * d));
    ex.copy(B.p, nullspace, (size_t)(n * d * m));
    std::vector<amg::Level> levels;
    amg::Csr coarse;
    int rounds = 0;
    st = amg::setup_hierarchy(ex, A, B, m, theta, coarse_dofs, levels, coarse, &rounds);
    for (auto &l : levels) {
        if (st == FE_OK) {
            AmgLevel L;
            L.A = to_block_csr(l.A), L.P = to_block_csr(l.P), L.PT = to_block_csr(l.PT);
            L.dinv.assign(l.dinv.p, l.dinv.p + l.A.n * l.A.rd * l.A.rd);
            L.agg.assign(l.agg.p, l.agg.p + l.A.n);
            L.lmax = l.lmax;
            h->levels.push_back(std::move(L));
        }
        amg::release(ex, l);
    }
    if (st != FE_OK) return st;
    h->coarse = to_block_csr(coarse);
    amg::release(ex, coarse);
    return coarse_inverse(h, "fe_amg_build_parallel_host");
}

}  // namespace
}  // namespace fe

using namespace fe;

extern "C" {

int fe_amg_build_host(int64_t n_nodes, int32_t d, const int64_t *blk_ptr, const int32_t *blk_col,
                      const double *vals, int32_t m, const double *nullspace, double theta, int64_t coarse_dofs,
                      fe_amg *out) {
    if (!out || n_nodes < 0 || d < 1 || d > 6 || m < 1 || m > 6 || (n_nodes > 0 && (!blk_ptr || !blk_col ||
                                                                                     !vals || !nullspace))) {
        set_error("fe_amg_build_host: bad arguments");
        return FE_BAD_INPUT;
    }
    *out = nullptr;
    fe_amg_s *h = new fe_amg_s();
    BlockCsr A;
    A.n = n_nodes, A.rd = A.cd = d;
    A.ptr.assign(blk_ptr, blk_ptr + n_nodes + 1);
    A.col.assign(blk_col, blk_col + A.ptr[n_nodes]);
    A.val.assign(vals, vals + (size_t)A.ptr[n_nodes] * d * d);
    std::vector<double> B(nullspace, nullspace + (size_t)n_nodes * d * m);
    int bm = m;
    while (A.n * A.rd > coarse_dofs && h->levels.size() < 12) {
        AmgLevel L;
        const int dd = A.rd;
        std::vector<double> dinv = block_diag_pinv(A);
        L.lmax = lmax_lanczos(A, dinv);
        int32_t na = 0;
        L.agg = aggregate(A, theta, &na);
        // tentative prolongator and coarse near-null space
        BlockCsr Pt;
        Pt.n = A.n, Pt.rd = dd, Pt.cd = bm;
        Pt.ptr.resize((size_t)A.n + 1);
        Pt.col.resize((size_t)A.n);
        Pt.val.assign((size_t)A.n * dd * bm, 0.0);
        for (int64_t i = 0; i <= A.n; ++i) Pt.ptr[i] = i;
        std::vector<double> Bc((size_t)na * bm * bm, 0.0);
        std::vector<std::vector<int64_t>> members((size_t)na);
        for (int64_t i = 0; i < A.n; ++i) members[L.agg[i]].push_back(i);
        std::vector<double> X, Q;
        for (int32_t a = 0; a < na; ++a) {
            const auto &nodes = members[a];
            const int k = (int)nodes.size() * dd;
            X.assign((size_t)k * bm, 0.0);
            for (size_t t = 0; t < nodes.size(); ++t)
                for (int c = 0; c < dd; ++c)
                    for (int j = 0; j < bm; ++j)
                        X[(t * dd + c) * bm + j] = B[((size_t)nodes[t] * dd + c) * bm + j];
            double R[36];
            qr_mgs(X, k, bm, Q, R);
            for (size_t t = 0; t < nodes.size(); ++t) {
                const int64_t i = nodes[t];
                Pt.col[i] = a;
                for (int c = 0; c < dd; ++c)
                    for (int j = 0; j < bm; ++j)
                        Pt.val[((size_t)i * dd + c) * bm + j] = Q[(size_t)j * k + t * dd + c];
            }
            for (int r = 0; r < bm * bm; ++r) Bc[(size_t)a * bm * bm + r] = R[r];
        }
        // smoothed prolongator P = P_tent - w D^-1 (A P_tent)
        BlockCsr AP = spgemm(A, Pt, na);
        const double w = 4.0 / (3.0 * L.lmax);
        BlockCsr P = AP;
        const int bs = dd * bm;
        parallel_chunks(A.n, [&](int64_t lo, int64_t hi, int) {
        for (int64_t i = lo; i < hi; ++i)
            for (int64_t s = P.ptr[i]; s < P.ptr[i + 1]; ++s) {
                double t[36];
                const double *di = &dinv[(size_t)i * dd * dd];
                for (int x = 0; x < dd; ++x)
                    for (int z = 0; z < bm; ++z) {
                        double acc = 0.0;
                        for (int y = 0; y < dd; ++y) acc += di[x * dd + y] * AP.val[(size_t)s * bs + y * bm + z];
                        t[x * bm + z] = -w * acc;
                    }
                if (P.col[s] == Pt.col[i])
                    for (int r = 0; r < bs; ++r) t[r] += Pt.val[(size_t)i * bs + r];
                for (int r = 0; r < bs; ++r) P.val[(size_t)s * bs + r] = t[r];
            }
        });
        // Galerkin coarse operator P^T (A P)
        BlockCsr APs = spgemm(A, P, na);
        BlockCsr PT = transpose(P, na);
        BlockCsr Ac = spgemm(PT, APs, na);
        L.A = std::move(A);
        L.P = std::move(P);
        L.PT = std::move(PT);
        L.dinv = std::move(dinv);
        h->levels.push_back(std::move(L));
        A = std::move(Ac);
        B.swap(Bc);
        (void)bm;
    }
    h->coarse = std::move(A);
    const int st = coarse_inverse(h, "fe_amg_build_host");
    if (st != FE_OK) {
        fe_amg_destroy(h);
        return st;
    }
    *out = h;
    return FE_OK;
}

// The same hierarchy inputs, set up by the parallel passes of the device setup
// (independent-set aggregation, row-wise products) run on the host.
int fe_amg_build_parallel_host(int64_t n_nodes, int32_t d, const int64_t *blk_ptr, const int32_t *blk_col,
                               const double *vals, int32_t m, const double *nullspace, double theta,
                               int64_t coarse_dofs, fe_amg *out) {
    if (!out || n_nodes < 0 || d < 1 || d > 6 || m < 1 || m > 6 || (n_nodes > 0 && (!blk_ptr || !blk_col ||
                                                                                     !vals || !nullspace))) {
        set_error("fe_amg_build_parallel_host: bad arguments");
        return FE_BAD_INPUT;
    }
    *out = nullptr;
    fe_amg_s *h = new fe_amg_s();
    const int st = build_parallel(h, n_nodes, d, blk_ptr, blk_col, vals, nullspace, m, theta, coarse_dofs);
    if (st != FE_OK) {
        fe_amg_destroy(h);
        return st;
    }
    *out = h;
    return FE_OK;
}

}  // extern "C"

namespace fe {
namespace {

// FP32 copies of a host hierarchy and its cycle vectors, viewed as the shared cycle
// (fe_amg_cycle.cuh) sees the device's.
struct HostCycle {
    std::vector<std::vector<float>> store;
    std::vector<amg::CycleLevel> levels;
    amg::CycleCoarse coarse;
    explicit HostCycle(const fe_amg_s *h) {
        auto f32 = [](const std::vector<double> &v) { return std::vector<float>(v.begin(), v.end()); };
        const size_t nl = h->levels.size();
        store.reserve(nl * 9 + 2);
        levels.resize(nl);
        for (size_t l = 0; l < nl; ++l) {
            const AmgLevel &H = h->levels[l];
            amg::CycleLevel &L = levels[l];
            L.n = H.A.n, L.d = H.A.rd, L.m = H.P.cd, L.lmax = H.lmax, L.nc = H.PT.n;
            L.aptr = H.A.ptr.data(), L.acol = H.A.col.data();
            L.pptr = H.P.ptr.data(), L.pcol = H.P.col.data();
            L.tptr = H.PT.ptr.data(), L.tcol = H.PT.col.data();
            store.push_back(f32(H.A.val)), L.a = store.back().data();
            store.push_back(f32(H.dinv)), L.dinv = store.back().data();
            store.push_back(f32(H.P.val)), L.p = store.back().data();
            store.push_back(f32(H.PT.val)), L.pt = store.back().data();
            float **vec[5] = {&L.r, &L.x, &L.t, &L.dir, &L.zn};
            for (float **v : vec) {
                store.emplace_back((size_t)std::max<int64_t>(L.n * L.d, 1), 0.0f);
                *v = store.back().data();
            }
        }
        coarse.n = h->coarse.n * h->coarse.rd;
        coarse.inv = h->coarse_inv.data();
        store.emplace_back((size_t)std::max<int64_t>(coarse.n, 1), 0.0f), coarse.r = store.back().data();
        store.emplace_back((size_t)std::max<int64_t>(coarse.n, 1), 0.0f), coarse.x = store.back().data();
    }
};

}  // namespace
}  // namespace fe

extern "C" {

// One V-cycle of the device's FP32 sequence (amg::precondition, fe_amg_cycle.cuh) run
// on the host: FP32 copies of the levels, r rounded to FP32, x widened to FP64.
int fe_amg_vcycle_host_f32(fe_amg h, int32_t k_smooth, const double *r, double *x) {
    if (!h || !r || !x || k_smooth < 1 || h->levels.empty()) {
        set_error("fe_amg_vcycle_host_f32: bad arguments");
        return FE_BAD_INPUT;
    }
    HostCycle c(h);
    HostEx ex;
    return amg::precondition(ex, c.levels, c.coarse, k_smooth, r, x);
}

// The device's multigrid PCG (amg::pcg around the FP32 cycle) run on the host, on the
// hierarchy's level-0 matrix: x from zero, to ||r|| <= tol ||b||.
int fe_amg_pcg_host(fe_amg h, int32_t k_smooth, const double *b, double tol, int32_t max_iter, double *x,
                    int32_t *iters, double *relres, int32_t *status) {
    if (!h || !b || !x || !iters || !relres || !status || k_smooth < 1 || h->levels.empty() || max_iter < 1) {
        set_error("fe_amg_pcg_host: bad arguments");
        return FE_BAD_INPUT;
    }
    HostCycle c(h);
    HostEx ex;
    const BlockCsr &A = h->levels[0].A;
    const size_t nd = (size_t)(A.n * A.rd);
    std::vector<double> r(nd), p(nd), q(nd), z(nd);
    const amg::PcgVectors v{x, r.data(), p.data(), q.data(), z.data()};
    auto precond = [&]() { return amg::precondition(ex, c.levels, c.coarse, k_smooth, v.r, v.z); };
    int it = 0, st = 0;
    FE_CHECK(amg::pcg(ex, A.n, A.rd, A.ptr.data(), A.col.data(), A.val.data(), b, v, precond, tol, max_iter, &it,
                      relres, &st));
    *iters = it, *status = st;
    return FE_OK;
}

// One V-cycle x = M^-1 r on the host (k Chebyshev steps before and after each coarse
// correction), the arithmetic of the device cycle row by row.
int fe_amg_vcycle_host(fe_amg h, int32_t k_smooth, const double *r, double *x) {
    if (!h || !r || !x || k_smooth < 1) {
        set_error("fe_amg_vcycle_host: bad arguments");
        return FE_BAD_INPUT;
    }
    const int64_t n = h->levels.empty() ? h->coarse.n * h->coarse.rd : h->levels[0].A.n * h->levels[0].A.rd;
    std::vector<double> rv(r, r + n), xv;
    vcycle_host(h, 0, k_smooth, rv, xv);
    std::copy(xv.begin(), xv.end(), x);
    return FE_OK;
}

int fe_amg_levels(fe_amg h, int32_t *n_levels) {
    if (!h || !n_levels) {
        set_error("fe_amg_levels: null argument");
        return FE_BAD_INPUT;
    }
    *n_levels = (int32_t)h->levels.size();
    return FE_OK;
}

// Level l < n_levels: its matrix and prolongator; l == n_levels: the coarsest matrix
// (no prolongator: nnzb_P = 0, n_coarse = 0).
int fe_amg_level_info(fe_amg h, int32_t l, int64_t *n_nodes, int32_t *d, int64_t *nnzb_A, int64_t *nnzb_P,
                      int64_t *n_coarse, int32_t *m, double *lmax) {
    if (!h || l < 0 || l > (int32_t)h->levels.size()) {
        set_error("fe_amg_level_info: bad level");
        return FE_BAD_INPUT;
    }
    const bool last = l == (int32_t)h->levels.size();
    const BlockCsr &A = last ? h->coarse : h->levels[l].A;
    if (n_nodes) *n_nodes = A.n;
    if (d) *d = A.rd;
    if (nnzb_A) *nnzb_A = A.nnzb();
    if (nnzb_P) *nnzb_P = last ? 0 : h->levels[l].P.nnzb();
    if (n_coarse) *n_coarse = last ? 0 : (l + 1 < (int32_t)h->levels.size() ? h->levels[l + 1].A.n : h->coarse.n);
    if (m) *m = last ? 0 : h->levels[l].P.cd;
    if (lmax) *lmax = last ? 0.0 : h->levels[l].lmax;
    return FE_OK;
}

int fe_amg_level_matrix(fe_amg h, int32_t l, int32_t which, int64_t *ptr, int32_t *col, double *val) {
    if (!h || l < 0 || l > (int32_t)h->levels.size() || (which == 1 && l == (int32_t)h->levels.size())) {
        set_error("fe_amg_level_matrix: bad level");
        return FE_BAD_INPUT;
    }
    const BlockCsr &M = which == 1 ? h->levels[l].P : (l == (int32_t)h->levels.size() ? h->coarse : h->levels[l].A);
    if (ptr) std::copy(M.ptr.begin(), M.ptr.end(), ptr);
    if (col) std::copy(M.col.begin(), M.col.end(), col);
    if (val) std::copy(M.val.begin(), M.val.end(), val);
    return FE_OK;
}

int fe_amg_level_aggregates(fe_amg h, int32_t l, int32_t *agg) {
    if (!h || !agg || l < 0 || l >= (int32_t)h->levels.size()) {
        set_error("fe_amg_level_aggregates: bad level");
        return FE_BAD_INPUT;
    }
    std::copy(h->levels[l].agg.begin(), h->levels[l].agg.end(), agg);
    return FE_OK;
}

int fe_amg_destroy(fe_amg h) {
    delete h;
    return FE_OK;
}

}  // extern "C"
