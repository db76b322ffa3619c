// Continuity conditions and additive right-hand-side entries.
//
// Continuity (conditions.py:196-241, analysis.py:175-199): u[dof1] = value * u[dof2],
// one Lagrange multiplier each.  The conditions link DOFs into trees (a condition that
// would close a cycle is refused); on a tree the admissible vectors are t * s, s the
// scale of each DOF relative to the tree's root.  The solve is a projected PCG in FP64
// (the operator P A P and the preconditioner P M^-1 P on the admissible subspace, P the
// orthogonal projector, tree by tree x_T <- s (s.x_T) / (s.s)), with A the
// Dirichlet-eliminated K and M^-1 its node-block Jacobi inverse.  The multipliers come
// from the first block row, F - K u = C^T mu, solved tree by tree from the leaves.
//
// Additive entries (analysis.py:556-577, :681-708): the magnet-load contributions,
// which create_source_matrix adds with += after the loads; per DOF they are added in
// list order.
#include <algorithm>
#include <cmath>
#include <functional>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "fe_internal.h"

namespace fe {
namespace {

constexpr int kCT = 256;

inline int grid_c(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kCT - 1) / kCT, 152 * 8)); }

// y = A x for the node-block CSR of A (one thread per block row)
template <int D>
__global__ void kc_spmv(int64_t n_nodes, const int32_t *__restrict__ ptr, const int32_t *__restrict__ col,
                        const double *__restrict__ val, const double *__restrict__ x, double *__restrict__ y) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_nodes;
         r += (int64_t)gridDim.x * blockDim.x) {
        double acc[D];
#pragma unroll
        for (int a = 0; a < D; ++a) acc[a] = 0.0;
        for (int s = ptr[r]; s < ptr[r + 1]; ++s) {
            const int64_t c = col[s];
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
                for (int b = 0; b < D; ++b) acc[a] = fma(val[(int64_t)s * D * D + a * D + b], x[c * D + b], acc[a]);
        }
#pragma unroll
        for (int a = 0; a < D; ++a) y[r * D + a] = acc[a];
    }
}

// v <- P v: on every tree T, v_T <- s_T (s_T . v_T) / (s_T . s_T)
__global__ void kc_project(int64_t n_comp, const int64_t *__restrict__ cptr, const int64_t *__restrict__ cdof,
                           const double *__restrict__ cs, double *__restrict__ v) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n_comp;
         c += (int64_t)gridDim.x * blockDim.x) {
        double sv = 0.0, ss = 0.0;
        for (int64_t k = cptr[c]; k < cptr[c + 1]; ++k) {
            sv = fma(cs[k], v[cdof[k]], sv);
            ss = fma(cs[k], cs[k], ss);
        }
        const double t = sv / ss;
        for (int64_t k = cptr[c]; k < cptr[c + 1]; ++k) v[cdof[k]] = cs[k] * t;
    }
}

// z = M^-1 r with the node-block Jacobi inverse
template <int D>
__global__ void kc_precond(int64_t n_nodes, const double *__restrict__ dinv, const double *__restrict__ r,
                           double *__restrict__ z) {
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < n_nodes;
         n += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double acc = 0.0;
#pragma unroll
            for (int b = 0; b < D; ++b) acc = fma(dinv[n * D * D + a * D + b], r[n * D + b], acc);
            z[n * D + a] = acc;
        }
    }
}

// Dot products, deterministic: per-block partial sums, then one block sums them in
// block order.  NV products a_k . b_k at once.
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double sh[kCT / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < kCT / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;
}

__global__ void kc_dot2(int64_t n, const double *__restrict__ a0, const double *__restrict__ b0,
                        const double *__restrict__ a1, const double *__restrict__ b1, double *__restrict__ part) {
    double s0 = 0.0, s1 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        s0 = fma(a0[i], b0[i], s0);
        if (a1) s1 = fma(a1[i], b1[i], s1);
    }
    s0 = block_sum(s0);
    s1 = block_sum(s1);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = s0;
        part[gridDim.x + blockIdx.x] = s1;
    }
}

// out[k] = sum of the nb partials of product k; with keep_old, out[4] takes the old
// out[0] first (r.z of the previous iteration, for beta)
__global__ void kc_dot_final(int nb, const double *__restrict__ part, int nv, double *__restrict__ out, int keep_old) {
    for (int k = 0; k < nv; ++k) {
        double s = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[k * nb + i];
        s = block_sum(s);
        if (threadIdx.x == 0) {
            if (keep_old && k == 0) out[4] = out[0];
            out[k] = s;
        }
    }
}

// scalars: [0] r.z, [1] r.r, [2] p.q, [4] previous r.z
__global__ void kc_update(int64_t n, const double *__restrict__ sc, const double *__restrict__ p,
                          const double *__restrict__ q, double *__restrict__ x, double *__restrict__ r) {
    const double alpha = sc[0] / sc[2];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fma(alpha, p[i], x[i]);
        r[i] = fma(-alpha, q[i], r[i]);
    }
}

// r = b - q (q = A x)
__global__ void kc_update_r(int64_t n, const double *__restrict__ b, const double *__restrict__ q,
                            double *__restrict__ r) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = b[i] - q[i];
}

__global__ void kc_direction(int64_t n, const double *__restrict__ sc, const double *__restrict__ z,
                             double *__restrict__ p) {
    const double beta = sc[0] / sc[4];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fma(beta, p[i], z[i]);
}

// w_k = (F - K u)[dof_k] for the listed DOFs
template <int D>
__global__ void kc_residual_at(int64_t n, const int64_t *__restrict__ dofs, const int32_t *__restrict__ ptr,
                               const int32_t *__restrict__ col, const double *__restrict__ kval,
                               const double *__restrict__ F, const double *__restrict__ u, double *__restrict__ w) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = dofs[k], r = d / D;
        const int a = (int)(d - r * D);
        double acc = F[d];
        for (int s = ptr[r]; s < ptr[r + 1]; ++s) {
            const int64_t c = col[s];
#pragma unroll
            for (int b = 0; b < D; ++b) acc -= kval[(int64_t)s * D * D + a * D + b] * u[c * D + b];
        }
        w[k] = acc;
    }
}

// F[add_dof[k]] += add_val[add_ptr[k]], += add_val[add_ptr[k] + 1], ... in order
__global__ void kc_rhs_add(int64_t n, const int64_t *__restrict__ dof, const int64_t *__restrict__ ptr,
                           const double *__restrict__ val, int64_t n_dof, double *__restrict__ F, int *err) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = dof[k];
        if (d < 0 || d >= n_dof) {
            atomicOr(err, ERR_DOF_RANGE);
            continue;
        }
        double f = F[d];
        for (int64_t j = ptr[k]; j < ptr[k + 1]; ++j) f = __dadd_rn(f, val[j]);
        F[d] = f;
    }
}

template <int D>
int projected_pcg(fe_handle_s *h, const fe_solve_opts *o, fe_solve_stats *st) {
    cudaStream_t s = h->stream;
    const int64_t n = h->n_dof, nn = h->n_nodes;
    const int gn = grid_c(n), gnn = grid_c(nn), gc = grid_c(h->n_comp);
    DBuf<double> r, z, p, q, part, sc;
    struct Free {
        DBuf<double> *b[6];
        ~Free() {
            for (auto *x : b) dfree(*x);
        }
    } guard{{&r, &z, &p, &q, &part, &sc}};
    const size_t nv = (size_t)std::max<int64_t>(n, 1);
    FE_CHECK(dalloc(h->w.x, nv));
    FE_CHECK(dalloc(r, nv));
    FE_CHECK(dalloc(z, nv));
    FE_CHECK(dalloc(p, nv));
    FE_CHECK(dalloc(q, nv));
    FE_CHECK(dalloc(part, 2 * (size_t)gn));
    FE_CHECK(dalloc(sc, 8));
    double *x = h->w.x.p;
    auto project = [&](double *v) -> int {
        if (h->n_comp > 0) {
            kc_project<<<gc, kCT, 0, s>>>(h->n_comp, h->comp_ptr.p, h->comp_dof.p, h->comp_s.p, v);
            FE_LAUNCH_CHECK();
            h->launches += 1;
        }
        return FE_OK;
    };
    auto dots = [&](const double *a0, const double *b0, const double *a1, const double *b1, double *out,
                    int keep_old) -> int {
        kc_dot2<<<gn, kCT, 0, s>>>(n, a0, b0, a1, b1, part.p);
        kc_dot_final<<<1, kCT, 0, s>>>(gn, part.p, a1 ? 2 : 1, out, keep_old);
        FE_LAUNCH_CHECK();
        h->launches += 2;
        return FE_OK;
    };
    auto precond = [&]() -> int {
        kc_precond<D><<<gnn, kCT, 0, s>>>(nn, h->dinv.p, r.p, z.p);
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return project(z.p);
    };
    // x = 0, r = P b, z = P M^-1 r, p = z
    FE_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    FE_CUDA(cudaMemcpyAsync(r.p, h->b.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    FE_CHECK(project(r.p));
    FE_CHECK(precond());
    FE_CUDA(cudaMemcpyAsync(p.p, z.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    FE_CHECK(dots(r.p, z.p, r.p, r.p, sc.p, 0));   // sc[0] = r.z, sc[1] = r.r
    double host[8];
    FE_CUDA(cudaMemcpyAsync(host, sc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    const double bb = host[1];
    const double tol = o->tol > 0 ? o->tol : 1e-10;
    const int max_iter = o->max_iter > 0 ? o->max_iter : 200000;
    st->bnorm = std::sqrt(bb);
    int it = 0, status = FE_MAXITER;
    double rr = bb;
    if (!(bb > 0.0)) {
        status = std::isfinite(bb) ? FE_OK : FE_NONFINITE;
        rr = 0.0;
    }
    // stagnation: no halving of the best residual over 400 iterations ends the loop,
    // as converged with FE_SOLVE_ACCEPT_STAGNATION, else as FE_MAXITER
    const bool accept_stag = (o->flags & FE_SOLVE_ACCEPT_STAGNATION) != 0;
    double best = rr;
    int best_it = 0;
    bool stalled = false;
    // convergence is read back every 16 iterations
    while (status == FE_MAXITER && it < max_iter && !stalled) {
        const int batch = std::min(16, max_iter - it);
        for (int k = 0; k < batch; ++k) {
            kc_spmv<D><<<gnn, kCT, 0, s>>>(nn, h->blk_ptr.p, h->blk_col.p, h->aval.p, p.p, q.p);
            FE_LAUNCH_CHECK();
            h->launches += 1;
            FE_CHECK(project(q.p));
            FE_CHECK(dots(p.p, q.p, nullptr, nullptr, sc.p + 2, 0));
            kc_update<<<gn, kCT, 0, s>>>(n, sc.p, p.p, q.p, x, r.p);
            FE_LAUNCH_CHECK();
            FE_CHECK(precond());
            FE_CHECK(dots(r.p, z.p, r.p, r.p, sc.p, 1));
            kc_direction<<<gn, kCT, 0, s>>>(n, sc.p, z.p, p.p);
            FE_LAUNCH_CHECK();
            h->launches += 3;
        }
        it += batch;
        FE_CUDA(cudaMemcpyAsync(host, sc.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        rr = host[1];
        if (!std::isfinite(rr) || !std::isfinite(host[0])) {
            status = FE_NONFINITE;
        } else if (rr <= tol * tol * bb) {
            status = FE_OK;
        } else if (!(host[2] > 0.0) || !(host[0] > 0.0)) {
            status = FE_BREAKDOWN;
        } else if (rr < 0.25 * best) {
            best = rr, best_it = it;
        } else if (it - best_it >= 400) {
            stalled = true;
            if (accept_stag) status = FE_OK;
        }
    }
    // the reported residual is the true one, P (b - A x), recomputed in FP64
    double relres = 0.0;
    if (bb > 0.0 && status != FE_NONFINITE) {
        kc_spmv<D><<<gnn, kCT, 0, s>>>(nn, h->blk_ptr.p, h->blk_col.p, h->aval.p, x, q.p);
        FE_LAUNCH_CHECK();
        kc_update_r<<<gn, kCT, 0, s>>>(n, h->b.p, q.p, r.p);
        FE_LAUNCH_CHECK();
        h->launches += 2;
        FE_CHECK(project(r.p));
        FE_CHECK(dots(r.p, r.p, nullptr, nullptr, sc.p + 5, 0));
        FE_CUDA(cudaMemcpyAsync(host, sc.p + 5, sizeof(double), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        relres = std::sqrt(std::max(host[0], 0.0) / bb);
    }
    st->iterations = it;
    st->spmv = it + 1;
    st->outer = 0;
    st->relres = relres;
    st->status = status;
    return FE_OK;
}

// Multipliers of the continuity conditions: F - K u = C^T mu on the DOFs of every
// tree, from the leaves to the root (a DOF's multiplier row holds 1 at dof1 and
// -value at dof2).
int continuity_multipliers(fe_handle_s *h) {
    const int64_t m = (int64_t)h->comp_dof_h.size();
    h->mu_host.assign((size_t)h->n_cont, 0.0);
    if (m == 0) return FE_OK;
    DBuf<double> w;
    FE_CHECK(dalloc(w, (size_t)m));
    int st = with_dim(h->dim, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        kc_residual_at<D><<<grid_c(m), kCT, 0, h->stream>>>(m, h->comp_dof.p, h->blk_ptr.p, h->blk_col.p,
                                                             h->kval.p, h->F.p, h->w.x.p, w.p);
        return cudaGetLastError() == cudaSuccess ? FE_OK : FE_CUDA_ERR;
    });
    std::vector<double> wh((size_t)m);
    if (!st && cudaMemcpyAsync(wh.data(), w.p, m * sizeof(double), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
        st = FE_CUDA_ERR;
    if (!st && cudaStreamSynchronize(h->stream) != cudaSuccess) st = FE_CUDA_ERR;
    dfree(w);
    if (st) return st;
    h->launches += 1;
    std::unordered_map<int64_t, int64_t> pos;   // DOF -> its slot in comp_dof
    for (int64_t k = 0; k < m; ++k) pos[h->comp_dof_h[k]] = k;
    for (int64_t c = 0; c < h->n_comp; ++c) {
        // BFS order: every DOF after its parent, so the reverse visits leaves first
        for (int64_t k = h->comp_ptr_h[c + 1] - 1; k > h->comp_ptr_h[c]; --k) {
            const int64_t e = h->comp_edge_h[k], d = h->comp_dof_h[k];
            const double cd = d == h->cont_d1[e] ? 1.0 : -h->cont_v[e];
            const double mu = wh[k] / cd;
            h->mu_host[e] = mu;
            const int64_t parent = d == h->cont_d1[e] ? h->cont_d2[e] : h->cont_d1[e];
            const double cp = parent == h->cont_d1[e] ? 1.0 : -h->cont_v[e];
            wh[pos[parent]] -= cp * mu;
        }
    }
    return FE_OK;
}

}  // namespace

int set_continuity(fe_handle_s *h, int64_t n, const int64_t *d1, const int64_t *d2, const double *v) {
    if (n < 0 || (n > 0 && (!d1 || !d2 || !v))) {
        set_error("fe_set_continuity: bad condition list");
        return FE_BAD_INPUT;
    }
    std::vector<int64_t> a(d1, d1 + n), b(d2, d2 + n);
    std::vector<double> val(v, v + n);
    // union-find over the linked DOFs; a condition joining two DOFs already linked
    // closes a cycle (redundant or conflicting conditions)
    std::unordered_map<int64_t, int64_t> parent;
    std::function<int64_t(int64_t)> find = [&](int64_t x) {
        while (parent[x] != x) x = parent[x] = parent[parent[x]];
        return x;
    };
    for (int64_t k = 0; k < n; ++k) {
        if (a[k] < 0 || a[k] >= h->n_dof || b[k] < 0 || b[k] >= h->n_dof) {
            set_error("fe_set_continuity: DOF out of range");
            return FE_BAD_INPUT;
        }
        if (!(std::isfinite(val[k]) && val[k] != 0.0)) {
            set_error("fe_set_continuity: the value of a condition must be finite and non-zero");
            return FE_BAD_INPUT;
        }
        for (int64_t d : {a[k], b[k]})
            if (!parent.count(d)) parent[d] = d;
        const int64_t ra = find(a[k]), rb = find(b[k]);
        if (ra == rb) {
            set_error("fe_set_continuity: the conditions link a DOF to itself through a cycle (redundant or "
                      "conflicting conditions)");
            return FE_BAD_INPUT;
        }
        parent[ra] = rb;
    }
    // trees in order of first appearance, breadth first from the first DOF seen
    std::unordered_map<int64_t, std::vector<int64_t>> adj;   // DOF -> incident conditions
    std::vector<int64_t> first;
    for (int64_t k = 0; k < n; ++k)
        for (int64_t d : {a[k], b[k]}) {
            if (!adj.count(d)) first.push_back(d);
            adj[d].push_back(k);
        }
    std::unordered_map<int64_t, double> scale;
    std::vector<int64_t> cptr{0}, cdof, cedge;
    std::vector<double> cs;
    for (int64_t root : first) {
        if (scale.count(root)) continue;
        scale[root] = 1.0;
        size_t head = cdof.size();
        cdof.push_back(root);
        cedge.push_back(-1);
        cs.push_back(1.0);
        while (head < cdof.size()) {
            const int64_t d = cdof[head++];
            for (int64_t k : adj[d]) {
                const int64_t o = d == a[k] ? b[k] : a[k];
                if (scale.count(o)) continue;
                // u[a] = value * u[b]
                const double so = d == a[k] ? scale[d] / val[k] : scale[d] * val[k];
                scale[o] = so;
                cdof.push_back(o);
                cedge.push_back(k);
                cs.push_back(so);
            }
        }
        cptr.push_back((int64_t)cdof.size());
    }
    h->n_cont = n;
    h->cont_d1 = std::move(a);
    h->cont_d2 = std::move(b);
    h->cont_v = std::move(val);
    h->comp_ptr_h = cptr;
    h->comp_dof_h = cdof;
    h->comp_edge_h = cedge;
    h->comp_s_h = cs;
    h->n_comp = (int64_t)cptr.size() - 1;
    h->mu_host.assign((size_t)n, 0.0);
    FE_CHECK(dalloc(h->comp_ptr, cptr.size()));
    FE_CHECK(dalloc(h->comp_dof, std::max<size_t>(cdof.size(), 1)));
    FE_CHECK(dalloc(h->comp_s, std::max<size_t>(cs.size(), 1)));
    FE_CUDA(cudaMemcpyAsync(h->comp_ptr.p, cptr.data(), cptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                            h->stream));
    if (!cdof.empty()) {
        FE_CUDA(cudaMemcpyAsync(h->comp_dof.p, cdof.data(), cdof.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                                h->stream));
        FE_CUDA(cudaMemcpyAsync(h->comp_s.p, cs.data(), cs.size() * sizeof(double), cudaMemcpyHostToDevice,
                                h->stream));
    }
    FE_CUDA(cudaStreamSynchronize(h->stream));
    h->have_solution = false;
    return FE_OK;
}

int solve_continuity(fe_handle_s *h, const fe_solve_opts *o, fe_solve_stats *st) {
    // a linked DOF that is also Dirichlet-constrained is not supported: with two such
    // DOFs on one tree the reference's saddle-point matrix is singular, with one its
    // value fixes the whole tree
    std::unordered_map<int64_t, int> linked;
    for (int64_t d : h->comp_dof_h) linked[d] = 1;
    for (int64_t d : h->bc_dof_host)
        if (linked.count(d)) {
            set_error("fe_solve: a DOF with a continuity condition also has a Dirichlet condition");
            return FE_BAD_INPUT;
        }
    FE_CUDA(cudaEventRecord(h->events[6], h->stream));
    FE_CHECK(with_dim(h->dim, [&](auto dc) { return projected_pcg<decltype(dc)::value>(h, o, st); }));
    FE_CHECK(recover_multipliers(h));
    FE_CHECK(continuity_multipliers(h));
    FE_CUDA(cudaEventRecord(h->events[7], h->stream));
    FE_CUDA(cudaEventSynchronize(h->events[7]));
    float ms = 0;
    FE_CUDA(cudaEventElapsedTime(&ms, h->events[6], h->events[7]));
    st->solve_ms = ms;
    st->assemble_ms = h->last_assemble_ms;
    h->have_solution = true;
    return FE_OK;
}

int set_rhs_additions(fe_handle_s *h, int64_t n, const int64_t *dof, const double *value) {
    if (n < 0 || (n > 0 && (!dof || !value))) {
        set_error("fe_set_rhs_additions: bad list");
        return FE_BAD_INPUT;
    }
    // group by DOF, keeping list order within a DOF
    std::vector<int64_t> order((size_t)n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t i, int64_t j) { return dof[i] < dof[j]; });
    std::vector<int64_t> udof, ptr{0};
    std::vector<double> val;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t i = order[k];
        if (k == 0 || dof[i] != dof[order[k - 1]]) {
            if (k > 0) ptr.push_back(k);
            udof.push_back(dof[i]);
        }
        val.push_back(value[i]);
    }
    if (n > 0) ptr.push_back(n);
    h->n_add_dofs = (int64_t)udof.size();
    FE_CHECK(dalloc(h->add_dof, std::max<size_t>(udof.size(), 1)));
    FE_CHECK(dalloc(h->add_ptr, ptr.size()));
    FE_CHECK(dalloc(h->add_val, std::max<size_t>(val.size(), 1)));
    if (n > 0) {
        FE_CUDA(cudaMemcpyAsync(h->add_dof.p, udof.data(), udof.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                                h->stream));
        FE_CUDA(cudaMemcpyAsync(h->add_ptr.p, ptr.data(), ptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                                h->stream));
        FE_CUDA(cudaMemcpyAsync(h->add_val.p, val.data(), val.size() * sizeof(double), cudaMemcpyHostToDevice,
                                h->stream));
    }
    FE_CUDA(cudaStreamSynchronize(h->stream));
    h->f_ready = h->sys_ready = false;
    return FE_OK;
}

int apply_rhs_additions(fe_handle_s *h) {
    if (h->n_add_dofs == 0) return FE_OK;
    kc_rhs_add<<<grid_c(h->n_add_dofs), kCT, 0, h->stream>>>(h->n_add_dofs, h->add_dof.p, h->add_ptr.p,
                                                               h->add_val.p, h->n_dof, h->F.p, h->err.p);
    FE_LAUNCH_CHECK();
    h->launches += 1;
    return FE_OK;
}

}  // namespace fe

using namespace fe;

extern "C" {

int fe_set_continuity(fe_handle h, int64_t n, const int64_t *dof1_host, const int64_t *dof2_host,
                      const double *value_host) {
    if (!h) {
        set_error("fe_set_continuity: null handle");
        return FE_BAD_INPUT;
    }
    return set_continuity(h, n, dof1_host, dof2_host, value_host);
}

int fe_set_rhs_additions(fe_handle h, int64_t n, const int64_t *dof_host, const double *value_host) {
    if (!h) {
        set_error("fe_set_rhs_additions: null handle");
        return FE_BAD_INPUT;
    }
    return set_rhs_additions(h, n, dof_host, value_host);
}

}  // extern "C"
