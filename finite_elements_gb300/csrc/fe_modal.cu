// Modal analysis: generalized eigenpairs K v = lambda M v of the assembled
// stiffness and mass (no Dirichlet conditions: modal_analysis works on
// k_matrix_sparse / m_matrix_sparse, finite_elements/analysis.py:741-796).
//
// Lanczos in the M inner product on an operator T that is self-adjoint there:
//   smallest: T = (K - sigma M)^-1 M, shift sigma < 0 below the spectrum of the
//             positive semidefinite K, so K - sigma M is SPD and each step is one PCG
//             solve with the library's solver; theta = 1 / (lambda - sigma) puts the
//             smallest lambda (rigid-body zeros included) at the top of T's spectrum;
//   largest:  T = M^-1 K, each step one PCG solve with M; theta = lambda.
// The basis is kept on the device and re-orthogonalized in full against every earlier
// vector, twice (classical Gram-Schmidt twice), which keeps the projected matrix
// tridiagonal to rounding.  The small tridiagonal matrix is diagonalized on the host
// (cyclic Jacobi rotations); Ritz vectors are formed on the device and their true
// residuals ||K x - lambda M x|| / (||K x|| + max(|lambda|, |lambda|_max) ||M x||)
// reported (|lambda|_max over the k computed: a rigid-body zero is measured against
// the spectrum's scale, not against its own rounding).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "fe_internal.h"

namespace fe {
namespace {

constexpr int kMT = 256;

// y = A x for a node-block CSR matrix (FP64 values [nnzb][D][D]).
template <int D>
__global__ void __launch_bounds__(kMT)
km_bsr_spmv(int64_t n_nodes, const int32_t *__restrict__ ptr, const int32_t *__restrict__ col,
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

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double sh[kMT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < kMT / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;   // valid in thread 0
}

// part[i][blockIdx.x] = partial sum of V_i . y over this block's rows (grid: x = parts,
// y = vectors); deterministic (fixed partition, fixed order).
__global__ void __launch_bounds__(kMT)
km_dots(int64_t n, const double *__restrict__ V, int64_t ld, const double *__restrict__ y, double *__restrict__ part) {
    const double *v = V + blockIdx.y * ld;
    double acc = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        acc = fma(v[r], y[r], acc);
    const double t = block_sum(acc);
    if (threadIdx.x == 0) part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
}

__global__ void __launch_bounds__(kMT) km_dots_final(int parts, const double *__restrict__ part, double *__restrict__ out) {
    double acc = 0.0;
    for (int p = threadIdx.x; p < parts; p += blockDim.x) acc += part[(int64_t)blockIdx.x * parts + p];
    const double t = block_sum(acc);
    if (threadIdx.x == 0) out[blockIdx.x] = t;
}

// w += sign * sum_i V_i c_i (c on the device, nv entries)
__global__ void __launch_bounds__(kMT)
km_gemv(int64_t n, int nv, const double *__restrict__ V, int64_t ld, const double *__restrict__ c, double sign,
        double *__restrict__ w) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int i = 0; i < nv; ++i) acc = fma(V[i * ld + r], c[i], acc);
        w[r] = fma(sign, acc, w[r]);
    }
}

// y = s x; also called in place (y == x), so the pointers are not restrict-qualified
__global__ void __launch_bounds__(kMT) km_scale(int64_t n, const double *x, double s, double *y) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        y[r] = s * x[r];
}

// deterministic pseudo-random start vector in [-1, 1) (splitmix64 of the index)
__global__ void __launch_bounds__(kMT) km_start(int64_t n, double *__restrict__ v) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long z = (unsigned long long)r + 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        v[r] = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    }
}

// a smooth, non-rigid test field for the automatic shift: ((x - xmin) / L)^2 in every
// component
__global__ void __launch_bounds__(kMT)
km_smooth(int64_t n_nodes, int D, int cdim, const double *__restrict__ coords, double xmin, double inv_len,
          double *__restrict__ v) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_nodes;
         r += (int64_t)gridDim.x * blockDim.x) {
        const double t = (coords[cdim * r] - xmin) * inv_len;
        for (int a = 0; a < D; ++a) v[r * D + a] = t * t;
    }
}

inline int grid1(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kMT - 1) / kMT, 152 * 16)); }

struct Modal {
    fe_handle_s *h;
    int64_t n;
    // scratch owned by this call: the Lanczos basis V (m + 1 vectors), work vectors,
    // reduction partials; freed on every exit
    DBuf<double> part, cdev, tmp, V, w, Mw, Kx;
    std::vector<double> chost;
    int parts = 1;

    ~Modal() {
        dfree(part), dfree(cdev), dfree(tmp), dfree(V), dfree(w), dfree(Mw), dfree(Kx);
    }

    int spmv(const DBuf<double> &A, const double *x, double *y) {
        FE_CHECK(with_dim(h->dim, [&](auto dc) {
            constexpr int D = decltype(dc)::value;
            km_bsr_spmv<D><<<grid1(h->n_nodes), kMT, 0, h->stream>>>(h->n_nodes, h->blk_ptr.p, h->blk_col.p, A.p, x, y);
            return FE_OK;
        }));
        FE_LAUNCH_CHECK();
        h->launches += 1;
        return FE_OK;
    }
    // chost[0..nv) = V_i . y
    int dots(const double *V, int64_t ld, int nv, const double *y) {
        km_dots<<<dim3(parts, nv), kMT, 0, h->stream>>>(n, V, ld, y, part.p);
        km_dots_final<<<nv, kMT, 0, h->stream>>>(parts, part.p, cdev.p);
        FE_LAUNCH_CHECK();
        h->launches += 2;
        chost.resize(nv);
        FE_CUDA(cudaMemcpyAsync(chost.data(), cdev.p, nv * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
        return FE_OK;
    }
    int dot(const double *x, const double *y, double *out) {
        FE_CHECK(dots(x, 0, 1, y));
        *out = chost[0];
        return FE_OK;
    }
};

// Eigen-decomposition of the symmetric m x m matrix a (row-major, overwritten) by
// cyclic Jacobi rotations: eigenvalues in w, eigenvectors in the columns of v.
void jacobi_eigen(int m, std::vector<double> &a, std::vector<double> &w, std::vector<double> &v) {
    v.assign((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i) v[(size_t)i * m + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int p = 0; p < m; ++p) {
            diag += a[(size_t)p * m + p] * a[(size_t)p * m + p];
            for (int q = p + 1; q < m; ++q) off += a[(size_t)p * m + q] * a[(size_t)p * m + q];
        }
        if (off <= 1e-30 * diag || off == 0.0) break;
        for (int p = 0; p < m; ++p)
            for (int q = p + 1; q < m; ++q) {
                const double apq = a[(size_t)p * m + q];
                if (apq == 0.0) continue;
                const double app = a[(size_t)p * m + p], aqq = a[(size_t)q * m + q];
                // rotation that zeroes a_pq: tan of the angle is the smaller root of
                // t^2 + 2 zeta t - 1 = 0, zeta = (a_qq - a_pp) / (2 a_pq)
                const double zeta = (aqq - app) / (2.0 * apq);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(zeta * zeta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < m; ++r) {
                    const double arp = a[(size_t)r * m + p], arq = a[(size_t)r * m + q];
                    a[(size_t)r * m + p] = c * arp - s * arq;
                    a[(size_t)r * m + q] = s * arp + c * arq;
                }
                for (int r = 0; r < m; ++r) {
                    const double apr = a[(size_t)p * m + r], aqr = a[(size_t)q * m + r];
                    a[(size_t)p * m + r] = c * apr - s * aqr;
                    a[(size_t)q * m + r] = s * apr + c * aqr;
                }
                for (int r = 0; r < m; ++r) {
                    const double vrp = v[(size_t)r * m + p], vrq = v[(size_t)r * m + q];
                    v[(size_t)r * m + p] = c * vrp - s * vrq;
                    v[(size_t)r * m + q] = s * vrp + c * vrq;
                }
            }
    }
    w.resize(m);
    for (int i = 0; i < m; ++i) w[i] = a[(size_t)i * m + i];
}

}  // namespace

int modal(fe_handle_s *h, int which, int k, double sigma, int steps, int precision, double *eigvals,
          double *eigvecs, double *resid) {
    const int64_t n = h->n_dof;
    if (!h->k_ready || !h->m_ready) {
        set_error("fe_modal: assemble K and M first (FE_ASSEMBLE_K | FE_ASSEMBLE_M)");
        return FE_NOT_READY;
    }
    if (which != FE_MODAL_SMALLEST && which != FE_MODAL_LARGEST) {
        set_error("fe_modal: which must be FE_MODAL_SMALLEST or FE_MODAL_LARGEST");
        return FE_BAD_INPUT;
    }
    if (k < 1 || k > n) {
        set_error("fe_modal: k must be in 1 .. n_dof");
        return FE_BAD_INPUT;
    }
    if (precision != FE_PREC_FP64 && precision != FE_PREC_MIXED_CG64) {
        set_error("fe_modal: precision must be FE_PREC_FP64 or FE_PREC_MIXED_CG64");
        return FE_BAD_INPUT;
    }
    const int m_default = which == FE_MODAL_SMALLEST ? std::max(3 * k, 2 * k + 30) : std::max(6 * k, 200);
    const int m = (int)std::min<int64_t>(n, steps > 0 ? steps : m_default);
    if (m < k) {
        set_error("fe_modal: fewer Lanczos steps than eigenpairs");
        return FE_BAD_INPUT;
    }
    Modal md;
    md.h = h;
    md.n = n;
    md.parts = (int)std::min<int64_t>(64, std::max<int64_t>(1, (n + kMT - 1) / kMT));
    DBuf<double> &V = md.V, &w = md.w, &Mw = md.Mw, &Kx = md.Kx;
    FE_CHECK(dalloc(V, (size_t)(m + 1) * n));
    FE_CHECK(dalloc(w, (size_t)n));
    FE_CHECK(dalloc(Mw, (size_t)n));
    FE_CHECK(dalloc(Kx, (size_t)n));
    FE_CHECK(dalloc(md.part, (size_t)md.parts * (m + 1)));
    FE_CHECK(dalloc(md.cdev, (size_t)m + 1));
    FE_CHECK(dalloc(md.tmp, 1));
    cudaStream_t s = h->stream;

    // automatic shift: 1% of the Rayleigh quotient of a smooth field, below zero
    if (which == FE_MODAL_SMALLEST && !(sigma < 0.0)) {
        const int cd = h->cdim;
        std::vector<double> xy(cd * h->n_nodes);
        FE_CUDA(cudaMemcpyAsync(xy.data(), h->coords.p, xy.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        double xmin = INFINITY, xmax = -INFINITY;
        for (int64_t i = 0; i < h->n_nodes; ++i) xmin = std::min(xmin, xy[cd * i]), xmax = std::max(xmax, xy[cd * i]);
        const double len = xmax > xmin ? xmax - xmin : 1.0;
        km_smooth<<<grid1(h->n_nodes), kMT, 0, s>>>(h->n_nodes, h->dim, cd, h->coords.p, xmin, 1.0 / len, w.p);
        FE_LAUNCH_CHECK();
        double vkv = 0, vmv = 0;
        FE_CHECK(md.spmv(h->kval, w.p, Mw.p));
        FE_CHECK(md.dot(w.p, Mw.p, &vkv));
        FE_CHECK(md.spmv(h->mval, w.p, Mw.p));
        FE_CHECK(md.dot(w.p, Mw.p, &vmv));
        if (!(vkv > 0.0) || !(vmv > 0.0)) {
            set_error("fe_modal: cannot pick a shift (pass sigma < 0)");
            return FE_BAD_INPUT;
        }
        sigma = -0.01 * vkv / vmv;
    }

    // the operator's solve matrix: K - sigma M (smallest) or M (largest), no Dirichlet
    // conditions; the multipliers of any set conditions are left alone meanwhile
    const int64_t n_bc_saved = h->n_bc;
    h->n_bc = 0;
    auto restore = [&]() {
        h->n_bc = n_bc_saved;
        h->sys_ready = false;            // the static system is rebuilt by fe_assemble
        h->have_solution = false;
        h->w.lmax[0] = h->w.lmax[1] = 0.0;
    };
    int rc = which == FE_MODAL_SMALLEST ? build_system(h, 1.0, -sigma, false) : build_system(h, 0.0, 1.0, false);
    if (rc == FE_OK) rc = check_error_word(h, "fe_modal");
    if (rc != FE_OK || h->singular) {
        restore();
        if (rc == FE_OK) {
            set_error("fe_modal: the solve matrix has a singular diagonal block");
            rc = FE_BREAKDOWN;
        }
        return rc;
    }
    const DBuf<double> &B = which == FE_MODAL_SMALLEST ? h->mval : h->kval;   // T = A^-1 B

    fe_solve_opts so;
    memset(&so, 0, sizeof(so));
    so.precision = precision;
    so.tol = 1e-12;
    so.cheb_degree = 8;
    so.cheb_ratio = 1000.0;
    so.flags = FE_SOLVE_ACCEPT_STAGNATION;

    std::vector<double> alpha, beta, acc;
    // v_0: pseudo-random, M-normalized
    km_start<<<grid1(n), kMT, 0, s>>>(n, V.p);
    FE_LAUNCH_CHECK();
    double nrm = 0.0;
    if (rc == FE_OK) rc = md.spmv(h->mval, V.p, Mw.p);
    if (rc == FE_OK) rc = md.dot(V.p, Mw.p, &nrm);
    if (rc == FE_OK) km_scale<<<grid1(n), kMT, 0, s>>>(n, V.p, 1.0 / sqrt(nrm), V.p);
    int mm = m;
    for (int j = 0; j < m && rc == FE_OK; ++j) {
        double *vj = V.p + (size_t)j * n;
        // w = T v_j: solve A w = B v_j
        rc = md.spmv(B, vj, h->b.p);
        fe_solve_stats st;
        memset(&st, 0, sizeof(st));
        if (rc == FE_OK) rc = solve(h, &so, &st);
        if (rc == FE_OK && st.status != FE_OK) {
            set_error("fe_modal: an inner PCG solve did not converge");
            rc = st.status;
        }
        if (rc != FE_OK) break;
        FE_CUDA(cudaMemcpyAsync(w.p, h->w.x.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        // Gram-Schmidt twice against v_0 .. v_j in the M inner product
        acc.assign(j + 1, 0.0);
        for (int pass = 0; pass < 2 && rc == FE_OK; ++pass) {
            rc = md.spmv(h->mval, w.p, Mw.p);
            if (rc == FE_OK) rc = md.dots(V.p, n, j + 1, Mw.p);
            if (rc != FE_OK) break;
            for (int i = 0; i <= j; ++i) acc[i] += md.chost[i];
            FE_CUDA(cudaMemcpyAsync(md.cdev.p, md.chost.data(), (j + 1) * sizeof(double), cudaMemcpyHostToDevice, s));
            km_gemv<<<grid1(n), kMT, 0, s>>>(n, j + 1, V.p, n, md.cdev.p, -1.0, w.p);
            FE_LAUNCH_CHECK();
        }
        if (rc != FE_OK) break;
        alpha.push_back(acc[j]);
        double bb = 0.0;
        rc = md.spmv(h->mval, w.p, Mw.p);
        if (rc == FE_OK) rc = md.dot(w.p, Mw.p, &bb);
        if (rc != FE_OK) break;
        const double b = sqrt(std::max(bb, 0.0));
        if (j + 1 == m) break;
        if (!(b > 1e-13 * fabs(acc[j]))) {   // invariant subspace reached
            mm = j + 1;
            break;
        }
        beta.push_back(b);
        km_scale<<<grid1(n), kMT, 0, s>>>(n, w.p, 1.0 / b, V.p + (size_t)(j + 1) * n);
        FE_LAUNCH_CHECK();
    }
    if (rc != FE_OK) {
        restore();
        return rc;
    }
    mm = (int)alpha.size();
    if (mm < k) {
        restore();
        set_error("fe_modal: the Krylov space closed before k eigenpairs");
        return FE_BREAKDOWN;
    }
    // Ritz pairs of the tridiagonal projection
    std::vector<double> T((size_t)mm * mm, 0.0), theta, Y;
    for (int i = 0; i < mm; ++i) T[(size_t)i * mm + i] = alpha[i];
    for (int i = 0; i + 1 < mm; ++i) T[(size_t)i * mm + i + 1] = T[(size_t)(i + 1) * mm + i] = beta[i];
    jacobi_eigen(mm, T, theta, Y);
    std::vector<int> order(mm);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return theta[a] > theta[b]; });
    std::vector<double> lam(k);
    for (int i = 0; i < k; ++i)
        lam[i] = which == FE_MODAL_SMALLEST ? sigma + 1.0 / theta[order[i]] : theta[order[i]];
    std::vector<int> by_lambda(k);
    std::iota(by_lambda.begin(), by_lambda.end(), 0);
    std::sort(by_lambda.begin(), by_lambda.end(), [&](int a, int b) { return lam[a] < lam[b]; });
    // eigenvalue scale of the residuals: a zero (rigid-body) eigenvalue is measured
    // against the largest computed one instead of against its own rounding
    double lam_ref = 0.0;
    for (int i = 0; i < k; ++i) lam_ref = std::max(lam_ref, fabs(lam[i]));
    std::vector<double> y(mm);
    for (int t = 0; t < k && rc == FE_OK; ++t) {
        const int i = by_lambda[t];
        for (int l = 0; l < mm; ++l) y[l] = Y[(size_t)l * mm + order[i]];
        FE_CUDA(cudaMemsetAsync(w.p, 0, n * sizeof(double), s));
        FE_CUDA(cudaMemcpyAsync(md.cdev.p, y.data(), mm * sizeof(double), cudaMemcpyHostToDevice, s));
        km_gemv<<<grid1(n), kMT, 0, s>>>(n, mm, V.p, n, md.cdev.p, 1.0, w.p);
        FE_LAUNCH_CHECK();
        double xx = 0.0;
        rc = md.dot(w.p, w.p, &xx);
        if (rc != FE_OK) break;
        km_scale<<<grid1(n), kMT, 0, s>>>(n, w.p, 1.0 / sqrt(xx), w.p);
        // true residual K x - lambda M x
        double kk = 0, mmx = 0, rr = 0;
        rc = md.spmv(h->kval, w.p, Kx.p);
        if (rc == FE_OK) rc = md.spmv(h->mval, w.p, Mw.p);
        if (rc == FE_OK) rc = md.dot(Kx.p, Kx.p, &kk);
        if (rc == FE_OK) rc = md.dot(Mw.p, Mw.p, &mmx);
        if (rc != FE_OK) break;
        const double lm = lam[i];
        FE_CUDA(cudaMemcpyAsync(md.tmp.p, &lm, sizeof(double), cudaMemcpyHostToDevice, s));
        km_gemv<<<grid1(n), kMT, 0, s>>>(n, 1, Mw.p, n, md.tmp.p, -1.0, Kx.p);    // Kx -= lambda M x
        FE_LAUNCH_CHECK();
        rc = md.dot(Kx.p, Kx.p, &rr);
        if (rc != FE_OK) break;
        eigvals[t] = lam[i];
        if (resid) resid[t] = sqrt(rr) / (sqrt(kk) + std::max(fabs(lam[i]), lam_ref) * sqrt(mmx) + 1e-300);
        if (eigvecs)
            FE_CUDA(cudaMemcpyAsync(eigvecs + (size_t)t * n, w.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    if (rc == FE_OK) rc = cudaStreamSynchronize(s) == cudaSuccess ? FE_OK : FE_CUDA_ERR;
    restore();
    return rc;
}

}  // namespace fe
