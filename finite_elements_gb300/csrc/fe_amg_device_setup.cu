// Device setup of the smoothed-aggregation hierarchy: amg::setup_hierarchy
// (fe_amg_passes.cuh, the passes fe_amg_build_parallel_host runs on the host) on the
// device executor -- every pass one grid-stride kernel over its rows, int64 prefix
// sums on the device between the passes that size the next ones -- and the dense
// inverse of the coarsest matrix (at most 4096 DOFs) by Gauss-Jordan elimination on the
// device.
#include <algorithm>
#include <cmath>
#include <functional>
#include <vector>

#include "fe_amg_dev.h"
#include "fe_amg_par.cuh"
#include "fe_grid_sync.cuh"

namespace fe {
namespace {

constexpr int kST = 256;                 // threads per block
constexpr int kScanPer = 8;              // elements per thread in the scans
constexpr int kScanTile = kST * kScanPer;

inline int grid_s(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kST - 1) / kST, 152 * 8)); }

#define FE_ROWS(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------- int64 exclusive scan

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v) {
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive prefix of v over the block's threads; *total = the block's sum
__device__ int64_t block_excl_scan(int64_t v, int64_t *total) {
    __shared__ int64_t warp_sum[kST / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t inc = warp_incl_scan(v);
    if (lane == 31) warp_sum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int64_t w = lane < kST / 32 ? warp_sum[lane] : 0;
        const int64_t wi = warp_incl_scan(w);
        if (lane < kST / 32) warp_sum[lane] = wi - w;   // exclusive prefix of the warp sums
        if (lane == kST / 32 - 1) *total = wi;
    }
    __syncthreads();
    const int64_t out = warp_sum[wid] + inc - v;
    __syncthreads();
    return out;
}

__global__ void ks_tile_sums(const int64_t *__restrict__ in, int64_t n, int64_t *__restrict__ part) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    int64_t v = 0;
    for (int k = 0; k < kScanPer; ++k)
        if (base + k < n) v += in[base + k];
    __shared__ int64_t tot;
    block_excl_scan(v, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// serial exclusive scan of the tile sums (a few thousand at most); out[n] = total
__global__ void ks_scan_tiles(int64_t nt, int64_t *part, int64_t *out, int64_t n) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int64_t run = 0;
    for (int64_t t = 0; t < nt; ++t) {
        const int64_t v = part[t];
        part[t] = run;
        run += v;
    }
    out[n] = run;
}

__global__ void ks_tile_scan(const int64_t *__restrict__ in, int64_t n, const int64_t *__restrict__ part,
                             int64_t *__restrict__ out) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    int64_t local[kScanPer];
    int64_t v = 0;
    for (int k = 0; k < kScanPer; ++k) {
        local[k] = base + k < n ? in[base + k] : 0;
        v += local[k];
    }
    __shared__ int64_t tot;
    int64_t run = part[blockIdx.x] + block_excl_scan(v, &tot);
    for (int k = 0; k < kScanPer; ++k)
        if (base + k < n) out[base + k] = run, run += local[k];
}

// out[0..n] = exclusive prefix sums of in[0..n), out[n] the total (also returned)
int scan64(const int64_t *in, int64_t n, int64_t *out, int64_t *total, DBuf<int64_t> &tmp, cudaStream_t s) {
    const int64_t nt = std::max<int64_t>(1, (n + kScanTile - 1) / kScanTile);
    FE_CHECK(dalloc(tmp, (size_t)nt));
    ks_tile_sums<<<(unsigned)nt, kST, 0, s>>>(in, n, tmp.p);
    ks_scan_tiles<<<1, 1, 0, s>>>(nt, tmp.p, out, n);
    ks_tile_scan<<<(unsigned)nt, kST, 0, s>>>(in, n, tmp.p, out);
    FE_LAUNCH_CHECK();
    FE_CUDA(cudaMemcpyAsync(total, out + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    return FE_OK;
}

// ---------------------------------------------------------------- device executor

template <typename F>
__global__ void k_rows(int64_t n, F f) {
    FE_ROWS(i, n) f(i);
}

__device__ __forceinline__ double block_sum_d(double v) {
    __shared__ double sh[kST / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < kST / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;
}

__global__ void kd_dot(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *part) {
    double s = 0.0;
    FE_ROWS(i, n) s = fma(a[i], b[i], s);
    s = block_sum_d(s);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void kd_dot_final(int nb, const double *__restrict__ part, double *out) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[i];
    s = block_sum_d(s);
    if (threadIdx.x == 0) *out = s;
}

// y = D^-1 A x (FP64) with G lanes of a warp per block row (a strided share of its
// blocks each, then a shuffle sum): the power iterations of the lmax estimates
template <int D, int G>
__global__ void __launch_bounds__(kST) kd_dinv_product(int64_t n, amg::PassDinvProduct f) {
    const int sub = threadIdx.x & (G - 1);
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
    const int64_t rows_padded = ((n + groups - 1) / groups) * groups;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; i < rows_padded; i += groups) {
        double acc[D];
#pragma unroll
        for (int a = 0; a < D; ++a) acc[a] = 0.0;
        if (i < n) {
            for (int64_t s = f.ptr[i] + sub; s < f.ptr[i + 1]; s += G) {
                const double *b = f.val + s * D * D;
                const double *xc = f.x + (int64_t)f.col[s] * D;
#pragma unroll
                for (int a = 0; a < D; ++a)
#pragma unroll
                    for (int k = 0; k < D; ++k) acc[a] = fma(b[a * D + k], xc[k], acc[a]);
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int a = 0; a < D; ++a) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], o);
        if (i < n && sub == 0)
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double v = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) v = fma(f.dinv[i * D * D + a * D + k], acc[k], v);
                f.y[i * D + a] = v;
            }
    }
}

template <int D>
int launch_dinv_product(int64_t n, const amg::PassDinvProduct &f, cudaStream_t s) {
    const double mean = n > 0 ? (double)f.nnzb / (double)n : 0.0;
    const int G = mean < 4 ? 2 : mean < 10 ? 4 : mean < 24 ? 8 : 32;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n * G + kST - 1) / kST, 152 * 8));
    switch (G) {
        case 2: kd_dinv_product<D, 2><<<grid, kST, 0, s>>>(n, f); break;
        case 4: kd_dinv_product<D, 4><<<grid, kST, 0, s>>>(n, f); break;
        case 8: kd_dinv_product<D, 8><<<grid, kST, 0, s>>>(n, f); break;
        default: kd_dinv_product<D, 32><<<grid, kST, 0, s>>>(n, f); break;
    }
    FE_LAUNCH_CHECK();
    return FE_OK;
}

struct DevEx {
    cudaStream_t s;
    DBuf<int64_t> scan_tmp;
    DBuf<double> part, sc;
    explicit DevEx(cudaStream_t st) : s(st) {}
    ~DevEx() { dfree(scan_tmp), dfree(part), dfree(sc); }
    template <class T>
    int alloc(DBuf<T> &b, size_t n) { return dalloc(b, n); }
    template <class T>
    void release(DBuf<T> &b) { dfree(b); }
    template <class T>
    int copy(T *dst, const T *src, size_t n) {
        if (n) FE_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
        return FE_OK;
    }
    template <class T>
    int read(T *dst, const T *src, size_t n) {
        if (n) FE_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        return FE_OK;
    }
    template <class F>
    int rows(int64_t n, const F &f) {
        if (n <= 0) return FE_OK;
        k_rows<F><<<grid_s(n), kST, 0, s>>>(n, f);
        FE_LAUNCH_CHECK();
        return FE_OK;
    }
    // the power iterations' product with lanes per row; other block sizes row by row
    int rows(int64_t n, const amg::PassDinvProduct &f) {
        if (n <= 0) return FE_OK;
        switch (f.d) {
            case 1: return launch_dinv_product<1>(n, f, s);
            case 2: return launch_dinv_product<2>(n, f, s);
            case 3: return launch_dinv_product<3>(n, f, s);
            case 6: return launch_dinv_product<6>(n, f, s);
            default:
                k_rows<amg::PassDinvProduct><<<grid_s(n), kST, 0, s>>>(n, f);
                FE_LAUNCH_CHECK();
                return FE_OK;
        }
    }
    int scan(const int64_t *in, int64_t n, int64_t *out, int64_t *total) { return scan64(in, n, out, total, scan_tmp, s); }
    int dot(const double *a, const double *b, int64_t n, double *out) {
        const int g = grid_s(n);
        FE_CHECK(dalloc(part, (size_t)g));
        FE_CHECK(dalloc(sc, 1));
        kd_dot<<<g, kST, 0, s>>>(n, a, b, part.p);
        kd_dot_final<<<1, kST, 0, s>>>(g, part.p, sc.p);
        FE_LAUNCH_CHECK();
        return read(out, sc.p, 1);
    }
};

// ---------------------------------------------------------------- inputs of level 0

struct PassPtr64 {
    const int32_t *p32; int64_t *p64;
    FE_HD void operator()(int64_t i) const { p64[i] = p32[i]; }
};

// near-null space per node: rigid-body modes (d = 2: 3, d = 3: 6) or the constant (d = 1)
struct PassNullspace {
    int d, cdim, m; const double *xy; double *B;
    FE_HD void operator()(int64_t i) const {
        const double x = xy[i * cdim], y = xy[i * cdim + 1], z = cdim == 3 ? xy[i * cdim + 2] : 0.0;
        double *b = &B[i * d * m];
        for (int k = 0; k < d * m; ++k) b[k] = 0.0;
        if (d == 1) {
            b[0] = 1.0;
        } else if (d == 2) {
            b[0 * m + 0] = 1.0, b[1 * m + 1] = 1.0, b[0 * m + 2] = -y, b[1 * m + 2] = x;
        } else {
            for (int k = 0; k < 3; ++k) b[k * m + k] = 1.0;
            b[0 * m + 3] = -y, b[1 * m + 3] = x;
            b[1 * m + 4] = -z, b[2 * m + 4] = y;
            b[0 * m + 5] = z, b[2 * m + 5] = -x;
        }
    }
};

struct PassZeroRows {
    const int64_t *dof; int m; double *B;
    FE_HD void operator()(int64_t k) const {
        for (int j = 0; j < m; ++j) B[dof[k] * m + j] = 0.0;
    }
};

template <typename T>
int to_host(std::vector<T> &dst, const DBuf<T> &src, size_t n, cudaStream_t s) {
    dst.resize(n);
    if (n) FE_CUDA(cudaMemcpyAsync(dst.data(), src.p, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    return FE_OK;
}

int csr_to_host(const DevCsr &D, BlockCsr &H, cudaStream_t s) {
    H.n = D.n, H.rd = D.rd, H.cd = D.cd;
    FE_CHECK(to_host(H.ptr, D.ptr, (size_t)D.n + 1, s));
    FE_CHECK(to_host(H.col, D.col, (size_t)D.nnzb, s));
    FE_CHECK(to_host(H.val, D.val, (size_t)D.nnzb * D.rd * D.cd, s));
    return FE_OK;
}

// ---------------------------------------------------------------- coarsest inverse
// Dense inverse of the coarsest matrix by Gauss-Jordan elimination without pivoting
// (the matrix is symmetric positive definite once 1e-12 of its largest diagonal entry
// is added, as the host version does), in place, one pivot k after the other, every new
// value from old ones:
//   others:  a_ij - a_ik a_kj / a_kk      (i != k, j != k)
//   row k:   a_kj / a_kk (j != k);  column k: -a_ik / a_kk (i != k);  pivot: 1 / a_kk

constexpr int kMaxCoarse = 4096;   // DOFs of the coarsest level (a 128 MB inverse)

__global__ void kc_dense_fill(int64_t nb_rows, int cd, const int64_t *__restrict__ ptr,
                              const int32_t *__restrict__ col, const double *__restrict__ val, int64_t n,
                              double *__restrict__ M) {
    FE_ROWS(i, nb_rows)
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s)
        for (int a = 0; a < cd; ++a)
            for (int b = 0; b < cd; ++b) M[(i * cd + a) * n + (int64_t)col[s] * cd + b] = val[(s * cd + a) * cd + b];
}

// one block: the diagonal gets 1e-12 of its largest magnitude added
__global__ void kc_regularise(int64_t n, double *M) {
    __shared__ double sh[kST / 32];
    double m = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(M[i * n + i]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < kST / 32; ++w) t = fmax(t, sh[w]);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) M[i * n + i] += 1e-12 * t;
}

// All pivots in one cooperative launch, one grid barrier per pivot.  Warp w owns rows
// w, w + W, ... and lane l the columns l, l + 32, ... of them, so every element has one
// owner for the whole elimination.  Pivot k's new values come from old values only --
// the element itself, a_ik, a_kj and a_kk -- and the old pivot row and column are read
// from buffers (piv[k & 1]) that the owners filled while computing the previous pivot,
// so a pivot's updates do not race with its readers; the owners of row and column k + 1
// fill piv[(k + 1) & 1] on the way.  piv[b] holds the row (n values) then the column.
// A zero or non-finite pivot stops every block at the same step (*singular = 1).
__global__ void __launch_bounds__(kST) kc_gauss_jordan(int64_t n, double *M, double *piv, unsigned *bar, int *err,
                                                       int *singular) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = 0; k < n; ++k) {
        const double *row = piv + (k & 1) * 2 * n, *colv = row + n;
        double *nrow = piv + ((k + 1) & 1) * 2 * n, *ncol = nrow + n;
        const double p = __ldcg(row + k);
        if (p == 0.0 || !isfinite(p)) {
            if (w0 == 0 && lane == 0) *singular = 1;
            return;
        }
        const double ip = 1.0 / p;
        for (int64_t i = w0; i < n; i += W) {
            const double aik = __ldcg(colv + i);
            for (int64_t j = lane; j < n; j += 32) {
                const double akj = __ldcg(row + j);
                double v;
                if (i == k) v = j == k ? ip : akj * ip;
                else if (j == k) v = -aik * ip;
                else v = fma(-aik * ip, akj, M[i * n + j]);
                M[i * n + j] = v;
                if (i == k + 1) nrow[j] = v;
                if (j == k + 1) ncol[i] = v;
            }
        }
        if (!grid_sync_bounded(bar, err)) return;
    }
}

// piv[0] = row 0 and column 0 of M (the first pivot's)
__global__ void kc_first_pivot(int64_t n, const double *__restrict__ M, double *__restrict__ piv) {
    FE_ROWS(j, n) {
        piv[j] = M[j];
        piv[n + j] = M[j * n];
    }
}

int coarse_inverse_device(const DevCsr &C, DevAmg &G, cudaStream_t s) {
    const int64_t n = C.n * C.rd;
    if (n > kMaxCoarse) {
        set_error("multigrid setup: coarsest level too large for its dense solve");
        return FE_BAD_INPUT;
    }
    G.nc = n;
    FE_CHECK(dalloc(G.cinv, (size_t)std::max<int64_t>(n * n, 1)));
    if (n == 0) return FE_OK;
    DBuf<int> flag;   // [0] singular, [1] [2] the grid barrier, [3] its error word
    DBuf<double> piv;   // the pivot row and column, two generations
    FE_CHECK(dalloc(flag, 4));
    FE_CHECK(dalloc(piv, (size_t)4 * n));
    struct Free {
        DBuf<int> &f;
        DBuf<double> &p;
        ~Free() { dfree(f), dfree(p); }
    } fr{flag, piv};
    FE_CUDA(cudaMemsetAsync(flag.p, 0, 4 * sizeof(int), s));
    FE_CUDA(cudaMemsetAsync(G.cinv.p, 0, (size_t)n * n * sizeof(double), s));
    kc_dense_fill<<<grid_s(C.n), kST, 0, s>>>(C.n, C.rd, C.ptr.p, C.col.p, C.val.p, n, G.cinv.p);
    kc_regularise<<<1, kST, 0, s>>>(n, G.cinv.p);
    kc_first_pivot<<<grid_s(n), kST, 0, s>>>(n, G.cinv.p, piv.p);
    FE_LAUNCH_CHECK();
    // the cooperative grid: every SM's resident blocks of the kernel
    int dev = 0, sms = 0, per_sm = 0;
    FE_CUDA(cudaGetDevice(&dev));
    FE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)kc_gauss_jordan, kST, 0));
    const int64_t want = (n + kST / 32 - 1) / (kST / 32);   // a warp per row
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * std::max(per_sm, 1)));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kST);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FE_CUDA(cudaLaunchKernelEx(&cfg, kc_gauss_jordan, n, G.cinv.p, piv.p, (unsigned *)(flag.p + 1), flag.p + 3,
                               flag.p));
    int host[4] = {0, 0, 0, 0};
    FE_CUDA(cudaMemcpyAsync(host, flag.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    if (host[3]) {
        set_error("multigrid setup: a grid barrier of the coarsest inverse timed out");
        return FE_CUDA_ERR;
    }
    if (host[0]) {
        set_error("multigrid setup: singular coarsest matrix");
        return FE_BREAKDOWN;
    }
    return FE_OK;
}

}  // namespace

int amg_setup_device(fe_handle_s *h, double theta, int64_t coarse_dofs, DevAmg &G) {
    cudaStream_t s = h->stream;
    DevEx ex(s);
    const int D = h->dim;
    const int64_t n0 = h->n_nodes;
    const int m = D == 2 ? 3 : D == 3 ? 6 : 1;
    // level-0 operator (own copies, int64 row pointers) and near-null space, both
    // handed over to setup_hierarchy
    DevCsr A;
    DBuf<double> B;
    A.n = n0, A.rd = A.cd = D, A.nnzb = h->nnzb;
    int st = FE_OK;
    if ((st = dalloc(A.ptr, (size_t)n0 + 1)) || (st = dalloc(A.col, (size_t)std::max<int64_t>(h->nnzb, 1))) ||
        (st = dalloc(A.val, (size_t)std::max<int64_t>(h->nnzb * D * D, 1))) ||
        (st = dalloc(B, (size_t)std::max<int64_t>(n0 * D * m, 1))) ||
        (st = ex.rows(n0 + 1, PassPtr64{h->blk_ptr.p, A.ptr.p})) ||
        (st = ex.copy(A.col.p, h->blk_col.p, (size_t)h->nnzb)) ||
        (st = ex.copy(A.val.p, h->aval.p, (size_t)(h->nnzb * D * D))) ||
        (st = ex.rows(n0, PassNullspace{D, h->cdim, m, h->coords.p, B.p})) ||
        (st = ex.rows(h->n_bc, PassZeroRows{h->bc_dof.p, m, B.p}))) {
        drelease(A);
        dfree(B);
        return st;
    }
    std::vector<amg::Level> levels;
    st = amg::setup_hierarchy(ex, A, B, m, theta, coarse_dofs, levels, G.coarse, &G.mis_rounds);
    // the levels move into G (released with it, also after a failure)
    for (auto &l : levels) {
        DevLevel L;
        L.A = l.A, L.P = l.P, L.PT = l.PT, L.dinv = l.dinv, L.agg = l.agg, L.lmax = l.lmax;
        G.L.push_back(L);
    }
    FE_CHECK(st);
    // coarsest level: its dense inverse, on the device
    return coarse_inverse_device(G.coarse, G, s);
}

int amg_download(const DevAmg &G, fe_amg_s *out, cudaStream_t s) {
    out->levels.resize(G.L.size());
    for (size_t l = 0; l < G.L.size(); ++l) {
        const DevLevel &D = G.L[l];
        AmgLevel &H = out->levels[l];
        FE_CHECK(csr_to_host(D.A, H.A, s));
        FE_CHECK(csr_to_host(D.P, H.P, s));
        FE_CHECK(csr_to_host(D.PT, H.PT, s));
        FE_CHECK(to_host(H.dinv, D.dinv, (size_t)D.A.n * D.A.rd * D.A.rd, s));
        FE_CHECK(to_host(H.agg, D.agg, (size_t)D.A.n, s));
        H.lmax = D.lmax;
    }
    FE_CHECK(csr_to_host(G.coarse, out->coarse, s));
    FE_CHECK(to_host(out->coarse_inv, G.cinv, (size_t)(G.nc * G.nc), s));
    FE_CUDA(cudaStreamSynchronize(s));
    return FE_OK;
}

}  // namespace fe

using namespace fe;

extern "C" int fe_amg_build_device(fe_handle h, double theta, int64_t coarse_dofs, fe_amg *out) {
    if (!h || !out) {
        set_error("fe_amg_build_device: bad arguments");
        return FE_BAD_INPUT;
    }
    *out = nullptr;
    if (!h->sys_ready) {
        set_error("fe_amg_build_device: the system is not assembled");
        return FE_NOT_READY;
    }
    DevAmg G;
    FE_CHECK(amg_setup_device(h, theta, coarse_dofs, G));
    fe_amg_s *a = new fe_amg_s();
    const int st = amg_download(G, a, h->stream);
    if (st != FE_OK) {
        fe_amg_destroy(a);
        return st;
    }
    *out = a;
    return FE_OK;
}
