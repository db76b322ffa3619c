// Device setup of the smoothed-aggregation hierarchy: the passes of
// fe_amg_build_parallel_host (fe_amg_setup.cu) as grid-stride loops over the row
// operations of fe_amg_par.cuh, with int64 prefix sums between the passes that size the
// next ones.  Only the coarsest matrix (a few hundred DOFs) goes to the host, for its
// dense inverse.
//
// WORK IN PROGRESS: not yet run on a GPU.
#include <algorithm>
#include <cmath>
#include <functional>
#include <vector>

#include "fe_amg_dev.h"
#include "fe_amg_par.cuh"

namespace fe {
namespace {

constexpr int kST = 256;                 // threads per block
constexpr int kScanPer = 8;              // elements per thread in the scans
constexpr int kScanTile = kST * kScanPer;
constexpr int kMaxRounds = 256;          // independent-set rounds per level

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

// ---------------------------------------------------------------- setup kernels

__global__ void kd_ptr64(int64_t n, const int32_t *__restrict__ p32, int64_t *__restrict__ p64) {
    FE_ROWS(i, n + 1) p64[i] = p32[i];
}

__global__ void kd_iota(int64_t n, int64_t *__restrict__ p) {
    FE_ROWS(i, n + 1) p[i] = i;
}

// near-null space per node: rigid-body modes (d = 2: 3, d = 3: 6) or the constant (d = 1)
__global__ void kd_nullspace(int64_t n, int d, int cdim, int m, const double *__restrict__ xy, double *__restrict__ B) {
    FE_ROWS(i, n) {
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
}

__global__ void kd_zero_rows(int64_t nb, const int64_t *__restrict__ dof, int m, double *__restrict__ B) {
    FE_ROWS(k, nb) for (int j = 0; j < m; ++j) B[dof[k] * m + j] = 0.0;
}

__global__ void kd_dinv(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                        const double *__restrict__ val, int d, double *__restrict__ dinv) {
    FE_ROWS(i, n) {
        double *o = &dinv[i * d * d];
        for (int k = 0; k < d * d; ++k) o[k] = 0.0;
        for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s)
            if (col[s] == i) amg::sym_pinv(&val[s * d * d], d, o);
    }
}

__global__ void kd_power_start(int64_t nd, double *__restrict__ x) {
    FE_ROWS(i, nd) x[i] = 1.0 + (double)(i % 7) / 7.0;
}

__global__ void kd_dinv_product(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                const double *__restrict__ val, const double *__restrict__ dinv, int d,
                                const double *__restrict__ x, double *__restrict__ y) {
    FE_ROWS(i, n) amg::row_dinv_product(ptr, col, val, dinv, d, x, i, y);
}

// x = y / sqrt(*yy)
__global__ void kd_normalise(int64_t nd, const double *__restrict__ y, const double *__restrict__ yy,
                             double *__restrict__ x) {
    const double inv = 1.0 / sqrt(*yy);
    FE_ROWS(i, nd) x[i] = y[i] * inv;
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

__global__ void kd_block_norms(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                               const double *__restrict__ val, int d, double *__restrict__ nrm, double *__restrict__ dg) {
    FE_ROWS(i, n) amg::row_block_norms(ptr, col, val, d, i, nrm, dg);
}

__global__ void kd_strength(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                            const double *__restrict__ nrm, const double *__restrict__ dg, double theta,
                            uint8_t *__restrict__ strong) {
    FE_ROWS(i, n) amg::row_strength(ptr, col, nrm, dg, theta, i, strong);
}

__global__ void kd_state_init(int64_t n, uint32_t *__restrict__ state) {
    FE_ROWS(i, n) state[i] = amg::kUndecided;
}

__global__ void kd_mis_key(int64_t n, const uint32_t *__restrict__ state, uint64_t *__restrict__ key) {
    FE_ROWS(i, n) key[i] = amg::mis_key(state[i], i);
}

__global__ void kd_max_key(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                           const uint8_t *__restrict__ strong, const uint64_t *__restrict__ in, uint64_t *__restrict__ out) {
    FE_ROWS(i, n) amg::row_max_key(ptr, col, strong, in, i, out);
}

__global__ void kd_mis_decide(int64_t n, const uint64_t *__restrict__ m2, uint32_t *__restrict__ state,
                              unsigned long long *undecided) {
    unsigned long long u = 0;
    FE_ROWS(i, n) u += (unsigned long long)amg::mis_decide(m2, i, state);
    for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
    if ((threadIdx.x & 31) == 0 && u) atomicAdd(undecided, u);
}

__global__ void kd_root_flags(int64_t n, const uint32_t *__restrict__ state, int64_t *__restrict__ flag) {
    FE_ROWS(i, n) flag[i] = state[i] == amg::kIn ? 1 : 0;
}

__global__ void kd_roots(int64_t n, const uint32_t *__restrict__ state, const int64_t *__restrict__ off,
                         int32_t *__restrict__ rank, int32_t *__restrict__ roots) {
    FE_ROWS(i, n) {
        if (state[i] == amg::kIn) {
            rank[i] = (int32_t)off[i];
            roots[off[i]] = (int32_t)i;
        } else {
            rank[i] = -1;
        }
    }
}

__global__ void kd_join_root(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                             const uint8_t *__restrict__ strong, const double *__restrict__ nrm,
                             const uint32_t *__restrict__ state, const int32_t *__restrict__ rank,
                             int32_t *__restrict__ agg1) {
    FE_ROWS(i, n) amg::row_join_root(ptr, col, strong, nrm, state, rank, i, agg1);
}

__global__ void kd_join_neighbour(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                  const uint8_t *__restrict__ strong, const double *__restrict__ nrm,
                                  const int32_t *__restrict__ agg1, int32_t *__restrict__ agg, int *unassigned) {
    int u = 0;
    FE_ROWS(i, n) {
        amg::row_join_neighbour(ptr, col, strong, nrm, agg1, i, agg);
        u += agg[i] < 0;
    }
    if (u) atomicAdd(unassigned, u);
}

__global__ void kd_member_bound(int64_t na, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                const int32_t *__restrict__ roots, int64_t *__restrict__ bound) {
    FE_ROWS(c, na) bound[c] = amg::agg_member_bound(ptr, col, roots, c);
}

__global__ void kd_members(int64_t na, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                           const int32_t *__restrict__ roots, const int32_t *__restrict__ agg,
                           const int64_t *__restrict__ boff, int32_t *__restrict__ cand, int64_t *__restrict__ cnt) {
    FE_ROWS(c, na) cnt[c] = amg::agg_members(ptr, col, roots, agg, c, cand + boff[c]);
}

// rows of candidates -> packed rows: dst[off[r] ..] = src[boff[r] ..], off[r+1]-off[r] entries
__global__ void kd_pack_rows(int64_t n, const int64_t *__restrict__ boff, const int64_t *__restrict__ off,
                             const int32_t *__restrict__ src, int32_t *__restrict__ dst) {
    FE_ROWS(r, n) {
        const int64_t len = off[r + 1] - off[r];
        for (int64_t k = 0; k < len; ++k) dst[off[r] + k] = src[boff[r] + k];
    }
}

__global__ void kd_qr(int64_t na, const int64_t *__restrict__ mptr, const int32_t *__restrict__ mem, int d, int m,
                      double *__restrict__ pt, double *__restrict__ Bc) {
    FE_ROWS(c, na) amg::aggregate_qr(mem + mptr[c], mptr[c + 1] - mptr[c], d, m, pt, Bc + c * m * m);
}

__global__ void kd_prod_bound(int64_t n, const int64_t *__restrict__ aptr, const int32_t *__restrict__ acol,
                              const int64_t *__restrict__ bptr, int64_t *__restrict__ bound) {
    FE_ROWS(i, n) bound[i] = amg::row_product_bound(aptr, acol, bptr, i);
}

__global__ void kd_prod_cols(int64_t n, const int64_t *__restrict__ aptr, const int32_t *__restrict__ acol,
                             const int64_t *__restrict__ bptr, const int32_t *__restrict__ bcol,
                             const int64_t *__restrict__ boff, int32_t *__restrict__ cand, int64_t *__restrict__ cnt) {
    FE_ROWS(i, n) cnt[i] = amg::row_product_columns(aptr, acol, bptr, bcol, i, cand + boff[i]);
}

__global__ void kd_prod_vals(int64_t n, const int64_t *__restrict__ aptr, const int32_t *__restrict__ acol,
                             const double *__restrict__ aval, int ra, int ca, const int64_t *__restrict__ bptr,
                             const int32_t *__restrict__ bcol, const double *__restrict__ bval, int cb,
                             const int64_t *__restrict__ cptr, const int32_t *__restrict__ ccol,
                             double *__restrict__ cval) {
    FE_ROWS(i, n) amg::row_product_values(aptr, acol, aval, ra, ca, bptr, bcol, bval, cb, cptr, ccol, cval, i);
}

__global__ void kd_smooth(int64_t n, const int64_t *__restrict__ pptr, const int32_t *__restrict__ pcol,
                          double *__restrict__ pval, const double *__restrict__ dinv, const double *__restrict__ ptent,
                          const int32_t *__restrict__ agg, int d, int m, double w) {
    FE_ROWS(i, n) amg::row_smooth_prolongator(pptr, pcol, pval, dinv, ptent, agg, d, m, w, i);
}

__global__ void kd_restr_bound(int64_t na, const int64_t *__restrict__ mptr, const int32_t *__restrict__ mem,
                               const int64_t *__restrict__ aptr, int64_t *__restrict__ bound) {
    FE_ROWS(c, na) bound[c] = amg::row_restriction_bound(mptr, mem, aptr, c);
}

__global__ void kd_restr_cols(int64_t na, const int64_t *__restrict__ mptr, const int32_t *__restrict__ mem,
                              const int64_t *__restrict__ aptr, const int32_t *__restrict__ acol,
                              const int64_t *__restrict__ boff, int32_t *__restrict__ cand, int64_t *__restrict__ cnt) {
    FE_ROWS(c, na) cnt[c] = amg::row_restriction_columns(mptr, mem, aptr, acol, c, cand + boff[c]);
}

__global__ void kd_restr_vals(int64_t na, const int64_t *__restrict__ rptr, const int32_t *__restrict__ rcol,
                              double *__restrict__ rval, const int64_t *__restrict__ pptr,
                              const int32_t *__restrict__ pcol, const double *__restrict__ pval, int d, int m) {
    FE_ROWS(c, na) amg::row_restriction_values(rptr, rcol, rval, pptr, pcol, pval, d, m, c);
}

// ---------------------------------------------------------------- host side of the passes

// Runs f at scope exit unless disarmed.
template <typename F>
struct Defer {
    F f;
    bool armed = true;
    ~Defer() {
        if (armed) f();
    }
};
template <typename F>
Defer<F> defer(F f) {
    return Defer<F>{f};
}

struct Scratch {
    DBuf<int64_t> bound, boff, cnt, scan;
    DBuf<int32_t> cand;
    ~Scratch() { dfree(bound), dfree(boff), dfree(cnt), dfree(scan), dfree(cand); }
};

// The rows of a row-wise pass whose candidates are sized by `bound_launch` and reduced
// to sorted distinct columns by `cols_launch`: C.ptr and C.col of n rows.
template <typename Bound, typename Cols>
int distinct_rows(int64_t n, Bound bound_launch, Cols cols_launch, DevCsr &C, Scratch &S, cudaStream_t s) {
    FE_CHECK(dalloc(S.bound, (size_t)std::max<int64_t>(n, 1)));
    FE_CHECK(dalloc(S.boff, (size_t)n + 1));
    FE_CHECK(dalloc(S.cnt, (size_t)std::max<int64_t>(n, 1)));
    bound_launch(S.bound.p);
    FE_LAUNCH_CHECK();
    int64_t total = 0;
    FE_CHECK(scan64(S.bound.p, n, S.boff.p, &total, S.scan, s));
    FE_CHECK(dalloc(S.cand, (size_t)std::max<int64_t>(total, 1)));
    cols_launch(S.boff.p, S.cand.p, S.cnt.p);
    FE_LAUNCH_CHECK();
    FE_CHECK(dalloc(C.ptr, (size_t)n + 1));
    int64_t nnzb = 0;
    FE_CHECK(scan64(S.cnt.p, n, C.ptr.p, &nnzb, S.scan, s));
    C.nnzb = nnzb;
    FE_CHECK(dalloc(C.col, (size_t)std::max<int64_t>(nnzb, 1)));
    kd_pack_rows<<<grid_s(n), kST, 0, s>>>(n, S.boff.p, C.ptr.p, S.cand.p, C.col.p);
    FE_LAUNCH_CHECK();
    return FE_OK;
}

// C = A B
int product_dev(const DevCsr &A, const DevCsr &B, DevCsr &C, Scratch &S, cudaStream_t s) {
    C.n = A.n, C.rd = A.rd, C.cd = B.cd;
    const int64_t n = A.n;
    FE_CHECK(distinct_rows(
        n,
        [&](int64_t *bound) {
            kd_prod_bound<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, B.ptr.p, bound);
        },
        [&](const int64_t *boff, int32_t *cand, int64_t *cnt) {
            kd_prod_cols<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, B.ptr.p, B.col.p, boff, cand, cnt);
        },
        C, S, s));
    FE_CHECK(dalloc(C.val, (size_t)std::max<int64_t>(C.nnzb * C.rd * C.cd, 1)));
    kd_prod_vals<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, A.rd, A.cd, B.ptr.p, B.col.p, B.val.p, B.cd,
                                           C.ptr.p, C.col.p, C.val.p);
    FE_LAUNCH_CHECK();
    return FE_OK;
}

// largest eigenvalue of D^-1 A: 30 power iterations, then the Rayleigh quotient
int lmax_dev(const DevCsr &A, const double *dinv, double *lmax, cudaStream_t s) {
    const int d = A.rd;
    const int64_t n = A.n, nd = n * d;
    DBuf<double> x, y, part, sc;
    struct Free {
        DBuf<double> *b[4];
        ~Free() {
            for (auto *p : b) dfree(*p);
        }
    } fr{{&x, &y, &part, &sc}};
    const int g = grid_s(nd);
    FE_CHECK(dalloc(x, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(dalloc(y, (size_t)std::max<int64_t>(nd, 1)));
    FE_CHECK(dalloc(part, (size_t)g));
    FE_CHECK(dalloc(sc, 3));
    kd_power_start<<<g, kST, 0, s>>>(nd, x.p);
    for (int it = 0; it < 30; ++it) {
        kd_dinv_product<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, dinv, d, x.p, y.p);
        kd_dot<<<g, kST, 0, s>>>(nd, y.p, y.p, part.p);
        kd_dot_final<<<1, kST, 0, s>>>(g, part.p, sc.p);
        kd_normalise<<<g, kST, 0, s>>>(nd, y.p, sc.p, x.p);
    }
    kd_dinv_product<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, dinv, d, x.p, y.p);
    kd_dot<<<g, kST, 0, s>>>(nd, x.p, y.p, part.p);
    kd_dot_final<<<1, kST, 0, s>>>(g, part.p, sc.p + 1);
    kd_dot<<<g, kST, 0, s>>>(nd, x.p, x.p, part.p);
    kd_dot_final<<<1, kST, 0, s>>>(g, part.p, sc.p + 2);
    FE_LAUNCH_CHECK();
    double hsc[3];
    FE_CUDA(cudaMemcpyAsync(hsc, sc.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    *lmax = hsc[1] / hsc[2];
    if (!std::isfinite(*lmax) || !(*lmax > 0.0)) {
        set_error("multigrid setup: the largest eigenvalue estimate is not positive");
        return FE_BREAKDOWN;
    }
    return FE_OK;
}

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

}  // namespace

int amg_setup_device(fe_handle_s *h, double theta, int64_t coarse_dofs, DevAmg &G) {
    cudaStream_t s = h->stream;
    const int D = h->dim;
    const int64_t n0 = h->n_nodes;
    // level-0 operator: the eliminated system matrix, own copies with int64 row pointers
    DevCsr A;
    A.n = n0, A.rd = A.cd = D, A.nnzb = h->nnzb;
    FE_CHECK(dalloc(A.ptr, (size_t)n0 + 1));
    FE_CHECK(dalloc(A.col, (size_t)std::max<int64_t>(h->nnzb, 1)));
    FE_CHECK(dalloc(A.val, (size_t)std::max<int64_t>(h->nnzb * D * D, 1)));
    kd_ptr64<<<grid_s(n0 + 1), kST, 0, s>>>(n0, h->blk_ptr.p, A.ptr.p);
    FE_LAUNCH_CHECK();
    if (h->nnzb > 0) {
        FE_CUDA(cudaMemcpyAsync(A.col.p, h->blk_col.p, h->nnzb * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
        FE_CUDA(cudaMemcpyAsync(A.val.p, h->aval.p, h->nnzb * D * D * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    int m = D == 2 ? 3 : D == 3 ? 6 : 1;
    DBuf<double> B, Bc, nrm, dg;
    DBuf<uint8_t> strong;
    DBuf<uint32_t> state;
    DBuf<uint64_t> key, m1, m2;
    DBuf<int32_t> rank, roots, agg1, mem;
    DBuf<int64_t> flags, roff, mptr;
    DBuf<unsigned long long> ucount;
    DBuf<int> unassigned;
    struct Free {
        std::vector<std::function<void()>> f;
        ~Free() {
            for (auto &x : f) x();
        }
    } fr;
    fr.f = {[&] { dfree(B), dfree(Bc), dfree(nrm), dfree(dg), dfree(strong), dfree(state); },
            [&] { dfree(key), dfree(m1), dfree(m2), dfree(rank), dfree(roots), dfree(agg1), dfree(mem); },
            [&] { dfree(flags), dfree(roff), dfree(mptr), dfree(ucount), dfree(unassigned); },
            [&] { A.release(); }};
    FE_CHECK(dalloc(B, (size_t)std::max<int64_t>(n0 * D * m, 1)));
    kd_nullspace<<<grid_s(n0), kST, 0, s>>>(n0, D, h->cdim, m, h->coords.p, B.p);
    if (h->n_bc > 0) kd_zero_rows<<<grid_s(h->n_bc), kST, 0, s>>>(h->n_bc, h->bc_dof.p, m, B.p);
    FE_LAUNCH_CHECK();
    FE_CHECK(dalloc(ucount, 1));
    FE_CHECK(dalloc(unassigned, 1));
    Scratch S;
    while (A.n * A.rd > coarse_dofs && G.L.size() < 12) {
        DevLevel L;
        DevCsr Mem, Pt, AP, Ac;   // member lists, tentative prolongator, A P, Galerkin product
        auto level_guard = defer([&] { L.release(), Mem.release(), Pt.release(), AP.release(), Ac.release(); });
        const int dd = A.rd;
        const int64_t n = A.n;
        FE_CHECK(dalloc(L.dinv, (size_t)std::max<int64_t>(n * dd * dd, 1)));
        kd_dinv<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, dd, L.dinv.p);
        FE_LAUNCH_CHECK();
        FE_CHECK(lmax_dev(A, L.dinv.p, &L.lmax, s));
        // strength and the independent set
        FE_CHECK(dalloc(nrm, (size_t)std::max<int64_t>(A.nnzb, 1)));
        FE_CHECK(dalloc(strong, (size_t)std::max<int64_t>(A.nnzb, 1)));
        FE_CHECK(dalloc(dg, (size_t)std::max<int64_t>(n, 1)));
        kd_block_norms<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, dd, nrm.p, dg.p);
        kd_strength<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, nrm.p, dg.p, theta, strong.p);
        FE_CHECK(dalloc(state, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(dalloc(key, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(dalloc(m1, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(dalloc(m2, (size_t)std::max<int64_t>(n, 1)));
        kd_state_init<<<grid_s(n), kST, 0, s>>>(n, state.p);
        FE_LAUNCH_CHECK();
        int rounds = 0;
        for (;;) {
            if (++rounds > kMaxRounds) {
                set_error("multigrid setup: the independent set did not settle");
                return FE_BREAKDOWN;
            }
            FE_CUDA(cudaMemsetAsync(ucount.p, 0, sizeof(unsigned long long), s));
            kd_mis_key<<<grid_s(n), kST, 0, s>>>(n, state.p, key.p);
            kd_max_key<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, strong.p, key.p, m1.p);
            kd_max_key<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, strong.p, m1.p, m2.p);
            kd_mis_decide<<<grid_s(n), kST, 0, s>>>(n, m2.p, state.p, ucount.p);
            FE_LAUNCH_CHECK();
            unsigned long long und = 0;
            FE_CUDA(cudaMemcpyAsync(&und, ucount.p, sizeof(und), cudaMemcpyDeviceToHost, s));
            FE_CUDA(cudaStreamSynchronize(s));
            if (und == 0) break;
        }
        G.mis_rounds += rounds;
        // roots in node order, aggregates
        FE_CHECK(dalloc(flags, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(dalloc(roff, (size_t)n + 1));
        kd_root_flags<<<grid_s(n), kST, 0, s>>>(n, state.p, flags.p);
        FE_LAUNCH_CHECK();
        int64_t na = 0;
        FE_CHECK(scan64(flags.p, n, roff.p, &na, S.scan, s));
        FE_CHECK(dalloc(rank, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(dalloc(roots, (size_t)std::max<int64_t>(na, 1)));
        FE_CHECK(dalloc(agg1, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(dalloc(L.agg, (size_t)std::max<int64_t>(n, 1)));
        kd_roots<<<grid_s(n), kST, 0, s>>>(n, state.p, roff.p, rank.p, roots.p);
        kd_join_root<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, strong.p, nrm.p, state.p, rank.p, agg1.p);
        FE_CUDA(cudaMemsetAsync(unassigned.p, 0, sizeof(int), s));
        kd_join_neighbour<<<grid_s(n), kST, 0, s>>>(n, A.ptr.p, A.col.p, strong.p, nrm.p, agg1.p, L.agg.p,
                                                    unassigned.p);
        FE_LAUNCH_CHECK();
        int left = 0;
        FE_CUDA(cudaMemcpyAsync(&left, unassigned.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaStreamSynchronize(s));
        if (left != 0 || na == 0) {
            set_error("multigrid setup: a node was left without an aggregate");
            return FE_BREAKDOWN;
        }
        // members of every aggregate in node order (rows = aggregates, no values)
        Mem.n = na;
        FE_CHECK(distinct_rows(
            na,
            [&](int64_t *bound) {
                kd_member_bound<<<grid_s(na), kST, 0, s>>>(na, A.ptr.p, A.col.p, roots.p, bound);
            },
            [&](const int64_t *boff, int32_t *cand, int64_t *cnt) {
                kd_members<<<grid_s(na), kST, 0, s>>>(na, A.ptr.p, A.col.p, roots.p, L.agg.p, boff, cand, cnt);
            },
            Mem, S, s));
        if (Mem.nnzb != n) {
            set_error("multigrid setup: aggregate members do not cover the nodes");
            return FE_BREAKDOWN;
        }
        // tentative prolongator: B's rows, one QR per aggregate in place
        Pt.n = n, Pt.rd = dd, Pt.cd = m, Pt.nnzb = n;
        FE_CHECK(dalloc(Pt.ptr, (size_t)n + 1));
        FE_CHECK(dalloc(Pt.col, (size_t)std::max<int64_t>(n, 1)));
        FE_CHECK(dalloc(Pt.val, (size_t)std::max<int64_t>(n * dd * m, 1)));
        kd_iota<<<grid_s(n + 1), kST, 0, s>>>(n, Pt.ptr.p);
        FE_CUDA(cudaMemcpyAsync(Pt.col.p, L.agg.p, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
        FE_CUDA(cudaMemcpyAsync(Pt.val.p, B.p, n * dd * m * sizeof(double), cudaMemcpyDeviceToDevice, s));
        FE_CHECK(dalloc(Bc, (size_t)std::max<int64_t>(na * m * m, 1)));
        kd_qr<<<grid_s(na), kST, 0, s>>>(na, Mem.ptr.p, Mem.col.p, dd, m, Pt.val.p, Bc.p);
        FE_LAUNCH_CHECK();
        // P = P_t - w D^-1 A P_t, then A_c = P^T (A P)
        FE_CHECK(product_dev(A, Pt, L.P, S, s));
        const double w = 4.0 / (3.0 * L.lmax);
        kd_smooth<<<grid_s(n), kST, 0, s>>>(n, L.P.ptr.p, L.P.col.p, L.P.val.p, L.dinv.p, Pt.val.p, L.agg.p, dd, m, w);
        FE_LAUNCH_CHECK();
        Pt.release();
        FE_CHECK(product_dev(A, L.P, AP, S, s));
        L.PT.n = na, L.PT.rd = m, L.PT.cd = dd;
        FE_CHECK(distinct_rows(
            na,
            [&](int64_t *bound) {
                kd_restr_bound<<<grid_s(na), kST, 0, s>>>(na, Mem.ptr.p, Mem.col.p, A.ptr.p, bound);
            },
            [&](const int64_t *boff, int32_t *cand, int64_t *cnt) {
                kd_restr_cols<<<grid_s(na), kST, 0, s>>>(na, Mem.ptr.p, Mem.col.p, A.ptr.p, A.col.p, boff, cand, cnt);
            },
            L.PT, S, s));
        FE_CHECK(dalloc(L.PT.val, (size_t)std::max<int64_t>(L.PT.nnzb * m * dd, 1)));
        kd_restr_vals<<<grid_s(na), kST, 0, s>>>(na, L.PT.ptr.p, L.PT.col.p, L.PT.val.p, L.P.ptr.p, L.P.col.p,
                                                 L.P.val.p, dd, m);
        FE_LAUNCH_CHECK();
        Mem.release();
        FE_CHECK(product_dev(L.PT, AP, Ac, S, s));
        AP.release();
        FE_CUDA(cudaStreamSynchronize(s));
        L.A = A;            // the level keeps the operator's buffers
        A = Ac;             // and the next level starts from the Galerkin product
        Ac = DevCsr();
        std::swap(B, Bc);
        G.L.push_back(L);
        L = DevLevel();     // now owned by G
    }
    // coarsest level: its dense inverse on the host
    G.coarse = A;
    A = DevCsr();
    BlockCsr C;
    FE_CHECK(csr_to_host(G.coarse, C, s));
    FE_CUDA(cudaStreamSynchronize(s));
    std::vector<double> inv;
    FE_CHECK(coarse_inverse_of(C, inv, "multigrid setup"));
    G.nc = C.n * C.rd;
    FE_CHECK(dalloc(G.cinv, std::max<size_t>(inv.size(), 1)));
    if (!inv.empty())
        FE_CUDA(cudaMemcpyAsync(G.cinv.p, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    FE_CUDA(cudaStreamSynchronize(s));
    return FE_OK;
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
