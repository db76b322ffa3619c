// Row operations of the smoothed-aggregation V-cycle, shared by the host cycle
// (fe_amg_setup.cu) and the device kernels that run it: each function computes one
// block row, so a kernel is a loop of these over rows and the host cycle the same
// loop run serially.  Blocks are row-major, rd x cd, at most 6 x 6.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define FE_HD __host__ __device__ __forceinline__
#else
#define FE_HD inline
#endif

namespace fe {
namespace amg {

// out[0..rd) = sum over the blocks of row i of B_s x[col_s]; T is double (host cycle,
// setup) or float (device cycle)
template <typename T>
FE_HD void row_product(const int64_t *ptr, const int32_t *col, const T *val, int rd, int cd, const T *x,
                       int64_t i, T *out) {
    for (int a = 0; a < rd; ++a) out[a] = T(0);
    for (int64_t s = ptr[i]; s < ptr[i + 1]; ++s) {
        const T *b = val + s * rd * cd;
        const T *xc = x + (int64_t)col[s] * cd;
        for (int a = 0; a < rd; ++a) {
            T acc = T(0);
            for (int k = 0; k < cd; ++k) acc += b[a * cd + k] * xc[k];
            out[a] += acc;
        }
    }
}

// One Chebyshev row update on D^-1 A z = D^-1 r (d x d blocks):
//   res = D_i^-1 (r_i - (A z_in)_i),  dir_i = a dir_i + b res,  z_out_i = z_in_i + dir_i
// with first: dir_i = b res (a and the old dir unused).
template <typename T>
FE_HD void row_chebyshev(const int64_t *ptr, const int32_t *col, const T *val, const T *dinv, int d, const T *r,
                         const T *z_in, T *dir, T *z_out, T a, T b, bool first, int64_t i) {
    T az[6], t[6];
    row_product(ptr, col, val, d, d, z_in, i, az);
    for (int k = 0; k < d; ++k) t[k] = r[i * d + k] - az[k];
    for (int p = 0; p < d; ++p) {
        T res = T(0);
        for (int k = 0; k < d; ++k) res += dinv[i * d * d + p * d + k] * t[k];
        const T dn = first ? b * res : a * dir[i * d + p] + b * res;
        dir[i * d + p] = dn;
        z_out[i * d + p] = z_in[i * d + p] + dn;
    }
}

// t_i = r_i - (A x)_i
template <typename T>
FE_HD void row_residual(const int64_t *ptr, const int32_t *col, const T *val, int d, const T *r, const T *x, T *t,
                        int64_t i) {
    T ax[6];
    row_product(ptr, col, val, d, d, x, i, ax);
    for (int k = 0; k < d; ++k) t[i * d + k] = r[i * d + k] - ax[k];
}

// x_i += (P x_c)_i  (P: d x m blocks)
template <typename T>
FE_HD void row_prolong_add(const int64_t *ptr, const int32_t *col, const T *val, int d, int m, const T *xc, T *x,
                           int64_t i) {
    T px[6];
    row_product(ptr, col, val, d, m, xc, i, px);
    for (int k = 0; k < d; ++k) x[i * d + k] += px[k];
}

// r_c,I = (P^T t)_I  (P^T: m x d blocks)
template <typename T>
FE_HD void row_restrict(const int64_t *ptr, const int32_t *col, const T *val, int m, int d, const T *t, T *rc,
                        int64_t I) {
    T out[6];
    row_product(ptr, col, val, m, d, t, I, out);
    for (int k = 0; k < m; ++k) rc[I * m + k] = out[k];
}

}  // namespace amg
}  // namespace fe
