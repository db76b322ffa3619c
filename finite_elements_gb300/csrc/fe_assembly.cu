// Assembly on the device: element kernels, the sort-based pattern build, the
// segmented reduction of element blocks into node-block CSR slots, loads with the
// reference's last-wins semantics, Dirichlet elimination, and the exports in the
// exact layouts scipy builds (finite_elements/analysis.py:617-708, :345-405).
//
// Layout in HBM.  DOFs are interleaved node-major (dof = node*d + comp,
// finite_elements/core.py:89-108), so K is stored as a CSR of d x d node blocks:
// blk_ptr[n_nodes+1], blk_col[nnzb], values [nnzb][d][d] row-major.  The scalar CSR
// scipy returns is this matrix with every block row expanded and the multiplier
// entries appended; the export kernels produce it on the device.
#include <algorithm>
#include <vector>

#include "fe_element.cuh"
#include "fe_internal.h"

namespace fe {
namespace {


struct Tri {
    double x1, y1, x2, y2, x3, y3;
};

__device__ __forceinline__ Tri load_tri(const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                        int64_t e) {
    int n0 = conn[3 * e], n1 = conn[3 * e + 1], n2 = conn[3 * e + 2];
    double2 p0 = reinterpret_cast<const double2 *>(coords)[n0];
    double2 p1 = reinterpret_cast<const double2 *>(coords)[n1];
    double2 p2 = reinterpret_cast<const double2 *>(coords)[n2];
    return Tri{p0.x, p0.y, p1.x, p1.y, p2.x, p2.y};
}

// (x2-x1)(y3-y1) - (x3-x1)(y2-y1): twice the signed area in the vertex order used by
// element_to_node_factors (elements.py:33) and the triangle area.
__device__ __forceinline__ double det_123(const Tri &t) {
    return sub(mul(sub(t.x2, t.x1), sub(t.y3, t.y1)), mul(sub(t.x3, t.x1), sub(t.y2, t.y1)));
}

__device__ __forceinline__ double tri_area(const Tri &t) { return dvd(fabs(det_123(t)), 2.0); }

// Shape-function coefficients (a_i, b_i, c_i), N_i(p_j) = delta_ij.
__device__ __forceinline__ void form_functions(const Tri &t, double a[3], double b[3], double c[3]) {
    double det = det_123(t);
    a[0] = dvd(sub(mul(t.x2, t.y3), mul(t.x3, t.y2)), det);
    a[1] = dvd(sub(mul(t.x3, t.y1), mul(t.x1, t.y3)), det);
    a[2] = dvd(sub(mul(t.x1, t.y2), mul(t.x2, t.y1)), det);
    b[0] = dvd(sub(t.y2, t.y3), det);
    b[1] = dvd(sub(t.y3, t.y1), det);
    b[2] = dvd(sub(t.y1, t.y2), det);
    c[0] = dvd(sub(t.x3, t.x2), det);
    c[1] = dvd(sub(t.x1, t.x3), det);
    c[2] = dvd(sub(t.x2, t.x1), det);
}

// |detJ| * (a_i + 0.5 b_i x2 + 0.5 c_i y2 + 0.5 b_i x3 + 0.5 c_i y3), term order of
// elements.py:46-51.
__device__ __forceinline__ void node_factors(const Tri &t, double f[3]) {
    double a[3], b[3], c[3];
    form_functions(t, a, b, c);
    double dj = fabs(det_123(t));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double hb = mul(0.5, b[i]), hc = mul(0.5, c[i]);
        double s = add(a[i], mul(hb, t.x2));
        s = add(s, mul(hc, t.y2));
        s = add(s, mul(hb, t.x3));
        s = add(s, mul(hc, t.y3));
        f[i] = mul(dj, s);
    }
}

// ---------------------------------------------------------------- mesh checks

__global__ void k_validate_conn(const int32_t *__restrict__ conn, int64_t n3, int64_t n_nodes,
                                int *err, int *max_node) {
    int local_max = -1;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n3;
         k += (int64_t)gridDim.x * blockDim.x) {
        int v = conn[k];
        if (v < 0 || v >= n_nodes) atomicOr(err, ERR_CONN_RANGE);
        local_max = max(local_max, v);
    }
    for (int o = 16; o > 0; o >>= 1) local_max = max(local_max, __shfl_xor_sync(0xffffffffu, local_max, o));
    if ((threadIdx.x & 31) == 0) atomicMax(max_node, local_max);
}

// ---------------------------------------------------------------- pattern build
// Counting sort of the npe*E (element, local vertex) incidences by node, a per-node
// sort of each incidence list (element order), then per node the sorted set of nodes
// sharing an element with it: the block columns of that node's block row.

__global__ void k_count_incidence(const int32_t *__restrict__ conn, int64_t n3, int32_t *cnt) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n3;
         k += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[conn[k]], 1);
}

__global__ void k_fill_incidence(const int32_t *__restrict__ conn, int64_t n3,
                                 const int32_t *__restrict__ inc_ptr, int32_t *cursor,
                                 int32_t *__restrict__ inc) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n3;
         k += (int64_t)gridDim.x * blockDim.x) {
        int node = conn[k];
        int pos = inc_ptr[node] + atomicAdd(&cursor[node], 1);
        inc[pos] = (int32_t)k;   // element*npe + local vertex
    }
}

__device__ __forceinline__ void insertion_sort(int32_t *a, int n) {
    for (int i = 1; i < n; ++i) {
        int32_t v = a[i];
        int j = i - 1;
        while (j >= 0 && a[j] > v) {
            a[j + 1] = a[j];
            --j;
        }
        a[j + 1] = v;
    }
}

// Sort each node's incidence list, gather the nodes of its elements into cand[]
// (npe per incidence), sort them and count the distinct ones.
__global__ void k_node_neighbours(int64_t n_nodes, int npe, const int32_t *__restrict__ conn,
                                  const int32_t *__restrict__ inc_ptr, int32_t *__restrict__ inc,
                                  int32_t *__restrict__ cand, int32_t *__restrict__ nb_cnt) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_nodes;
         r += (int64_t)gridDim.x * blockDim.x) {
        int s = inc_ptr[r], e = inc_ptr[r + 1], d = e - s;
        insertion_sort(inc + s, d);
        int32_t *c = cand + npe * (int64_t)s;
        for (int t = 0; t < d; ++t) {
            int el = inc[s + t] / npe;
            for (int j = 0; j < npe; ++j) c[npe * t + j] = conn[(int64_t)npe * el + j];
        }
        insertion_sort(c, npe * d);
        int u = 0;
        for (int t = 0; t < npe * d; ++t)
            if (t == 0 || c[t] != c[t - 1]) ++u;
        nb_cnt[r] = u;
    }
}

__global__ void k_write_pattern(int64_t n_nodes, int npe, const int32_t *__restrict__ inc_ptr,
                                const int32_t *__restrict__ cand, const int32_t *__restrict__ blk_ptr,
                                int32_t *__restrict__ blk_col, int32_t *__restrict__ blk_row) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_nodes;
         r += (int64_t)gridDim.x * blockDim.x) {
        int s = inc_ptr[r], d = inc_ptr[r + 1] - s;
        const int32_t *c = cand + npe * (int64_t)s;
        int o = blk_ptr[r];
        for (int t = 0; t < npe * d; ++t)
            if (t == 0 || c[t] != c[t - 1]) {
                blk_col[o] = c[t];
                blk_row[o] = (int32_t)r;
                ++o;
            }
    }
}

// ---------------------------------------------------------------- element kernels

// Plane-elasticity Ke (elements.py:395-453, :466-511).  B uses the signed
// detJ = (x1-x3)(y2-y3) - (y1-y3)(x2-x3); the zero entries of B and D contribute
// exact zeros, so Ke[2i+a][2j+b] reduces to two products per entry in the order of
// (B^T D) B.  Ke = (t * area) * M, area = |detJ|/2.  128 elements per block are
// staged in shared memory and written back as one contiguous, coalesced range.
constexpr int kElemBlock = 128;

__global__ void __launch_bounds__(kElemBlock)
k_elastic_ke(int64_t n_elem, const double *__restrict__ coords, const int32_t *__restrict__ conn,
             const double *__restrict__ E, const double *__restrict__ nu,
             const double *__restrict__ thick, int plane_strain, double *__restrict__ ke_out,
             int *err) {
    __shared__ double tile[kElemBlock * 36];
    for (int64_t base = (int64_t)blockIdx.x * kElemBlock; base < n_elem;
         base += (int64_t)gridDim.x * kElemBlock) {
        int64_t e = base + threadIdx.x;
        double *my = tile + threadIdx.x * 36;
        if (e < n_elem) {
            Tri t = load_tri(coords, conn, e);
            double det = sub(mul(sub(t.x1, t.x3), sub(t.y2, t.y3)), mul(sub(t.y1, t.y3), sub(t.x2, t.x3)));
            double inv = dvd(1.0, det);
            // beta_i = y-differences / det, gamma_i = x-differences / det
            double be[3] = {mul(inv, sub(t.y2, t.y3)), mul(inv, sub(t.y3, t.y1)), mul(inv, sub(t.y1, t.y2))};
            double ga[3] = {mul(inv, sub(t.x3, t.x2)), mul(inv, sub(t.x1, t.x3)), mul(inv, sub(t.x2, t.x1))};
            double Em = E[e], v = nu[e];
            double a = plane_strain ? dvd(mul(Em, v), mul(add(1.0, v), sub(1.0, mul(2.0, v))))
                                    : dvd(mul(Em, v), sub(1.0, mul(v, v)));
            double bb = dvd(Em, mul(2.0, add(1.0, v)));
            double c = add(a, mul(2.0, bb));
            double ta = mul(thick[e], tri_area(t));
            if (!isfinite(ta) || !isfinite(inv) || !isfinite(c)) atomicOr(err, ERR_NONFINITE);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                // rows 2i and 2i+1 of B^T D
                double r0c = mul(be[i], c), r0a = mul(be[i], a), r0b = mul(ga[i], bb);
                double r1a = mul(ga[i], a), r1c = mul(ga[i], c), r1b = mul(be[i], bb);
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    double m00 = add(mul(r0c, be[j]), mul(r0b, ga[j]));
                    double m01 = add(mul(r0a, ga[j]), mul(r0b, be[j]));
                    double m10 = add(mul(r1a, be[j]), mul(r1b, ga[j]));
                    double m11 = add(mul(r1c, ga[j]), mul(r1b, be[j]));
                    my[(2 * i) * 6 + 2 * j] = mul(ta, m00);
                    my[(2 * i) * 6 + 2 * j + 1] = mul(ta, m01);
                    my[(2 * i + 1) * 6 + 2 * j] = mul(ta, m10);
                    my[(2 * i + 1) * 6 + 2 * j + 1] = mul(ta, m11);
                }
            }
        }
        __syncthreads();
        int64_t cnt = min((int64_t)kElemBlock, n_elem - base) * 36;
        double *dst = ke_out + base * 36;
        for (int64_t k = threadIdx.x; k < cnt; k += kElemBlock) dst[k] = tile[k];
        __syncthreads();
    }
}

// Magnetostatic Ke_ij = ((1/mu) * (b_i b_j + c_i c_j)) * area (elements.py:93-118).
__global__ void __launch_bounds__(kElemBlock)
k_magnetic_ke(int64_t n_elem, const double *__restrict__ coords, const int32_t *__restrict__ conn,
              const double *__restrict__ mu, double *__restrict__ ke_out, int *err) {
    __shared__ double tile[kElemBlock * 9];
    for (int64_t base = (int64_t)blockIdx.x * kElemBlock; base < n_elem;
         base += (int64_t)gridDim.x * kElemBlock) {
        int64_t e = base + threadIdx.x;
        double *my = tile + threadIdx.x * 9;
        if (e < n_elem) {
            Tri t = load_tri(coords, conn, e);
            double a[3], b[3], c[3];
            form_functions(t, a, b, c);
            double area = tri_area(t);
            double im = dvd(1.0, mu[e]);
            if (!isfinite(area) || !isfinite(im) || !isfinite(b[0])) atomicOr(err, ERR_NONFINITE);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    my[3 * i + j] = mul(mul(im, add(mul(b[i], b[j]), mul(c[i], c[j]))), area);
        }
        __syncthreads();
        int64_t cnt = min((int64_t)kElemBlock, n_elem - base) * 9;
        double *dst = ke_out + base * 9;
        for (int64_t k = threadIdx.x; k < cnt; k += kElemBlock) dst[k] = tile[k];
        __syncthreads();
    }
}

// Mass scale (rho * area * t) / 12 of elements.py:530-531; Me = scale * P.
__global__ void k_mass_scale(int64_t n_elem, const double *__restrict__ coords,
                             const int32_t *__restrict__ conn, const double *__restrict__ rho,
                             const double *__restrict__ thick, double *__restrict__ out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem;
         e += (int64_t)gridDim.x * blockDim.x) {
        Tri t = load_tri(coords, conn, e);
        out[e] = dvd(mul(mul(rho[e], tri_area(t)), thick[e]), 12.0);
    }
}

// Tetrahedron elasticity Ke = V (B^T D) B (elements.py:808-827) with the isotropic D
// of elements.py:779-796: coef = E/((1+nu)(1-2nu)), normal diagonal coef*(1-nu),
// normal off-diagonal coef*nu, shear coef*((1-2nu)/2).  The zeros of B and D add
// exact zeros, so entry (3i+a, 3j+b) is a sum of two or three products of row a of
// B_i^T D with column b of B_j.  32 elements per block are staged in shared memory
// (144 doubles each) and written back as one contiguous range.
constexpr int kTetBlock = 32;

__global__ void __launch_bounds__(kTetBlock)
k_elastic_tet_ke(int64_t n_elem, const double *__restrict__ coords, const int32_t *__restrict__ conn,
                 const double *__restrict__ E, const double *__restrict__ nu, double *__restrict__ ke_out,
                 int *err) {
    __shared__ double tile[kTetBlock * 144];
    for (int64_t base = (int64_t)blockIdx.x * kTetBlock; base < n_elem; base += (int64_t)gridDim.x * kTetBlock) {
        const int64_t e = base + threadIdx.x;
        double *my = tile + threadIdx.x * 144;
        if (e < n_elem) {
            const TetGrad t = tet_gradients(coords, conn, e);
            const double Em = E[e], v = nu[e];
            const double coef = dvd(Em, mul(add(1.0, v), sub(1.0, mul(2.0, v))));
            const double cn = mul(coef, sub(1.0, v)), cl = mul(coef, v);
            const double cg = mul(coef, dvd(sub(1.0, mul(2.0, v)), 2.0));
            if (!t.finite || !isfinite(t.vol) || !isfinite(cn) || !isfinite(cg)) atomicOr(err, ERR_NONFINITE);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const double gx = t.g[i][0], gy = t.g[i][1], gz = t.g[i][2];
                const double ux = mul(gx, cn), vy = mul(gy, cn), wz = mul(gz, cn);
                const double lx = mul(gx, cl), ly = mul(gy, cl), lz = mul(gz, cl);
                const double sx = mul(gx, cg), sy = mul(gy, cg), sz = mul(gz, cg);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const double hx = t.g[j][0], hy = t.g[j][1], hz = t.g[j][2];
                    double *row0 = my + (3 * i) * 12 + 3 * j, *row1 = row0 + 12, *row2 = row1 + 12;
                    row0[0] = mul(t.vol, add(add(mul(ux, hx), mul(sy, hy)), mul(sz, hz)));
                    row0[1] = mul(t.vol, add(mul(lx, hy), mul(sy, hx)));
                    row0[2] = mul(t.vol, add(mul(lx, hz), mul(sz, hx)));
                    row1[0] = mul(t.vol, add(mul(ly, hx), mul(sx, hy)));
                    row1[1] = mul(t.vol, add(add(mul(vy, hy), mul(sx, hx)), mul(sz, hz)));
                    row1[2] = mul(t.vol, add(mul(ly, hz), mul(sz, hy)));
                    row2[0] = mul(t.vol, add(mul(lz, hx), mul(sx, hz)));
                    row2[1] = mul(t.vol, add(mul(lz, hy), mul(sy, hz)));
                    row2[2] = mul(t.vol, add(add(mul(wz, hz), mul(sy, hy)), mul(sx, hx)));
                }
            }
        }
        __syncthreads();
        const int64_t cnt = min((int64_t)kTetBlock, n_elem - base) * 144;
        double *dst = ke_out + base * 144;
        for (int64_t k = threadIdx.x; k < cnt; k += kTetBlock) dst[k] = tile[k];
        __syncthreads();
    }
}

// Tetrahedron mass scale (rho * V) / 20 of elements.py:845-858; Me = scale * P12,
// P12 block (i, j) = (i == j ? 2 : 1) * I_3.
__global__ void k_mass_scale_tet(int64_t n_elem, const double *__restrict__ coords,
                                 const int32_t *__restrict__ conn, const double *__restrict__ rho,
                                 double *__restrict__ out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem;
         e += (int64_t)gridDim.x * blockDim.x)
        out[e] = dvd(mul(rho[e], tet_gradients(coords, conn, e).vol), 20.0);
}

__global__ void k_node_factors(int64_t n, const int64_t *__restrict__ elems, int64_t n_elem,
                               const double *__restrict__ coords, const int32_t *__restrict__ conn,
                               double *__restrict__ out, int *err) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t e = elems[k];
        if (e < 0 || e >= n_elem) {
            atomicOr(err, ERR_ELEM_RANGE);
            continue;
        }
        double f[3];
        node_factors(load_tri(coords, conn, e), f);
        out[3 * k] = f[0];
        out[3 * k + 1] = f[1];
        out[3 * k + 2] = f[2];
    }
}

// ---------------------------------------------------------------- segmented reduction
// One thread per block slot (row node r, column node m): walk r's incidence list in
// element order and add block (i, j) of every element whose vertex j is m.  The sum
// runs in element order, as the reference's dict merge does (analysis.py:390-395),
// with no atomics: the result is the same on every run.
template <int D, int NPE>
__global__ void k_reduce_stiffness(int64_t nnzb, const int32_t *__restrict__ blk_row,
                                   const int32_t *__restrict__ blk_col, const int32_t *__restrict__ inc_ptr,
                                   const int32_t *__restrict__ inc, const int32_t *__restrict__ conn,
                                   const double *__restrict__ ke, double *__restrict__ kval) {
    constexpr int NL = NPE * D;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nnzb;
         s += (int64_t)gridDim.x * blockDim.x) {
        int r = blk_row[s], m = blk_col[s];
        double acc[D * D];
#pragma unroll
        for (int k = 0; k < D * D; ++k) acc[k] = 0.0;
        int a0 = inc_ptr[r], a1 = inc_ptr[r + 1];
        for (int t = a0; t < a1; ++t) {
            int code = inc[t];
            int e = code / NPE, i = code - NPE * e;
#pragma unroll
            for (int j = 0; j < NPE; ++j) {
                if (conn[NPE * (int64_t)e + j] == m) {
                    const double *blk = ke + (int64_t)e * NL * NL + (i * D) * NL + j * D;
#pragma unroll
                    for (int a = 0; a < D; ++a)
#pragma unroll
                        for (int b = 0; b < D; ++b) acc[a * D + b] = __dadd_rn(acc[a * D + b], blk[a * NL + b]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < D * D; ++k) kval[s * D * D + k] = acc[k];
    }
}

// Mass blocks: Me block (i, j) = scale * (i == j ? 2 : 1) * I_D (elements.py:514-519,
// :830-843).
template <int D, int NPE>
__global__ void k_reduce_mass(int64_t nnzb, const int32_t *__restrict__ blk_row,
                              const int32_t *__restrict__ blk_col, const int32_t *__restrict__ inc_ptr,
                              const int32_t *__restrict__ inc, const int32_t *__restrict__ conn,
                              const double *__restrict__ scale, double *__restrict__ mval) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nnzb;
         s += (int64_t)gridDim.x * blockDim.x) {
        int r = blk_row[s], m = blk_col[s];
        double diag = 0.0;
        int a0 = inc_ptr[r], a1 = inc_ptr[r + 1];
        for (int t = a0; t < a1; ++t) {
            int code = inc[t];
            int e = code / NPE, i = code - NPE * e;
#pragma unroll
            for (int j = 0; j < NPE; ++j)
                if (conn[NPE * (int64_t)e + j] == m) diag = __dadd_rn(diag, __dmul_rn(scale[e], i == j ? 2.0 : 1.0));
        }
        // the off-diagonal entries of the block are sums of exact zeros
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b = 0; b < D; ++b) mval[s * D * D + a * D + b] = a == b ? diag : 0.0;
    }
}

// ---------------------------------------------------------------- loads
// The reference keeps, per (node, dimension), the last load of its list
// (analysis.py:71-110).  Every load carries its list position as seq; an atomicMax
// picks the winner, then the winner alone writes F.

__global__ void k_init_loads(int64_t n_dof, double *F, long long *seq) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_dof;
         k += (int64_t)gridDim.x * blockDim.x) {
        F[k] = 0.0;
        seq[k] = -1;
    }
}

__global__ void k_node_load_seq(int64_t n, const int64_t *__restrict__ dof, const int64_t *__restrict__ sq,
                                int64_t n_dof, long long *seq, int *err) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t d = dof[k];
        if (d < 0 || d >= n_dof) {
            atomicOr(err, ERR_DOF_RANGE);
            continue;
        }
        atomicMax(&seq[d], (long long)sq[k]);
    }
}

__global__ void k_node_load_write(int64_t n, const int64_t *__restrict__ dof, const int64_t *__restrict__ sq,
                                  const double *__restrict__ val, int64_t n_dof,
                                  const long long *__restrict__ seq, double *F) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t d = dof[k];
        if (d < 0 || d >= n_dof) continue;
        if (seq[d] == sq[k]) F[d] = val[k];
    }
}

// Set of each element occurrence (binary search of the set pointers).
__global__ void k_load_set_of(int64_t n_occ, const int64_t *__restrict__ set_ptr, int64_t n_sets,
                              int32_t *__restrict__ set_of) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_occ;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = n_sets - 1;
        while (lo < hi) {
            int64_t mid = (lo + hi + 1) / 2;
            if (set_ptr[mid] <= k) lo = mid;
            else hi = mid - 1;
        }
        set_of[k] = (int32_t)lo;
    }
}

// sum(elem.area for elem in elements) of loads.py:32, left to right, one thread per
// set so that the rounding is that of the reference's sequential sum.
__global__ void k_load_area_total(int64_t n_sets, const int64_t *__restrict__ set_ptr,
                                  const int64_t *__restrict__ elems, int64_t n_elem,
                                  const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                  double *__restrict__ total, int *err) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_sets;
         s += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int64_t k = set_ptr[s]; k < set_ptr[s + 1]; ++k) {
            int64_t e = elems[k];
            if (e < 0 || e >= n_elem) {
                atomicOr(err, ERR_ELEM_RANGE);
                continue;
            }
            acc = __dadd_rn(acc, tri_area(load_tri(coords, conn, e)));
        }
        total[s] = acc;
    }
}

template <bool WRITE>
__global__ void k_element_loads(int64_t n_occ, const int32_t *__restrict__ set_of,
                                const int64_t *__restrict__ elems, const double *__restrict__ set_val,
                                const int32_t *__restrict__ set_dim, const double *__restrict__ total,
                                int64_t seq_base, int D, int64_t n_elem,
                                const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                long long *seq, double *F, int *err) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_occ;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t e = elems[k];
        if (e < 0 || e >= n_elem) continue;
        int s = set_of[k];
        int dm = set_dim[s];
        if (dm < 1 || dm > D) {
            atomicOr(err, ERR_DOF_RANGE);
            continue;
        }
        double f[3] = {0, 0, 0}, per = 0.0;
        if (WRITE) {
            Tri t = load_tri(coords, conn, e);
            node_factors(t, f);
            per = dvd(mul(set_val[s], tri_area(t)), total[s]);
        }
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            int64_t dof = (int64_t)conn[3 * e + p] * D + (dm - 1);
            long long sq = seq_base + 3 * k + p;
            if (!WRITE) atomicMax(&seq[dof], sq);
            else if (seq[dof] == sq) F[dof] = mul(per, f[p]);
        }
    }
}

// ---------------------------------------------------------------- Dirichlet elimination

__global__ void k_bc_map(int64_t n_bc, const int64_t *__restrict__ dof, int64_t n_dof,
                         int32_t *bc_of_dof, int *err) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n_bc;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t d = dof[k];
        if (d < 0 || d >= n_dof) {
            atomicOr(err, ERR_DOF_RANGE);
            continue;
        }
        bc_of_dof[d] = (int32_t)k;
    }
}

// A = K with every constrained row and column replaced by the identity's.
template <int D>
__global__ void k_eliminate(int64_t nnzb, const int32_t *__restrict__ blk_row,
                            const int32_t *__restrict__ blk_col, const int32_t *__restrict__ bc_of_dof,
                            const double *__restrict__ kval, const double *__restrict__ mval, double ka,
                            double mb, double *__restrict__ aval, float *__restrict__ aval32) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nnzb;
         s += (int64_t)gridDim.x * blockDim.x) {
        int r = blk_row[s], m = blk_col[s];
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b = 0; b < D; ++b) {
                int64_t rd = (int64_t)r * D + a, cd = (int64_t)m * D + b;
                // the system matrix ka K + mb M (K alone for the static solve)
                double v = mval ? ka * kval[s * D * D + a * D + b] + mb * mval[s * D * D + a * D + b]
                                : kval[s * D * D + a * D + b];
                if (bc_of_dof[rd] >= 0 || bc_of_dof[cd] >= 0) v = (rd == cd) ? 1.0 : 0.0;
                aval[s * D * D + a * D + b] = v;
                aval32[s * D * D + a * D + b] = (float)v;
            }
    }
}

// Difference form of A: (A x)_r = sum_{m != r} A_rm (x_m - x_r) + S_r x_r with the
// block row sum S_r = sum_m A_rm, which vanishes at interior nodes (K annihilates
// translations).  Evaluated this way, rounding scales with the differences of x
// between neighbours instead of with x.  S_r is summed in double-double (TwoSum), so
// its own error is eps64 * |S_r| rather than eps64 * sum |A_rm|.  Writes S_r in FP64
// (for the FP64 true residual) and the FP32 copy of A with S_r in the diagonal slot
// (for the mixed solver's SpMV).
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
    s = __dadd_rn(a, b);
    double bb = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

template <int D>
__global__ void k_diff_form(int64_t n_nodes, const int32_t *__restrict__ blk_ptr,
                            const int32_t *__restrict__ blk_col, const double *__restrict__ aval,
                            double *__restrict__ srow, float *__restrict__ aval32) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_nodes;
         r += (int64_t)gridDim.x * blockDim.x) {
        double hi[D * D], lo[D * D];
#pragma unroll
        for (int k = 0; k < D * D; ++k) hi[k] = 0.0, lo[k] = 0.0;
        int diag = -1;
        for (int s = blk_ptr[r]; s < blk_ptr[r + 1]; ++s) {
            if (blk_col[s] == (int)r) diag = s;
#pragma unroll
            for (int k = 0; k < D * D; ++k) {
                double t, e;
                two_sum(hi[k], aval[(int64_t)s * D * D + k], t, e);
                hi[k] = t;
                lo[k] = __dadd_rn(lo[k], e);
            }
        }
#pragma unroll
        for (int k = 0; k < D * D; ++k) {
            double S = __dadd_rn(hi[k], lo[k]);
            srow[r * D * D + k] = S;
            if (diag >= 0) aval32[(int64_t)diag * D * D + k] = (float)S;
        }
    }
}

// b = F - K[:, c] g on free rows, b = g on constrained rows.
template <int D>
__global__ void k_eliminated_rhs(int64_t n_nodes, const int32_t *__restrict__ blk_ptr,
                                 const int32_t *__restrict__ blk_col, const int32_t *__restrict__ bc_of_dof,
                                 const double *__restrict__ bc_val, const double *__restrict__ kval,
                                 const double *__restrict__ F, double *__restrict__ b) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_nodes;
         r += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < D; ++a) {
            int64_t rd = r * D + a;
            int k = bc_of_dof[rd];
            if (k >= 0) {
                b[rd] = bc_val[k];
                continue;
            }
            double acc = F[rd];
            for (int s = blk_ptr[r]; s < blk_ptr[r + 1]; ++s) {
                int m = blk_col[s];
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    int kc = bc_of_dof[(int64_t)m * D + c];
                    if (kc >= 0) acc -= kval[(int64_t)s * D * D + a * D + c] * bc_val[kc];
                }
            }
            b[rd] = acc;
        }
    }
}

__device__ __forceinline__ int find_col(const int32_t *__restrict__ cols, int lo, int hi, int key) {
    // first index in [lo, hi) with cols[idx] == key, or -1
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (cols[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Inverse of one D x D block (row-major): 1/v, the 2 x 2 adjugate formula, or the
// 3 x 3 cofactors over the determinant.  False when the block is singular.
template <int D>
__device__ __forceinline__ bool invert_block(const double *a, double *o) {
    if constexpr (D == 1) {
        const double inv = 1.0 / a[0];
        o[0] = inv;
        return a[0] != 0.0 && isfinite(inv);
    } else if constexpr (D == 2) {
        const double det = a[0] * a[3] - a[1] * a[2];
        const double id = 1.0 / det;
        o[0] = a[3] * id, o[1] = -a[1] * id, o[2] = -a[2] * id, o[3] = a[0] * id;
        return det != 0.0 && isfinite(id);
    } else {
        const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8];
        const double c02 = a[3] * a[7] - a[4] * a[6];
        const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
        const double id = 1.0 / det;
        o[0] = c00 * id, o[1] = (a[2] * a[7] - a[1] * a[8]) * id, o[2] = (a[1] * a[5] - a[2] * a[4]) * id;
        o[3] = c01 * id, o[4] = (a[0] * a[8] - a[2] * a[6]) * id, o[5] = (a[2] * a[3] - a[0] * a[5]) * id;
        o[6] = c02 * id, o[7] = (a[1] * a[6] - a[0] * a[7]) * id, o[8] = (a[0] * a[4] - a[1] * a[3]) * id;
        return det != 0.0 && isfinite(id);
    }
}

// Inverse of every diagonal block of A (node-block Jacobi).
template <int D>
__global__ void k_block_jacobi(int64_t n_nodes, const int32_t *__restrict__ blk_ptr,
                               const int32_t *__restrict__ blk_col, const double *__restrict__ aval,
                               double *__restrict__ dinv, float *__restrict__ dinv32, int *err) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_nodes;
         r += (int64_t)gridDim.x * blockDim.x) {
        int lo = blk_ptr[r], hi = blk_ptr[r + 1];
        int s = find_col(blk_col, lo, hi, (int)r);
        bool found = s < hi && blk_col[s] == (int)r;
        double a[D * D], o[D * D];
#pragma unroll
        for (int k = 0; k < D * D; ++k) a[k] = found ? aval[(int64_t)s * D * D + k] : 0.0;
        if (!invert_block<D>(a, o) || !found) {
            atomicOr(err, ERR_SINGULAR_BLOCK);
#pragma unroll
            for (int k = 0; k < D * D; ++k) o[k] = 0.0;
        }
#pragma unroll
        for (int k = 0; k < D * D; ++k) {
            dinv[r * D * D + k] = o[k];
            dinv32[r * D * D + k] = (float)o[k];
        }
    }
}

// ---------------------------------------------------------------- SELL-32 copy for the solver
// Row r carries a row-sum entry when its block row sum S_r is not rounding noise: S_r
// vanishes exactly (K annihilates rigid translations) except on rows that lost
// columns to the Dirichlet elimination, so a row keeps it when some entry exceeds
// 1e-12 of the largest diagonal entry.
template <int D>
__device__ __forceinline__ bool has_row_sum(const double *__restrict__ srow, const double *__restrict__ d64row) {
    double smax = 0.0, dmax = 0.0;
#pragma unroll
    for (int q = 0; q < D * D; ++q) smax = fmax(smax, fabs(srow[q])), dmax = fmax(dmax, fabs(d64row[q]));
    return smax > 1e-12 * dmax;
}

// Width of each slice: the largest entry count of its 32 rows -- off-diagonal blocks
// plus the row-sum entry -- (rows past the end count 0), stored as 32 * width so that
// a scan gives the slice offsets.
template <int D>
__global__ void k_sell_widths(int64_t n_nodes, int64_t n_slices, const int32_t *__restrict__ blk_ptr,
                              const int32_t *__restrict__ blk_col, const double *__restrict__ aval,
                              const double *__restrict__ srow, int32_t *__restrict__ len) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t sl = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < n_slices; sl += warps) {
        int64_t r = sl * 32 + lane;
        int w = 0;
        if (r < n_nodes) {
            const int lo = blk_ptr[r], hi = blk_ptr[r + 1];
            const int s = find_col(blk_col, lo, hi, (int)r);
            const bool found = s < hi && blk_col[s] == (int)r;
            w = hi - lo - (found ? 1 : 0);
            if (found && has_row_sum<D>(srow + r * D * D, aval + (int64_t)s * D * D)) ++w;
        }
        w = max(w, 0);
        for (int o = 16; o > 0; o >>= 1) w = max(w, __shfl_xor_sync(0xffffffffu, w, o));
        if (lane == 0) len[sl] = 32 * w;
    }
}

// D^-1 B for one block row (r's inverse diagonal block times block B), in FP64.
template <int D>
__device__ __forceinline__ void scale_block(const double *__restrict__ dinv_r, const double *__restrict__ b,
                                            double *out) {
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) acc = fma(dinv_r[i * D + k], b[k * D + j], acc);
            out[i * D + j] = acc;
        }
}

// SELL-32 fill.  Columns as int32 (col) and as 16-bit offsets c - r (dcol, usable when
// no offset overflows: *dcol_over stays 0).  FP64 copy: the eliminated blocks A_rm and
// the diagonal A_rr (diag64).
// FP32 copy, prescaled by the node-block Jacobi inverse for the Chebyshev steps and in
// difference form: blocks D_r^-1 A_rm applied to x_m - x_r and, where S_r is not
// rounding noise, a first entry with column r holding D_r^-1 S_r, applied to x_r
// itself (a zero block in the FP64 copy).  dblk32 keeps A_rr in FP32 so that a product
// with the FP32 copy can be scaled back to A x.
template <int D>
__global__ void k_sell_fill(int64_t n_nodes, int64_t n_slices, const int32_t *__restrict__ blk_ptr,
                            const int32_t *__restrict__ blk_col, const double *__restrict__ aval,
                            const double *__restrict__ srow, const double *__restrict__ dinv,
                            const int32_t *__restrict__ off, int32_t *__restrict__ col, double *__restrict__ v64,
                            float *__restrict__ v32, double *__restrict__ d64, float *__restrict__ d32,
                            float *__restrict__ dblk32, int16_t *__restrict__ dcol, int *__restrict__ dcol_over) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_slices * 32;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t sl = r >> 5, lane = r & 31;
        const int64_t base = off[sl];
        const int w = (off[sl + 1] - off[sl]) >> 5;
        int k = 0;
        if (r < n_nodes) {
            const double *dr = dinv + r * D * D;
            double sc[D * D];
            scale_block<D>(dr, srow + r * D * D, sc);
#pragma unroll
            for (int q = 0; q < D * D; ++q) d32[r * D * D + q] = (float)sc[q];
            const int lo = blk_ptr[r], hi = blk_ptr[r + 1];
            const int sd = find_col(blk_col, lo, hi, (int)r);
            if (sd < hi && blk_col[sd] == (int)r && has_row_sum<D>(srow + r * D * D, aval + (int64_t)sd * D * D)) {
                const int64_t e = base + lane;
                col[e] = (int32_t)r;
                dcol[e] = 0;
#pragma unroll
                for (int q = 0; q < D * D; ++q) {
                    v64[e * D * D + q] = 0.0;
                    v32[e * D * D + q] = (float)sc[q];
                }
                k = 1;
            }
            for (int s = blk_ptr[r]; s < blk_ptr[r + 1]; ++s) {
                const int c = blk_col[s];
                if (c == (int)r) {
#pragma unroll
                    for (int q = 0; q < D * D; ++q) {
                        d64[r * D * D + q] = aval[(int64_t)s * D * D + q];
                        dblk32[r * D * D + q] = (float)aval[(int64_t)s * D * D + q];
                    }
                    continue;
                }
                const int64_t e = base + 32 * (int64_t)k + lane;
                col[e] = c;
                const int64_t off_c = (int64_t)c - r;
                if (off_c < -32768 || off_c > 32767) atomicOr(dcol_over, 1);
                dcol[e] = (int16_t)max((int64_t)-32768, min((int64_t)32767, off_c));
                scale_block<D>(dr, aval + (int64_t)s * D * D, sc);
#pragma unroll
                for (int q = 0; q < D * D; ++q) {
                    v64[e * D * D + q] = aval[(int64_t)s * D * D + q];
                    v32[e * D * D + q] = (float)sc[q];
                }
                ++k;
            }
        }
        // padding: the row itself (or node 0 past the end) with a zero block
        for (; k < w; ++k) {
            const int64_t e = base + 32 * (int64_t)k + lane;
            col[e] = r < n_nodes ? (int32_t)r : 0;
            dcol[e] = r < n_nodes ? (int16_t)0 : (int16_t)max((int64_t)-32768, -r);
#pragma unroll
            for (int q = 0; q < D * D; ++q) {
                v64[e * D * D + q] = 0.0;
                v32[e * D * D + q] = 0.0f;
            }
        }
    }
}

// ---------------------------------------------------------------- exports
// Augmented CSR of create_matrix: DOF row (r, a) holds the d*deg(r) block columns in
// order, then its multiplier column n_dof + k if the DOF is constrained; multiplier row
// k holds column dof_k.  Row lengths first, then a scan, then the fill.

__global__ void k_aug_row_len(int64_t n_rows_dof, int D, const int32_t *__restrict__ blk_ptr,
                              const int32_t *__restrict__ bc_of_dof, int64_t n_bc, int64_t n_rows,
                              int32_t *__restrict__ len) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (i < n_rows_dof) {
            int64_t r = i / D;
            len[i] = D * (blk_ptr[r + 1] - blk_ptr[r]) + (bc_of_dof && bc_of_dof[i] >= 0 ? 1 : 0);
        } else {
            len[i] = 1;
        }
    }
}

// transpose = 1: write the value of (col, row) in place of (row, col) -- CSC of a
// matrix whose pattern is symmetric.
__global__ void k_aug_fill(int64_t n_rows_dof, int D, int64_t n_dof, const int32_t *__restrict__ blk_ptr,
                           const int32_t *__restrict__ blk_col, const double *__restrict__ val,
                           const int32_t *__restrict__ bc_of_dof, const int64_t *__restrict__ bc_dof,
                           int64_t n_rows, const int32_t *__restrict__ row_off, int transpose,
                           int32_t *__restrict__ indices, double *__restrict__ data, int *err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t o = row_off[i];
        if (i < n_rows_dof) {
            int64_t r = i / D;
            int a = (int)(i - r * D);
            for (int s = blk_ptr[r]; s < blk_ptr[r + 1]; ++s) {
                int m = blk_col[s];
                int st = s;
                if (transpose) {
                    int lo = blk_ptr[m], hi = blk_ptr[m + 1];
                    st = find_col(blk_col, lo, hi, (int)r);
                    if (st >= hi || blk_col[st] != (int)r) {
                        atomicOr(err, ERR_PATTERN);
                        st = s;
                    }
                }
                for (int b = 0; b < D; ++b) {
                    indices[o] = m * D + b;
                    data[o] = transpose ? val[(int64_t)st * D * D + b * D + a]
                                        : val[(int64_t)st * D * D + a * D + b];
                    ++o;
                }
            }
            if (bc_of_dof && bc_of_dof[i] >= 0) {
                indices[o] = (int32_t)(n_dof + bc_of_dof[i]);
                data[o] = 1.0;
            }
        } else {
            int64_t k = i - n_dof;
            indices[o] = (int32_t)bc_dof[k];
            data[o] = 1.0;
        }
    }
}

int sync_err(fe_handle_s *h) {
    FE_CUDA(cudaMemcpyAsync(h->err_host, h->err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    FE_CUDA(cudaStreamSynchronize(h->stream));
    return FE_OK;
}

}  // namespace

int check_error_word(fe_handle_s *h, const char *where) {
    FE_CHECK(sync_err(h));
    int e = *h->err_host;
    if (!e) return FE_OK;
    FE_CUDA(cudaMemsetAsync(h->err.p, 0, sizeof(int), h->stream));
    if (e == ERR_SINGULAR_BLOCK) {
        // a singular diagonal block (a node no element touches) makes the system
        // singular, as in the reference, where spsolve then returns NaN: the solve
        // reports FE_BREAKDOWN instead of the assembly failing
        h->singular = true;
        return FE_OK;
    }
    std::string msg = std::string(where) + ":";
    if (e & ERR_CONN_RANGE) msg += " connectivity index out of range;";
    if (e & ERR_DOF_RANGE) msg += " load/condition DOF or dimension out of range;";
    if (e & ERR_ELEM_RANGE) msg += " element index out of range;";
    if (e & ERR_NONFINITE) msg += " non-finite element value (degenerate element or bad material);";
    if (e & ERR_SINGULAR_BLOCK) msg += " singular diagonal block (node without stiffness);";
    if (e & ERR_PATTERN) msg += " inconsistent pattern;";
    set_error(msg);
    if (e & ERR_NONFINITE) return FE_NONFINITE;
    if (e & ERR_SINGULAR_BLOCK) return FE_BREAKDOWN;
    return FE_BAD_INPUT;
}

int validate_mesh(fe_handle_s *h) {
    DBuf<int32_t> mx;
    FE_CHECK(dalloc(mx, 1));
    int init = -1;
    FE_CUDA(cudaMemcpyAsync(mx.p, &init, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    int64_t n3 = h->n_elem * h->npe;
    if (n3 > 0) {
        k_validate_conn<<<grid_for(n3), kThreads, 0, h->stream>>>(h->conn.p, n3, h->n_nodes, h->err.p, mx.p);
        FE_LAUNCH_CHECK();
        h->launches += 1;
    }
    int m = -1;
    FE_CUDA(cudaMemcpyAsync(&m, mx.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    int st = check_error_word(h, "fe_mesh_create");
    dfree(mx);
    h->max_node = m;
    return st;
}

int build_pattern(fe_handle_s *h) {
    if (h->pattern_ready) return FE_OK;
    cudaStream_t s = h->stream;
    const int npe = h->npe;
    int64_t n = h->n_nodes, n3 = h->n_elem * npe;
    FE_CHECK(dalloc(h->counts, (size_t)n + 1));
    FE_CHECK(dalloc(h->inc_ptr, (size_t)n + 1));
    FE_CHECK(dalloc(h->inc, (size_t)std::max<int64_t>(n3, 1)));
    FE_CHECK(dalloc(h->cand, (size_t)std::max<int64_t>(npe * n3, 1)));
    FE_CUDA(cudaMemsetAsync(h->counts.p, 0, (n + 1) * sizeof(int32_t), s));
    if (n3 > 0) {
        k_count_incidence<<<grid_for(n3), kThreads, 0, s>>>(h->conn.p, n3, h->counts.p);
        FE_LAUNCH_CHECK();
    }
    int64_t tot = 0;
    FE_CHECK(exclusive_scan_i32(h->counts.p, h->inc_ptr.p, n, &tot, h->scan_tmp, s));
    FE_CUDA(cudaMemsetAsync(h->counts.p, 0, (n + 1) * sizeof(int32_t), s));
    if (n3 > 0) {
        k_fill_incidence<<<grid_for(n3), kThreads, 0, s>>>(h->conn.p, n3, h->inc_ptr.p, h->counts.p, h->inc.p);
        FE_LAUNCH_CHECK();
    }
    k_node_neighbours<<<grid_for(n), kThreads, 0, s>>>(n, npe, h->conn.p, h->inc_ptr.p, h->inc.p, h->cand.p,
                                                        h->counts.p);
    FE_LAUNCH_CHECK();
    FE_CHECK(dalloc(h->blk_ptr, (size_t)n + 1));
    int64_t nnzb = 0;
    FE_CHECK(exclusive_scan_i32(h->counts.p, h->blk_ptr.p, n, &nnzb, h->scan_tmp, s));
    FE_CHECK(dalloc(h->blk_col, (size_t)std::max<int64_t>(nnzb, 1)));
    FE_CHECK(dalloc(h->blk_row, (size_t)std::max<int64_t>(nnzb, 1)));
    k_write_pattern<<<grid_for(n), kThreads, 0, s>>>(n, npe, h->inc_ptr.p, h->cand.p, h->blk_ptr.p, h->blk_col.p,
                                                      h->blk_row.p);
    FE_LAUNCH_CHECK();
    h->nnzb = nnzb;
    h->launches += (n3 > 0 ? 2 : 0) + 2 + 2 * 3;
    dfree(h->cand);
    h->pattern_ready = true;
    return FE_OK;
}

int assemble_stiffness(fe_handle_s *h) {
    cudaStream_t s = h->stream;
    const int D = h->dim, NL = h->npe * D;
    FE_CHECK(dalloc(h->ke, (size_t)std::max<int64_t>(h->n_elem * NL * NL, 1)));
    if (h->n_elem > 0) {
        if (h->kind == FE_KIND_ELASTIC_TRI)
            k_elastic_ke<<<grid_for(h->n_elem, kElemBlock, 152 * 64), kElemBlock, 0, s>>>(
                h->n_elem, h->coords.p, h->conn.p, h->E.p, h->nu.p, h->thick.p, h->plane == FE_PLANE_STRAIN, h->ke.p,
                h->err.p);
        else if (h->kind == FE_KIND_ELASTIC_TET)
            k_elastic_tet_ke<<<grid_for(h->n_elem, kTetBlock, 152 * 64), kTetBlock, 0, s>>>(
                h->n_elem, h->coords.p, h->conn.p, h->E.p, h->nu.p, h->ke.p, h->err.p);
        else
            k_magnetic_ke<<<grid_for(h->n_elem, kElemBlock, 152 * 64), kElemBlock, 0, s>>>(
                h->n_elem, h->coords.p, h->conn.p, h->mu.p, h->ke.p, h->err.p);
        FE_LAUNCH_CHECK();
    }
    if (h->n_elem > 0) h->launches += 1;
    FE_CHECK(dalloc(h->kval, (size_t)std::max<int64_t>(h->nnzb * D * D, 1)));
    if (h->nnzb > 0) {
        int g = grid_for(h->nnzb, kThreads, 152 * 64);
        FE_CHECK(with_dim(D, [&](auto dc) {
            constexpr int DD = decltype(dc)::value;
            constexpr int NPE = DD == 3 ? 4 : 3;   // tetrahedra carry 3 DOF per node, triangles 1 or 2
            k_reduce_stiffness<DD, NPE><<<g, kThreads, 0, s>>>(h->nnzb, h->blk_row.p, h->blk_col.p, h->inc_ptr.p,
                                                               h->inc.p, h->conn.p, h->ke.p, h->kval.p);
            return FE_OK;
        }));
        FE_LAUNCH_CHECK();
    }
    if (h->nnzb > 0) h->launches += 1;
    h->k_ready = true;
    return FE_OK;
}

int assemble_mass(fe_handle_s *h) {
    if ((h->kind != FE_KIND_ELASTIC_TRI && h->kind != FE_KIND_ELASTIC_TET) || !h->have_rho) {
        set_error("mass matrices need elasticity elements with a mass density");
        return FE_NOT_READY;
    }
    cudaStream_t s = h->stream;
    const int D = h->dim;
    FE_CHECK(dalloc(h->me_scale, (size_t)std::max<int64_t>(h->n_elem, 1)));
    if (h->n_elem > 0) {
        if (h->kind == FE_KIND_ELASTIC_TET)
            k_mass_scale_tet<<<grid_for(h->n_elem), kThreads, 0, s>>>(h->n_elem, h->coords.p, h->conn.p, h->rho.p,
                                                                      h->me_scale.p);
        else
            k_mass_scale<<<grid_for(h->n_elem), kThreads, 0, s>>>(h->n_elem, h->coords.p, h->conn.p, h->rho.p,
                                                                  h->thick.p, h->me_scale.p);
        FE_LAUNCH_CHECK();
    }
    FE_CHECK(dalloc(h->mval, (size_t)std::max<int64_t>(h->nnzb * D * D, 1)));
    if (h->nnzb > 0) {
        const int g = grid_for(h->nnzb, kThreads, 152 * 64);
        if (h->kind == FE_KIND_ELASTIC_TET)
            k_reduce_mass<3, 4><<<g, kThreads, 0, s>>>(h->nnzb, h->blk_row.p, h->blk_col.p, h->inc_ptr.p, h->inc.p,
                                                       h->conn.p, h->me_scale.p, h->mval.p);
        else
            k_reduce_mass<2, 3><<<g, kThreads, 0, s>>>(h->nnzb, h->blk_row.p, h->blk_col.p, h->inc_ptr.p, h->inc.p,
                                                       h->conn.p, h->me_scale.p, h->mval.p);
        FE_LAUNCH_CHECK();
    }
    h->launches += (h->n_elem > 0 ? 1 : 0) + (h->nnzb > 0 ? 1 : 0);
    h->m_ready = true;
    return FE_OK;
}

int assemble_loads(fe_handle_s *h) {
    cudaStream_t s = h->stream;
    FE_CHECK(dalloc(h->F, (size_t)std::max<int64_t>(h->n_dof, 1)));
    FE_CHECK(dalloc(h->load_seq, (size_t)std::max<int64_t>(h->n_dof, 1)));
    k_init_loads<<<grid_for(h->n_dof), kThreads, 0, s>>>(h->n_dof, h->F.p, h->load_seq.p);
    FE_LAUNCH_CHECK();
    if (h->n_node_loads > 0) {
        k_node_load_seq<<<grid_for(h->n_node_loads), kThreads, 0, s>>>(h->n_node_loads, h->nl_dof.p, h->nl_seq.p,
                                                                       h->n_dof, h->load_seq.p, h->err.p);
        FE_LAUNCH_CHECK();
    }
    if (h->n_load_elems > 0) {
        FE_CHECK(dalloc(h->ls_of_occ, (size_t)h->n_load_elems));
        FE_CHECK(dalloc(h->ls_area_total, (size_t)h->n_load_sets));
        k_load_set_of<<<grid_for(h->n_load_elems), kThreads, 0, s>>>(h->n_load_elems, h->ls_ptr.p, h->n_load_sets,
                                                                     h->ls_of_occ.p);
        FE_LAUNCH_CHECK();
        k_load_area_total<<<grid_for(h->n_load_sets, 32), 32, 0, s>>>(h->n_load_sets, h->ls_ptr.p, h->ls_elems.p,
                                                                      h->n_elem, h->coords.p, h->conn.p,
                                                                      h->ls_area_total.p, h->err.p);
        FE_LAUNCH_CHECK();
        k_element_loads<false><<<grid_for(h->n_load_elems), kThreads, 0, s>>>(
            h->n_load_elems, h->ls_of_occ.p, h->ls_elems.p, h->ls_val.p, h->ls_dim.p, h->ls_area_total.p,
            h->load_seq_base, h->dim, h->n_elem, h->coords.p, h->conn.p, h->load_seq.p, h->F.p, h->err.p);
        FE_LAUNCH_CHECK();
    }
    if (h->n_node_loads > 0) {
        k_node_load_write<<<grid_for(h->n_node_loads), kThreads, 0, s>>>(
            h->n_node_loads, h->nl_dof.p, h->nl_seq.p, h->nl_val.p, h->n_dof, h->load_seq.p, h->F.p);
        FE_LAUNCH_CHECK();
    }
    if (h->n_load_elems > 0) {
        k_element_loads<true><<<grid_for(h->n_load_elems), kThreads, 0, s>>>(
            h->n_load_elems, h->ls_of_occ.p, h->ls_elems.p, h->ls_val.p, h->ls_dim.p, h->ls_area_total.p,
            h->load_seq_base, h->dim, h->n_elem, h->coords.p, h->conn.p, h->load_seq.p, h->F.p, h->err.p);
        FE_LAUNCH_CHECK();
    }
    // magnet-load contributions, added after the loads (analysis.py:681-708)
    FE_CHECK(apply_rhs_additions(h));
    h->launches += 1 + (h->n_node_loads > 0 ? 2 : 0) + (h->n_load_elems > 0 ? 4 : 0);
    h->f_ready = true;
    return FE_OK;
}

int apply_dirichlet(fe_handle_s *h) { return build_system(h, 1.0, 0.0, true); }

// System matrix ka K + mb M (mb != 0 needs M), with the Dirichlet elimination when
// use_bc, its difference form, block-Jacobi inverses and the SELL copies; the
// eliminated right-hand side when the loads are assembled.
int build_system(fe_handle_s *h, double ka, double mb, bool use_bc) {
    cudaStream_t s = h->stream;
    const int D = h->dim;
    const double *mv = mb != 0.0 ? h->mval.p : nullptr;
    FE_CHECK(dalloc(h->bc_of_dof, (size_t)std::max<int64_t>(h->n_dof, 1)));
    FE_CUDA(cudaMemsetAsync(h->bc_of_dof.p, 0xff, h->n_dof * sizeof(int32_t), s));
    if (use_bc && h->n_bc > 0) {
        k_bc_map<<<grid_for(h->n_bc), kThreads, 0, s>>>(h->n_bc, h->bc_dof.p, h->n_dof, h->bc_of_dof.p, h->err.p);
        FE_LAUNCH_CHECK();
    }
    size_t nv = (size_t)std::max<int64_t>(h->nnzb * D * D, 1);
    FE_CHECK(dalloc(h->aval, nv));
    FE_CHECK(dalloc(h->aval32, nv));
    FE_CHECK(dalloc(h->b, (size_t)std::max<int64_t>(h->n_dof, 1)));
    FE_CHECK(dalloc(h->dinv, (size_t)std::max<int64_t>(h->n_nodes * D * D, 1)));
    FE_CHECK(dalloc(h->srow, (size_t)std::max<int64_t>(h->n_nodes * D * D, 1)));
    FE_CHECK(dalloc(h->dinv32, (size_t)std::max<int64_t>(h->n_nodes * D * D, 1)));
    int gs = grid_for(h->nnzb, kThreads, 152 * 64), gn = grid_for(h->n_nodes, kThreads, 152 * 64);
    FE_CHECK(with_dim(D, [&](auto dc) {
        constexpr int DD = decltype(dc)::value;
        if (h->nnzb > 0)
            k_eliminate<DD><<<gs, kThreads, 0, s>>>(h->nnzb, h->blk_row.p, h->blk_col.p, h->bc_of_dof.p, h->kval.p,
                                                    mv, ka, mb, h->aval.p, h->aval32.p);
        k_diff_form<DD><<<gn, kThreads, 0, s>>>(h->n_nodes, h->blk_ptr.p, h->blk_col.p, h->aval.p, h->srow.p,
                                                h->aval32.p);
        if (h->f_ready)
            k_eliminated_rhs<DD><<<gn, kThreads, 0, s>>>(h->n_nodes, h->blk_ptr.p, h->blk_col.p, h->bc_of_dof.p,
                                                         h->bc_val.p, h->kval.p, h->F.p, h->b.p);
        k_block_jacobi<DD><<<gn, kThreads, 0, s>>>(h->n_nodes, h->blk_ptr.p, h->blk_col.p, h->aval.p, h->dinv.p,
                                                   h->dinv32.p, h->err.p);
        return FE_OK;
    }));
    FE_LAUNCH_CHECK();
    h->launches += (use_bc && h->n_bc > 0 ? 1 : 0) + (h->nnzb > 0 ? 1 : 0) + 2 + (h->f_ready ? 1 : 0);
    FE_CHECK(build_sell(h));
    h->w.lmax[0] = h->w.lmax[1] = 0.0;   // a new matrix: new Chebyshev bounds
    h->sys_generation += 1;
    h->sys_ready = true;
    return FE_OK;
}

int build_sell(fe_handle_s *h) {
    cudaStream_t s = h->stream;
    const int D = h->dim;
    const int64_t n_slices = (h->n_nodes + 31) / 32;
    h->n_slices = n_slices;
    FE_CHECK(dalloc(h->counts, (size_t)std::max<int64_t>(n_slices, h->n_nodes) + 1));
    FE_CHECK(dalloc(h->sell_off, (size_t)n_slices + 1));
    if (n_slices > 0) {
        FE_CHECK(with_dim(D, [&](auto dc) {
            constexpr int DD = decltype(dc)::value;
            k_sell_widths<DD><<<grid_for(n_slices * 32), kThreads, 0, s>>>(h->n_nodes, n_slices, h->blk_ptr.p,
                                                                          h->blk_col.p, h->aval.p, h->srow.p,
                                                                          h->counts.p);
            return FE_OK;
        }));
        FE_LAUNCH_CHECK();
    }
    int64_t total = 0;
    FE_CHECK(exclusive_scan_i32(h->counts.p, h->sell_off.p, n_slices, &total, h->scan_tmp, s));
    size_t ne = (size_t)std::max<int64_t>(total, 1);
    FE_CHECK(dalloc(h->sell_col, ne));
    FE_CHECK(dalloc(h->sell_dcol, ne));
    FE_CHECK(dalloc(h->sell_over, 1));
    FE_CUDA(cudaMemsetAsync(h->sell_over.p, 0, sizeof(int), s));
    FE_CHECK(dalloc(h->sell_val64, ne * D * D));
    FE_CHECK(dalloc(h->sell_val32, ne * D * D));
    FE_CHECK(dalloc(h->diag64, (size_t)std::max<int64_t>(h->n_nodes * D * D, 1)));
    FE_CHECK(dalloc(h->diag32, (size_t)std::max<int64_t>(h->n_nodes * D * D, 1)));
    FE_CHECK(dalloc(h->dblk32, (size_t)std::max<int64_t>(h->n_nodes * D * D, 1)));
    // a node without elements has no diagonal block to copy: leave zeros there
    FE_CUDA(cudaMemsetAsync(h->diag64.p, 0, h->n_nodes * D * D * sizeof(double), s));
    FE_CUDA(cudaMemsetAsync(h->diag32.p, 0, h->n_nodes * D * D * sizeof(float), s));
    FE_CUDA(cudaMemsetAsync(h->dblk32.p, 0, h->n_nodes * D * D * sizeof(float), s));
    if (n_slices > 0) {
        int g = grid_for(n_slices * 32, kThreads, 152 * 64);
        FE_CHECK(with_dim(D, [&](auto dc) {
            constexpr int DD = decltype(dc)::value;
            k_sell_fill<DD><<<g, kThreads, 0, s>>>(h->n_nodes, n_slices, h->blk_ptr.p, h->blk_col.p, h->aval.p,
                                                   h->srow.p, h->dinv.p, h->sell_off.p, h->sell_col.p,
                                                   h->sell_val64.p, h->sell_val32.p, h->diag64.p, h->diag32.p,
                                                   h->dblk32.p, h->sell_dcol.p, h->sell_over.p);
            return FE_OK;
        }));
        FE_LAUNCH_CHECK();
    }
    int over = 1;
    FE_CUDA(cudaMemcpyAsync(&over, h->sell_over.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FE_CUDA(cudaStreamSynchronize(s));
    h->sell_c16 = (over == 0);
    h->launches += (n_slices > 0 ? 2 : 0) + 3;
    return FE_OK;
}

int element_node_factors(fe_handle_s *h, int64_t n, const int64_t *elems_dev, double *out_dev) {
    if (n <= 0) return FE_OK;
    k_node_factors<<<grid_for(n), kThreads, 0, h->stream>>>(n, elems_dev, h->n_elem, h->coords.p, h->conn.p,
                                                            out_dev, h->err.p);
    FE_LAUNCH_CHECK();
    h->launches += 1;
    return check_error_word(h, "fe_element_node_factors");
}

// Shapes follow scipy's inference from the largest index present
// (analysis.py:661 and :401): the augmented matrix spans n_dof + n_bc when there is a
// condition, otherwise the DOFs of the largest node any element uses.
int export_sizes(fe_handle_s *h, int which, int64_t *nrows, int64_t *ncols, int64_t *nnz) {
    const int D = h->dim;
    int64_t elem_dofs = (int64_t)(h->max_node + 1) * D;
    int64_t dof_nnz = h->nnzb * D * D;  // every stored block expands to D*D entries
    if (which == FE_MAT_K_AUGMENTED) {
        int64_t n = h->n_bc > 0 ? h->n_dof + h->n_bc : elem_dofs;
        *nrows = *ncols = n;
        *nnz = dof_nnz + 2 * h->n_bc;
    } else if (which == FE_MAT_K_CSC || which == FE_MAT_M_CSC) {
        *nrows = *ncols = elem_dofs;
        *nnz = dof_nnz;
    } else {
        set_error("unknown matrix selector");
        return FE_BAD_INPUT;
    }
    return FE_OK;
}

int export_csr(fe_handle_s *h, int which, int64_t *indptr_host, int32_t *indices_host, double *data_host) {
    cudaStream_t s = h->stream;
    const int D = h->dim;
    int64_t nrows, ncols, nnz;
    FE_CHECK(export_sizes(h, which, &nrows, &ncols, &nnz));
    const double *val = nullptr;
    bool aug = which == FE_MAT_K_AUGMENTED;
    if (which == FE_MAT_M_CSC) {
        if (!h->m_ready) {
            set_error("mass matrix not assembled");
            return FE_NOT_READY;
        }
        val = h->mval.p;
    } else {
        if (!h->k_ready) {
            set_error("stiffness matrix not assembled");
            return FE_NOT_READY;
        }
        val = h->kval.p;
    }
    if (aug && h->n_bc > 0 && !h->bc_of_dof.p) {
        set_error("conditions not applied");
        return FE_NOT_READY;
    }
    int64_t n_rows_dof = aug && h->n_bc > 0 ? h->n_dof : nrows;
    DBuf<int32_t> len, off, idx;
    DBuf<double> dat;
    FE_CHECK(dalloc(len, (size_t)nrows + 1));
    FE_CHECK(dalloc(off, (size_t)nrows + 1));
    FE_CHECK(dalloc(idx, (size_t)std::max<int64_t>(nnz, 1)));
    FE_CHECK(dalloc(dat, (size_t)std::max<int64_t>(nnz, 1)));
    const int32_t *bcmap = aug && h->n_bc > 0 ? h->bc_of_dof.p : nullptr;
    if (nrows > 0) {
        k_aug_row_len<<<grid_for(nrows), kThreads, 0, s>>>(n_rows_dof, D, h->blk_ptr.p, bcmap, h->n_bc, nrows,
                                                           len.p);
        FE_LAUNCH_CHECK();
    }
    int64_t total = 0;
    FE_CHECK(exclusive_scan_i32(len.p, off.p, nrows, &total, h->scan_tmp, s));
    if (total != nnz) {
        dfree(len), dfree(off), dfree(idx), dfree(dat);
        set_error("export size mismatch");
        return FE_BAD_INPUT;
    }
    if (nrows > 0) {
        k_aug_fill<<<grid_for(nrows), kThreads, 0, s>>>(n_rows_dof, D, h->n_dof, h->blk_ptr.p, h->blk_col.p, val,
                                                        bcmap, h->bc_dof.p, nrows, off.p, aug ? 0 : 1, idx.p,
                                                        dat.p, h->err.p);
        FE_LAUNCH_CHECK();
    }
    std::vector<int32_t> off_h((size_t)nrows + 1);
    FE_CUDA(cudaMemcpyAsync(off_h.data(), off.p, (nrows + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (nnz > 0) {
        FE_CUDA(cudaMemcpyAsync(indices_host, idx.p, nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        FE_CUDA(cudaMemcpyAsync(data_host, dat.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    h->launches += (nrows > 0 ? 2 : 0) + 3;
    int st = check_error_word(h, "fe_export_csr");
    for (int64_t i = 0; i <= nrows; ++i) indptr_host[i] = off_h[i];
    dfree(len), dfree(off), dfree(idx), dfree(dat);
    return st;
}

int export_element_matrices(fe_handle_s *h, int which, double *out_host) {
    const int NL = h->npe * h->dim;
    if (which == FE_ASSEMBLE_K) {
        if (!h->k_ready) {
            set_error("stiffness not assembled");
            return FE_NOT_READY;
        }
        FE_CUDA(cudaMemcpyAsync(out_host, h->ke.p, h->n_elem * NL * NL * sizeof(double), cudaMemcpyDeviceToHost,
                                h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
        return FE_OK;
    }
    if (which == FE_ASSEMBLE_M) {
        if (!h->m_ready) {
            set_error("mass not assembled");
            return FE_NOT_READY;
        }
        std::vector<double> sc((size_t)h->n_elem);
        FE_CUDA(cudaMemcpyAsync(sc.data(), h->me_scale.p, h->n_elem * sizeof(double), cudaMemcpyDeviceToHost,
                                h->stream));
        FE_CUDA(cudaStreamSynchronize(h->stream));
        // P = (1 + delta_ij) per node pair times I_D (elements.py:514-519, :830-843)
        const int D = h->dim;
        for (int64_t e = 0; e < h->n_elem; ++e)
            for (int r = 0; r < NL; ++r)
                for (int c = 0; c < NL; ++c) {
                    const double p = (r % D != c % D) ? 0.0 : (r / D == c / D ? 2.0 : 1.0);
                    out_host[e * NL * NL + r * NL + c] = sc[e] * p;
                }
        return FE_OK;
    }
    set_error("unknown element matrix selector");
    return FE_BAD_INPUT;
}

}  // namespace fe
