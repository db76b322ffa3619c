// Per-element post-processing of a solution, the first consumers of solve():
//   elasticity: strain = B q, stress = (D B) q, energy = 0.5 (q^T Ke) q
//               (finite_elements/results.py:809-830, :769-781; elements.py:275-292)
//   magnetostatics: B = (sum_i c_i A_i, -sum_i b_i A_i)  (results.py:121-152)
// q is the element's DOF vector gathered from the solution (node-major, dimension
// minor).  One thread per element; the arithmetic follows the reference's evaluation
// order with explicit round-to-nearest operations, like the element kernels.
#include "fe_element.cuh"
#include "fe_internal.h"

namespace fe {
namespace {


__global__ void k_post_elastic(int64_t n_elem, const double *__restrict__ coords, const int32_t *__restrict__ conn,
                               const double *__restrict__ E, const double *__restrict__ nu, int plane_strain,
                               const double *__restrict__ ke, const double *__restrict__ u,
                               double *__restrict__ strain, double *__restrict__ stress, double *__restrict__ energy) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem;
         e += (int64_t)gridDim.x * blockDim.x) {
        int nd[3] = {conn[3 * e], conn[3 * e + 1], conn[3 * e + 2]};
        double x[3], y[3], q[6];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            x[i] = coords[2 * (int64_t)nd[i]];
            y[i] = coords[2 * (int64_t)nd[i] + 1];
            q[2 * i] = u[2 * (int64_t)nd[i]];
            q[2 * i + 1] = u[2 * (int64_t)nd[i] + 1];
        }
        // B (elements.py:403-414): (1/detJ) * data, signed detJ
        const double det = sub(mul(sub(x[0], x[2]), sub(y[1], y[2])), mul(sub(y[0], y[2]), sub(x[1], x[2])));
        const double inv = dvd(1.0, det);
        const double yc[3] = {sub(y[1], y[2]), sub(y[2], y[0]), sub(y[0], y[1])};
        const double xc[3] = {sub(x[2], x[1]), sub(x[0], x[2]), sub(x[1], x[0])};
        double B[3][6];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            B[0][2 * i] = mul(inv, yc[i]);
            B[0][2 * i + 1] = 0.0;
            B[1][2 * i] = 0.0;
            B[1][2 * i + 1] = mul(inv, xc[i]);
            B[2][2 * i] = mul(inv, xc[i]);
            B[2][2 * i + 1] = mul(inv, yc[i]);
        }
        const double Em = E[e], v = nu[e];
        const double a = plane_strain ? dvd(mul(Em, v), mul(add(1.0, v), sub(1.0, mul(2.0, v))))
                                      : dvd(mul(Em, v), sub(1.0, mul(v, v)));
        const double b = dvd(Em, mul(2.0, add(1.0, v)));
        const double c = add(a, mul(2.0, b));
        const double D[3][3] = {{c, a, 0.0}, {a, c, 0.0}, {0.0, 0.0, b}};
        // strain = B q ; DB = D B ; stress = (D B) q
        double DB[3][6];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                double s = mul(D[r][0], B[0][k]);
                s = add(s, mul(D[r][1], B[1][k]));
                DB[r][k] = add(s, mul(D[r][2], B[2][k]));
            }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            double s = 0.0, t = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                s = add(s, mul(B[r][k], q[k]));
                t = add(t, mul(DB[r][k], q[k]));
            }
            strain[3 * e + r] = s;
            stress[3 * e + r] = t;
        }
        // energy = 0.5 * ((q^T Ke) q)
        const double *K = ke + e * 36;
        double en = 0.0;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            double w = 0.0;
#pragma unroll
            for (int i = 0; i < 6; ++i) w = add(w, mul(q[i], K[i * 6 + j]));
            en = add(en, mul(w, q[j]));
        }
        energy[e] = mul(0.5, en);
    }
}

// Tetrahedron: strain = B q with the rows (xx, yy, zz, xy, yz, zx) of elements.py:743-748
// (the zeros of B dropped), stress = D strain with the isotropic D of
// elements.py:779-796, energy = 0.5 (q^T Ke) q.
__global__ void k_post_elastic_tet(int64_t n_elem, const double *__restrict__ coords,
                                   const int32_t *__restrict__ conn, const double *__restrict__ E,
                                   const double *__restrict__ nu, const double *__restrict__ ke,
                                   const double *__restrict__ u, double *__restrict__ strain,
                                   double *__restrict__ stress, double *__restrict__ energy) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem;
         e += (int64_t)gridDim.x * blockDim.x) {
        const TetGrad t = tet_gradients(coords, conn, e);
        double q[12];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int64_t n = conn[4 * e + i];
#pragma unroll
            for (int a = 0; a < 3; ++a) q[3 * i + a] = u[3 * n + a];
        }
        double eps[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const double gx = t.g[i][0], gy = t.g[i][1], gz = t.g[i][2];
            const double ui = q[3 * i], vi = q[3 * i + 1], wi = q[3 * i + 2];
            eps[0] = add(eps[0], mul(gx, ui));
            eps[1] = add(eps[1], mul(gy, vi));
            eps[2] = add(eps[2], mul(gz, wi));
            eps[3] = add(eps[3], add(mul(gy, ui), mul(gx, vi)));
            eps[4] = add(eps[4], add(mul(gz, vi), mul(gy, wi)));
            eps[5] = add(eps[5], add(mul(gz, ui), mul(gx, wi)));
        }
        const double Em = E[e], v = nu[e];
        const double coef = dvd(Em, mul(add(1.0, v), sub(1.0, mul(2.0, v))));
        const double cn = mul(coef, sub(1.0, v)), cl = mul(coef, v);
        const double cg = mul(coef, dvd(sub(1.0, mul(2.0, v)), 2.0));
        double sig[6];
        sig[0] = add(add(mul(cn, eps[0]), mul(cl, eps[1])), mul(cl, eps[2]));
        sig[1] = add(add(mul(cl, eps[0]), mul(cn, eps[1])), mul(cl, eps[2]));
        sig[2] = add(add(mul(cl, eps[0]), mul(cl, eps[1])), mul(cn, eps[2]));
        sig[3] = mul(cg, eps[3]);
        sig[4] = mul(cg, eps[4]);
        sig[5] = mul(cg, eps[5]);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            strain[6 * e + k] = eps[k];
            stress[6 * e + k] = sig[k];
        }
        const double *K = ke + e * 144;
        double en = 0.0;
#pragma unroll 1
        for (int j = 0; j < 12; ++j) {
            double w = 0.0;
#pragma unroll
            for (int i = 0; i < 12; ++i) w = add(w, mul(q[i], K[i * 12 + j]));
            en = add(en, mul(w, q[j]));
        }
        energy[e] = mul(0.5, en);
    }
}

__global__ void k_post_magnetic(int64_t n_elem, const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                const double *__restrict__ A, double *__restrict__ Bf) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem;
         e += (int64_t)gridDim.x * blockDim.x) {
        int nd[3] = {conn[3 * e], conn[3 * e + 1], conn[3 * e + 2]};
        double x[3], y[3], a[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            x[i] = coords[2 * (int64_t)nd[i]];
            y[i] = coords[2 * (int64_t)nd[i] + 1];
            a[i] = A[nd[i]];
        }
        // form-function coefficients b_i, c_i (N_i = a_i + b_i x + c_i y)
        const double det = sub(mul(sub(x[1], x[0]), sub(y[2], y[0])), mul(sub(x[2], x[0]), sub(y[1], y[0])));
        const double bb[3] = {dvd(sub(y[1], y[2]), det), dvd(sub(y[2], y[0]), det), dvd(sub(y[0], y[1]), det)};
        const double cc[3] = {dvd(sub(x[2], x[1]), det), dvd(sub(x[0], x[2]), det), dvd(sub(x[1], x[0]), det)};
        double bx = add(add(mul(cc[0], a[0]), mul(cc[1], a[1])), mul(cc[2], a[2]));
        double by = sub(sub(mul(-bb[0], a[0]), mul(bb[1], a[1])), mul(bb[2], a[2]));
        Bf[2 * e] = bx;
        Bf[2 * e + 1] = by;
    }
}

}  // namespace
}  // namespace fe

using namespace fe;

extern "C" {

int fe_post_elastic(fe_handle h, const double *u_host, double *strain_host, double *stress_host,
                    double *energy_host) {
    if (!h || !strain_host || !stress_host || !energy_host) {
        set_error("fe_post_elastic: null argument");
        return FE_BAD_INPUT;
    }
    if ((h->kind != FE_KIND_ELASTIC_TRI && h->kind != FE_KIND_ELASTIC_TET) || !h->k_ready) {
        set_error("fe_post_elastic: needs an assembled elasticity handle");
        return FE_NOT_READY;
    }
    if (!u_host && !h->have_solution) {
        set_error("fe_post_elastic: no displacement given and no solution yet");
        return FE_NOT_READY;
    }
    const int64_t ne = h->n_elem;
    const int nc = h->kind == FE_KIND_ELASTIC_TET ? 6 : 3;   // strain / stress components
    DBuf<double> ud, out;
    int st = dalloc(out, (size_t)std::max<int64_t>((2 * nc + 1) * ne, 1));
    const double *u = h->w.x.p;
    if (!st && u_host) {
        st = dalloc(ud, (size_t)std::max<int64_t>(h->n_dof, 1));
        if (!st && cudaMemcpyAsync(ud.p, u_host, h->n_dof * sizeof(double), cudaMemcpyHostToDevice, h->stream) !=
                       cudaSuccess)
            st = FE_CUDA_ERR;
        u = ud.p;
    }
    if (!st && ne > 0) {
        if (nc == 6)
            k_post_elastic_tet<<<grid_for(ne), kThreads, 0, h->stream>>>(ne, h->coords.p, h->conn.p, h->E.p, h->nu.p,
                                                                        h->ke.p, u, out.p, out.p + 6 * ne,
                                                                        out.p + 12 * ne);
        else
            k_post_elastic<<<grid_for(ne), kThreads, 0, h->stream>>>(ne, h->coords.p, h->conn.p, h->E.p, h->nu.p,
                                                                    h->plane == FE_PLANE_STRAIN, h->ke.p, u, out.p,
                                                                    out.p + 3 * ne, out.p + 6 * ne);
        if (cudaGetLastError() != cudaSuccess) st = FE_CUDA_ERR;
        h->launches += 1;
    }
    if (!st && ne > 0 &&
        (cudaMemcpyAsync(strain_host, out.p, nc * ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream) ||
         cudaMemcpyAsync(stress_host, out.p + nc * ne, nc * ne * sizeof(double), cudaMemcpyDeviceToHost,
                         h->stream) ||
         cudaMemcpyAsync(energy_host, out.p + 2 * nc * ne, ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream)))
        st = FE_CUDA_ERR;
    if (!st && cudaStreamSynchronize(h->stream) != cudaSuccess) st = FE_CUDA_ERR;
    if (st == FE_CUDA_ERR) set_error("fe_post_elastic: CUDA failure");
    dfree(ud), dfree(out);
    return st;
}

int fe_post_magnetic(fe_handle h, const double *a_host, double *field_host) {
    if (!h || !field_host) {
        set_error("fe_post_magnetic: null argument");
        return FE_BAD_INPUT;
    }
    if (h->kind != FE_KIND_MAGNETIC_TRI) {
        set_error("fe_post_magnetic: needs a magnetostatic handle");
        return FE_NOT_READY;
    }
    if (!a_host && !h->have_solution) {
        set_error("fe_post_magnetic: no potential given and no solution yet");
        return FE_NOT_READY;
    }
    const int64_t ne = h->n_elem;
    DBuf<double> ad, out;
    int st = dalloc(out, (size_t)std::max<int64_t>(2 * ne, 1));
    const double *a = h->w.x.p;
    if (!st && a_host) {
        st = dalloc(ad, (size_t)std::max<int64_t>(h->n_dof, 1));
        if (!st && cudaMemcpyAsync(ad.p, a_host, h->n_dof * sizeof(double), cudaMemcpyHostToDevice, h->stream) !=
                       cudaSuccess)
            st = FE_CUDA_ERR;
        a = ad.p;
    }
    if (!st && ne > 0) {
        k_post_magnetic<<<grid_for(ne), kThreads, 0, h->stream>>>(ne, h->coords.p, h->conn.p, a, out.p);
        if (cudaGetLastError() != cudaSuccess) st = FE_CUDA_ERR;
        h->launches += 1;
    }
    if (!st && ne > 0 &&
        cudaMemcpyAsync(field_host, out.p, 2 * ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
        st = FE_CUDA_ERR;
    if (!st && cudaStreamSynchronize(h->stream) != cudaSuccess) st = FE_CUDA_ERR;
    if (st == FE_CUDA_ERR) set_error("fe_post_magnetic: CUDA failure");
    dfree(ad), dfree(out);
    return st;
}

}  // extern "C"
