// Element arithmetic shared by the element kernels and the post-processing: explicit
// round-to-nearest operations (no contracted multiply-adds, so element values round
// as the reference's numpy expressions do) and the linear tetrahedron's gradients.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fe {
namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// Linear tetrahedron (elements.py:719-748): B = (1/(6V)) [coefficients] where the
// coefficients (b_i, c_i, d_i) of node i are 6V grad N_i, so B holds the shape-function
// gradients g_i.  With a = p1-p0, b = p2-p0, c = p3-p0 and det = a.(b x c) the signed
// 6V: g_1 = (b x c)/det, g_2 = (c x a)/det, g_3 = (a x b)/det and
// g_0 = ((p3-p1) x (p2-p1))/det (= -(g_1+g_2+g_3) without the cancellation).
// vol = |det|/6 is the unsigned volume.
struct TetGrad {
    double g[4][3];
    double vol;
    bool finite;
};

__device__ __forceinline__ void cross3(double ax, double ay, double az, double bx, double by, double bz,
                                       double o[3]) {
    o[0] = sub(mul(ay, bz), mul(az, by));
    o[1] = sub(mul(az, bx), mul(ax, bz));
    o[2] = sub(mul(ax, by), mul(ay, bx));
}

__device__ __forceinline__ TetGrad tet_gradients(const double *__restrict__ coords, const int32_t *__restrict__ conn,
                                                 int64_t e) {
    double p[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t n = conn[4 * e + i];
#pragma unroll
        for (int k = 0; k < 3; ++k) p[i][k] = coords[3 * n + k];
    }
    double a[3], b[3], c[3], f[3], q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a[k] = sub(p[1][k], p[0][k]);
        b[k] = sub(p[2][k], p[0][k]);
        c[k] = sub(p[3][k], p[0][k]);
        f[k] = sub(p[3][k], p[1][k]);
        q[k] = sub(p[2][k], p[1][k]);
    }
    double cr[4][3];
    cross3(f[0], f[1], f[2], q[0], q[1], q[2], cr[0]);
    cross3(b[0], b[1], b[2], c[0], c[1], c[2], cr[1]);
    cross3(c[0], c[1], c[2], a[0], a[1], a[2], cr[2]);
    cross3(a[0], a[1], a[2], b[0], b[1], b[2], cr[3]);
    const double det = add(add(mul(a[0], cr[1][0]), mul(a[1], cr[1][1])), mul(a[2], cr[1][2]));
    const double inv = dvd(1.0, det);
    TetGrad t;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) t.g[i][k] = mul(inv, cr[i][k]);
    t.vol = dvd(fabs(det), 6.0);
    t.finite = isfinite(inv) && det != 0.0;
    return t;
}

}  // namespace
}  // namespace fe
