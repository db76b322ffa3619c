"""CPU model of a smoothed-aggregation multigrid preconditioner for the elasticity
systems of this path.

TEST INFRASTRUCTURE ONLY.  Nothing in ``finite_elements_gb300`` imports this module.
The reference solves with a direct factorisation (scipy spsolve, analysis.py:798-830)
and has no multigrid; this model is the oracle for a device multilevel
preconditioner, the step beyond the Chebyshev preconditioner on the device.  It
restates published smoothed aggregation (Vanek, Mandel and Brezina, "Algebraic
multigrid by smoothed aggregation for second and fourth order elliptic problems",
Computing 56, 1996):

* strength of connection between node blocks: ||A_ij||_1 >= theta sqrt(||A_ii|| ||A_jj||);
* greedy aggregation: a node whose strong neighbours are all free starts an aggregate
  with them, the nodes left join an aggregate of a strong neighbour;
* tentative prolongator: per aggregate, the QR factors of the near-null space (the
  rigid-body modes: two translations and the rotation (-y, x) in 2D) restricted to
  its DOFs; the R factors are the coarse near-null space;
* smoothed prolongator P = (I - 4/(3 lmax) D^-1 A) P_tent, D the block diagonal, lmax
  the largest eigenvalue of D^-1 A from 10 Lanczos steps (lmax_lanczos);
* Galerkin coarse operators P^T A P down to a few hundred DOFs, solved directly;
* V-cycle with Chebyshev(k) pre- and post-smoothing on D^-1 A, interval
  [lmax/30, 1.05 lmax].
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def block_diag_inv(A, d):
    """Block-diagonal (pseudo-)inverse of A with d x d blocks, as a CSR matrix."""
    n = A.shape[0] // d
    Ac = A.tocsr()
    Dm = np.zeros((n, d, d))
    for a in range(d):
        for b in range(d):
            Dm[:, a, b] = np.asarray(Ac[np.arange(n) * d + a, np.arange(n) * d + b]).reshape(-1)
    Di = np.linalg.pinv(Dm)
    rows = np.repeat(np.arange(n * d), d)
    cols = (np.arange(n)[:, None, None] * d + np.arange(d)[None, None, :]).repeat(d, axis=1).reshape(-1)
    return sp.csr_matrix((Di.reshape(-1), (rows, cols)), shape=A.shape)


def power_start(n):
    """Deterministic start vector of the eigenvalue estimates: 1 + (i mod 7) / 7."""
    return 1.0 + (np.arange(n) % 7) / 7.0


def lmax_power(A, Minv, it=30):
    """Largest eigenvalue of Minv A by power iteration (Rayleigh quotient)."""
    x = power_start(A.shape[0])
    for _ in range(it):
        x = Minv @ (A @ x)
        x /= np.linalg.norm(x)
    return float(x @ (Minv @ (A @ x)) / (x @ x))


def lmax_lanczos(A, Minv, steps=10):
    """Largest eigenvalue of Minv A from the Lanczos matrix of `steps` iterations of CG
    on A x = b preconditioned by Minv, b = power_start (the coefficients alpha_j, beta_j
    give T with diagonal 1/alpha_j + beta_{j-1}/alpha_{j-1} and off-diagonal
    sqrt(beta_j)/alpha_j; Saad, Iterative Methods for Sparse Linear Systems, 6.7.3).
    Stops early when p.Ap or r.z vanish."""
    r = power_start(A.shape[0])
    z = Minv @ r
    p = z.copy()
    rz = float(r @ z)
    rz0 = rz
    al, be = [], []
    for j in range(steps):
        if not rz > 0:
            break
        q = A @ p
        pq = float(p @ q)
        if not (pq > 0 and np.isfinite(pq)):
            break
        alpha = rz / pq
        al.append(alpha)
        r = r - alpha * q
        z = Minv @ r
        rzn = float(r @ z)
        be.append(rzn / rz)
        rz = rzn
        if j + 1 < steps:
            p = z + be[-1] * p
        if not rzn > 1e-28 * rz0:
            break
    m = len(al)
    if m == 0:
        raise ValueError("lmax_lanczos: no Lanczos step")
    dg = np.array([1.0 / al[j] + (be[j - 1] / al[j - 1] if j > 0 else 0.0) for j in range(m)])
    off = np.array([np.sqrt(max(be[j], 0.0)) / al[j] for j in range(m - 1)])
    T = np.diag(dg) + np.diag(off, 1) + np.diag(off, -1)
    return float(np.linalg.eigvalsh(T)[-1])


def chebyshev(A, Minv, lmax, ratio, k):
    """k steps of Chebyshev on Minv A z = Minv r over [1.05 lmax / ratio, 1.05 lmax];
    returns apply(r, x0=None)."""
    hi = 1.05 * lmax
    lo = hi / ratio
    theta, delta = (hi + lo) / 2, (hi - lo) / 2
    sigma = theta / delta

    def apply(r, x0=None):
        rho = 1 / sigma
        z = np.zeros_like(r) if x0 is None else x0.copy()
        d = (Minv @ (r - A @ z) if x0 is not None else Minv @ r) / theta
        for _ in range(k):
            z = z + d
            res = Minv @ (r - A @ z)
            rn = 1 / (2 * sigma - rho)
            d = rn * rho * d + 2 * rn / delta * res
            rho = rn
        return z
    return apply


def aggregate(A, d, theta=0.08):
    """Node aggregates (agg[i] = aggregate of node i) and their number."""
    n = A.shape[0] // d
    R = sp.kron(sp.eye(n), np.ones((1, d)), format="csr")
    S = (R @ abs(A.tocsr()) @ R.T).tocsr()
    diag = S.diagonal()
    S = S.tocoo()
    keep = (S.row != S.col) & (S.data >= theta * np.sqrt(diag[S.row] * diag[S.col]))
    S = sp.csr_matrix((np.ones(keep.sum()), (S.row[keep], S.col[keep])), shape=(n, n))
    agg = -np.ones(n, np.int64)
    na = 0
    for i in range(n):
        nb = S.indices[S.indptr[i]:S.indptr[i + 1]]
        if agg[i] < 0 and np.all(agg[nb] < 0):
            agg[i] = na
            agg[nb] = na
            na += 1
    for i in range(n):
        if agg[i] < 0:
            nb = S.indices[S.indptr[i]:S.indptr[i + 1]]
            nb = nb[agg[nb] >= 0]
            if nb.size:
                agg[i] = agg[nb[0]]
            else:
                agg[i] = na
                na += 1
    return agg, na


def qr_positive(X, tol=1e-12):
    """Thin QR by modified Gram-Schmidt with a non-negative diagonal of R; a column
    whose remainder is below tol times its norm gives a zero column of Q and a zero
    row of R (rank-deficient aggregates keep the block size)."""
    k, m = X.shape
    Q = np.zeros((k, m))
    R = np.zeros((m, m))
    for j in range(m):
        v = X[:, j].astype(np.float64).copy()
        nrm0 = np.sqrt(v @ v)
        for i in range(j):
            R[i, j] = Q[:, i] @ v
            v -= R[i, j] * Q[:, i]
        nrm = np.sqrt(v @ v)
        if nrm > tol * max(nrm0, 1e-300) and nrm > 0:
            R[j, j] = nrm
            Q[:, j] = v / nrm
    return Q, R


def tentative(agg, na, B, d):
    """P_tent (n d x na m) and the coarse near-null space (na m x m)."""
    m = B.shape[1]
    order = np.argsort(agg, kind="stable")
    starts = np.searchsorted(agg[order], np.arange(na + 1))
    rows, cols, vals = [], [], []
    Bc = np.zeros((na * m, m))
    for a in range(na):
        nodes = order[starts[a]:starts[a + 1]]
        dofs = (nodes[:, None] * d + np.arange(d)[None, :]).reshape(-1)
        Q, Rr = qr_positive(B[dofs])
        if Q.shape[1] < m:
            Q = np.hstack([Q, np.zeros((Q.shape[0], m - Q.shape[1]))])
            Rr = np.vstack([Rr, np.zeros((m - Rr.shape[0], m))])
        for j in range(m):
            rows += dofs.tolist()
            cols += [a * m + j] * dofs.size
            vals += Q[:, j].tolist()
        Bc[a * m:(a + 1) * m] = Rr
    return sp.csr_matrix((vals, (rows, cols)), shape=(agg.size * d, na * m)), Bc


class SmoothedAggregation:
    """Hierarchy and V-cycle.  ``work`` counts fine-operator-application equivalents
    (nnz-weighted) of the cycles applied so far."""

    def __init__(self, A, B, d=2, coarse=400, k_smooth=3, theta=0.08):
        self.levels = []
        A = A.tocsr()
        while A.shape[0] > coarse and len(self.levels) < 12:
            Minv = block_diag_inv(A, d)
            lm = lmax_lanczos(A, Minv)
            agg, na = aggregate(A, d, theta)
            Pt, Bc = tentative(agg, na, B, d)
            P = (Pt - (4.0 / (3.0 * lm)) * (Minv @ (A @ Pt))).tocsr()
            self.levels.append((A, Minv, lm, P))
            A, B, d = (P.T @ A @ P).tocsr(), Bc, B.shape[1]
        Ac = sp.csc_matrix(A)
        self.lu = spla.splu(sp.csc_matrix(Ac + 1e-12 * abs(Ac.diagonal()).max() * sp.eye(Ac.shape[0])))
        self.coarse_size = Ac.shape[0]
        self.k = k_smooth
        self.smooth = [chebyshev(A, Minv, lm, 30.0, k_smooth) for A, Minv, lm, _ in self.levels]
        self.work = 0.0

    def __call__(self, r, lvl=0):
        if lvl == len(self.levels):
            return self.lu.solve(r)
        A, _, _, P = self.levels[lvl]
        w = A.nnz / self.levels[0][0].nnz
        x = self.smooth[lvl](r)
        x = x + P @ self(P.T @ (r - A @ x), lvl + 1)
        x = self.smooth[lvl](r, x)
        self.work += (2 * self.k + 4) * w
        return x


def rigid_modes_2d(xy):
    """The three rigid-body modes of plane elasticity at the nodes xy (n, 2), node-major."""
    n = xy.shape[0]
    B = np.zeros((2 * n, 3))
    B[0::2, 0] = 1.0
    B[1::2, 1] = 1.0
    B[0::2, 2] = -xy[:, 1]
    B[1::2, 2] = xy[:, 0]
    return B


def rigid_modes_3d(xyz):
    """The six rigid-body modes of 3D elasticity at the nodes xyz (n, 3), node-major:
    three translations and the rotations about z, x and y."""
    n = xyz.shape[0]
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    B = np.zeros((3 * n, 6))
    for k in range(3):
        B[k::3, k] = 1.0
    B[0::3, 3], B[1::3, 3] = -y, x
    B[1::3, 4], B[2::3, 4] = -z, y
    B[0::3, 5], B[2::3, 5] = z, -x
    return B


def pcg(A, b, M, tol=1e-8, maxit=20000):
    """PCG from x = 0 to ||r|| <= tol ||b||: (x, iterations)."""
    x = np.zeros_like(b)
    r = b.copy()
    z = M(r)
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    for it in range(1, maxit + 1):
        q = A @ p
        al = rz / (p @ q)
        x += al * p
        r -= al * q
        if np.linalg.norm(r) <= tol * bn:
            return x, it
        z = M(r)
        rz, rz_old = r @ z, rz
        p = z + rz / rz_old * p
    return x, maxit
