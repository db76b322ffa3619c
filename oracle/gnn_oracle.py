"""CPU oracle of the warm-start graph network -- TEST INFRASTRUCTURE ONLY.

A torch (CPU, float64) restatement of the network, features and loss that
libfe_gb300.so implements in CUDA (fe_gnn_*), used to check its forward values and
its hand-written backward against autograd.  The warm start has no counterpart in
the reference project; its definition is the library's (include/fe_gb300.h):

  features (16 per node): x_n, y_n (bounding-box normalised), sin/cos(pi x_n),
  sin/cos(pi y_n), sin(2 pi x_n), sin(2 pi y_n), constrained flags (x, y), then
  graph-level values broadcast to every node: the direction of the total load sum b~,
  the load moments sum b~_y x_n / sum|b~| and sum b~_x y_n / sum|b~|, the mean of
  log10 E over the elements - 10.5 and 10 (mean nu - 0.3);
  h0 = relu(f W0 + b0); h_{l+1} = h_l + relu([h_l, mean_nbr h_l] W_l + b_l + mean(h_l) U_l);
  u_hat = (P S)^32 P (h_6 Wd + bd), P zeroing the constrained DOFs and
  S = (I + mean_nbr) / 2 a low-pass step;
  loss = 1 - (u.b~)^2 / ((u.A u) e*).
With bf16=True the GEMM inputs are rounded to bfloat16 as the tensor-core kernels do.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from oracle import fe_oracle as O

HID, NF, NLAYER, NSMOOTH = 64, 16, 6, 32


def split_params(p):
    p = torch.as_tensor(np.asarray(p, np.float64))
    out, o = {}, 0

    def take(name, shape):
        nonlocal o
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape).clone()
        o += n

    take("W0", (NF, HID))
    take("b0", (HID,))
    for l in range(NLAYER):
        take(f"W{l + 1}", (2 * HID, HID))
        take(f"b{l + 1}", (HID,))
        take(f"U{l + 1}", (HID, HID))
    take("Wd", (HID, 2))
    take("bd", (2,))
    assert o == p.numel()
    return out


def flatten_grads(tensors):
    order = ["W0", "b0"]
    for l in range(NLAYER):
        order += [f"W{l + 1}", f"b{l + 1}", f"U{l + 1}"]
    order += ["Wd", "bd"]
    return np.concatenate([tensors[k].grad.detach().numpy().reshape(-1) for k in order])


def eliminated_system(prob):
    """A (identity rows/columns on constrained DOFs), b, g_ext, b~ = b - A g (0 on
    constrained DOFs), constrained mask."""
    data, row, col = O.k_matrix_data(prob)
    nd = prob.n_dof
    K = sp.csr_matrix((data, (row, col)), shape=(nd, nd))
    lk, lv = O.node_loads(prob)
    F = np.zeros(nd)
    np.add.at(F, lk, lv)
    bc_dof, bc_val = O.boundary_conditions(prob)
    mask = np.zeros(nd, bool)
    mask[bc_dof] = True
    Kc = K.tocoo()
    keep = ~(mask[Kc.row] | mask[Kc.col])
    A = (sp.coo_matrix((Kc.data[keep], (Kc.row[keep], Kc.col[keep])), shape=(nd, nd)).tocsr()
         + sp.diags(mask.astype(float)))
    g = np.zeros(nd)
    g[bc_dof] = bc_val
    b = F - K @ g
    b[mask] = g[mask]
    bt = b - A @ g
    bt[mask] = 0.0
    return A, b, g, bt, mask


def features(prob, A, bt, mask):
    n = prob.n_nodes
    xy = prob.coords
    mn = xy.min(axis=0).astype(np.float32).astype(np.float64)
    mx = xy.max(axis=0).astype(np.float32).astype(np.float64)
    L = max(mx[0] - mn[0], mx[1] - mn[1])
    xn, yn = (xy[:, 0] - mn[0]) / L, (xy[:, 1] - mn[1]) / L
    b2 = bt.reshape(n, 2)
    sx, sy = b2[:, 0].sum(), b2[:, 1].sum()
    sa = np.abs(b2).sum()
    fn = np.hypot(sx, sy)
    f = np.zeros((n, NF))
    f[:, 0], f[:, 1] = xn, yn
    f[:, 2], f[:, 3] = np.sin(np.pi * xn), np.cos(np.pi * xn)
    f[:, 4], f[:, 5] = np.sin(np.pi * yn), np.cos(np.pi * yn)
    f[:, 6], f[:, 7] = np.sin(2 * np.pi * xn), np.sin(2 * np.pi * yn)
    f[:, 8], f[:, 9] = mask[0::2], mask[1::2]
    f[:, 10] = sx / fn if fn > 0 else 0.0
    f[:, 11] = sy / fn if fn > 0 else 0.0
    f[:, 12] = (b2[:, 1] * xn).sum() / sa if sa > 0 else 0.0
    f[:, 13] = (b2[:, 0] * yn).sum() / sa if sa > 0 else 0.0
    f[:, 14] = np.log10(prob.E).mean() - 10.5
    f[:, 15] = (prob.nu.mean() - 0.3) * 10.0
    return f


def neighbour_mean_matrix(prob):
    """Row-normalised adjacency of the nodes sharing an element (no self loops)."""
    n = prob.n_nodes
    c = prob.conn.astype(np.int64)
    r = np.concatenate([c[:, i] for i in range(3) for j in range(3) if i != j])
    q = np.concatenate([c[:, j] for i in range(3) for j in range(3) if i != j])
    Adj = sp.csr_matrix((np.ones(r.size), (r, q)), shape=(n, n))
    Adj.data[:] = 1.0
    Adj.sum_duplicates()
    Adj.data[:] = 1.0
    deg = np.asarray(Adj.sum(axis=1)).reshape(-1)
    inv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)
    return sp.diags(inv) @ Adj


def _bf(x, on):
    return x.to(torch.bfloat16).to(torch.float64) if on else x


def loss_and_grad(prob, params, energy, bf16=False, fit_solution=None):
    """(loss, gradient in the library's parameter order, u_hat, features).  With
    fit_solution = x the loss is the mean-squared error of u_hat against
    (x - g) / RMS(x - g) on the free DOFs instead of the energy loss."""
    A, b, g, bt, mask = eliminated_system(prob)
    f = torch.as_tensor(features(prob, A, bt, mask))
    P = {k: v.requires_grad_(True) for k, v in split_params(params).items()}
    Mn = neighbour_mean_matrix(prob).tocoo()
    Mt = torch.sparse_coo_tensor(np.vstack([Mn.row, Mn.col]), Mn.data, Mn.shape)
    h = torch.relu(_bf(f, bf16) @ _bf(P["W0"], bf16) + P["b0"])
    for l in range(1, NLAYER + 1):
        m = torch.sparse.mm(Mt, h)
        gm = h.mean(dim=0, keepdim=True)
        z = _bf(torch.cat([h, m], dim=1), bf16) @ _bf(P[f"W{l}"], bf16) + P[f"b{l}"] + gm @ P[f"U{l}"]
        h = h + torch.relu(z)
    keep = torch.as_tensor(~mask.reshape(-1, 2)).to(torch.float64)
    u = (h @ P["Wd"] + P["bd"]) * keep
    for _ in range(NSMOOTH):
        u = 0.5 * (u + torch.sparse.mm(Mt, u)) * keep
    u = u.reshape(-1)
    At = torch.sparse_csr_tensor(torch.as_tensor(A.indptr, dtype=torch.int64),
                                 torch.as_tensor(A.indices, dtype=torch.int64),
                                 torch.as_tensor(A.data), A.shape)
    Au = (At @ u.reshape(-1, 1)).reshape(-1)
    btt = torch.as_tensor(bt)
    a = u @ btt
    c = u @ Au
    if fit_solution is not None:
        free = ~mask
        d = np.asarray(fit_solution)[: prob.n_dof] - g
        sigma = np.sqrt(np.mean(d[free] ** 2))
        t = torch.as_tensor(np.where(free, d / sigma, 0.0))
        fm = torch.as_tensor(free.astype(np.float64))
        loss = (((u - t) * fm) ** 2).sum() / free.sum()
    else:
        loss = 1.0 - a * a / (c * energy)
    loss.backward()
    return float(loss), flatten_grads(P), u.detach().numpy(), f.numpy()


def solution_energy(prob):
    """b~ . (x - g) for the oracle's own solution."""
    A, b, g, bt, mask = eliminated_system(prob)
    import scipy.sparse.linalg as spla
    x = spla.spsolve(A.tocsc(), b)
    return float(bt @ (x - g))
