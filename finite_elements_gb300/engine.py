"""One problem on the GPU: the host-side ordering logic of the reference plus calls
into libfe_gb300.so for every piece of arithmetic.

Host work here is list bookkeeping only, O(number of loads and conditions):

* Dirichlet conditions are de-duplicated exactly as the reference's dict round trip
  does (finite_elements/analysis.py:28-68, :249-265): a Python dict keyed by
  (node, dimension), filled in list order, so the LAST value wins and the multiplier
  order is that of first insertion.  Element conditions get their values from the
  device (element_to_node_factors, elements.py:18-53).
* Loads keep their list position as a sequence number (user NodeLoads, then element
  loads, then edge loads, analysis.py:465-469); the device keeps the last one per
  (node, dimension) (analysis.py:71-110) and does all the arithmetic.
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import Handle, SolveOpts, SolveStats, ptr
from .problem import ELASTIC, ELASTIC3D, Problem


# solve precisions: plain FP64 PCG; FP32 Krylov + FP64 iterative refinement; FP64 CG
# recurrence with the FP32 Chebyshev preconditioner
PRECISIONS = {"fp64": _lib.FE_PREC_FP64, "mixed": _lib.FE_PREC_MIXED, "mixed-cg64": _lib.FE_PREC_MIXED_CG64}


def check_plane_flags(plane_strain, plane_stress):
    """The checks and messages of ElasticityElement.d_matrix (elements.py:265-273)."""
    if plane_strain and plane_stress:
        raise ValueError('just one of plane_strain or plane_stress can be True')
    if not plane_strain and not plane_stress:
        raise ValueError('one of plane_strain or plane_stress must be True')


def dirichlet_count(prob: Problem):
    """Number of multiplier rows: the distinct (node, dimension) keys of the node,
    element and edge conditions (analysis.py:28-68, :249-265)."""
    d = prob.dim
    keys = set((prob.node_bc_node * d + prob.node_bc_dim - 1).tolist())
    for e, dm in zip(prob.element_bc_element.tolist(), prob.element_bc_dim.tolist()):
        keys.update((prob.conn[e].astype(np.int64) * d + dm - 1).tolist())
    keys.update((prob.edge_bc_nodes * d + prob.edge_bc_dim[:, None] - 1).reshape(-1).tolist())
    return len(keys)


def _index_dtype(n):
    return np.int32 if n < 2 ** 31 else np.int64


class GpuSystem:
    """Device handle of one Problem, assembled on construction (K and F; M on demand)."""

    def __init__(self, prob: Problem, assemble=True):
        self.prob = prob
        self.dim = prob.dim
        if prob.elastic:
            check_plane_flags(prob.plane_strain, prob.plane_stress)
        if prob.kind == ELASTIC3D and (prob.element_loads or prob.element_bc_element.size):
            # element loads and conditions go through element_to_node_factors (and an
            # area), which the reference defines on triangles only (elements.py:18-53)
            raise AttributeError("'ElasticityTetrahedralElement3D' object has no attribute "
                                 "'element_to_node_factors'")
        kind = {ELASTIC: _lib.FE_KIND_ELASTIC_TRI, ELASTIC3D: _lib.FE_KIND_ELASTIC_TET}.get(
            prob.kind, _lib.FE_KIND_MAGNETIC_TRI)
        self.handle = Handle(kind, prob.coords, prob.conn)
        h = self.handle
        if prob.elastic:
            mode = _lib.FE_PLANE_STRAIN if prob.plane_strain else _lib.FE_PLANE_STRESS
            rho = prob.rho if prob.rho is not None else None
            thick = prob.thickness if prob.kind == ELASTIC else None
            h.call("fe_set_elastic_materials", ptr(prob.E), ptr(prob.nu), ptr(thick),
                   ptr(rho), mode)
        else:
            h.call("fe_set_mu", ptr(prob.mu))
        self.bc_dof, self.bc_value = self._dirichlet()
        h.call("fe_set_dirichlet", len(self.bc_dof), ptr(self.bc_dof), ptr(self.bc_value))
        self._set_loads()
        self._set_continuity()
        self.m_assembled = False
        if assemble:
            self.assemble()

    # ------------------------------------------------------------ host bookkeeping

    def _dof(self, node, dim):
        """positions[(node_index, dim)] (core.py:89-108): KeyError outside the table."""
        node = int(node)
        dim = int(dim)
        if not (0 <= node < self.prob.n_nodes) or not (1 <= dim <= self.dim):
            raise KeyError((node, dim))
        return node * self.dim + dim - 1

    def _element_factors(self, elements):
        elements = np.ascontiguousarray(elements, dtype=np.int64)
        out = np.empty((elements.size, 3))
        if elements.size:
            self.handle.call("fe_element_node_factors", elements.size, ptr(elements), ptr(out))
        return out

    def condition_list(self):
        """(DOFs, values) of every condition before de-duplication, in the order of
        c_matrix_boundary_conditions (analysis.py:252-256): node conditions, element
        conditions times element_to_node_factors (analysis.py:201-220), edge
        conditions halved (analysis.py:222-239)."""
        p = self.prob
        keys, vals = [], []
        for n, d, v in zip(p.node_bc_node.tolist(), p.node_bc_dim.tolist(), p.node_bc_value.tolist()):
            keys.append(self._dof(n, d))
            vals.append(v)
        if p.element_bc_element.size:
            fac = self._element_factors(p.element_bc_element)
            for k, (e, d, v) in enumerate(zip(p.element_bc_element.tolist(), p.element_bc_dim.tolist(),
                                              p.element_bc_value.tolist())):
                for i, node in enumerate(p.conn[e].tolist()):
                    keys.append(self._dof(node, d))
                    vals.append(v * fac[k, i])
        for (a, b), d, v in zip(p.edge_bc_nodes.tolist(), p.edge_bc_dim.tolist(), p.edge_bc_value.tolist()):
            keys += [self._dof(a, d), self._dof(b, d)]
            vals += [v * 0.5, v * 0.5]
        return keys, vals

    def load_list(self):
        """(DOFs, values) of every load before de-duplication, in the order of
        source_c_matrix_loads (analysis.py:465-469): user NodeLoads, element loads
        (value * area / total area, loads.py:32-34, times element_to_node_factors per
        point), edge loads halved.  The device computes the same values during
        assembly; this host copy serves the reference's intermediate lists."""
        p = self.prob
        keys = [self._dof(n, d) for n, d in zip(p.node_load_node.tolist(), p.node_load_dim.tolist())]
        vals = list(p.node_load_value.tolist())
        for ls in p.element_loads:
            pts = p.coords[p.conn[ls.elements]]
            area = np.abs((pts[:, 1, 0] - pts[:, 0, 0]) * (pts[:, 2, 1] - pts[:, 0, 1])
                          - (pts[:, 2, 0] - pts[:, 0, 0]) * (pts[:, 1, 1] - pts[:, 0, 1])) / 2.0
            total = 0
            for a in area.tolist():
                total += a
            fac = self._element_factors(ls.elements)
            for k, e in enumerate(ls.elements.tolist()):
                per = ls.value * area[k] / total
                for i, node in enumerate(p.conn[e].tolist()):
                    keys.append(self._dof(node, ls.dimension))
                    vals.append(per * fac[k, i])
        for (a, b), d, v in zip(p.edge_load_nodes.tolist(), p.edge_load_dim.tolist(), p.edge_load_value.tolist()):
            keys += [self._dof(a, d), self._dof(b, d)]
            vals += [v * 0.5, v * 0.5]
        return keys, vals

    def _dirichlet(self):
        table = {}
        for k, v in zip(*self.condition_list()):
            table[k] = v
        dof = np.fromiter(table.keys(), dtype=np.int64, count=len(table))
        val = np.fromiter(table.values(), dtype=np.float64, count=len(table))
        return dof, val

    def _set_loads(self):
        p = self.prob
        n_user = p.node_load_node.size
        dofs = [self._dof(n, d) for n, d in zip(p.node_load_node.tolist(), p.node_load_dim.tolist())]
        vals = list(p.node_load_value.tolist())
        seqs = list(range(n_user))
        # element loads (triangles): sets in order, occurrence k, point i -> seq n_user + 3k + i
        n_occ = 0
        if p.element_loads:
            set_ptr = np.zeros(len(p.element_loads) + 1, np.int64)
            for s, ls in enumerate(p.element_loads):
                if not (1 <= ls.dimension <= self.dim):
                    raise KeyError((int(ls.elements[0]) if ls.elements.size else -1, ls.dimension))
                set_ptr[s + 1] = set_ptr[s] + ls.elements.size
            elems = np.ascontiguousarray(np.concatenate([ls.elements for ls in p.element_loads]), np.int64)
            values = np.array([ls.value for ls in p.element_loads], np.float64)
            dims = np.array([ls.dimension for ls in p.element_loads], np.int32)
            n_occ = int(set_ptr[-1])
            self.handle.call("fe_set_element_loads", len(p.element_loads), ptr(set_ptr), ptr(elems),
                             ptr(values), ptr(dims), n_user)
        else:
            self.handle.call("fe_set_element_loads", 0, None, None, None, None, n_user)
        # edge loads: half the value to each end point, after every element load
        base = n_user + 3 * n_occ
        for j, ((a, b), d, v) in enumerate(zip(p.edge_load_nodes.tolist(), p.edge_load_dim.tolist(),
                                               p.edge_load_value.tolist())):
            dofs += [self._dof(a, d), self._dof(b, d)]
            vals += [v * 0.5, v * 0.5]
            seqs += [base + 2 * j, base + 2 * j + 1]
        dof_a = np.array(dofs, np.int64)
        val_a = np.array(vals, np.float64)
        seq_a = np.array(seqs, np.int64)
        self.handle.call("fe_set_node_loads", dof_a.size, ptr(dof_a), ptr(val_a), ptr(seq_a))
        # magnet loads: added after the loads, indexed by node (analysis.py:556-577)
        if p.magnet_loads:
            from .loads import magnet_contributions
            parts = [magnet_contributions(p.coords, p.conn, m.elements, m.non_contour_nodes, m.magnetization)
                     for m in p.magnet_loads]
            nodes = np.ascontiguousarray(np.concatenate([a for a, _ in parts]), np.int64)
            vals = np.ascontiguousarray(np.concatenate([v for _, v in parts]), np.float64)
            self.handle.call("fe_set_rhs_additions", nodes.size, ptr(nodes), ptr(vals))

    def _set_continuity(self):
        """Continuity conditions, DOF = node index as in analysis.py:186-189."""
        p = self.prob
        if p.n_cont:
            self.handle.call("fe_set_continuity", p.n_cont, ptr(p.cont_node1), ptr(p.cont_node2),
                             ptr(p.cont_value))

    # ------------------------------------------------------------ device work

    def assemble(self, mass=False):
        flags = _lib.FE_ASSEMBLE_K | _lib.FE_ASSEMBLE_F
        if mass:
            flags |= _lib.FE_ASSEMBLE_M
            self.m_assembled = True
        self.handle.call("fe_assemble", flags)

    def _export(self, which):
        nr, nc, nnz = _i64(), _i64(), _i64()
        self.handle.call("fe_export_sizes", which, nr, nc, nnz)
        nrows, ncols, nz = nr.value, nc.value, nnz.value
        indptr = np.empty(nrows + 1, np.int64)
        indices = np.empty(max(nz, 1), np.int32)
        data = np.empty(max(nz, 1), np.float64)
        self.handle.call("fe_export_csr", which, ptr(indptr), ptr(indices), ptr(data))
        idt = _index_dtype(max(nz, nrows, ncols))
        return (data[:nz], indices[:nz].astype(idt, copy=False), indptr.astype(idt)), (nrows, ncols)

    def continuity_triplets(self):
        """(data, row, col) of c_matrix_continuity_conditions (analysis.py:175-199):
        row n_nodes + len(node_loads) + i, columns the two node indices, data
        (1, 1, -value, -value)."""
        p = self.prob
        i = np.arange(p.n_cont, dtype=np.int64)
        row_c = p.n_nodes + p.node_load_node.size + i
        data = np.stack([np.ones(p.n_cont), np.ones(p.n_cont), -p.cont_value, -p.cont_value], 1).reshape(-1)
        row = np.stack([row_c, p.cont_node1, row_c, p.cont_node2], 1).reshape(-1)
        col = np.stack([p.cont_node1, row_c, p.cont_node2, row_c], 1).reshape(-1)
        return data, row, col

    def create_matrix(self):
        arrays, shape = self._export(_lib.FE_MAT_K_AUGMENTED)
        m = sp.csr_matrix(arrays, shape=shape)
        if self.prob.n_cont:
            # the continuity entries at the reference's own rows, then scipy's duplicate
            # summation and shape inference from the largest index
            coo = m.tocoo()
            d, r, c = self.continuity_triplets()
            m = sp.csr_matrix((np.r_[coo.data, d], (np.r_[coo.row, r], np.r_[coo.col, c])))
        return m

    def create_source_matrix(self):
        n = self.prob.n_dof + len(self.bc_dof)
        out = np.empty(n, np.float64)
        self.handle.call("fe_export_rhs", ptr(out))
        # n*dim + n_cont + n_bc rows; the continuity rows have no source (analysis.py:737-739)
        return np.r_[out, np.zeros(self.prob.n_cont)].reshape(-1, 1)

    def k_matrix_sparse(self):
        arrays, shape = self._export(_lib.FE_MAT_K_CSC)
        return sp.csc_matrix(arrays, shape=shape)

    def m_matrix_sparse(self):
        if not self.m_assembled:
            self.assemble(mass=True)
        arrays, shape = self._export(_lib.FE_MAT_M_CSC)
        return sp.csc_matrix(arrays, shape=shape)

    def element_matrices(self, which="K"):
        nl = self.prob.npe * self.dim
        out = np.empty((self.prob.n_elements, nl * nl))
        if which == "M" and not self.m_assembled:
            self.assemble(mass=True)
        sel = _lib.FE_ASSEMBLE_K if which == "K" else _lib.FE_ASSEMBLE_M
        self.handle.call("fe_export_element_matrices", sel, ptr(out))
        return out

    def solve(self, precision="fp64", tol=None, cheb_degree=0, max_iter=0, x0=None, lanes=0,
              accept_stagnation=False, inner_tol=0.0, cheb_ratio=0.0, chunk=0, max_outer=0,
              want_host=True, restart_each_step=False, x0_device_ptr=None, x0_if_better=False,
              multigrid=False):
        """Solve the eliminated system on the GPU.  precision: "fp64", "mixed" or
        "mixed-cg64" (see PRECISIONS).  x0 / x0_device_ptr: warm start; with
        x0_if_better it is kept only when its true residual beats the zero start.
        multigrid: PCG with an FP64 recurrence preconditioned by one FP32
        smoothed-aggregation V-cycle per iteration, the hierarchy set up on the device
        (precision and Chebyshev options are not used; x0 and x0_if_better are).
        Returns (x, stats): x holds n_dof + n_bc values (u then the multipliers) or
        None with want_host=False."""
        o = SolveOpts()
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        o.precision = PRECISIONS[precision]
        o.cheb_degree = cheb_degree
        o.max_iter = max_iter
        o.max_outer = max_outer
        o.tol = tol if tol is not None else (1e-12 if precision == "fp64" else 1e-8)
        o.inner_tol = inner_tol
        o.cheb_ratio = cheb_ratio
        x0a = None
        if x0 is not None:
            x0a = np.ascontiguousarray(x0, dtype=np.float64)[: self.prob.n_dof]
            o.x0 = x0a.ctypes.data
        elif x0_device_ptr is not None:
            o.x0 = x0_device_ptr
            o.x0_device = 1
        o.lanes = lanes
        o.chunk = chunk
        o.flags = ((_lib.FE_SOLVE_ACCEPT_STAGNATION if accept_stagnation else 0)
                   | (_lib.FE_SOLVE_RESTART_EACH_STEP if restart_each_step else 0)
                   | (_lib.FE_SOLVE_X0_IF_BETTER if x0_if_better else 0)
                   | (_lib.FE_SOLVE_MULTIGRID if multigrid else 0))
        st = SolveStats()
        x = np.empty(self.prob.n_dof + len(self.bc_dof) + self.prob.n_cont) if want_host else None
        lib = _lib.load()
        status = lib.fe_solve(self.handle.h, o, ptr(x) if want_host else None, st)
        if status not in (_lib.FE_OK, _lib.FE_MAXITER, _lib.FE_BREAKDOWN, _lib.FE_NONFINITE):
            _lib.check(status, "fe_solve")
        return x, st

    def post(self, x=None):
        """Per-element results of a solution (the handle's last one when x is None):
        elasticity -> dict(strain (E,3), stress (E,3), energy (E,)), with 6 strain and
        stress components (xx, yy, zz, xy, yz, zx) on tetrahedra; magnetostatics ->
        dict(field (E,2))."""
        ne = self.prob.n_elements
        xa = None if x is None else np.ascontiguousarray(np.asarray(x, np.float64)[: self.prob.n_dof])
        if self.prob.elastic:
            nc = 6 if self.prob.kind == ELASTIC3D else 3
            strain, stress, energy = np.empty((ne, nc)), np.empty((ne, nc)), np.empty(ne)
            self.handle.call("fe_post_elastic", ptr(xa), ptr(strain), ptr(stress), ptr(energy))
            return {"strain": strain, "stress": stress, "energy": energy}
        field = np.empty((ne, 2))
        self.handle.call("fe_post_magnetic", ptr(xa), ptr(field))
        return {"field": field}

    def modal(self, k, which="smallest", sigma=0.0, steps=0, precision="fp64"):
        """k eigenpairs of K v = lambda M v (no Dirichlet conditions), by increasing
        eigenvalue: (eigenvalues (k,), eigenvectors (k, n_dof) of unit 2-norm,
        relative residuals (k,)).  which: "smallest" (shift-invert, sigma < 0 or 0 for
        an automatic shift) or "largest"."""
        if which not in ("smallest", "largest"):
            raise ValueError("Order parameter should be either 'largest' or 'smallest'")
        lib = _lib.load()
        self.handle.call("fe_assemble", _lib.FE_ASSEMBLE_K | _lib.FE_ASSEMBLE_M)
        vals, res = np.empty(k), np.empty(k)
        vecs = np.empty((k, self.prob.n_dof))
        status = lib.fe_modal(self.handle.h, _lib.FE_MODAL_SMALLEST if which == "smallest" else _lib.FE_MODAL_LARGEST,
                              int(k), float(sigma), int(steps), PRECISIONS[precision], ptr(vals), ptr(vecs), ptr(res))
        _lib.check(status, "fe_modal")
        return vals, vecs, res

    def sell_info(self):
        """Stored SELL-32 entries (padding included) and whether the FP32 kernels use
        16-bit column offsets."""
        ne, c16 = _i64(), ctypes.c_int32()
        self.handle.call("fe_sell_info", ne, c16)
        return {"entries": ne.value, "col16": bool(c16.value)}

    def info(self):
        nd, nb, nblk = _i64(), _i64(), _i64()
        self.handle.call("fe_info", nd, nb, nblk)
        return {"n_dof": nd.value, "n_bc": nb.value, "n_blocks": nblk.value}

    def close(self):
        self.handle.close()


def _i64():
    return ctypes.c_int64()
