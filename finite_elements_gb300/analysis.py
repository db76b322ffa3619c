"""Drop-in ``FiniteElementAnalysis`` running the assembly-and-solve path on the GPU.

Same constructor, methods, return types and error behaviour as the reference's
``finite_elements.analysis.FiniteElementAnalysis`` (finite_elements/analysis.py:141-173,
:580-830) for what it solves:

* ``create_matrix()`` -> scipy CSR of the augmented system [[K, C^T], [C, 0]], same
  pattern (explicit zeros kept), same indices, values to rounding (analysis.py:617-663);
* ``create_source_matrix()`` -> (n*dim + n_bc, 1) array (analysis.py:665-708);
* ``solve()`` -> ``Result(mesh, list)`` with u then the multipliers (analysis.py:798-830);
* ``k_matrix_sparse()`` / ``m_matrix_sparse()`` -> scipy CSC (analysis.py:345-405).

Instead of scipy's sparse LU on the saddle system, the GPU eliminates the Dirichlet
DOFs, solves the SPD system with PCG and recovers each multiplier from the first
block row, lambda_i = (F - K u)[dof_i].  Magnet loads become additive right-hand-side
entries (analysis.py:556-577).  Continuity conditions enter create_matrix at the
reference's own rows n_nodes + len(node_loads) + i (analysis.py:175-199), and solve()
raises scipy's dimension-mismatch ValueError wherever those rows make the matrix and
the right-hand side disagree in size, as spsolve does; where they agree (the rows
follow the Dirichlet rows) the GPU solves with a projected FP64 PCG and returns the
continuity multipliers after the Dirichlet ones.
"""
from __future__ import annotations

import warnings

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .engine import GpuSystem, check_plane_flags, dirichlet_count
from .mesh import ArrayMesh
from .problem import ELASTIC, ELASTIC3D, MAGNETIC, ElementLoadSet, MagnetLoadSet, Problem
from .results import Result

DEFAULT_SOLVER = {"precision": "fp64", "tol": 1e-14, "accept_stagnation": True, "cheb_degree": 0}


class SolverConvergenceError(RuntimeError):
    """PCG stopped at its iteration cap above the requested tolerance."""


class FeSolveError(RuntimeError):
    """Strict mode (``solver={"strict": True}``): a singular or non-finite system raises
    this instead of returning the NaN vector spsolve would return."""

    def __init__(self, status, stats):
        RuntimeError.__init__(self, f"solve failed with status {status}: {stats}")
        self.status = status
        self.stats = stats


def _element_kind(element):
    if hasattr(element, "mu_total"):
        return MAGNETIC
    if hasattr(element, "elasticity_modulus"):
        return ELASTIC3D if len(element.points) == 4 else ELASTIC
    raise NotImplementedError(f"element type {type(element).__name__} is not a linear triangle "
                              "or tetrahedron of the GPU path")


class FiniteElementAnalysis:
    """See the module docstring.  ``solver`` (optional) overrides the solve options
    (``precision`` "fp64" / "mixed" / "mixed-cg64", ``tol``, ``cheb_degree``,
    ``max_iter``, ``x0`` ...; ``strict`` raises FeSolveError on a singular or
    non-finite system instead of returning NaN)."""

    def __init__(self, mesh, element_loads, edge_loads, node_loads, magnet_loads,
                 continuity_conditions, node_boundary_conditions, edge_boundary_conditions,
                 element_boundary_conditions, plane_strain: bool = None, plane_stress: bool = None,
                 solver=None):
        self.mesh = mesh
        self.element_loads = element_loads
        self.edge_loads = edge_loads
        self.node_loads = node_loads
        self.magnet_loads = magnet_loads
        self.continuity_conditions = continuity_conditions
        self.node_boundary_conditions = node_boundary_conditions
        self.edge_boundary_conditions = edge_boundary_conditions
        self.element_boundary_conditions = element_boundary_conditions
        self.plane_strain = plane_strain
        self.plane_stress = plane_stress
        self.solver = dict(DEFAULT_SOLVER, **(solver or {}))
        self._problem = None
        self._system = None
        self._boundary_conditions = None
        self._positions = None
        self.last_stats = None

    @classmethod
    def from_problem(cls, problem: Problem, mesh=None, solver=None):
        """Analysis of an array-only Problem (no per-element Python objects)."""
        if mesh is None:
            mesh = ArrayMesh(problem.coords, problem.conn)
        obj = cls(mesh, [], [], [], [], [], [], [], [], problem.plane_strain, problem.plane_stress,
                  solver=solver)
        obj._problem = problem
        return obj

    # ------------------------------------------------------------ modal analysis

    def modal_analysis(self, order, k, steps=0, precision="fp64"):
        """k eigenpairs of K v = lambda M v on the matrices without conditions
        (analysis.py:741-796): ``order`` 'smallest' or 'largest'.  Returns (eigenvalues
        (k,), eigenvectors (k, n_dof)) by increasing eigenvalue, the vectors of unit
        2-norm.  The GPU runs shift-invert Lanczos ('smallest') or Lanczos on M^-1 K
        ('largest') in the M inner product.  Unlike the reference's 'smallest' branch,
        which inverts K although a free body makes it singular, the values are the
        exact generalized eigenvalues (rigid-body modes at zero) and real."""
        if order not in ("largest", "smallest"):
            raise ValueError("Order parameter should be either 'largest' or 'smallest'")
        vals, vecs, _ = self.system().modal(k, which=order, steps=steps, precision=precision)
        return vals, vecs

    # ------------------------------------------------------------ reference properties

    @property
    def dimension(self):
        if self._problem is not None and isinstance(self.mesh, ArrayMesh):
            return self._problem.dim
        return self.mesh.elements_groups[0].elements[0].dimension

    @property
    def elements_name(self):
        return self.mesh.elements_groups[0].elements[0].__class__.__name__

    @property
    def positions(self):
        if not self._positions:
            d, n = self.dimension, len(self.mesh.nodes)
            self._positions = {(i, j + 1): i * d + j for i in range(n) for j in range(d)}
        return self._positions

    # ------------------------------------------------------------ flattening

    def problem(self) -> Problem:
        """The analysis as arrays (mesh walk of analysis.py:326-338, :714-735)."""
        if self._problem is not None:
            return self._problem
        mesh = self.mesh
        nodes = mesh.nodes
        index = mesh.node_to_index
        elements = [el for g in mesh.elements_groups for el in g.elements]
        if not elements:
            raise ValueError("the mesh has no element")
        kind = _element_kind(elements[0])
        cdim, npe = (3, 4) if kind == ELASTIC3D else (2, 3)
        coords = np.array([[float(p[k]) for k in range(cdim)] for p in nodes],
                          dtype=np.float64).reshape(-1, cdim)
        conn = np.array([[index[p] for p in el.points] for el in elements], dtype=np.int32).reshape(-1, npe)
        by_id = {id(el): k for k, el in enumerate(elements)}
        by_points = {}

        def element_index(el):
            k = by_id.get(id(el))
            if k is None:
                if not by_points:
                    by_points.update({tuple(r): k for k, r in enumerate(conn.tolist())})
                k = by_points.get(tuple(index[p] for p in el.points))
                if k is None:
                    raise ValueError("an element of a load or condition is not part of the mesh")
            return k

        kw = {}
        if kind in (ELASTIC, ELASTIC3D):
            kw = dict(E=[el.elasticity_modulus for el in elements],
                      nu=[el.poisson_ratio for el in elements],
                      thickness=[getattr(el, "thickness", 1.0) for el in elements],
                      plane_strain=self.plane_strain, plane_stress=self.plane_stress)
            rho = [el.mass_density for el in elements]
            if all(r is not None for r in rho):
                kw["rho"] = rho
        else:
            kw = dict(mu=[el.mu_total for el in elements])
        nl = self.node_loads
        el_loads = [ElementLoadSet(np.array([element_index(e) for e in ld.elements], np.int64),
                                   ld.value, ld.dimension) for ld in self.element_loads]
        magnets = [MagnetLoadSet(np.array([element_index(e) for e in ml.elements], np.int64),
                                 np.array([index[p] for p in ml.non_contour_nodes], np.int64),
                                 (float(ml.magnetization_vector[0]), float(ml.magnetization_vector[1])))
                   for ml in self.magnet_loads]
        cc = self.continuity_conditions
        prob = Problem(
            kind, coords, conn, **kw,
            node_load_node=[index[ld.node] for ld in nl], node_load_dim=[ld.dimension for ld in nl],
            node_load_value=[ld.value for ld in nl], element_loads=el_loads,
            edge_load_nodes=[[index[ld.edge.start], index[ld.edge.end]] for ld in self.edge_loads],
            edge_load_dim=[ld.dimension for ld in self.edge_loads],
            edge_load_value=[ld.value for ld in self.edge_loads],
            node_bc_node=[index[c.application] for c in self.node_boundary_conditions],
            node_bc_dim=[c.dimension for c in self.node_boundary_conditions],
            node_bc_value=[c.value for c in self.node_boundary_conditions],
            element_bc_element=[element_index(c.application) for c in self.element_boundary_conditions],
            element_bc_dim=[c.dimension for c in self.element_boundary_conditions],
            element_bc_value=[c.value for c in self.element_boundary_conditions],
            edge_bc_nodes=[[index[c.application.start], index[c.application.end]]
                           for c in self.edge_boundary_conditions],
            edge_bc_dim=[c.dimension for c in self.edge_boundary_conditions],
            edge_bc_value=[c.value for c in self.edge_boundary_conditions],
            magnet_loads=magnets, cont_node1=[index[c.node1] for c in cc],
            cont_node2=[index[c.node2] for c in cc], cont_value=[c.value for c in cc])
        self._problem = prob
        return prob

    def system(self) -> GpuSystem:
        if self._system is None:
            prob = self.problem()
            if prob.elastic:
                check_plane_flags(self.plane_strain, self.plane_stress)
                prob.plane_strain, prob.plane_stress = self.plane_strain, self.plane_stress
            self._system = GpuSystem(prob)
        return self._system

    # ------------------------------------------------------------ reference API

    def create_matrix(self):
        sysm = self.system()
        self._boundary_conditions = list(zip(sysm.bc_dof.tolist(), sysm.bc_value.tolist()))
        return sysm.create_matrix()

    def create_source_matrix(self):
        if self._boundary_conditions is None:
            # the reference sizes F with len(self._boundary_conditions), which only
            # create_matrix sets (analysis.py:737-739)
            raise TypeError("object of type 'NoneType' has no len()")
        return self.system().create_source_matrix()

    def k_matrix_sparse(self):
        return self.system().k_matrix_sparse()

    def m_matrix_sparse(self):
        if not self.problem().elastic:
            raise AttributeError("'MagneticElement2D' object has no attribute 'elementary_mass_matrix'")
        return self.system().m_matrix_sparse()

    def k_matrix(self, method_name):
        if method_name == 'dense':
            return self.k_matrix_sparse().toarray()
        if method_name == 'sparse':
            return self.k_matrix_sparse()
        raise NotImplementedError(
            f'Class {self.__class__.__name__} does not implement {method_name} k matrix')

    def m_matrix(self, method_name):
        if method_name == 'dense':
            return self.m_matrix_sparse().toarray()
        if method_name == 'sparse':
            return self.m_matrix_sparse()
        raise NotImplementedError(
            f'Class {self.__class__.__name__} does not implement {method_name} m matrix')

    def element_matrices(self, which="K"):
        """(E, (npe*dim)^2) row-major element matrices from the GPU element kernels."""
        return self.system().element_matrices(which)

    # ------------------------------------------------------------ intermediate lists
    # The reference's building blocks (analysis.py:175-577), for callers that use them.
    # Triplet lists are numpy arrays here: at the sizes this path serves, Python lists
    # of the element matrices would not fit in host memory.

    def _element_dofs(self):
        prob = self.problem()
        d = prob.dim
        return (prob.conn.astype(np.int64)[:, :, None] * d + np.arange(d)[None, None, :]).reshape(
            prob.n_elements, -1)

    def get_row_col_indices(self, element):
        """row = each local DOF repeated len(L) times, col = L tiled (analysis.py:714-735)."""
        index = self.mesh.node_to_index
        d = element.dimension
        L = [index[p] * d + i for p in element.points for i in range(d)]
        return [r for r in L for _ in L], L * len(L)

    def _triplets(self, which):
        ke = self.element_matrices(which).reshape(-1)
        L = self._element_dofs()
        n = L.shape[1]
        return ke, np.repeat(L, n, axis=1).reshape(-1), np.tile(L, (1, n)).reshape(-1)

    def k_matrix_data(self):
        """(data, row, col) of every element matrix in group and element order
        (analysis.py:324-339), the values from the GPU element kernels."""
        return self._triplets("K")

    def m_matrix_data(self):
        """As k_matrix_data for the mass matrices (analysis.py:356-369)."""
        if not self.problem().elastic:
            raise AttributeError("'MagneticElement2D' object has no attribute 'elementary_mass_matrix'")
        return self._triplets("M")

    def matrix_dense(self, method_name):
        """Dense (n*dim)^2 sum of the triplets of ``method_name`` (analysis.py:373-390)."""
        if not hasattr(self, method_name):
            raise NotImplementedError(f'Class {self.__class__.__name__} does not implement {method_name}')
        data, row, col = getattr(self, method_name)()
        n = self.problem().n_dof
        m = np.zeros((n, n))
        np.add.at(m, (np.asarray(row), np.asarray(col)), np.asarray(data))
        return m

    def matrix_sparse(self, method_name):
        """csc_matrix of the merged triplets of ``method_name`` (analysis.py:387-405); K
        and M come from the device's merge (fe_export_csr)."""
        if method_name == 'k_matrix_data':
            return self.k_matrix_sparse()
        if method_name == 'm_matrix_data':
            return self.m_matrix_sparse()
        if not hasattr(self, method_name):
            raise NotImplementedError(f'Class {self.__class__.__name__} does not implement {method_name}')
        data, row, col = getattr(self, method_name)()
        merged = {}
        for v, r, c in zip(np.asarray(data).tolist(), np.asarray(row).tolist(), np.asarray(col).tolist()):
            merged[(r, c)] = merged[(r, c)] + v if (r, c) in merged else v
        keys = list(merged)
        return sp.csc_matrix((list(merged.values()), ([k[0] for k in keys], [k[1] for k in keys])))

    def k_matrix_dense(self):
        return self.matrix_dense('k_matrix_data')

    def m_matrix_dense(self):
        return self.matrix_dense('m_matrix_data')

    def elements_permeability(self):
        """mu_total of the first element of every group (analysis.py:292-306)."""
        if isinstance(self.mesh, ArrayMesh):
            prob = self.problem()
            return [float(prob.mu[int(a)]) for a in self.mesh.group_ptr[:-1]]
        return [g.elements[0].mu_total for g in self.mesh.elements_groups]

    def c_matrix_boundary_conditions(self):
        """(data, row, col): for de-duplicated condition i at DOF p, (n*dim + i, p) and
        (p, n*dim + i), both 1 (analysis.py:241-279)."""
        sysm = self.system()
        self._boundary_conditions = list(zip(sysm.bc_dof.tolist(), sysm.bc_value.tolist()))
        nd = self.problem().n_dof
        data, row, col = [], [], []
        for i, p in enumerate(sysm.bc_dof.tolist()):
            data.extend((1, 1))
            row.extend((nd + i, p))
            col.extend((p, nd + i))
        return data, row, col

    def c_matrix_continuity_conditions(self):
        """(data, row, col) at the reference's rows n_nodes + len(node_loads) + i
        (analysis.py:175-199)."""
        d, r, c = self.system().continuity_triplets()
        return d.tolist(), r.tolist(), c.tolist()

    def get_source_matrix_length(self):
        """n*dim + n_continuity + n_bc (analysis.py:737-739); TypeError before
        create_matrix, as in the reference."""
        if self._boundary_conditions is None:
            raise TypeError("object of type 'NoneType' has no len()")
        prob = self.problem()
        return prob.n_dof + prob.n_cont + len(self._boundary_conditions)

    def source_c_matrix_boundary_conditions(self):
        """(values, rows n*dim + i) of the de-duplicated conditions (analysis.py:509-543)."""
        sysm = self.system()
        self._boundary_conditions = list(zip(sysm.bc_dof.tolist(), sysm.bc_value.tolist()))
        nd = self.problem().n_dof
        return sysm.bc_value.tolist(), [nd + i for i in range(len(sysm.bc_dof))]

    def source_c_matrix_magnet_loads(self):
        """(values, node rows) of the magnet loads (analysis.py:556-577)."""
        from .loads import magnet_contributions
        prob = self.problem()
        data, rows = [], []
        for m in prob.magnet_loads:
            r, v = magnet_contributions(prob.coords, prob.conn, m.elements, m.non_contour_nodes, m.magnetization)
            data += v.tolist()
            rows += r.tolist()
        return data, rows

    def source_c_matrix_loads(self):
        """(values, DOF rows) of the de-duplicated loads, last value per (node, dimension)
        in first-insertion order (analysis.py:457-489, :71-110)."""
        prob, sysm = self.problem(), self.system()
        keys, vals = sysm.load_list()
        table = {}
        for k, v in zip(keys, vals):
            table[k] = v
        return list(table.values()), list(table.keys())

    def _node_objects(self, keys_values, cls):
        nodes = self.mesh.nodes
        d = self.problem().dim
        return [cls(nodes[k // d], v, k % d + 1) for k, v in keys_values]

    def loads_element_to_node(self):
        """NodeLoads of the element loads, per element and point (analysis.py:407-429)."""
        from .loads import NodeLoad
        prob, sysm = self.problem(), self.system()
        n_user = prob.node_load_node.size
        keys, vals = sysm.load_list()
        n_el = len(keys) - n_user - 2 * prob.edge_load_dim.size
        return self._node_objects(zip(keys[n_user:n_user + n_el], vals[n_user:n_user + n_el]), NodeLoad)

    def loads_edge_to_node(self):
        """NodeLoads of the edge loads, half to each end (analysis.py:431-447)."""
        from .loads import NodeLoad
        prob, sysm = self.problem(), self.system()
        keys, vals = sysm.load_list()
        m = 2 * prob.edge_load_dim.size
        return self._node_objects(zip(keys[len(keys) - m:], vals[len(vals) - m:]), NodeLoad)

    def boundary_conditions_element_to_node(self):
        """NodeBoundaryConditions of the element conditions (analysis.py:201-220)."""
        from .conditions import NodeBoundaryCondition
        keys, vals = self.system().condition_list()
        prob = self.problem()
        a = prob.node_bc_node.size
        b = len(keys) - 2 * prob.edge_bc_dim.size
        return self._node_objects(zip(keys[a:b], vals[a:b]), NodeBoundaryCondition)

    def boundary_conditions_edge_to_node(self):
        """NodeBoundaryConditions of the edge conditions (analysis.py:222-239)."""
        from .conditions import NodeBoundaryCondition
        keys, vals = self.system().condition_list()
        m = 2 * self.problem().edge_bc_dim.size
        return self._node_objects(zip(keys[len(keys) - m:], vals[len(vals) - m:]), NodeBoundaryCondition)

    def _check_shapes(self):
        """spsolve's check of the reference's create_matrix against its
        create_source_matrix: with continuity conditions the matrix spans its largest
        row index + 1 (analysis.py:186-199, :656), the right-hand side
        n*dim + n_cont + n_bc rows (analysis.py:737-739)."""
        prob = self.problem()
        if not prob.n_cont:
            return
        n_bc = dirichlet_count(prob)
        top = max(int(prob.conn.max()) + 1 if prob.conn.size else 0, 0) * prob.dim
        if n_bc:
            top = max(top, prob.n_dof + n_bc)
        top = max(top, prob.n_nodes + prob.node_load_node.size + prob.n_cont,
                  int(max(prob.cont_node1.max(), prob.cont_node2.max())) + 1)
        n_f = prob.n_dof + prob.n_cont + n_bc
        if top != n_f:
            raise ValueError(f"matrix - rhs dimension mismatch (({top}, {top}) - {n_f})")

    def solve(self):
        """PCG on the GPU in place of spsolve (analysis.py:798-830)."""
        self._check_shapes()
        sysm = self.system()
        self._boundary_conditions = list(zip(sysm.bc_dof.tolist(), sysm.bc_value.tolist()))
        opts = dict(self.solver)
        strict = opts.pop("strict", False)
        x, st = sysm.solve(**opts)
        self.last_stats = st.as_dict()
        from . import _lib
        if strict and st.status in (_lib.FE_BREAKDOWN, _lib.FE_NONFINITE):
            raise FeSolveError(_lib.STATUS_NAMES.get(st.status, st.status), self.last_stats)
        if st.status in (_lib.FE_BREAKDOWN, _lib.FE_NONFINITE):
            # scipy's spsolve warns and returns NaN for an exactly singular matrix; the
            # reference turns the warning into NotImplementedError when it is raised
            try:
                warnings.warn("Matrix is exactly singular", spla.MatrixRankWarning)
            except spla.MatrixRankWarning as exc:
                print('MatricRankWarning')
                raise NotImplementedError from exc
            x = np.full(x.shape, np.nan)
        elif st.status == _lib.FE_MAXITER:
            raise SolverConvergenceError(
                f"PCG stopped after {st.iterations} iterations at relative residual {st.relres:.3e}")
        return Result(self.mesh, list(x), dimension=self.problem().dim)
