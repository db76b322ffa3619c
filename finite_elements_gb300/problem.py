"""Flat, array-only description of one assembly-and-solve problem.

This is the layout that crosses the C ABI: node coordinates, triangle connectivity,
per-element material arrays and the load / condition lists of the reference's
``FiniteElementAnalysis`` (finite_elements/analysis.py:141-167), each reduced to node
indices, 1-based dimensions and values.  List order is kept exactly, because the
reference's load and condition de-duplication depends on it (analysis.py:28-110,
:252-265, :465-475).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

ELASTIC = "elastic"
MAGNETIC = "magnetic"
ELASTIC3D = "elastic3d"

# DOF per node, nodes per element and coordinates per node of each kind
_DIM = {ELASTIC: 2, MAGNETIC: 1, ELASTIC3D: 3}
_NPE = {ELASTIC: 3, MAGNETIC: 3, ELASTIC3D: 4}


def _f64(a, n=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))
    if n is not None and a.shape[0] == 1 and n != 1:
        a = np.full(n, a[0])
    return a


def _i64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64).reshape(-1))


@dataclass
class ElementLoadSet:
    """One ``ElementsLoad``: a total ``value`` spread over ``elements`` by area
    (finite_elements/loads.py:24-35), applied in 1-based ``dimension``."""

    elements: np.ndarray
    value: float
    dimension: int


@dataclass
class MagnetLoadSet:
    """One ``MagnetLoad`` (loads.py:105-147): its triangles, the nodes that are not on
    the magnet's contour, and the magnetization vector (mx, my)."""

    elements: np.ndarray
    non_contour_nodes: np.ndarray
    magnetization: tuple


@dataclass
class Problem:
    """Everything the GPU path needs for one analysis, as arrays.

    kind            "elastic" (plane triangles, 2 DOF per node), "magnetic" (triangles,
                    1 DOF per node) or "elastic3d" (linear tetrahedra, 3 DOF per node)
    coords          (n, 2) float64 node coordinates, in ``mesh.nodes`` order ((n, 3)
                    for "elastic3d")
    conn            (E, 3) int32 node indices, groups then elements in mesh order ((E, 4)
                    for "elastic3d")
    E, nu, thickness, rho   (E,) float64 elastic material per element (no thickness in 3D)
    mu              (E,) float64 absolute permeability per element (magnetic)
    plane_strain, plane_stress   the reference's two flags (elements.py:251-273)
    node_loads      (node, dim, value) triples in user order
    element_loads   list of ElementLoadSet in user order
    edge_loads      (node_a, node_b, dim, value) in user order
    node_bcs        (node, dim, value) in user order
    element_bcs     (element, dim, value) in user order
    edge_bcs        (node_a, node_b, dim, value) in user order
    magnet_loads    list of MagnetLoadSet in user order (triangles)
    continuity      (node1, node2, value) in user order: u[node1] = value * u[node2],
                    the reference indexing the DOF by the node index
                    (analysis.py:175-199)
    """

    kind: str
    coords: np.ndarray
    conn: np.ndarray
    E: np.ndarray | None = None
    nu: np.ndarray | None = None
    thickness: np.ndarray | None = None
    rho: np.ndarray | None = None
    mu: np.ndarray | None = None
    plane_strain: bool | None = None
    plane_stress: bool | None = None
    node_load_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    node_load_dim: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    node_load_value: np.ndarray = field(default_factory=lambda: np.zeros(0))
    element_loads: list = field(default_factory=list)
    edge_load_nodes: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int64))
    edge_load_dim: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    edge_load_value: np.ndarray = field(default_factory=lambda: np.zeros(0))
    node_bc_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    node_bc_dim: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    node_bc_value: np.ndarray = field(default_factory=lambda: np.zeros(0))
    element_bc_element: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    element_bc_dim: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    element_bc_value: np.ndarray = field(default_factory=lambda: np.zeros(0))
    edge_bc_nodes: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int64))
    edge_bc_dim: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    edge_bc_value: np.ndarray = field(default_factory=lambda: np.zeros(0))
    magnet_loads: list = field(default_factory=list)
    cont_node1: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    cont_node2: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    cont_value: np.ndarray = field(default_factory=lambda: np.zeros(0))

    def __post_init__(self):
        if self.kind not in _DIM:
            raise ValueError(f"unknown problem kind {self.kind!r}")
        cdim = 3 if self.kind == ELASTIC3D else 2
        self.coords = np.ascontiguousarray(np.asarray(self.coords, np.float64).reshape(-1, cdim))
        self.conn = np.ascontiguousarray(np.asarray(self.conn, np.int32).reshape(-1, _NPE[self.kind]))
        ne = self.conn.shape[0]
        for name in ("E", "nu", "thickness", "rho", "mu"):
            v = getattr(self, name)
            if v is not None:
                setattr(self, name, _f64(v, ne))
        for name in ("node_load_node", "node_load_dim", "node_bc_node", "node_bc_dim",
                     "element_bc_element", "element_bc_dim", "edge_load_dim", "edge_bc_dim",
                     "cont_node1", "cont_node2"):
            setattr(self, name, _i64(getattr(self, name)))
        for name in ("node_load_value", "node_bc_value", "element_bc_value",
                     "edge_load_value", "edge_bc_value", "cont_value"):
            setattr(self, name, _f64(getattr(self, name)))
        self.edge_load_nodes = _i64(self.edge_load_nodes).reshape(-1, 2)
        self.edge_bc_nodes = _i64(self.edge_bc_nodes).reshape(-1, 2)
        self.element_loads = [ElementLoadSet(_i64(s.elements), float(s.value), int(s.dimension))
                              for s in self.element_loads]
        self.magnet_loads = [MagnetLoadSet(_i64(s.elements), _i64(s.non_contour_nodes),
                                           (float(s.magnetization[0]), float(s.magnetization[1])))
                             for s in self.magnet_loads]

    @property
    def dim(self) -> int:
        return _DIM[self.kind]

    @property
    def npe(self) -> int:
        """Nodes per element."""
        return _NPE[self.kind]

    @property
    def elastic(self) -> bool:
        return self.kind in (ELASTIC, ELASTIC3D)

    @property
    def n_nodes(self) -> int:
        return self.coords.shape[0]

    @property
    def n_elements(self) -> int:
        return self.conn.shape[0]

    @property
    def n_dof(self) -> int:
        return self.n_nodes * self.dim

    @property
    def n_cont(self) -> int:
        return self.cont_node1.size
