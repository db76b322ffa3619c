"""Light mesh types standing in for the parts of ``volmdlr.mesh`` the analysis reads.

The reference builds its meshes from volmdlr objects and the analysis only touches a
small surface of them:

* ``Mesh.nodes`` / ``Mesh.node_to_index`` / ``Mesh.elements_groups``
  (finite_elements/analysis.py:274, :487, :716; core.py:89-108);
* ``ElementsGroup.elements`` (analysis.py:326-327);
* ``TriangularElement2D.points`` / ``.area`` / ``.form_functions``
  (elements.py:35-44, :100-116, :508, :530; loads.py:32-34);
* ``TetrahedralElement.points`` / ``.volume`` / ``.form_functions``
  (elements.py:719-748, :808-858);
* edge objects with ``.start`` / ``.end`` (analysis.py:232-233, :441-442);
* for magnet loads, ``TriangularElement2D.linear_elements`` with ``.points``,
  ``.interior_normal`` and ``.length()``, and ``Vector2D.Dot`` (loads.py:129-147,
  analysis.py:556-577).

volmdlr is not a dependency of this package, so these classes provide that surface.
Real volmdlr objects with the same attributes work as well (the analysis only
duck-types them).  ``ArrayMesh`` is the bulk form: node coordinates and
connectivity as arrays, so that meshes of millions of triangles never become Python
objects on the host.
"""
from __future__ import annotations

import math

import numpy as np


class Point2D:
    """A 2D point, hashed and compared by its coordinates (like volmdlr.Point2D)."""

    __slots__ = ("x", "y")

    def __init__(self, x, y):
        self.x = float(x)
        self.y = float(y)

    def __getitem__(self, i):
        return (self.x, self.y)[i]

    def __iter__(self):
        yield self.x
        yield self.y

    def __len__(self):
        return 2

    def __hash__(self):
        return hash((self.x, self.y))

    def __eq__(self, other):
        return (isinstance(other, Point2D) and self.x == other.x and self.y == other.y)

    def __repr__(self):
        return f"{type(self).__name__}({self.x!r}, {self.y!r})"


class Node2D(Point2D):
    """A mesh node (volmdlr.mesh.Node2D)."""


class Vector2D(Point2D):
    """A 2D vector (volmdlr.Vector2D): the dot product and the scaling MagnetLoad uses.
    Built from (x, y) or from one (x, y) sequence."""

    def __init__(self, x, y=None):
        if y is None:
            x, y = x
        Point2D.__init__(self, x, y)

    def Dot(self, other):
        return self.x * other[0] + self.y * other[1]

    def dot(self, other):
        return self.x * other[0] + self.y * other[1]

    def Norm(self):
        return math.sqrt(self.x ** 2 + self.y ** 2)

    def norm(self):
        return math.sqrt(self.x ** 2 + self.y ** 2)

    def normalize(self):
        """In place, as volmdlr's Vector2D.normalize."""
        n = self.norm()
        self.x /= n
        self.y /= n

    def __truediv__(self, k):
        return Vector2D(self.x / k, self.y / k)

    def __neg__(self):
        return Vector2D(-self.x, -self.y)


class LinearElement:
    """An edge of a triangle with the unit normal pointing into that triangle
    (volmdlr.mesh.LinearElement).  Two edges are equal when they join the same two
    points, in either direction, so that counting edges over a set of triangles finds
    its contour (loads.py:129-147)."""

    def __init__(self, start, end, interior_normal):
        self.points = [start, end]
        self.interior_normal = interior_normal

    def length(self):
        (x1, y1), (x2, y2) = self.points
        return math.sqrt((x2 - x1) ** 2 + (y2 - y1) ** 2)

    def __hash__(self):
        return hash(self.points[0]) + hash(self.points[1])

    def __eq__(self, other):
        a, b = self.points
        c, d = other.points
        return (a == c and b == d) or (a == d and b == c)


class Point3D:
    """A 3D point, hashed and compared by its coordinates (like volmdlr.Point3D)."""

    __slots__ = ("x", "y", "z")

    def __init__(self, x, y, z):
        self.x = float(x)
        self.y = float(y)
        self.z = float(z)

    def __getitem__(self, i):
        return (self.x, self.y, self.z)[i]

    def __iter__(self):
        yield self.x
        yield self.y
        yield self.z

    def __len__(self):
        return 3

    def __hash__(self):
        return hash((self.x, self.y, self.z))

    def __eq__(self, other):
        return (isinstance(other, Point3D) and self.x == other.x and self.y == other.y
                and self.z == other.z)

    def __repr__(self):
        return f"{type(self).__name__}({self.x!r}, {self.y!r}, {self.z!r})"


class Node3D(Point3D):
    """A 3D mesh node (volmdlr.mesh.Node3D)."""


class LineSegment2D:
    """An edge between two points; edge loads and edge conditions read ``start``/``end``."""

    def __init__(self, start, end, name=""):
        self.start = start
        self.end = end
        self.name = name

    @property
    def points(self):
        return [self.start, self.end]


class TriangularElement2D:
    """A 3-node triangle.

    ``area`` is the unsigned area |detJ|/2 and ``form_functions`` the three rows
    (a_i, b_i, c_i) of the linear shape functions N_i = a_i + b_i x + c_i y with
    N_i(p_j) = delta_ij -- the two volmdlr quantities the reference consumes
    (elements.py:100-116, :35-44, :508, :530).
    """

    def __init__(self, points, name=""):
        self.points = list(points)
        self.name = name

    def _xy(self):
        return [(float(p[0]), float(p[1])) for p in self.points]

    @property
    def area(self):
        (x1, y1), (x2, y2), (x3, y3) = self._xy()
        return abs((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1)) / 2.0

    @property
    def form_functions(self):
        (x1, y1), (x2, y2), (x3, y3) = self._xy()
        det = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1)
        a = ((x2 * y3 - x3 * y2) / det, (x3 * y1 - x1 * y3) / det, (x1 * y2 - x2 * y1) / det)
        b = ((y2 - y3) / det, (y3 - y1) / det, (y1 - y2) / det)
        c = ((x3 - x2) / det, (x1 - x3) / det, (x2 - x1) / det)
        return [[a[i], b[i], c[i]] for i in range(3)]

    @property
    def center(self):
        xy = self._xy()
        return Vector2D(sum(p[0] for p in xy) / 3.0, sum(p[1] for p in xy) / 3.0)

    @property
    def linear_elements(self):
        """The edges (p1, p2), (p2, p3), (p3, p1), each with its unit normal turned
        towards the opposite vertex."""
        out = []
        for i in range(3):
            a, b, c = self.points[i], self.points[(i + 1) % 3], self.points[(i + 2) % 3]
            n = interior_normal(a, b, c)
            out.append(LinearElement(a, b, Vector2D(n[0], n[1])))
        return out


def interior_normal(a, b, c):
    """Unit normal of the edge a -> b pointing to the side of c: the edge direction
    turned by +90 degrees, negated when it points away from c."""
    tx, ty = float(b[0]) - float(a[0]), float(b[1]) - float(a[1])
    length = math.sqrt(tx * tx + ty * ty)
    nx, ny = -ty / length, tx / length
    if nx * (float(c[0]) - float(a[0])) + ny * (float(c[1]) - float(a[1])) < 0:
        nx, ny = -nx, -ny
    return nx, ny


class TetrahedralElement:
    """A 4-node linear tetrahedron.

    ``volume`` is the unsigned volume |det[p1-p0, p2-p0, p3-p0]|/6 and
    ``form_functions`` the four rows (a_i, b_i, c_i, d_i) with
    N_i = (a_i + b_i x + c_i y + d_i z) / (6 V), N_i(p_j) = delta_ij: the convention under
    which the reference's B = (1/(6V)) [b_i, c_i, d_i ...] (elements.py:719-748) is the
    matrix of shape-function gradients.
    """

    def __init__(self, points, name=""):
        self.points = list(points)
        self.name = name

    def _xyz(self):
        return np.array([[float(p[0]), float(p[1]), float(p[2])] for p in self.points])

    @property
    def volume(self):
        p = self._xyz()
        a, n = p[1] - p[0], np.cross(p[2] - p[0], p[3] - p[0])
        return abs(a[0] * n[0] + a[1] * n[1] + a[2] * n[2]) / 6.0

    @property
    def form_functions(self):
        p = self._xyz()
        coef = np.linalg.inv(np.hstack([np.ones((4, 1)), p]))   # column i: N_i = coef[:, i] . (1, x, y, z)
        return [list(6.0 * self.volume * coef[:, i]) for i in range(4)]

    @property
    def center(self):
        c = self._xyz().mean(axis=0)
        return Point3D(*c)


class ElementsGroup:
    """An ordered list of elements (volmdlr.mesh.ElementsGroup)."""

    def __init__(self, elements, name=""):
        self.elements = list(elements)
        self.name = name


class Mesh:
    """A mesh of element groups.

    ``nodes`` lists every distinct element point in order of first appearance
    (group order, element order, point order) and ``node_to_index`` maps a point to
    its position there.  Callers may overwrite both, as the reference's own scripts do
    to keep a mesh file's node order (scripts/Elasticity/beam2d_example_3.py:72-73).
    """

    def __init__(self, elements_groups, name=""):
        self.elements_groups = list(elements_groups)
        self.name = name
        nodes, index = [], {}
        for group in self.elements_groups:
            for element in group.elements:
                for p in element.points:
                    if p not in index:
                        index[p] = len(nodes)
                        nodes.append(p)
        self.nodes = nodes
        self.node_to_index = index


class ArrayMesh:
    """A mesh held as arrays: ``coords`` (n, 2) float64 and ``conn`` (E, 3) int32, or
    ``coords`` (n, 3) and ``conn`` (E, 4) for tetrahedra.

    ``group_ptr`` splits the elements into consecutive groups (group g is
    ``conn[group_ptr[g]:group_ptr[g+1]]``).  Per-element material arrays live in the
    analysis, not here.  ``nodes`` / ``node_to_index`` are built on first use only.
    """

    def __init__(self, coords, conn, group_ptr=None, name=""):
        coords = np.asarray(coords, dtype=np.float64)
        conn = np.asarray(conn, dtype=np.int32)
        cdim = coords.shape[1] if coords.ndim == 2 else 2
        npe = conn.shape[1] if conn.ndim == 2 else 3
        self.coords = np.ascontiguousarray(coords).reshape(-1, cdim)
        self.conn = np.ascontiguousarray(conn).reshape(-1, npe)
        if group_ptr is None:
            group_ptr = [0, self.conn.shape[0]]
        self.group_ptr = np.asarray(group_ptr, dtype=np.int64)
        self.name = name
        self._nodes = None
        self._node_to_index = None

    @property
    def n_nodes(self):
        return self.coords.shape[0]

    @property
    def n_elements(self):
        return self.conn.shape[0]

    @property
    def nodes(self):
        if self._nodes is None:
            node = Node3D if self.coords.shape[1] == 3 else Node2D
            self._nodes = [node(*c) for c in self.coords.tolist()]
        return self._nodes

    @property
    def node_to_index(self):
        if self._node_to_index is None:
            self._node_to_index = {p: i for i, p in enumerate(self.nodes)}
        return self._node_to_index

    def as_arrays(self):
        return self.coords, self.conn
