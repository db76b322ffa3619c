"""Result containers (finite_elements/results.py:23-54) and the GPU-computed
per-element results of elasticity and magnetostatic solutions."""
from __future__ import annotations

import math

import numpy as np

MU = 4 * math.pi * 1e-7   # finite_elements/core.py:31


class PerItem:
    """Per-element (or per-node) results: an array, one row per element (node) in mesh
    order, that can also be indexed by the mesh's element (node) objects, as the
    reference's dicts are ({element: value}, results.py:639-830).  Integer indices,
    slices and index arrays address rows; ``keys()``, ``values()`` and ``items()``
    and iteration follow the dict."""

    def __init__(self, values, keys_fn):
        self._values = values
        self._keys_fn = keys_fn
        self._by_id = None
        self._by_eq = None

    def __array__(self, dtype=None, copy=None):
        return np.asarray(self._values, dtype=dtype)

    @property
    def shape(self):
        return self._values.shape

    @property
    def ndim(self):
        return self._values.ndim

    @property
    def dtype(self):
        return self._values.dtype

    def __len__(self):
        return len(self._values)

    def _row(self, key):
        if self._by_id is None:
            keys = self._keys_fn()
            self._by_id = {id(k): i for i, k in enumerate(keys)}
            self._by_eq = {}
            for i, k in enumerate(keys):
                try:
                    self._by_eq.setdefault(k, i)
                except TypeError:
                    pass
        i = self._by_id.get(id(key))
        if i is None:
            i = self._by_eq[key]
        return i

    def __getitem__(self, key):
        if isinstance(key, (int, np.integer, slice, tuple, list, np.ndarray)):
            return self._values[key]
        return self._values[self._row(key)]

    def keys(self):
        return list(self._keys_fn())

    def values(self):
        return list(self._values)

    def items(self):
        return list(zip(self._keys_fn(), self._values))

    def __iter__(self):
        return iter(self._keys_fn())

    def __repr__(self):
        return f"PerItem({self._values!r})"


def _element_keys(mesh):
    if hasattr(mesh, "as_arrays"):
        return lambda: range(mesh.n_elements)
    return lambda: [el for g in mesh.elements_groups for el in g.elements]


def _node_keys(mesh):
    return lambda: mesh.nodes


class Result:
    """``mesh`` and ``result_vector``: n_nodes*dim displacements (or potentials)
    followed by one Lagrange multiplier per Dirichlet condition.  ``dimension`` comes
    from the mesh's first element (the reference's rule) or, for an array mesh, from
    the analysis that produced the result."""

    def __init__(self, mesh, result_vector, dimension=None):
        self.mesh = mesh
        self.result_vector = result_vector
        self._dimension = dimension

    @property
    def dimension(self):
        if self._dimension is not None:
            return self._dimension
        return self.mesh.elements_groups[0].elements[0].dimension


def mesh_arrays(mesh):
    """(coords (n, 2|3), conn (E, 3|4)) of an ArrayMesh or of a mesh of element objects
    (nodes in ``mesh.nodes`` order, elements in group order)."""
    if hasattr(mesh, "as_arrays"):
        return mesh.as_arrays()
    index = mesh.node_to_index
    first = mesh.elements_groups[0].elements[0]
    npe = len(first.points)
    cdim = 3 if npe == 4 else 2
    coords = np.array([[float(p[k]) for k in range(cdim)] for p in mesh.nodes], np.float64).reshape(-1, cdim)
    conn = np.array([[index[p] for p in el.points] for g in mesh.elements_groups for el in g.elements],
                    np.int64).reshape(-1, npe)
    return coords, conn


def write_vtk(file_name, coords, conn, point_scalars=(), point_vectors=()):
    """Legacy ASCII VTK unstructured grid of linear triangles (cell type 5) or linear
    tetrahedra (cell type 10, when conn has 4 columns) with point data:
    ``point_scalars`` / ``point_vectors`` are (name, (n,) or (n, 2|3)) pairs."""
    coords = np.asarray(coords, np.float64)
    conn = np.asarray(conn, np.int64)
    npe = conn.shape[1] if conn.ndim == 2 else 3
    conn = conn.reshape(-1, npe)
    n, e = coords.shape[0], conn.shape[0]
    xyz = coords if coords.shape[1] == 3 else np.hstack([coords[:, :2], np.zeros((n, 1))])
    out = ["# vtk DataFile Version 3.0", "finite element result", "ASCII", "DATASET UNSTRUCTURED_GRID",
           f"POINTS {n} double"]
    out += [f"{x!r} {y!r} {z!r}" for x, y, z in xyz.tolist()]
    out += [f"CELLS {e} {(npe + 1) * e}"] + [f"{npe} " + " ".join(map(str, row)) for row in conn.tolist()]
    out += [f"CELL_TYPES {e}"] + (["10"] if npe == 4 else ["5"]) * e
    if point_scalars or point_vectors:
        out.append(f"POINT_DATA {n}")
    for name, v in point_scalars:
        out += [f"SCALARS {name} float 1", "LOOKUP_TABLE default"] + [repr(float(t)) for t in np.asarray(v)]
    for name, v in point_vectors:
        v = np.asarray(v, np.float64).reshape(n, -1)
        if v.shape[1] == 2:
            v = np.hstack([v, np.zeros((n, 1))])
        out += [f"VECTORS {name} float"] + [f"{a!r} {b!r} {c!r}" for a, b, c in v.tolist()]
    with open(file_name, "w", encoding="utf-8") as f:
        f.write("\n".join(out) + "\n")


def _system_for(mesh, plane_strain=None, plane_stress=None):
    """A GPU system for a mesh of elasticity or magnetic elements (stiffness only:
    the post-processing reads element matrices and geometry)."""
    from .analysis import FiniteElementAnalysis
    fea = FiniteElementAnalysis(mesh, [], [], [], [], [], [], [], [], plane_strain, plane_stress)
    return fea.system()


class ElasticityResults2D(Result):
    """Per-element strain, stress and energy of a plane-elasticity solution
    (finite_elements/results.py:930, :700-830), computed by the GPU kernels.
    Arrays follow the mesh's element order (groups, then elements).  Strain and stress
    rows are (xx, yy, xy)."""

    _ncomp = 2

    def __init__(self, mesh, result_vector, plane_strain, plane_stress, system=None):
        Result.__init__(self, mesh, result_vector)
        self.plane_strain = plane_strain
        self.plane_stress = plane_stress
        self._system = system
        self._post = None

    def _compute(self):
        if self._post is None:
            if self._system is None:
                self._system = _system_for(self.mesh, self.plane_strain, self.plane_stress)
            self._post = self._system.post(np.asarray(self.result_vector, np.float64))
        return self._post

    @property
    def strain(self):
        return PerItem(self._compute()["strain"], _element_keys(self.mesh))

    @property
    def stress(self):
        return PerItem(self._compute()["stress"], _element_keys(self.mesh))

    @property
    def energy_per_element(self):
        return PerItem(self._compute()["energy"], _element_keys(self.mesh))

    @property
    def energy(self):
        return float(np.sum(self._compute()["energy"]))

    @property
    def displacement_vectors_per_node(self):
        n, d = len(self.mesh.nodes), self._ncomp
        return PerItem(np.asarray(self.result_vector[: d * n], np.float64).reshape(n, d), _node_keys(self.mesh))

    @property
    def displacements_per_element(self):
        """(E, npe*d) element DOF vectors, node-major (results.py:677-700), real part."""
        coords, conn = mesh_arrays(self.mesh)
        u = np.real(np.asarray(self.displacement_vectors_per_node))
        return PerItem(u[np.asarray(conn, np.int64)].reshape(conn.shape[0], -1), _element_keys(self.mesh))

    def deformed_nodes_m(self, amplitude=1):
        """(n, d) node coordinates moved by amplitude times the displacement
        (results.py:587-616), in mesh.nodes order."""
        coords, _ = mesh_arrays(self.mesh)
        return coords[:, : self._ncomp] + amplitude * np.real(np.asarray(self.displacement_vectors_per_node))

    @property
    def deformed_nodes(self):
        return self.deformed_nodes_m()

    def deformed_mesh_m(self, amplitude=1):
        """The mesh on the deformed nodes, as an ArrayMesh with the same connectivity
        and node order (results.py:549-585)."""
        from .mesh import ArrayMesh
        _, conn = mesh_arrays(self.mesh)
        return ArrayMesh(self.deformed_nodes_m(amplitude), conn)

    @property
    def deformed_mesh(self):
        return self.deformed_mesh_m()

    def displacement_per_node_x(self):
        return np.asarray(self.displacement_vectors_per_node)[:, 0]

    def displacement_per_node_y(self):
        return np.asarray(self.displacement_vectors_per_node)[:, 1]

    def axial_strain_x(self):
        return np.asarray(self.strain)[:, 0]

    def axial_strain_y(self):
        return np.asarray(self.strain)[:, 1]

    def axial_stress_x(self):
        return np.asarray(self.stress)[:, 0]

    def axial_stress_y(self):
        return np.asarray(self.stress)[:, 1]

    def shear_strain_xy(self):
        return np.asarray(self.strain)[:, 2]

    def shear_stress_xy(self):
        return np.asarray(self.stress)[:, 2]

    def generate_vtk_file(self, file_name_output):
        """The mesh with the displacement as point data, ``Displacement_Magnitude``
        (scalars) and ``Displacement_Vectors`` (vectors, z = 0 in 2D), as the
        reference's writer appends them (results.py:832-871).  The reference copies the
        mesh part from Gmsh's own VTK export; here the whole file is written."""
        if file_name_output[-3:] != "vtk":
            file_name_output += ".vtk"
        coords, conn = mesh_arrays(self.mesh)
        u = np.asarray(self.displacement_vectors_per_node)
        write_vtk(file_name_output, coords, conn,
                  point_scalars=[("Displacement_Magnitude", np.sqrt(np.sum(u * u, axis=1)))],
                  point_vectors=[("Displacement_Vectors", u)])
        return file_name_output


class ElasticityResults3D(ElasticityResults2D):
    """Per-element strain, stress and energy of a linear-tetrahedron solution
    (finite_elements/results.py:1468-1680); strain and stress rows are
    (xx, yy, zz, xy, yz, zx), the rows of the 3D B (elements.py:743-748)."""

    _ncomp = 3

    def displacement_per_node_z(self):
        return np.asarray(self.displacement_vectors_per_node)[:, 2]

    def axial_strain_z(self):
        return np.asarray(self.strain)[:, 2]

    def axial_stress_z(self):
        return np.asarray(self.stress)[:, 2]

    def shear_strain_xy(self):
        return np.asarray(self.strain)[:, 3]

    def shear_strain_yz(self):
        return np.asarray(self.strain)[:, 4]

    def shear_strain_zx(self):
        return np.asarray(self.strain)[:, 5]

    def shear_stress_xy(self):
        return np.asarray(self.stress)[:, 3]

    def shear_stress_yz(self):
        return np.asarray(self.stress)[:, 4]

    def shear_stress_zx(self):
        return np.asarray(self.stress)[:, 5]


class MagneticResults(Result):
    """Per-element magnetic flux density B = curl A of a magnetostatic solution
    (finite_elements/results.py:57-152), computed by the GPU kernel."""

    def __init__(self, mesh, result_vector, system=None):
        Result.__init__(self, mesh, result_vector)
        self._system = system
        self._field = None

    def _b(self):
        if self._field is None:
            if self._system is None:
                self._system = _system_for(self.mesh)
            self._field = self._system.post(np.asarray(self.result_vector, np.float64))["field"]
        return self._field

    @property
    def magnetic_field_per_element(self):
        return PerItem(self._b(), _element_keys(self.mesh))

    @property
    def magnetic_field_norm(self):
        b = self._b()
        return np.hypot(b[:, 0], b[:, 1])

    # ---- air-gap quantities (results.py:82-243), host arithmetic on the device's B field

    def _elements(self):
        return [el for g in self.mesh.elements_groups for el in g.elements]

    def _group_range(self, group):
        """Element range of a group of the mesh: the group object itself, or its name."""
        start = 0
        for g in self.mesh.elements_groups:
            n = len(g.elements)
            if g is group or (isinstance(group, str) and getattr(g, "name", None) == group):
                return range(start, start + n)
            start += n
        raise ValueError(f"no elements group {getattr(group, 'name', group)!r} in the mesh")

    def _polar(self, idx):
        """Element centres (x1 + x2 + x3) / 3, their norm, and (B . e_r, B . e_theta)
        with e_r the unit centre direction and e_theta = (-e_r[1], e_r[0])."""
        coords, conn = mesh_arrays(self.mesh)
        p = coords[np.asarray(conn, np.int64)[idx]]
        cx = (p[:, 0, 0] + p[:, 1, 0] + p[:, 2, 0]) / 3.0
        cy = (p[:, 0, 1] + p[:, 1, 1] + p[:, 2, 1]) / 3.0
        r = np.sqrt(cx ** 2 + cy ** 2)
        ex, ey = cx / r, cy / r
        b = self._b()[idx]
        br = b[:, 0] * ex + b[:, 1] * ey
        bt = b[:, 0] * -ey + b[:, 1] * ex
        return r, br, bt, b, p

    def brbtetha(self, gap_elements_group):
        """B_r * B_theta of every element of the group (results.py:82-106)."""
        _, br, bt, _, _ = self._polar(np.array(list(self._group_range(gap_elements_group)), np.int64))
        return list(br * bt)

    def maxwell_stress_tensor(self, element):
        """[sigma_rr, sigma_r_theta, sigma_theta_theta] of one element (results.py:154-181)."""
        k = next(i for i, el in enumerate(self._elements()) if el is element)
        _, br, bt, b, _ = self._polar(np.array([k]))
        nb2 = np.sqrt(b[0, 0] ** 2 + b[0, 1] ** 2) ** 2
        return [1 / MU * br[0] ** 2 - 1 / (2 * MU) * nb2, 1 / MU * br[0] * bt[0],
                1 / MU * bt[0] ** 2 - 1 / (2 * MU) * nb2]

    def torque(self, air_gap_elements_group_name, length_motor, radius_stator, radius_rotor):
        """Arkkio's torque (results.py:183-243): length / (mu0 (r_s - r_r)) times the sum
        over the air-gap elements of |centre| B_r B_theta area, summed in element order."""
        idx = np.array(list(self._group_range(air_gap_elements_group_name)), np.int64)
        r, br, bt, _, p = self._polar(idx)
        area = np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1])
                      - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])) / 2.0
        somme = 0
        for term in (r * br * bt * area).tolist():
            somme += term
        return length_motor / (MU * (radius_stator - radius_rotor)) * somme
