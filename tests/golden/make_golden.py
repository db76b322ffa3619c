"""Generate the golden vectors under tests/golden/ by running the reference itself.

The reference package (``finite_elements``) imports volmdlr, dessia_common and
matplotlib, none of which is installed, and reads its version through
pkg_resources.  This script puts minimal stand-ins for those four into
``sys.modules`` (volmdlr.mesh is served by ``finite_elements_gb300.mesh``, which
implements the attributes the reference reads) and then imports the reference's own
``finite_elements.analysis`` / ``elements`` / ``loads`` / ``conditions`` modules from
the reference checkout and runs ``create_matrix()``, ``create_source_matrix()``,
``solve()``, ``k_matrix_sparse()`` and ``m_matrix_sparse()`` on each case.

Each case is stored as ``<name>.npz`` holding the problem as arrays (the inputs the
GPU path takes) and the reference's outputs.  Run from the repository root:

    python tests/golden/make_golden.py [/path/to/reference [case ...]]
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from finite_elements_gb300 import mesh as fmesh          # noqa: E402
from finite_elements_gb300 import meshgen                # noqa: E402
from finite_elements_gb300.problem import (ELASTIC, ELASTIC3D, ElementLoadSet, MagnetLoadSet,  # noqa: E402
                                          Problem)


class _Anything:
    """Accepts any construction / call / attribute access (plotting stand-in)."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()


def _permissive_module(name, **attrs):
    mod = types.ModuleType(name)
    mod.__dict__.update(attrs)
    mod.__getattr__ = lambda attr: _Anything
    return mod


def install_stubs():
    class DessiaObject:
        def __init__(self, name='', **kwargs):
            self.name = name

    dc = _permissive_module("dessia_common")
    dcc = _permissive_module("dessia_common.core", DessiaObject=DessiaObject)
    dc.core = dcc
    vm = _permissive_module("volmdlr", Point2D=fmesh.Point2D, Point3D=fmesh.Point3D, Vector2D=fmesh.Vector2D)
    vmm = _permissive_module("volmdlr.mesh", Node2D=fmesh.Node2D, Node3D=fmesh.Node3D,
                             TriangularElement2D=fmesh.TriangularElement2D,
                             TetrahedralElement=fmesh.TetrahedralElement,
                             ElementsGroup=fmesh.ElementsGroup, Mesh=fmesh.Mesh)
    vm.mesh = vmm
    mpl = _permissive_module("matplotlib")
    for sub in ("pyplot", "colors", "tri"):
        m = _permissive_module("matplotlib." + sub)
        setattr(mpl, sub, m)
        sys.modules["matplotlib." + sub] = m
    pkr = types.ModuleType("pkg_resources")
    pkr.require = lambda name: [types.SimpleNamespace(version="0.2.0")]
    sys.modules.update({"dessia_common": dc, "dessia_common.core": dcc, "volmdlr": vm,
                        "volmdlr.mesh": vmm, "matplotlib": mpl, "pkg_resources": pkr})


def reference_objects(fe, prob: Problem, groups, names=None):
    """Build the reference's object graph for ``prob``: nodes, elements (wrapped as
    the reference's element classes), groups, mesh, loads and conditions."""
    if prob.kind == ELASTIC3D:
        nodes = [fmesh.Node3D(*c) for c in prob.coords.tolist()]
        tets = [fmesh.TetrahedralElement([nodes[i] for i in row]) for row in prob.conn.tolist()]
        elems = [fe.elements.ElasticityTetrahedralElement3D(
            t, float(prob.E[k]), float(prob.nu[k]), float(prob.rho[k])) for k, t in enumerate(tets)]
    else:
        nodes = [fmesh.Node2D(x, y) for x, y in prob.coords.tolist()]
        tris = [fmesh.TriangularElement2D([nodes[i] for i in row]) for row in prob.conn.tolist()]
        if prob.kind == ELASTIC:
            elems = [fe.elements.ElasticityTriangularElement2D(
                t, float(prob.E[k]), float(prob.nu[k]), float(prob.rho[k]), float(prob.thickness[k]))
                for k, t in enumerate(tris)]
        else:
            elems = [fe.elements.MagneticElement2D(t, float(prob.mu[k])) for k, t in enumerate(tris)]
    egroups = [fmesh.ElementsGroup(elems[a:b], names[g] if names else f"g{g}") for g, (a, b) in
               enumerate(zip(groups[:-1], groups[1:]))]
    mesh = fmesh.Mesh(egroups)
    mesh.nodes = nodes
    mesh.node_to_index = {p: i for i, p in enumerate(nodes)}
    node_loads = [fe.loads.NodeLoad(nodes[n], float(v), int(d)) for n, d, v in
                  zip(prob.node_load_node, prob.node_load_dim, prob.node_load_value)]
    element_loads = [fe.loads.ElementsLoad([elems[k] for k in s.elements.tolist()], s.value,
                                           s.dimension) for s in prob.element_loads]
    edge_loads = [fe.loads.EdgeLoad(fmesh.LineSegment2D(nodes[a], nodes[b]), float(v), int(d))
                  for (a, b), d, v in zip(prob.edge_load_nodes.tolist(), prob.edge_load_dim,
                                          prob.edge_load_value)]
    C = fe.conditions
    node_bcs = [C.NodeBoundaryCondition(nodes[n], float(v), int(d)) for n, d, v in
                zip(prob.node_bc_node, prob.node_bc_dim, prob.node_bc_value)]
    elem_bcs = [C.ElementBoundaryCondition(elems[k], float(v), int(d)) for k, d, v in
                zip(prob.element_bc_element, prob.element_bc_dim, prob.element_bc_value)]
    edge_bcs = [C.EdgeBoundaryCondition(fmesh.LineSegment2D(nodes[a], nodes[b]), float(v), int(d))
                for (a, b), d, v in zip(prob.edge_bc_nodes.tolist(), prob.edge_bc_dim,
                                        prob.edge_bc_value)]
    magnets = [fe.loads.MagnetLoad([elems[k] for k in m.elements.tolist()],
                                   [nodes[k] for k in m.non_contour_nodes.tolist()],
                                   fmesh.Vector2D(*m.magnetization)) for m in prob.magnet_loads]
    conts = [C.ContinuityCondition(nodes[a], nodes[b], float(v)) for a, b, v in
             zip(prob.cont_node1.tolist(), prob.cont_node2.tolist(), prob.cont_value.tolist())]
    return mesh, elems, node_loads, element_loads, edge_loads, node_bcs, elem_bcs, edge_bcs, magnets, conts


def run_reference(fe, prob: Problem, groups, names=None, motor=None):
    mesh, elems, nl, el, edl, nbc, ebc, edbc, mag, cont = reference_objects(fe, prob, groups, names)
    kw = {}
    if prob.elastic:
        kw = dict(plane_strain=prob.plane_strain, plane_stress=prob.plane_stress)
    analysis = fe.analysis.FiniteElementAnalysis(
        mesh=mesh, element_loads=el, edge_loads=edl, node_loads=nl, magnet_loads=mag,
        continuity_conditions=cont, node_boundary_conditions=nbc,
        edge_boundary_conditions=edbc, element_boundary_conditions=ebc, **kw)
    out = {}
    K = analysis.create_matrix()
    out["K_indptr"], out["K_indices"], out["K_data"] = K.indptr, K.indices, K.data
    out["K_shape"] = np.array(K.shape)
    out["F"] = analysis.create_source_matrix()[:, 0]
    try:
        res = analysis.solve()
        out["x"] = np.array(res.result_vector)
    except ValueError as exc:          # scipy's shape check of spsolve
        out["solve_error"] = np.array(str(exc))
    ks = analysis.k_matrix_sparse()
    out["Ks_indptr"], out["Ks_indices"], out["Ks_data"] = ks.indptr, ks.indices, ks.data
    out["Ks_shape"] = np.array(ks.shape)
    if prob.elastic:
        ms = analysis.m_matrix_sparse()
        out["Ms_indptr"], out["Ms_indices"], out["Ms_data"] = ms.indptr, ms.indices, ms.data
        out["Ms_shape"] = np.array(ms.shape)
        out["Ke"] = np.array([e.elementary_matrix(prob.plane_strain, prob.plane_stress)
                              for e in elems])
        out["Me"] = np.array([e.elementary_mass_matrix() for e in elems])
    else:
        out["Ke"] = np.array([e.elementary_matrix() for e in elems])
    if prob.kind != ELASTIC3D:
        out["factors"] = np.array([e.element_to_node_factors() for e in elems])
    if motor is not None:
        # the reference's air-gap post-processing on its own solution (results.py:82-243)
        mr = fe.results.MagneticResults(mesh, list(out["x"]))
        gap = next(g for g in mesh.elements_groups if g.name == motor["gap"])
        out["brbtetha"] = np.array(mr.brbtetha(gap))
        out["torque"] = np.array(mr.torque(motor["gap"], motor["length"], motor["r_stator"], motor["r_rotor"]))
        out["maxwell"] = np.array([mr.maxwell_stress_tensor(gap.elements[k]) for k in motor["maxwell_elements"]])
    bcs = analysis._boundary_conditions
    out["bc_dof"] = np.array([analysis.positions[(mesh.node_to_index[b.application],
                                                  b.dimension)] for b in bcs], np.int64)
    out["bc_value"] = np.array([b.value for b in bcs], np.float64)
    return out


def problem_arrays(prob: Problem, groups):
    a = {"kind": np.array(prob.kind), "coords": prob.coords, "conn": prob.conn,
         "groups": np.asarray(groups, np.int64)}
    for name in ("E", "nu", "thickness", "rho", "mu"):
        v = getattr(prob, name)
        if v is not None:
            a[name] = v
    a["plane"] = np.array([-1 if prob.plane_strain is None else int(bool(prob.plane_strain)),
                           -1 if prob.plane_stress is None else int(bool(prob.plane_stress))])
    for name in ("node_load_node", "node_load_dim", "node_load_value", "edge_load_nodes",
                 "edge_load_dim", "edge_load_value", "node_bc_node", "node_bc_dim",
                 "node_bc_value", "element_bc_element", "element_bc_dim", "element_bc_value",
                 "edge_bc_nodes", "edge_bc_dim", "edge_bc_value"):
        a[name] = getattr(prob, name)
    a["n_element_loads"] = np.array(len(prob.element_loads))
    for k, s in enumerate(prob.element_loads):
        a[f"element_load_{k}_elements"] = s.elements
        a[f"element_load_{k}_value"] = np.array(s.value)
        a[f"element_load_{k}_dim"] = np.array(s.dimension)
    a["n_magnet_loads"] = np.array(len(prob.magnet_loads))
    for k, m in enumerate(prob.magnet_loads):
        a[f"magnet_load_{k}_elements"] = m.elements
        a[f"magnet_load_{k}_non_contour"] = m.non_contour_nodes
        a[f"magnet_load_{k}_m"] = np.array(m.magnetization)
    for name in ("cont_node1", "cont_node2", "cont_value"):
        a[name] = getattr(prob, name)
    return a


# ---------------------------------------------------------------- cases


def case_ex1(plane):
    """scripts/Elasticity/beam2d_example_1.py:18-49: two triangles, E=30e6, nu=0.25,
    t=0.5, rho=2.7, -1000 at (3,2) in dimension 2, five node conditions."""
    coords = [(3, 0), (3, 2), (0, 0), (0, 2)]
    conn = [[0, 1, 2], [3, 2, 1]]
    prob = Problem(ELASTIC, coords, conn, E=30e6, nu=0.25, thickness=0.5, rho=2.7,
                   plane_strain=(plane == "strain"), plane_stress=(plane == "stress"),
                   node_load_node=[1], node_load_dim=[2], node_load_value=[-1000.0],
                   node_bc_node=[0, 3, 3, 2, 2], node_bc_dim=[2, 1, 2, 1, 2],
                   node_bc_value=[0, 0, 0, 0, 0])
    return prob, [0, 2]


def _strip_mesh(n_cells):
    """The 1-by-n strip of scripts/Elasticity/beam2d_example_2.py:37-67 and
    scripts/Magnetic/finite_element_beam.py:21-50, nodes in first-appearance order."""
    index, coords, conn = {}, [], []
    for i in range(n_cells):
        for tri in (((i, 0), (i + 1, 0), (i, 1)), ((i + 1, 1), (i + 1, 0), (i, 1))):
            row = []
            for p in tri:
                if p not in index:
                    index[p] = len(coords)
                    coords.append(p)
                row.append(index[p])
            conn.append(row)
    return np.array(coords, float), np.array(conn), index


def case_ex2():
    """scripts/Elasticity/beam2d_example_2.py:33-106: 18 triangles in 3 groups,
    E=210e9, nu=0.25, t=1, rho=7860, plane strain, -1e7 at (9,1), x=0 clamped."""
    coords, conn, index = _strip_mesh(9)
    x0 = [i for i, p in enumerate(coords.tolist()) if p[0] == 0]
    prob = Problem(ELASTIC, coords, conn, E=210e9, nu=0.25, thickness=1.0, rho=7860.0,
                   plane_strain=True, plane_stress=False,
                   node_load_node=[index[(9, 1)]], node_load_dim=[2], node_load_value=[-1e7],
                   node_bc_node=np.repeat(x0, 2), node_bc_dim=np.tile([1, 2], len(x0)),
                   node_bc_value=np.zeros(2 * len(x0)))
    return prob, [0, 6, 12, 18]


def case_mag_beam():
    """scripts/Magnetic/finite_element_beam.py:14-66: three permeability groups,
    ElementsLoad(group1[0:2], 1e10, 1), A=0 on the x=9 nodes."""
    coords, conn, index = _strip_mesh(9)
    mu0 = 4 * np.pi * 1e-7
    mu = np.repeat([mu0 * 100000, mu0, mu0 * 50000], 6)
    x9 = [i for i, p in enumerate(coords.tolist()) if abs(p[0] - 9) < 1e-6]
    prob = Problem("magnetic", coords, conn, mu=mu,
                   element_loads=[ElementLoadSet(np.array([0, 1]), 1e10, 1)],
                   node_bc_node=x9, node_bc_dim=np.ones(len(x9), int),
                   node_bc_value=np.zeros(len(x9)))
    return prob, [0, 6, 12, 18]


def case_quirks_elastic():
    """Every load and condition kind at once on a 6x3 plane-stress grid: repeated
    node loads and conditions (the last value wins), element loads whose
    (0, A, A) node factors overwrite a user load, edge loads overwriting element
    loads, element and edge conditions, non-zero prescribed values, per-element E
    and three groups."""
    rng = np.random.default_rng(7)
    nx, ny = 6, 3
    coords, conn = meshgen.rect_grid(nx, ny, 3.0, 1.5)
    ne = conn.shape[0]
    E = rng.uniform(50e9, 250e9, ne)
    prob = Problem(ELASTIC, coords, conn, E=E, nu=0.28, thickness=0.02, rho=2700.0,
                   plane_stress=True, plane_strain=False,
                   node_load_node=[27, 20, 27, 13, 6], node_load_dim=[2, 1, 2, 2, 1],
                   node_load_value=[-500.0, 40.0, -800.0, 75.0, 10.0],
                   element_loads=[ElementLoadSet(np.array([10, 11, 22]), 3e4, 2),
                                  ElementLoadSet(np.array([30, 31]), -1e4, 1)],
                   edge_load_nodes=[[27, 20], [13, 20]], edge_load_dim=[2, 1],
                   edge_load_value=[-300.0, 55.0],
                   node_bc_node=[0, 0, 7, 7, 14, 0], node_bc_dim=[1, 2, 1, 2, 1, 1],
                   node_bc_value=[0.0, 0.0, 1e-4, 0.0, 0.0, 2e-5],
                   element_bc_element=[2, 14], element_bc_dim=[2, 1],
                   element_bc_value=[3e-5, -1e-5],
                   edge_bc_nodes=[[21, 14]], edge_bc_dim=[2], edge_bc_value=[4e-5])
    return prob, [0, 12, 24, ne]


def case_quirks_magnetic():
    """Jittered 8x5 magnetostatic grid: two current regions of opposite sign sharing
    nodes, an edge load, repeated boundary conditions with different values."""
    rng = np.random.default_rng(3)
    nx, ny = 8, 5
    coords, conn = meshgen.rect_grid(nx, ny, 0.08, 0.05, jitter=0.3, rng=rng)
    ne = conn.shape[0]
    mu = np.where(np.arange(ne) % 7 == 0, 500.0, 1.0) * meshgen.MU0
    w = nx + 1
    boundary = [i for i in range(coords.shape[0]) if i % w in (0, nx) or i // w in (0, ny)]
    bv = np.zeros(len(boundary))
    bv[3] = 1e-6
    prob = Problem("magnetic", coords, conn, mu=mu,
                   element_loads=[ElementLoadSet(np.array([20, 21, 22, 23]), 2.5e3, 1),
                                  ElementLoadSet(np.array([23, 24, 37, 38]), -1.5e3, 1)],
                   edge_load_nodes=[[22, 23]], edge_load_dim=[1], edge_load_value=[7.0],
                   node_bc_node=boundary + [boundary[5]], node_bc_dim=[1] * (len(boundary) + 1),
                   node_bc_value=np.r_[bv, 3e-6])
    return prob, [0, 40, ne]


def case_tet_single():
    """scripts/Elasticity/beam3d_example_1.py:20-33: one tetrahedron (2,3,4), (6,3,2),
    (2,5,1), (4,3,6), E=210e9, nu=0.25, rho=7860, plane strain; the script stops at
    create_matrix, so three clamped vertices and a load on the fourth are added."""
    coords = [(2, 3, 4), (6, 3, 2), (2, 5, 1), (4, 3, 6)]
    prob = Problem(ELASTIC3D, coords, [[0, 1, 2, 3]], E=210e9, nu=0.25, rho=7860.0,
                   plane_strain=True, plane_stress=False,
                   node_load_node=[3, 3], node_load_dim=[3, 1], node_load_value=[-1000.0, 250.0],
                   node_bc_node=np.repeat([0, 1, 2], 3), node_bc_dim=np.tile([1, 2, 3], 3),
                   node_bc_value=np.zeros(9))
    return prob, [0, 1]


def case_tet_cantilever():
    """The solid cantilever of scripts/Elasticity/beam3d_example_2.py (x = 0 clamped,
    -1000 in dimension 3 on the x = 10, z = 2 edge, E=30e6, nu=0.25, rho=2.7, plane
    stress) on a jittered 5x2x2 Kuhn grid, in two groups."""
    p = meshgen.cantilever_3d(5, 2, 2, E=30e6, nu=0.25, rho=2.7, jitter=0.25, seed=5)
    return p, [0, 24, p.n_elements]


def case_tet_quirks():
    """Repeated node loads and conditions (the last value wins), edge loads and edge
    conditions, non-zero prescribed values and per-element E on a jittered 3x2x2 grid."""
    rng = np.random.default_rng(11)
    coords, conn = meshgen.box_tets(3, 2, 2, 1.5, 1.0, 1.0, jitter=0.2, rng=rng)
    ne = conn.shape[0]
    x = coords[:, 0]
    left = np.flatnonzero(x == 0.0)
    prob = Problem(ELASTIC3D, coords, conn, E=rng.uniform(50e9, 250e9, ne), nu=0.3, rho=2700.0,
                   plane_stress=True, plane_strain=False,
                   node_load_node=[35, 20, 35, 23, 11], node_load_dim=[3, 1, 3, 2, 1],
                   node_load_value=[-500.0, 40.0, -800.0, 75.0, 10.0],
                   edge_load_nodes=[[35, 31], [23, 19]], edge_load_dim=[3, 2],
                   edge_load_value=[-300.0, 55.0],
                   node_bc_node=np.r_[np.repeat(left, 3), left[0]],
                   node_bc_dim=np.r_[np.tile([1, 2, 3], left.size), 1],
                   node_bc_value=np.r_[np.zeros(3 * left.size), 2e-5],
                   edge_bc_nodes=[[3, 7]], edge_bc_dim=[2], edge_bc_value=[4e-5])
    return prob, [0, 30, ne]


def _grid_boundary(nx, ny):
    w = nx + 1
    left = [j * w for j in range(ny + 1)]
    right = [j * w + nx for j in range(ny + 1)]
    bottom = list(range(w))
    top = [ny * w + i for i in range(w)]
    return left, right, bottom, top


def case_mag_magnet():
    """A magnetostatic 10x6 grid with two magnets (magnetisation (8e5, 2e5) on a block
    of 12 triangles whose bottom edge from node 25 to node 26 is declared non-contour;
    (-3e5, 6e5) on 4 triangles), an element current load and A = 0 on the outer
    boundary."""
    nx, ny = 10, 6
    coords, conn = meshgen.rect_grid(nx, ny, 0.1, 0.06)
    ne = conn.shape[0]
    mu = np.where(np.arange(ne) % 5 == 0, 1000.0, 1.0) * meshgen.MU0
    left, right, bottom, top = _grid_boundary(nx, ny)
    boundary = sorted(set(left + right + bottom + top))
    block = [2 * (j * nx + i) + t for j in (2, 3) for i in (3, 4, 5) for t in (0, 1)]
    prob = Problem("magnetic", coords, conn, mu=mu,
                   element_loads=[ElementLoadSet(np.array([50, 51, 70]), 2e3, 1)],
                   node_bc_node=boundary, node_bc_dim=np.ones(len(boundary), np.int64),
                   node_bc_value=np.zeros(len(boundary)),
                   magnet_loads=[MagnetLoadSet(np.array(block), np.array([2 * 11 + 3, 2 * 11 + 4]), (8e5, 2e5)),
                                 MagnetLoadSet(np.array([2 * (4 * nx + 6), 2 * (4 * nx + 6) + 1,
                                                         2 * (2 * nx + 6), 2 * (2 * nx + 6) + 1]),
                                               np.array([], np.int64), (-3e5, 6e5))])
    return prob, [0, ne]


def case_mag_periodic():
    """A magnetostatic 8x5 grid with periodic (value 1) and anti-periodic (value -1)
    conditions between the interior nodes of its left and right edges, A = 0 on the
    bottom and top edges, a current load, and as many user NodeLoads as Dirichlet
    conditions -- the one arrangement in which the reference's continuity rows
    n + len(node_loads) + i land after the Dirichlet rows and spsolve accepts the
    system (analysis.py:186-189, :276)."""
    nx, ny = 8, 5
    rng = np.random.default_rng(21)
    coords, conn = meshgen.rect_grid(nx, ny, 0.08, 0.05, jitter=0.2, rng=rng)
    ne = conn.shape[0]
    left, right, bottom, top = _grid_boundary(nx, ny)
    bc = bottom + top
    inner_l, inner_r = left[1:-1], right[1:-1]
    interior = [j * (nx + 1) + i for j in range(1, ny) for i in range(1, nx)]
    nl_nodes = [interior[k % len(interior)] for k in range(len(bc))]
    prob = Problem("magnetic", coords, conn, mu=np.full(ne, meshgen.MU0),
                   element_loads=[ElementLoadSet(np.array([30, 31, 44, 45]), 5e2, 1)],
                   node_load_node=nl_nodes, node_load_dim=np.ones(len(bc), np.int64),
                   node_load_value=np.linspace(-1.0, 1.0, len(bc)),
                   node_bc_node=bc, node_bc_dim=np.ones(len(bc), np.int64), node_bc_value=np.zeros(len(bc)),
                   cont_node1=inner_l, cont_node2=inner_r,
                   cont_value=[1.0 if k % 2 == 0 else -1.0 for k in range(len(inner_l))])
    return prob, [0, ne]


def case_elastic_cont_mismatch():
    """Plane stress with one continuity condition and the usual few NodeLoads: the
    reference's continuity row n + len(node_loads) lands inside the DOF rows, the
    matrix and the right-hand side differ in size, and spsolve raises ValueError."""
    nx, ny = 4, 2
    coords, conn = meshgen.rect_grid(nx, ny, 2.0, 1.0)
    ne = conn.shape[0]
    left, right, _, _ = _grid_boundary(nx, ny)
    prob = Problem(ELASTIC, coords, conn, E=200e9, nu=0.3, thickness=0.01, rho=7800.0,
                   plane_stress=True, plane_strain=False,
                   node_load_node=[right[1]], node_load_dim=[2], node_load_value=[-100.0],
                   node_bc_node=np.repeat(left, 2), node_bc_dim=np.tile([1, 2], len(left)),
                   node_bc_value=np.zeros(2 * len(left)),
                   cont_node1=[right[0]], cont_node2=[right[2]], cont_value=[1.0])
    return prob, [0, ne]


def case_beam3d_msh(ref_root):
    """scripts/Elasticity/beam3d_example_2.py on the reference's own mesh file
    scripts/InputFiles/3D/beam3d_1.msh (Gmsh order kept): E=30e6, nu=0.25, rho=2.7,
    plane stress, -1000 in dimension 3 at the nodes with x = 10 and z = 2, the nodes
    with x = 0 clamped in dimensions 1, 2, 3."""
    from finite_elements_gb300 import gmsh
    m = gmsh.read_msh(os.path.join(ref_root, "scripts", "InputFiles", "3D", "beam3d_1.msh"))
    c, tets = m.coords, m.tetrahedra
    ne = tets.shape[0]
    tip = np.flatnonzero((c[:, 0] == 10) & (c[:, 2] == 2))
    x0 = np.flatnonzero(c[:, 0] == 0)
    prob = Problem(ELASTIC3D, c, tets, E=30e6, nu=0.25, rho=2.7, plane_strain=False, plane_stress=True,
                   node_load_node=tip, node_load_dim=np.full(tip.size, 3), node_load_value=np.full(tip.size, -1000.0),
                   node_bc_node=np.repeat(x0, 3), node_bc_dim=np.tile([1, 2, 3], x0.size),
                   node_bc_value=np.zeros(3 * x0.size))
    return prob, [int(v) for v in m.tet_group_ptr]


def case_beam2d_msh(ref_root):
    """scripts/Elasticity/beam2d_example_3.py on the reference's own mesh file
    scripts/InputFiles/2D/beam_2d_0.5.msh (Gmsh order kept): E=30e6, nu=0.25, t=1,
    rho=2.7, plane stress, -1000 in dimension 2 at node (10, 1), the nodes with x = 0
    clamped."""
    from finite_elements_gb300 import gmsh
    m = gmsh.read_msh(os.path.join(ref_root, "scripts", "InputFiles", "2D", "beam_2d_0.5.msh"))
    c = m.coords[:, :2]
    tip = np.flatnonzero((c[:, 0] == 10) & (c[:, 1] == 1))
    x0 = np.flatnonzero(c[:, 0] == 0)
    prob = Problem(ELASTIC, c, m.triangles, E=30e6, nu=0.25, thickness=1.0, rho=2.7, plane_strain=False,
                   plane_stress=True, node_load_node=tip, node_load_dim=[2], node_load_value=[-1000.0],
                   node_bc_node=np.repeat(x0, 2), node_bc_dim=np.tile([1, 2], x0.size),
                   node_bc_value=np.zeros(2 * x0.size))
    return prob, [int(v) for v in m.group_ptr]


def case_motor():
    """A motor-like annulus (scripts/Magnetic, the air-gap post-processing of
    results.py:82-243): an iron rotor ring with two magnets, the air gap in two radial
    layers, an iron stator ring carrying two opposite phase currents; A = 0 on the
    outer radius.  Groups "Rotor", "Gap ring", "Stator"."""
    nt = 48
    radii = [0.02, 0.028, 0.036, 0.0395, 0.04, 0.0405, 0.044, 0.052, 0.06]
    coords, conn = meshgen.annulus(radii, nt)
    ne = conn.shape[0]
    layer = np.repeat(np.arange(len(radii) - 1), 2 * nt)
    mu = np.where((layer <= 2) | (layer >= 5), 1000.0, 1.0) * meshgen.MU0
    rotor_mag = np.flatnonzero((layer == 2) & (np.arange(ne) % (2 * nt) < 12))
    rotor_mag2 = np.flatnonzero((layer == 2) & (np.arange(ne) % (2 * nt) >= 48) & (np.arange(ne) % (2 * nt) < 60))
    phase_a = np.flatnonzero((layer == 5) & (np.arange(ne) % (2 * nt) >= 6) & (np.arange(ne) % (2 * nt) < 18))
    phase_b = np.flatnonzero((layer == 5) & (np.arange(ne) % (2 * nt) >= 54) & (np.arange(ne) % (2 * nt) < 66))
    outer = np.arange((len(radii) - 1) * nt, len(radii) * nt)
    prob = Problem("magnetic", coords, conn, mu=mu,
                   element_loads=[ElementLoadSet(phase_a, 40.0, 1), ElementLoadSet(phase_b, -40.0, 1)],
                   magnet_loads=[MagnetLoadSet(rotor_mag, np.zeros(0, np.int64), (8e5, 3e5)),
                                 MagnetLoadSet(rotor_mag2, np.zeros(0, np.int64), (-8e5, -3e5))],
                   node_bc_node=outer, node_bc_dim=np.ones(nt, np.int64), node_bc_value=np.zeros(nt))
    groups = [0, 6 * nt, 10 * nt, ne]       # rotor: layers 0-2, gap: layers 3-4, stator: 5-7
    motor = {"gap": "Gap ring", "length": 0.1, "r_stator": 0.0405, "r_rotor": 0.0395,
             "maxwell_elements": [0, 17, 95, 150]}
    return prob, groups, ["Rotor", "Gap ring", "Stator"], motor


def cases(ref_root):
    yield "ex1_stress", case_ex1("stress")
    yield "ex1_strain", case_ex1("strain")
    yield "ex2_strain", case_ex2()
    yield "mag_beam", case_mag_beam()
    yield "quirks_elastic", case_quirks_elastic()
    yield "quirks_magnetic", case_quirks_magnetic()
    p = meshgen.cantilever_c1()
    yield "c1_cantilever", (p, [0, p.n_elements])
    p = meshgen.magnetostatic(40, 20, seed=1)
    yield "c2_magnetostatic_40x20", (p, [0, p.n_elements])
    p = meshgen.plane_strain_random(30, 15, seed=2)
    yield "c3_plane_strain_30x15", (p, [0, p.n_elements])
    yield "tet_single", case_tet_single()
    yield "tet_cantilever", case_tet_cantilever()
    yield "tet_quirks", case_tet_quirks()
    yield "mag_magnet", case_mag_magnet()
    yield "mag_periodic", case_mag_periodic()
    yield "elastic_cont_mismatch", case_elastic_cont_mismatch()
    yield "beam3d_msh", case_beam3d_msh(ref_root)
    yield "beam2d_msh", case_beam2d_msh(ref_root)
    yield "motor", case_motor()


def main():
    # the reference checkout: the first argument, $FE_REFERENCE_ROOT, or a directory
    # named "reference" beside this repository
    here = os.path.dirname(os.path.abspath(__file__))
    ref = (sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FE_REFERENCE_ROOT")
           or os.path.join(os.path.dirname(os.path.dirname(here)), "reference"))
    install_stubs()
    sys.path.insert(0, ref)
    import finite_elements.analysis      # noqa: F401  (the reference's own modules)
    import finite_elements.conditions    # noqa: F401
    import finite_elements.elements      # noqa: F401
    import finite_elements.loads         # noqa: F401
    import finite_elements.results       # noqa: F401
    fe = sys.modules["finite_elements"]
    only = set(sys.argv[2:])
    for name, case in cases(ref):
        if only and name not in only:
            continue
        prob, groups = case[0], case[1]
        names = case[2] if len(case) > 2 else None
        motor = case[3] if len(case) > 3 else None
        out = run_reference(fe, prob, groups, names, motor)
        arrays = problem_arrays(prob, groups)
        if names:
            arrays["group_names"] = np.array(names)
        if motor:
            arrays["motor"] = np.array([motor["length"], motor["r_stator"], motor["r_rotor"]])
            arrays["motor_maxwell_elements"] = np.array(motor["maxwell_elements"], np.int64)
        arrays.update({"ref_" + k: v for k, v in out.items()})
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(f"{name}: n_dof={prob.n_dof} nnz={out['K_data'].size} "
              f"n_bc={out['bc_dof'].size}")


if __name__ == "__main__":
    main()
