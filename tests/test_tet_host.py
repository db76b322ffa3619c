"""Host-side checks of the tetrahedron path (no GPU): the oracle's element against
the exact properties of linear elasticity, the Gmsh reader on tetrahedron meshes,
the VTK writer, and the refusals the reference's classes imply."""
import os

import numpy as np
import pytest

from finite_elements_gb300 import gmsh, meshgen
from finite_elements_gb300.problem import ELASTIC3D, ElementLoadSet, Problem
from oracle import fe_oracle as O

from conftest import reference_root

_REF = reference_root()
REF_3D = os.path.join(_REF, "scripts", "InputFiles", "3D") if _REF else ""


def test_box_tets_fill_the_box_and_conform():
    c, conn = meshgen.box_tets(3, 2, 2, 1.5, 1.0, 1.0, jitter=0.2, rng=np.random.default_rng(0))
    assert conn.shape == (72, 4)
    assert abs(O.tet_volume(c[conn]).sum() - 1.5) <= 1e-13
    # every interior face is shared by exactly two tetrahedra, boundary faces by one
    faces = np.sort(conn[:, [[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]]].reshape(-1, 3), axis=1)
    _, counts = np.unique(faces, axis=0, return_counts=True)
    assert set(counts.tolist()) <= {1, 2}
    assert (counts == 1).sum() == 2 * (3 * 2 * 2 + 3 * 2 * 2 + 2 * 2 * 2)   # 2 triangles per boundary cell face


def test_tet_stiffness_properties():
    prob = meshgen.cantilever_3d(3, 2, 2, jitter=0.25, seed=1)
    ke = O.tet_stiffness(prob).reshape(-1, 12, 12)
    p = O.element_points(prob)
    scale = np.abs(ke).max(axis=(1, 2))
    assert (np.abs(ke - ke.transpose(0, 2, 1)).max(axis=(1, 2)) <= 1e-14 * scale).all()
    # the six rigid-body modes are in the null space of every element
    for e in range(ke.shape[0]):
        x, y, z = p[e, :, 0], p[e, :, 1], p[e, :, 2]
        o, one = np.zeros(4), np.ones(4)
        modes = [np.stack(m, 1).reshape(-1) for m in
                 ((one, o, o), (o, one, o), (o, o, one), (-y, x, o), (o, -z, y), (z, o, -x))]
        for m in modes:
            assert np.abs(ke[e] @ m).max() <= 1e-12 * scale[e] * np.abs(m).max()
    # a uniform strain state: energy V/2 eps^T D eps
    eps = np.array([1e-3, -2e-4, 5e-4, 3e-4, -1e-4, 2e-4])
    E, nu = prob.E[0], prob.nu[0]
    D = O.d_matrix_3d(np.array([E]), np.array([nu]), False, True)[0]
    gx = np.array([[eps[0], eps[3] / 2, eps[5] / 2], [eps[3] / 2, eps[1], eps[4] / 2],
                   [eps[5] / 2, eps[4] / 2, eps[2]]])
    u = (p[0] @ gx.T).reshape(-1)
    V = O.tet_volume(p[:1])[0]
    assert abs(0.5 * u @ ke[0] @ u - 0.5 * V * eps @ D @ eps) <= 1e-12 * abs(0.5 * V * eps @ D @ eps)


def test_tet_mass_total_and_pattern():
    prob = meshgen.cantilever_3d(3, 2, 2)
    M = O.m_matrix_sparse(prob)
    total = np.asarray(M.sum(axis=1)).reshape(-1, 3)[:, 0].sum()
    assert abs(total - 7860.0 * 10 * 2 * 2) <= 1e-9 * total


def test_gmsh_tetrahedra_write_read(tmp_path):
    c, conn = meshgen.box_tets(2, 2, 1, 1.0, 1.0, 0.5)
    path = tmp_path / "box.msh"
    gmsh.write_msh(path, c, conn)
    m = gmsh.read_msh(path)
    np.testing.assert_array_equal(m.tetrahedra, conn)
    np.testing.assert_array_equal(m.coords, c)
    am = m.array_mesh()
    assert am.coords.shape == c.shape and am.conn.shape == conn.shape


@pytest.mark.skipif(not os.path.isdir(REF_3D),
                    reason="the reference checkout's scripts/InputFiles/3D is not present (set FE_REFERENCE_ROOT)")
@pytest.mark.parametrize("name,n_nodes,n_tets", [("beam3d_0.5", 46, 104), ("beam3d_1", 110, 253),
                                                 ("cube", 721, 2576)])
def test_gmsh_reads_the_reference_3d_inputs(name, n_nodes, n_tets):
    m = gmsh.read_msh(os.path.join(REF_3D, name + ".msh"))
    assert m.coords.shape == (n_nodes, 3) and m.tetrahedra.shape == (n_tets, 4)
    vol = O.tet_volume(m.coords[m.tetrahedra])
    assert (vol > 0).all()


def test_element_loads_on_tetrahedra_raise_like_the_reference():
    from finite_elements_gb300.engine import GpuSystem
    prob = meshgen.cantilever_3d(2, 1, 1)
    prob.element_loads = [ElementLoadSet(np.array([0]), 1.0, 1)]
    with pytest.raises(AttributeError):
        GpuSystem(prob)
    with pytest.raises(AttributeError):
        O.node_loads(prob)


def test_problem_shapes():
    prob = Problem(ELASTIC3D, np.zeros((4, 3)), [[0, 1, 2, 3]], E=1.0, nu=0.3, rho=1.0,
                   plane_strain=True, plane_stress=False)
    assert prob.dim == 3 and prob.npe == 4 and prob.n_dof == 12 and prob.elastic


def test_annulus_mesh():
    import math
    c, conn = meshgen.annulus([0.5, 0.75, 1.0], 24)
    assert conn.shape == (2 * 2 * 24, 3)
    p = c[conn]
    det = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    area = np.abs(det).sum() / 2
    # the polygonal annulus: 24 sectors of (R^2 - r^2) sin(2 pi / 24) / 2
    assert abs(area - 24 * (1.0 - 0.25) * math.sin(2 * math.pi / 24) / 2) <= 1e-12
    edges = np.sort(conn[:, [[0, 1], [1, 2], [0, 2]]].reshape(-1, 2), axis=1)
    _, counts = np.unique(edges, axis=0, return_counts=True)
    assert set(counts.tolist()) <= {1, 2} and (counts == 1).sum() == 2 * 24   # inner and outer circles


def test_dirichlet_count_matches_the_oracle():
    import golden_cases as gc
    from finite_elements_gb300.engine import dirichlet_count
    for name in gc.names():
        prob, _, ref = gc.load(name)
        assert dirichlet_count(prob) == ref["bc_dof"].size, name
