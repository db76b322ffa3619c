"""Gmsh 4.1 reader/writer and the VTK writer, on the CPU: a write/read round trip,
the reference's own beam meshes (scripts/InputFiles/2D, read where the reference
checkout is present) with the oracle's tip deflection converging to Euler-Bernoulli,
and the VTK file's sections."""
import glob
import os

import numpy as np
import pytest

from beam_cases import ANALYTIC_TIP, beam_problem
from finite_elements_gb300 import gmsh, meshgen

from conftest import reference_root

_REF = reference_root()
REF_MESHES = sorted(glob.glob(os.path.join(_REF, "scripts", "InputFiles", "2D", "beam_2d_*.msh"))
                    if _REF else [],
                    key=lambda f: -float(os.path.basename(f)[8:-4]))


def test_write_read_round_trip(tmp_path):
    coords, conn = meshgen.rect_grid(7, 3, 2.0, 1.0)
    f = tmp_path / "m.msh"
    gmsh.write_msh(f, coords, conn, node_tags=np.arange(11, 11 + coords.shape[0]))
    m = gmsh.read_msh(f)
    np.testing.assert_array_equal(m.coords[:, :2], coords)
    np.testing.assert_array_equal(m.triangles, conn)
    assert list(m.group_ptr) == [0, conn.shape[0]] and m.node_tags[0] == 11
    am = m.array_mesh()
    assert am.n_nodes == coords.shape[0] and am.n_elements == conn.shape[0]


def test_rejects_other_formats(tmp_path):
    f = tmp_path / "old.msh"
    f.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n")
    with pytest.raises(ValueError):
        gmsh.read_msh(f)


@pytest.mark.skipif(not REF_MESHES, reason="the reference checkout's scripts/InputFiles/2D/beam_2d_*.msh are "
                                           "not present (set FE_REFERENCE_ROOT)")
def test_reference_beam_meshes_and_euler_bernoulli():
    from oracle import fe_oracle as O
    errors = []
    for f in REF_MESHES:
        m = gmsh.read_msh(f)
        p = m.coords[m.triangles][:, :, :2]
        area = 0.5 * ((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1])
                      - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
        assert area.min() > 0 and abs(area.sum() - 10.0) <= 1e-12
        prob, tip = beam_problem(m.coords, m.triangles)
        x = np.array(O.solve(prob))
        errors.append(abs(x[2 * tip + 1] - ANALYTIC_TIP) / abs(ANALYTIC_TIP))
    assert all(b < a for a, b in zip(errors, errors[1:])), errors
    assert errors[-1] < 0.01


def test_vtk_file(tmp_path):
    from finite_elements_gb300.mesh import ArrayMesh
    from finite_elements_gb300.results import ElasticityResults2D
    coords, conn = meshgen.rect_grid(3, 2, 3.0, 1.0)
    n = coords.shape[0]
    u = np.column_stack([np.arange(n) * 1e-3, -np.arange(n) * 2e-3])
    res = ElasticityResults2D(ArrayMesh(coords, conn), list(u.reshape(-1)) + [0.0, 0.0], False, True)
    name = res.generate_vtk_file(str(tmp_path / "out"))
    assert name.endswith(".vtk")
    lines = open(name).read().splitlines()
    i = lines.index(f"POINTS {n} double")
    assert np.allclose([list(map(float, l.split())) for l in lines[i + 1:i + 1 + n]],
                       np.column_stack([coords, np.zeros(n)]))
    i = lines.index(f"CELLS {conn.shape[0]} {4 * conn.shape[0]}")
    assert [list(map(int, l.split())) for l in lines[i + 1:i + 1 + len(conn)]] == [[3, *c] for c in conn.tolist()]
    assert lines[lines.index(f"CELL_TYPES {len(conn)}") + 1] == "5"
    i = lines.index("SCALARS Displacement_Magnitude float 1")
    assert lines[i + 1] == "LOOKUP_TABLE default"
    np.testing.assert_allclose([float(v) for v in lines[i + 2:i + 2 + n]], np.hypot(u[:, 0], u[:, 1]))
    i = lines.index("VECTORS Displacement_Vectors float")
    np.testing.assert_allclose([list(map(float, l.split())) for l in lines[i + 1:i + 1 + n]],
                               np.column_stack([u, np.zeros(n)]))


def test_result_accessors_on_the_host():
    """Deformed nodes and per-element displacement vectors need no device work."""
    import numpy as np
    from finite_elements_gb300 import meshgen
    from finite_elements_gb300.mesh import ArrayMesh
    from finite_elements_gb300.results import ElasticityResults2D, ElasticityResults3D
    c, conn = meshgen.rect_grid(3, 2, 3.0, 2.0)
    u = np.arange(2 * len(c), dtype=float) * 1e-3
    r = ElasticityResults2D(ArrayMesh(c, conn), list(u) + [7.0], False, True)
    np.testing.assert_array_equal(r.deformed_nodes_m(2.0), c + 2.0 * u.reshape(-1, 2))
    np.testing.assert_array_equal(r.displacements_per_element[1], u.reshape(-1, 2)[conn[1]].reshape(-1))
    assert r.deformed_mesh.conn.shape == conn.shape
    c3, t3 = meshgen.box_tets(2, 1, 1, 2.0, 1.0, 1.0)
    u3 = np.linspace(0, 1, 3 * len(c3))
    r3 = ElasticityResults3D(ArrayMesh(c3, t3), list(u3), False, True)
    assert r3.displacements_per_element.shape == (t3.shape[0], 12)
    np.testing.assert_array_equal(r3.displacement_per_node_z(), u3[2::3])
    np.testing.assert_array_equal(r3.deformed_nodes, c3 + u3.reshape(-1, 3))


def test_per_item_results_index_like_the_reference_dicts():
    """Per-node and per-element results accept the mesh's node and element objects as
    keys, as the reference's dicts do, and integer rows, as arrays do."""
    import numpy as np
    from finite_elements_gb300 import elements as El, mesh as M
    from finite_elements_gb300.results import ElasticityResults2D
    pts = [M.Node2D(0, 0), M.Node2D(1, 0), M.Node2D(0, 1), M.Node2D(1, 1)]
    tris = [El.ElasticityTriangularElement2D(M.TriangularElement2D([pts[0], pts[1], pts[2]]), 1e9, 0.3, 1.0),
            El.ElasticityTriangularElement2D(M.TriangularElement2D([pts[3], pts[2], pts[1]]), 1e9, 0.3, 1.0)]
    mesh = M.Mesh([M.ElementsGroup(tris)])
    u = np.arange(8, dtype=float)
    r = ElasticityResults2D(mesh, list(u), False, True)
    d = r.displacement_vectors_per_node
    np.testing.assert_array_equal(d[M.Node2D(1, 1)], [6.0, 7.0])        # equal coordinates find the node
    np.testing.assert_array_equal(d[pts[1]], d[1])
    assert np.asarray(d).shape == (4, 2) and list(d.keys()) == mesh.nodes
    e = r.displacements_per_element
    np.testing.assert_array_equal(e[tris[1]], [6.0, 7.0, 4.0, 5.0, 2.0, 3.0])
    assert [k for k, _ in e.items()] == tris
