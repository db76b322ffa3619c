"""Host-side checks that need no GPU: the C ABI library loads and exports every
function include/fe_gb300.h declares; the Python bindings match; the flattening of
the drop-in object API reproduces the golden problem arrays."""
import os
import re
import subprocess

import numpy as np
import pytest

import golden_cases as gc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fe_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(fe_\w+)\s*\(", text, re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("fe_mesh_create", "fe_set_elastic_materials", "fe_set_mu", "fe_set_node_loads",
                 "fe_set_element_loads", "fe_set_dirichlet", "fe_assemble", "fe_export_csr",
                 "fe_export_rhs", "fe_solve", "fe_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from finite_elements_gb300 import _lib
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (fe_\w+)", out))
    assert set(declared_functions()) <= exported
    # the ctypes table covers the header
    assert set(declared_functions()) == set(_lib.exported_symbols())


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of fe_solve_opts and fe_solve_stats have the header's size
    and field offsets (a C probe compiled against include/fe_gb300.h)."""
    import ctypes
    import shutil
    from finite_elements_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = []
    for tag, cls in (("fe_solve_opts", _lib.SolveOpts), ("fe_solve_stats", _lib.SolveStats)):
        lines.append(f'printf("{tag} size %zu\\n", sizeof({tag}));')
        for name, _ in cls._fields_:
            lines.append(f'printf("{tag} {name} %zu\\n", offsetof({tag}, {name}));')
    src = tmp_path / "probe.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"fe_gb300.h\"\nint main(void) {\n"
                   + "\n".join(lines) + "\nreturn 0;\n}\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for tag, cls in (("fe_solve_opts", _lib.SolveOpts), ("fe_solve_stats", _lib.SolveStats)):
        assert int(got[f"{tag} size"]) == ctypes.sizeof(cls), tag
        for name, _ in cls._fields_:
            assert int(got[f"{tag} {name}"]) == getattr(cls, name).offset, (tag, name)


def test_bindings_accept_the_engine_argument_types():
    """ctypes converts arguments before the library runs: calls with the argument kinds
    the engine passes (numpy arrays through _lib.ptr) on a null handle must reach the
    library and come back with FE_BAD_INPUT, not fail in the conversion."""
    import ctypes
    from finite_elements_gb300 import _lib
    lib = _lib.load()
    a = np.zeros(8)
    assert lib.fe_modal(None, 0, 1, 0.0, 0, 0, _lib.ptr(a), _lib.ptr(a), _lib.ptr(a)) == _lib.FE_BAD_INPUT
    ne, c16 = ctypes.c_int64(), ctypes.c_int32()
    assert lib.fe_sell_info(None, ne, c16) == _lib.FE_BAD_INPUT
    cm, cn = ctypes.c_double(), ctypes.c_int64()
    assert lib.fe_profile_read(None, 2, ctypes.byref(cm), ctypes.byref(cn), ctypes.byref(cm),
                               ctypes.byref(cn)) == _lib.FE_BAD_INPUT


def test_library_calls_without_gpu_fail_loudly():
    """No CPU fallback: on a machine without a CUDA device the first call fails with
    a CUDA status."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from finite_elements_gb300 import _lib
    prob, _, _ = gc.load("ex1_stress")
    with pytest.raises(_lib.FeError) as e:
        _lib.Handle(_lib.FE_KIND_ELASTIC_TRI, prob.coords, prob.conn)
    assert e.value.status == _lib.FE_CUDA_ERR


def test_status_strings():
    from finite_elements_gb300 import _lib
    lib = _lib.load()
    assert lib.fe_status_string(_lib.FE_MAXITER) == b"FE_MAXITER"
    assert lib.fe_version() >= 1


def build_objects(name):
    """The golden case as drop-in objects (same construction as make_golden.py)."""
    from finite_elements_gb300 import conditions as C, elements as El, loads as L, mesh as M
    prob, groups, ref = gc.load(name)
    if prob.kind == "elastic3d":
        nodes = [M.Node3D(*c) for c in prob.coords.tolist()]
        tets = [M.TetrahedralElement([nodes[i] for i in row]) for row in prob.conn.tolist()]
        elems = [El.ElasticityTetrahedralElement3D(t, prob.E[k], prob.nu[k], prob.rho[k])
                 for k, t in enumerate(tets)]
    else:
        nodes = [M.Node2D(x, y) for x, y in prob.coords.tolist()]
        tris = [M.TriangularElement2D([nodes[i] for i in row]) for row in prob.conn.tolist()]
        if prob.kind == "elastic":
            elems = [El.ElasticityTriangularElement2D(t, prob.E[k], prob.nu[k], prob.rho[k], prob.thickness[k])
                     for k, t in enumerate(tris)]
        else:
            elems = [El.MagneticElement2D(t, prob.mu[k]) for k, t in enumerate(tris)]
    names = ref.get("_group_names")
    mesh = M.Mesh([M.ElementsGroup(elems[a:b], str(names[g]) if names is not None else "")
                   for g, (a, b) in enumerate(zip(groups[:-1], groups[1:]))])
    mesh.nodes = nodes
    mesh.node_to_index = {p: i for i, p in enumerate(nodes)}
    kw = dict(
        node_loads=[L.NodeLoad(nodes[n], v, d) for n, d, v in
                    zip(prob.node_load_node, prob.node_load_dim, prob.node_load_value)],
        element_loads=[L.ElementsLoad([elems[k] for k in s.elements], s.value, s.dimension)
                       for s in prob.element_loads],
        edge_loads=[L.EdgeLoad(M.LineSegment2D(nodes[a], nodes[b]), v, d) for (a, b), d, v in
                    zip(prob.edge_load_nodes.tolist(), prob.edge_load_dim, prob.edge_load_value)],
        node_boundary_conditions=[C.NodeBoundaryCondition(nodes[n], v, d) for n, d, v in
                                  zip(prob.node_bc_node, prob.node_bc_dim, prob.node_bc_value)],
        element_boundary_conditions=[C.ElementBoundaryCondition(elems[k], v, d) for k, d, v in
                                     zip(prob.element_bc_element, prob.element_bc_dim,
                                         prob.element_bc_value)],
        edge_boundary_conditions=[C.EdgeBoundaryCondition(M.LineSegment2D(nodes[a], nodes[b]), v, d)
                                  for (a, b), d, v in zip(prob.edge_bc_nodes.tolist(), prob.edge_bc_dim,
                                                          prob.edge_bc_value)])
    kw["magnet_loads"] = [L.MagnetLoad([elems[k] for k in m.elements.tolist()],
                                       [nodes[k] for k in m.non_contour_nodes.tolist()],
                                       M.Vector2D(*m.magnetization)) for m in prob.magnet_loads]
    kw["continuity_conditions"] = [C.ContinuityCondition(nodes[a], nodes[b], v) for a, b, v in
                                   zip(prob.cont_node1.tolist(), prob.cont_node2.tolist(),
                                       prob.cont_value.tolist())]
    if prob.elastic:
        kw.update(plane_strain=prob.plane_strain, plane_stress=prob.plane_stress)
    return prob, ref, mesh, kw


@pytest.mark.parametrize("name", gc.names())
def test_object_api_flattens_to_the_golden_problem(name):
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    prob, ref, mesh, kw = build_objects(name)
    fea = FiniteElementAnalysis(mesh=mesh, **kw)
    p = fea.problem()
    np.testing.assert_array_equal(p.coords, prob.coords)
    np.testing.assert_array_equal(p.conn, prob.conn)
    for f in ("node_load_node", "node_load_dim", "node_load_value", "node_bc_node", "node_bc_dim",
              "node_bc_value", "element_bc_element", "edge_bc_nodes", "edge_load_nodes"):
        np.testing.assert_array_equal(getattr(p, f), getattr(prob, f))
    assert len(p.element_loads) == len(prob.element_loads)
    for a, b in zip(p.element_loads, prob.element_loads):
        np.testing.assert_array_equal(a.elements, b.elements)
        assert a.value == b.value and a.dimension == b.dimension


def test_magnet_and_continuity_flatten_to_the_golden_problem():
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    for name in ("mag_magnet", "mag_periodic"):
        prob, ref, mesh, kw = build_objects(name)
        p = FiniteElementAnalysis(mesh=mesh, **kw).problem()
        for f in ("cont_node1", "cont_node2", "cont_value"):
            np.testing.assert_array_equal(getattr(p, f), getattr(prob, f))
        assert len(p.magnet_loads) == len(prob.magnet_loads)
        for a, b in zip(p.magnet_loads, prob.magnet_loads):
            np.testing.assert_array_equal(a.elements, b.elements)
            np.testing.assert_array_equal(a.non_contour_nodes, b.non_contour_nodes)
            assert a.magnetization == b.magnetization


def test_continuity_size_mismatch_raises_like_spsolve():
    """Where the reference's continuity rows make create_matrix and
    create_source_matrix disagree in size, solve() raises scipy's ValueError before
    any device work."""
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    prob, ref, mesh, kw = build_objects("elastic_cont_mismatch")
    with pytest.raises(ValueError) as e:
        FiniteElementAnalysis(mesh=mesh, **kw).solve()
    assert str(e.value) == str(ref["solve_error"])


def test_plane_flag_errors_match_reference():
    from finite_elements_gb300.engine import check_plane_flags
    with pytest.raises(ValueError, match="just one of plane_strain or plane_stress can be True"):
        check_plane_flags(True, True)
    with pytest.raises(ValueError, match="one of plane_strain or plane_stress must be True"):
        check_plane_flags(False, None)


def test_create_source_matrix_before_create_matrix_is_a_type_error():
    """The reference sizes F from state only create_matrix sets (analysis.py:737-739)."""
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    prob, ref, mesh, kw = build_objects("ex1_stress")
    with pytest.raises(TypeError):
        FiniteElementAnalysis(mesh=mesh, **kw).create_source_matrix()
