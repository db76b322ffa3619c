"""Linear-tetrahedron elasticity (elements.py:663-876) on the GPU against the oracle:
solves in every precision, per-element post-processing, modal analysis, meshes read
from Gmsh files, and the calls the reference does not define for tetrahedra.

Tolerances: FP64 and mixed-cg64 solutions ||x - x_ref|| <= 1e-10 ||x_ref||; the
mixed path to relative residual 1e-9, ||u - u_ref|| <= 1e-7 ||u_ref||; strain, stress
max |difference| <= 1e-12 max |oracle|, energy per element within 64 eps of the
sum of the magnitudes of its terms; elastic eigenvalues 1e-8
relative, the six rigid-body eigenvalues below 1e-6 of the first elastic one."""
import numpy as np
import pytest

from modal_cases import free_beam_3d

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def cantilever(gpu_lib):
    from finite_elements_gb300 import meshgen
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob = meshgen.cantilever_3d(12, 3, 3, jitter=0.2, seed=4)
    ref = np.array(O.solve(prob))
    s = GpuSystem(prob)
    yield s, prob, ref
    s.close()


@pytest.mark.parametrize("precision,cheb", [("fp64", 0), ("fp64", 8), ("mixed-cg64", 0), ("mixed-cg64", 32)])
def test_solve_matches_oracle(cantilever, precision, cheb):
    s, prob, ref = cantilever
    x, st = s.solve(precision=precision, tol=1e-13, cheb_degree=cheb, accept_stagnation=True)
    assert st.status == 0, st.as_dict()
    assert np.linalg.norm(x - ref) <= 1e-10 * np.linalg.norm(ref), st.as_dict()


@pytest.mark.parametrize("cheb", [0, 3])
def test_mixed_solve_matches_oracle(cantilever, cheb):
    s, prob, ref = cantilever
    n = prob.n_dof
    x, st = s.solve(precision="mixed", tol=1e-9, cheb_degree=cheb)
    assert st.status == 0 and st.relres <= 1e-9, st.as_dict()
    assert np.linalg.norm(x[:n] - ref[:n]) <= 1e-7 * np.linalg.norm(ref[:n])


def test_matrices_match_oracle(cantilever):
    from oracle import fe_oracle as O
    s, prob, _ = cantilever
    K = s.create_matrix()
    R = O.create_matrix(prob)
    np.testing.assert_array_equal(K.indptr, R.indptr)
    np.testing.assert_array_equal(K.indices, R.indices)
    assert relmax(K.data, R.data) <= 1e-13
    assert relmax(s.element_matrices("K"), O.tet_stiffness(prob)) <= 1e-13
    assert relmax(s.element_matrices("M"), O.tet_mass(prob)) <= 1e-15
    ms, mr = s.m_matrix_sparse(), O.m_matrix_sparse(prob)
    np.testing.assert_array_equal(ms.indices, mr.indices)
    assert relmax(ms.data, mr.data) <= 1e-15


def test_post_matches_oracle(cantilever):
    from oracle import fe_oracle as O
    s, prob, ref = cantilever
    out = s.post(ref)
    strain, stress, energy = O.elastic_post(prob, ref)
    assert out["strain"].shape == (prob.n_elements, 6)
    assert relmax(out["strain"], strain) <= 1e-12
    assert relmax(out["stress"], stress) <= 1e-12
    # energy: a sum of q_i Ke_ij q_j terms that cancel (Ke annihilates rigid motions),
    # bounded per element by the rounding of the sum of their magnitudes
    q = ref[: prob.n_dof].reshape(-1, 3)[prob.conn].reshape(-1, 12)
    ke = O.tet_stiffness(prob).reshape(-1, 12, 12)
    mag = 0.5 * np.einsum("ei,eij,ej->e", np.abs(q), np.abs(ke), np.abs(q))
    assert (np.abs(out["energy"] - energy) <= 64 * np.finfo(float).eps * mag).all()
    # the work of the loads equals twice the strain energy: F.u = sum q^T Ke q
    F = s.create_source_matrix()[: prob.n_dof, 0]
    u = ref[: prob.n_dof]
    assert abs(2 * out["energy"].sum() - F @ u) <= 1e-9 * abs(F @ u)


def test_results_3d_and_vtk(cantilever, tmp_path):
    from finite_elements_gb300.mesh import ArrayMesh
    from finite_elements_gb300.results import ElasticityResults3D
    s, prob, ref = cantilever
    mesh = ArrayMesh(prob.coords, prob.conn)
    res = ElasticityResults3D(mesh, list(ref), False, True, system=s)
    u = res.displacement_vectors_per_node
    assert u.shape == (prob.n_nodes, 3)
    np.testing.assert_array_equal(res.displacement_per_node_z(), ref[2: prob.n_dof: 3])
    assert res.shear_strain_zx().shape == (prob.n_elements,)
    path = res.generate_vtk_file(str(tmp_path / "beam3d"))
    text = open(path).read()
    assert f"CELLS {prob.n_elements} {5 * prob.n_elements}" in text
    assert text.count("\n10\n") >= 1 and "VECTORS Displacement_Vectors float" in text


@pytest.mark.parametrize("precision", ["fp64", "mixed-cg64"])
def test_smallest_modes_match_exact(gpu_lib, precision):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob = free_beam_3d(10, 2, 2)
    s = GpuSystem(prob)
    vals, vecs, res = s.modal(12, which="smallest", precision=precision)
    exact, _ = O.generalized_eigenpairs(prob, 12)
    assert np.abs(vals[:6]).max() <= 1e-6 * exact[6], vals[:6]
    np.testing.assert_allclose(vals[6:], exact[6:], rtol=1e-8)
    assert res.max() <= 1e-9, res
    s.close()


def test_gmsh_tetrahedra_round_trip_and_solve(gpu_lib, tmp_path):
    """A tetrahedron mesh written as Gmsh 4.1 and read back gives the same analysis."""
    from finite_elements_gb300 import gmsh, meshgen
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    from oracle import fe_oracle as O
    prob = meshgen.cantilever_3d(8, 2, 2, jitter=0.2, seed=9)
    path = tmp_path / "beam3d.msh"
    gmsh.write_msh(path, prob.coords, prob.conn)
    mesh = gmsh.read_msh(path).array_mesh()
    np.testing.assert_array_equal(mesh.conn, prob.conn)
    prob.coords = mesh.coords
    fea = FiniteElementAnalysis.from_problem(prob, mesh=mesh)
    x = np.array(fea.solve().result_vector)
    ref = np.array(O.solve(prob))
    assert np.linalg.norm(x - ref) <= 1e-10 * np.linalg.norm(ref)


def test_element_loads_and_factors_are_refused_on_tetrahedra(gpu_lib):
    from finite_elements_gb300 import _lib, meshgen
    prob = meshgen.cantilever_3d(2, 1, 1)
    lib = _lib.load()
    h = _lib.Handle(_lib.FE_KIND_ELASTIC_TET, prob.coords, prob.conn)
    ptr_ = np.array([0, 1], np.int64)
    el = np.array([0], np.int64)
    val = np.array([1.0])
    dims = np.array([1], np.int32)
    assert lib.fe_set_element_loads(h.h, 1, _lib.ptr(ptr_), _lib.ptr(el), _lib.ptr(val), _lib.ptr(dims),
                                    0) == _lib.FE_BAD_INPUT
    out = np.zeros(3)
    assert lib.fe_element_node_factors(h.h, 1, _lib.ptr(el), _lib.ptr(out)) == _lib.FE_BAD_INPUT
    h.close()


def test_larger_cantilever_precisions_agree(gpu_lib):
    """133k DOF: FP64 PCG and mixed-cg64 reach 1e-10 and agree to 1e-8; the FP64
    residual of both, recomputed on the host from the exported K, is at 1e-10."""
    from finite_elements_gb300 import meshgen
    from finite_elements_gb300.engine import GpuSystem
    prob = meshgen.cantilever_3d(100, 20, 20)
    s = GpuSystem(prob)
    x64, st64 = s.solve(precision="fp64", tol=1e-10, cheb_degree=16)
    xmp, stmp = s.solve(precision="mixed-cg64", tol=1e-10, cheb_degree=32)
    assert st64.status == 0 and stmp.status == 0, (st64.as_dict(), stmp.as_dict())
    n = prob.n_dof
    assert np.linalg.norm(xmp[:n] - x64[:n]) <= 1e-8 * np.linalg.norm(x64[:n])
    K = s.k_matrix_sparse().tocsr()
    F = s.create_source_matrix()[:n, 0]
    free = np.ones(n, bool)
    free[s.bc_dof] = False
    for x in (x64, xmp):
        r = (F - K @ x[:n])[free]
        assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(F[free])
    s.close()


def test_largest_modes_and_drop_in_modal_analysis(gpu_lib):
    """'largest' on the tetrahedral beam, and modal_analysis through the drop-in
    objects (scripts/ModalAnalysis/beam3d_1.py: order='smallest')."""
    from finite_elements_gb300 import elements as El, mesh as M
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob = free_beam_3d(6, 2, 2)
    s = GpuSystem(prob)
    vals, _, res = s.modal(4, which="largest", steps=prob.n_dof)
    exact, _ = O.generalized_eigenpairs(prob, 4, which="largest")
    np.testing.assert_allclose(vals, exact, rtol=1e-8)
    assert res.max() <= 1e-9
    s.close()
    nodes = [M.Node3D(*c) for c in prob.coords.tolist()]
    elems = [El.ElasticityTetrahedralElement3D(M.TetrahedralElement([nodes[i] for i in row]), 210e9, 0.25, 7860.0)
             for row in prob.conn.tolist()]
    mesh = M.Mesh([M.ElementsGroup(elems)])
    fea = FiniteElementAnalysis(mesh, [], [], [], [], [], [], [], [], plane_strain=False, plane_stress=True)
    vals, vecs = fea.modal_analysis(order="smallest", k=10)
    exact, _ = O.generalized_eigenpairs(prob, 10)
    assert vecs.shape == (10, prob.n_dof)
    np.testing.assert_allclose(vals[6:], exact[6:], rtol=1e-8)
