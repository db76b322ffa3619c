"""Modal analysis on the GPU (fe_modal) against the exact generalized eigenpairs of
K v = lambda M v (scipy eigsh, shift-invert for the smallest) on free beams.

Tolerances: elastic eigenvalues 1e-8 relative; the three rigid-body eigenvalues below
1e-6 of the first elastic one; eigenvectors of simple eigenvalues |cos| >= 1 - 1e-7
with the reference's; relative residuals ||K x - lambda M x|| / (||K x|| +
|lambda| ||M x||) <= 1e-9."""
import numpy as np
import pytest

from modal_cases import free_beam

pytestmark = pytest.mark.gpu


def check(vals, vecs, res, exact, exact_vecs, n_rigid):
    scale = exact[n_rigid]
    assert np.abs(vals[:n_rigid]).max() <= 1e-6 * scale, vals[:n_rigid]
    np.testing.assert_allclose(vals[n_rigid:], exact[n_rigid:], rtol=1e-8)
    assert res.max() <= 1e-9, res
    for i in range(n_rigid, len(vals)):
        gap = min(abs(exact[i] - exact[j]) for j in range(len(exact)) if j != i)
        if gap > 1e-6 * exact[i]:
            assert abs(vecs[i] @ exact_vecs[i]) >= 1 - 1e-7, (i, abs(vecs[i] @ exact_vecs[i]))


@pytest.mark.parametrize("nx,ny", [(20, 4), (80, 8)])
@pytest.mark.parametrize("precision", ["fp64", "mixed-cg64"])
def test_smallest_modes_match_exact(gpu_lib, nx, ny, precision):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob = free_beam(nx, ny)
    s = GpuSystem(prob)
    vals, vecs, res = s.modal(20, which="smallest", precision=precision)
    exact, exact_vecs = O.generalized_eigenpairs(prob, 20)
    check(vals, vecs, res, exact, exact_vecs, 3)
    s.close()


def test_largest_modes_match_exact(gpu_lib):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob = free_beam(20, 4)
    s = GpuSystem(prob)
    vals, vecs, res = s.modal(6, which="largest", steps=prob.n_dof)
    exact, exact_vecs = O.generalized_eigenpairs(prob, 6, which="largest")
    np.testing.assert_allclose(vals, exact, rtol=1e-8)
    assert res.max() <= 1e-9
    s.close()


def test_drop_in_modal_analysis_and_static_solve_afterwards(gpu_lib):
    """modal_analysis through the drop-in, then a static solve on the same analysis
    (the static system is rebuilt after the modal solve)."""
    import golden_cases as gc
    from test_abi_host import build_objects
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    prob, ref, mesh, kw = build_objects("c1_cantilever")
    fea = FiniteElementAnalysis(mesh=mesh, **kw)
    with pytest.raises(ValueError):
        fea.modal_analysis("middle", 4)
    vals, vecs = fea.modal_analysis("smallest", 8)
    assert vals.shape == (8,) and vecs.shape == (8, prob.n_dof) and np.all(np.diff(vals) >= 0)
    res = fea.solve()
    x = np.array(res.result_vector)
    assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])
