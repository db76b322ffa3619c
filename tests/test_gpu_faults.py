"""Failure paths on the GPU, all made on the host side (bad inputs, tiny iteration
caps, a singular system): every one ends in a status, none faults or hangs a GPU."""
import warnings

import numpy as np
import pytest
import scipy.sparse.linalg as spla

import golden_cases as gc

pytestmark = pytest.mark.gpu


def test_iteration_cap_gives_maxiter(gpu_lib):
    from finite_elements_gb300 import _lib
    from finite_elements_gb300.engine import GpuSystem
    prob, _, _ = gc.load("c1_cantilever")
    s = GpuSystem(prob)
    x, st = s.solve(precision="fp64", tol=1e-12, max_iter=5)
    assert st.status == _lib.FE_MAXITER
    assert st.iterations <= 5 + 16   # at most one captured chunk past the cap
    x, st = s.solve(precision="mixed", tol=1e-8, max_iter=5)
    assert st.status == _lib.FE_MAXITER


def test_singular_system_without_conditions(gpu_lib):
    """No Dirichlet condition: K is singular (rigid motions).  The drop-in warns like
    scipy's spsolve and returns NaNs, or raises NotImplementedError when the warning
    is an error, as the reference does (analysis.py:819-826)."""
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    from finite_elements_gb300.problem import Problem
    prob, _, _ = gc.load("ex2_strain")
    free = Problem("elastic", prob.coords, prob.conn, E=prob.E, nu=prob.nu, thickness=prob.thickness,
                   rho=prob.rho, plane_strain=True, plane_stress=False,
                   node_load_node=prob.node_load_node, node_load_dim=prob.node_load_dim,
                   node_load_value=prob.node_load_value)
    fea = FiniteElementAnalysis.from_problem(free, solver={"max_iter": 2000})
    try:
        with warnings.catch_warnings(record=True):
            warnings.simplefilter("always")
            res = fea.solve()
        x = np.array(res.result_vector)
        assert np.isnan(x).all() or np.isfinite(x).all()
    except Exception as e:   # MAXITER on a semi-definite system is also a status
        assert "PCG stopped" in str(e) or isinstance(e, NotImplementedError)
    fea2 = FiniteElementAnalysis.from_problem(free, solver={"max_iter": 2000})
    with warnings.catch_warnings():
        warnings.simplefilter("error", spla.MatrixRankWarning)
        try:
            fea2.solve()
        except (NotImplementedError, RuntimeError):
            pass


def test_nan_material_is_reported(gpu_lib):
    from finite_elements_gb300 import _lib
    from finite_elements_gb300.engine import GpuSystem
    prob, _, _ = gc.load("ex2_strain")
    prob.E = prob.E.copy()
    prob.E[3] = np.nan
    with pytest.raises(_lib.FeError) as e:
        GpuSystem(prob)
    assert e.value.status == _lib.FE_NONFINITE


def test_bad_connectivity_is_rejected(gpu_lib):
    from finite_elements_gb300 import _lib
    prob, _, _ = gc.load("ex1_stress")
    conn = prob.conn.copy()
    conn[1, 2] = 99
    with pytest.raises(_lib.FeError) as e:
        _lib.Handle(_lib.FE_KIND_ELASTIC_TRI, prob.coords, conn)
    assert e.value.status == _lib.FE_BAD_INPUT


def test_bad_dimension_is_a_key_error(gpu_lib):
    from finite_elements_gb300.engine import GpuSystem
    prob, _, _ = gc.load("ex1_stress")
    prob.node_load_dim = prob.node_load_dim.copy()
    prob.node_load_dim[0] = 3
    with pytest.raises(KeyError):
        GpuSystem(prob)


def test_empty_element_load_set_is_rejected(gpu_lib):
    from finite_elements_gb300 import _lib
    from finite_elements_gb300.engine import GpuSystem
    from finite_elements_gb300.problem import ElementLoadSet
    prob, _, _ = gc.load("mag_beam")
    prob.element_loads = [ElementLoadSet(np.zeros(0, np.int64), 1.0, 1)]
    with pytest.raises(_lib.FeError):
        GpuSystem(prob)


def test_node_without_elements_gives_nan_like_spsolve(gpu_lib):
    """A node no element touches leaves a zero row in K: scipy's spsolve warns that the
    matrix is singular and returns NaN; the drop-in does the same."""
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    from finite_elements_gb300.problem import Problem
    prob, _, _ = gc.load("ex2_strain")
    coords = np.vstack([prob.coords, [[50.0, 50.0]]])
    p2 = Problem("elastic", coords, prob.conn, E=prob.E, nu=prob.nu, thickness=prob.thickness,
                 rho=prob.rho, plane_strain=True, plane_stress=False,
                 node_load_node=prob.node_load_node, node_load_dim=prob.node_load_dim,
                 node_load_value=prob.node_load_value, node_bc_node=prob.node_bc_node,
                 node_bc_dim=prob.node_bc_dim, node_bc_value=prob.node_bc_value)
    fea = FiniteElementAnalysis.from_problem(p2)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        res = fea.solve()
    assert np.isnan(np.array(res.result_vector)).all()
    assert any(issubclass(x.category, spla.MatrixRankWarning) for x in w)


def test_strict_mode_raises_on_a_singular_system(gpu_lib):
    """solver={"strict": True}: the singular system of the test above raises
    FeSolveError with the BREAKDOWN status instead of returning NaN."""
    from finite_elements_gb300.analysis import FeSolveError, FiniteElementAnalysis
    from finite_elements_gb300.problem import Problem
    prob, _, _ = gc.load("ex2_strain")
    coords = np.vstack([prob.coords, [[50.0, 50.0]]])
    p2 = Problem("elastic", coords, prob.conn, E=prob.E, nu=prob.nu, thickness=prob.thickness,
                 rho=prob.rho, plane_strain=True, plane_stress=False,
                 node_load_node=prob.node_load_node, node_load_dim=prob.node_load_dim,
                 node_load_value=prob.node_load_value, node_bc_node=prob.node_bc_node,
                 node_bc_dim=prob.node_bc_dim, node_bc_value=prob.node_bc_value)
    fea = FiniteElementAnalysis.from_problem(p2, solver={"strict": True})
    with pytest.raises(FeSolveError) as e:
        fea.solve()
    assert "FE_BREAKDOWN" in str(e.value)
