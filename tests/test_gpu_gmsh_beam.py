"""The reference's beam study (scripts/Elasticity/beam2d_example_3.py) on the GPU:
structured meshes of the 10 x 1 cantilever written as Gmsh 4.1 files and read back,
solved by the drop-in analysis; tip deflections equal the oracle's (FP64 PCG to its
floor: 1e-9 on this one component -- the slender beam's condition number puts both
solvers' rounding near 1e-10 there) and converge to Euler-Bernoulli (error falling
with refinement, < 1% on the finest mesh); the mixed-precision solve gives the same
deflection to 1e-7."""
import numpy as np
import pytest

from beam_cases import ANALYTIC_TIP, beam_problem

pytestmark = pytest.mark.gpu


def test_gmsh_beam_converges_to_euler_bernoulli(gpu_lib, tmp_path):
    from finite_elements_gb300 import gmsh, meshgen
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    from oracle import fe_oracle as O
    errors = []
    for nx, ny in ((20, 2), (40, 4), (80, 8), (160, 16)):
        coords, conn = meshgen.rect_grid(nx, ny, 10.0, 1.0)
        f = tmp_path / f"beam_{nx}.msh"
        gmsh.write_msh(f, coords, conn)
        m = gmsh.read_msh(f)
        prob, tip = beam_problem(m.coords, m.triangles)
        res = FiniteElementAnalysis.from_problem(prob, mesh=m.array_mesh()).solve()
        x = np.array(res.result_vector)
        ref = np.array(O.solve(prob))
        assert abs(x[2 * tip + 1] - ref[2 * tip + 1]) <= 1e-9 * abs(ref[2 * tip + 1]), (nx, x[2 * tip + 1],
                                                                                     ref[2 * tip + 1])
        mixed = FiniteElementAnalysis.from_problem(prob, solver={"precision": "mixed-cg64", "tol": 1e-10,
                                                                 "cheb_degree": 16, "cheb_ratio": 1000}).solve()
        xm = np.array(mixed.result_vector)
        assert abs(xm[2 * tip + 1] - ref[2 * tip + 1]) <= 1e-7 * abs(ref[2 * tip + 1]), (nx, xm[2 * tip + 1],
                                                                                    ref[2 * tip + 1])
        errors.append(abs(x[2 * tip + 1] - ANALYTIC_TIP) / abs(ANALYTIC_TIP))
    assert all(b < a for a, b in zip(errors, errors[1:])), errors
    assert errors[-1] < 0.01
