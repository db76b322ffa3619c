"""Multigrid-preconditioned FP64 PCG (smoothed-aggregation V-cycle, work in progress)
against the oracle's direct solve: plane strain, tetrahedra and magnetostatics, each
to ||x - x_ref|| <= 1e-9 ||x_ref|| in a few tens of iterations."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems():
    from finite_elements_gb300 import meshgen
    return {
        "plane_strain": lambda: meshgen.plane_strain_random(60, 30, seed=3),
        "tet": lambda: meshgen.cantilever_3d(12, 3, 3, jitter=0.2, seed=4),
        "magnetic": lambda: meshgen.magnetostatic(60, 30, seed=5),
    }


@pytest.mark.parametrize("name", ["plane_strain", "tet", "magnetic"])
def test_multigrid_matches_oracle(gpu_lib, name):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob = _problems()[name]()
    ref = np.array(O.solve(prob))
    s = GpuSystem(prob)
    try:
        x, st = s.solve(precision="fp64", tol=1e-12, multigrid=True)
    finally:
        s.close()
    assert st.status == 0, st.as_dict()
    assert st.iterations <= 80, st.as_dict()
    assert np.linalg.norm(x - ref) <= 1e-9 * np.linalg.norm(ref), st.as_dict()
