"""Per-element post-processing on the GPU against the oracle (results.py:121-152,
:769-830): strain, stress, energy of elasticity solutions and the magnetic field of
magnetostatic ones.  Tolerance: max |difference| <= 1e-12 * max |oracle|."""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", [n for n in gc.names()])
def test_post_matches_oracle(gpu_lib, name):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob, _, ref = gc.load(name)
    s = GpuSystem(prob)
    x = ref["x"]
    res = s.post(x)
    if prob.kind == "elastic":
        strain, stress, energy = O.elastic_post(prob, x)
        assert relmax(res["strain"], strain) <= 1e-12
        assert relmax(res["stress"], stress) <= 1e-12
        assert relmax(res["energy"], energy) <= 1e-12
    else:
        assert relmax(res["field"], O.magnetic_field(prob, x)) <= 1e-12
    s.close()


def test_results_classes(gpu_lib):
    """The drop-in result objects built from (mesh, result_vector), as user scripts
    do (scripts/Elasticity/beam2d_example_1.py:72)."""
    from test_abi_host import build_objects
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    from finite_elements_gb300.results import ElasticityResults2D, MagneticResults
    from oracle import fe_oracle as O
    prob, ref, mesh, kw = build_objects("ex2_strain")
    res = FiniteElementAnalysis(mesh=mesh, **kw).solve()
    er = ElasticityResults2D(res.mesh, res.result_vector, prob.plane_strain, prob.plane_stress)
    strain, stress, energy = O.elastic_post(prob, ref["x"])
    assert relmax(er.strain, strain) <= 1e-9
    assert abs(er.energy - energy.sum()) <= 1e-9 * abs(energy.sum())
    prob, ref, mesh, kw = build_objects("mag_beam")
    res = FiniteElementAnalysis(mesh=mesh, **kw).solve()
    mr = MagneticResults(res.mesh, res.result_vector)
    assert relmax(mr.magnetic_field_per_element, O.magnetic_field(prob, ref["x"])) <= 1e-9
