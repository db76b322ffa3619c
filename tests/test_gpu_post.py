"""Per-element post-processing on the GPU against the oracle (results.py:121-152,
:769-830): strain, stress, energy of elasticity solutions and the magnetic field of
magnetostatic ones.

Tolerance: each value agrees with the oracle within 64 eps (1024 eps for tetrahedra,
whose B the oracle and the kernel compute by different formulas) times the sum of the
absolute values of the terms that make it (strain: |B| |q|, stress: |D| |B| |q|,
energy: 0.5 |q|^T |Ke| |q|, field: |b|, |c| times |A|).  That is the rounding bound
of a short dot product evaluated in another order; a plain relative bound would
fail on element energies, which are quadratic forms of near-rigid motions and so
cancel to far below their terms."""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def within(gpu, ref, scale, c=64.0):
    return bool(np.all(np.abs(gpu - ref) <= c * EPS * scale))


@pytest.mark.parametrize("name", gc.solvable_names())
def test_post_matches_oracle(gpu_lib, name):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob, _, ref = gc.load(name)
    s = GpuSystem(prob)
    x = ref["x"]
    res = s.post(x)
    if prob.elastic:
        strain, stress, energy = O.elastic_post(prob, x)
        d, nl = prob.dim, prob.npe * prob.dim
        q = np.abs(x[: prob.n_dof].reshape(-1, d)[prob.conn].reshape(-1, nl))
        if prob.kind == "elastic3d":
            B = np.abs(O.tet_b_matrix(O.element_points(prob)))
            D = np.abs(O.d_matrix_3d(prob.E, prob.nu, prob.plane_strain, prob.plane_stress))
        else:
            B = np.abs(O.b_matrix(O.element_points(prob)))
            D = np.abs(O.d_matrix(prob.E, prob.nu, prob.plane_strain, prob.plane_stress))
        ke = np.abs(O.element_stiffness(prob).reshape(-1, nl, nl))
        # tetrahedra: the oracle's B comes from the inverse of the 4x4 vertex matrix, the
        # kernel's from cross products over 6V; the two differ by a few eps of max |B|
        # per element, which the sums of |B| |q| over near-rigid motions can amplify to
        # ~80 eps on the reference's Gmsh beam (element condition numbers up to ~500)
        c = 1024.0 if prob.kind == "elastic3d" else 64.0
        assert within(res["strain"], strain, np.einsum("eij,ej->ei", B, q), c)
        assert within(res["stress"], stress, np.einsum("eij,ej->ei", np.matmul(D, B), q), c)
        assert within(res["energy"], energy, 0.5 * np.einsum("ei,eij,ej->e", q, ke, q), c)
    else:
        ff = np.abs(O.form_functions(O.element_points(prob)))
        A = np.abs(x[: prob.n_nodes][prob.conn])
        scale = np.stack([(ff[:, :, 2] * A).sum(axis=1), (ff[:, :, 1] * A).sum(axis=1)], axis=1)
        assert within(res["field"], O.magnetic_field(prob, x), scale)
    s.close()


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


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


def test_air_gap_post_processing_matches_the_reference(gpu_lib):
    """MagneticResults.brbtetha / maxwell_stress_tensor / torque (results.py:82-243) on
    the GPU solution and the GPU B field of the motor-like annulus, against the values
    the reference computed on its own solution.  Tolerance: 1e-9 relative to the sum of
    the magnitudes of the terms (each quantity is a short sum of products of B)."""
    from test_abi_host import build_objects
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    from finite_elements_gb300.results import MagneticResults
    prob, ref, mesh, kw = build_objects("motor")
    length, r_s, r_r = ref["_motor"].tolist()
    res = FiniteElementAnalysis(mesh=mesh, **kw).solve()
    mr = MagneticResults(res.mesh, res.result_vector)
    gap = next(g for g in mesh.elements_groups if g.name == "Gap ring")
    brbt = np.array(mr.brbtetha(gap))
    assert np.abs(brbt - ref["brbtetha"]).max() <= 1e-9 * np.abs(ref["brbtetha"]).max()
    t = mr.torque("Gap ring", length, r_s, r_r)
    idx = np.array(list(mr._group_range("Gap ring")))
    r, br, bt, _, p = mr._polar(idx)
    area = np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1])
                  - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])) / 2.0
    scale = length / (4e-7 * np.pi * (r_s - r_r)) * np.abs(r * br * bt * area).sum()
    assert abs(t - float(ref["torque"])) <= 1e-9 * scale
    for k, row in zip(ref["_motor_maxwell_elements"].tolist(), ref["maxwell"]):
        got = np.array(mr.maxwell_stress_tensor(gap.elements[k]))
        assert np.abs(got - row).max() <= 1e-9 * np.abs(row).max()
