"""The oracle against the golden vectors the reference itself produced
(tests/golden/make_golden.py ran finite_elements' own analysis code)."""
import numpy as np
import pytest

import golden_cases as gc
from oracle import fe_oracle as O

CASES = gc.names()


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    prob, groups, ref = gc.load(name)
    K = O.create_matrix(prob)
    # pattern and index arrays bit-exact, shape identical
    assert tuple(K.shape) == tuple(ref["K_shape"])
    np.testing.assert_array_equal(K.indptr, ref["K_indptr"])
    np.testing.assert_array_equal(K.indices, ref["K_indices"])
    scale = np.abs(ref["K_data"]).max()
    assert np.abs(K.data - ref["K_data"]).max() <= 1e-14 * scale
    F = O.create_source_matrix(prob)[:, 0]
    assert F.shape == ref["F"].shape
    assert np.abs(F - ref["F"]).max() <= 1e-14 * max(np.abs(ref["F"]).max(), 1e-300)
    if "x" in ref:
        x = np.array(O.solve(prob))
        assert np.linalg.norm(x - ref["x"]) <= 1e-12 * np.linalg.norm(ref["x"])
    else:
        with pytest.raises(ValueError) as e:
            O.solve(prob)
        assert str(e.value) == str(ref["solve_error"])
    ks = O.k_matrix_sparse(prob)
    np.testing.assert_array_equal(ks.indptr, ref["Ks_indptr"])
    np.testing.assert_array_equal(ks.indices, ref["Ks_indices"])
    assert np.abs(ks.data - ref["Ks_data"]).max() <= 1e-14 * np.abs(ref["Ks_data"]).max()
    bd, bv = O.boundary_conditions(prob)
    np.testing.assert_array_equal(bd, ref["bc_dof"])
    np.testing.assert_array_equal(bv, ref["bc_value"])
    ke = O.element_stiffness(prob)
    assert np.abs(ke - ref["Ke"]).max() <= 1e-14 * np.abs(ref["Ke"]).max()
    if "factors" in ref:      # triangles only: the reference has none for tetrahedra
        np.testing.assert_allclose(O.element_node_factors(prob), ref["factors"], rtol=0, atol=1e-15 *
                                   max(1.0, np.abs(ref["factors"]).max()))
    if "Ms_data" in ref:
        ms = O.m_matrix_sparse(prob)
        np.testing.assert_array_equal(ms.indices, ref["Ms_indices"])
        np.testing.assert_array_equal(ms.data, ref["Ms_data"])
        me = O.tet_mass(prob) if prob.kind == "elastic3d" else O.elastic_mass(prob)
        np.testing.assert_array_equal(me, ref["Me"])


def test_factor_quirk_is_zero_area_area():
    """element_to_node_factors evaluates to (0, A, A) (elements.py:46-53)."""
    prob, _, ref = gc.load("quirks_elastic")
    p = prob.coords[prob.conn]
    area = O.triangle_area(p)
    np.testing.assert_allclose(ref["factors"][:, 1], area, rtol=1e-12)
    np.testing.assert_allclose(ref["factors"][:, 2], area, rtol=1e-12)
    assert np.abs(ref["factors"][:, 0]).max() <= 1e-12 * area.max()


def test_magnet_source_matches_the_host_contour_code():
    """The drop-in's vectorised contour extraction (loads.magnet_contributions) gives
    the oracle's loop restatement of loads.py:129-147 entry for entry."""
    from finite_elements_gb300.loads import magnet_contributions
    prob, _, ref = gc.load("mag_magnet")
    rows, vals = O.magnet_source(prob)
    parts = [magnet_contributions(prob.coords, prob.conn, m.elements, m.non_contour_nodes, m.magnetization)
             for m in prob.magnet_loads]
    np.testing.assert_array_equal(np.concatenate([a for a, _ in parts]), rows)
    np.testing.assert_array_equal(np.concatenate([v for _, v in parts]), vals)
    # the non-contour edge 25-26 is skipped; the magnets add a net zero (closed contours)
    assert not any({a, b} == {25, 26} for a, b in rows.reshape(-1, 2).tolist())


def test_last_value_wins_dedup():
    """Repeated (node, dim) keys keep the LAST value in first-insertion order
    (analysis.py:28-110)."""
    keys = np.array([5, 3, 5, 7, 3])
    vals = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    k, v = O.dedup_last_wins(keys, vals)
    np.testing.assert_array_equal(k, [5, 3, 7])
    np.testing.assert_array_equal(v, [3.0, 5.0, 4.0])


def test_golden_cover_the_quirks():
    prob, _, ref = gc.load("quirks_elastic")
    # a repeated condition on (node 0, dim 1): 0.0 then 2e-5, the later value is kept
    assert ref["bc_dof"][0] == 0 and ref["bc_value"][0] == 2e-5
    # element loads overwrite the user load on node 27 dim 2, edge loads overwrite both
    lk, lv = O.node_load_list(prob)
    assert (lk == 27 * 2 + 1).sum() >= 2


def test_air_gap_post_processing_on_the_reference_field():
    """The drop-in's host arithmetic of brbtetha / maxwell_stress_tensor / torque
    (results.py:82-243), fed the oracle's B field of the reference's solution, gives
    the reference's values to rounding."""
    from test_abi_host import build_objects
    from finite_elements_gb300.results import MagneticResults
    prob, ref, mesh, kw = build_objects("motor")
    length, r_s, r_r = ref["_motor"].tolist()
    mr = MagneticResults(mesh, list(ref["x"]))
    mr._field = O.magnetic_field(prob, ref["x"])
    gap = next(g for g in mesh.elements_groups if g.name == "Gap ring")
    np.testing.assert_allclose(mr.brbtetha(gap), ref["brbtetha"], rtol=1e-12, atol=1e-13)
    assert abs(mr.torque("Gap ring", length, r_s, r_r) - float(ref["torque"])) <= 1e-11 * abs(float(ref["torque"]))
    for k, row in zip(ref["_motor_maxwell_elements"].tolist(), ref["maxwell"]):
        np.testing.assert_allclose(mr.maxwell_stress_tensor(gap.elements[k]), row, rtol=1e-12, atol=1e-6)
