"""The reference's intermediate building blocks through the drop-in (analysis.py:175-577):
triplet lists, dense and merged matrices, the condition and load lists and their
node objects, the source pieces, against the oracle and the golden vectors."""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["quirks_elastic", "quirks_magnetic", "tet_quirks", "mag_magnet", "mag_periodic"])
def test_intermediate_lists_match_the_oracle(gpu_lib, name):
    from test_abi_host import build_objects
    from finite_elements_gb300.analysis import FiniteElementAnalysis
    from oracle import fe_oracle as O
    prob, ref, mesh, kw = build_objects(name)
    fea = FiniteElementAnalysis(mesh=mesh, **kw)
    data, row, col = fea.k_matrix_data()
    od, orow, ocol = O.k_matrix_data(prob)
    np.testing.assert_array_equal(row, orow)
    np.testing.assert_array_equal(col, ocol)
    assert np.abs(data - od).max() <= 1e-13 * np.abs(od).max()
    K = fea.k_matrix_dense()
    assert K.shape == (prob.n_dof, prob.n_dof)
    assert np.abs(K - O.k_matrix_sparse(prob).toarray()).max() <= 1e-13 * np.abs(K).max()
    with pytest.raises(TypeError):
        fea.get_source_matrix_length()
    d, r, c = fea.c_matrix_boundary_conditions()
    bd, _ = O.boundary_conditions(prob)
    assert r[1::2] == bd.tolist() and r[0::2] == [prob.n_dof + i for i in range(bd.size)] and d == [1] * (2 * bd.size)
    assert fea.get_source_matrix_length() == ref["F"].size
    vals, rows = fea.source_c_matrix_loads()
    lk, lv = O.node_loads(prob)
    assert rows == lk.tolist()
    np.testing.assert_allclose(vals, lv, rtol=1e-14, atol=0)
    gv, grows = fea.source_c_matrix_boundary_conditions()
    assert grows == [prob.n_dof + i for i in range(bd.size)]
    mv, mrows = fea.source_c_matrix_magnet_loads()
    orow_m, oval_m = O.magnet_source(prob)
    assert mrows == orow_m.tolist() and mv == oval_m.tolist()
    cd, cr, cc = fea.c_matrix_continuity_conditions()
    od2, or2, oc2 = O.continuity_matrix_data(prob)
    assert cd == od2.tolist() and cr == or2.tolist() and cc == oc2.tolist()
    # F assembled from the pieces, as create_source_matrix does
    F = np.zeros(fea.get_source_matrix_length())
    for v, i in zip(vals + mv + gv, rows + mrows + grows):
        F[i] += v
    assert np.abs(F - ref["F"]).max() <= 1e-13 * max(np.abs(ref["F"]).max(), 1e-300)
    # node-object lists: element and edge loads / conditions in the reference's order
    el = fea.loads_element_to_node() + fea.loads_edge_to_node()
    ek = [mesh.node_to_index[ld.node] * prob.dim + ld.dimension - 1 for ld in el]
    keys, _ = fea.system().load_list()
    assert ek == keys[prob.node_load_node.size:]
    bl = fea.boundary_conditions_element_to_node() + fea.boundary_conditions_edge_to_node()
    bk = [mesh.node_to_index[c.application] * prob.dim + c.dimension - 1 for c in bl]
    ckeys, _ = fea.system().condition_list()
    assert bk == ckeys[prob.node_bc_node.size:]
    if prob.elastic:
        md, mr, mc = fea.m_matrix_data()
        omd, omr, omc = O.m_matrix_data(prob)
        np.testing.assert_array_equal(mr, omr)
        assert np.abs(md - omd).max() <= 1e-15 * np.abs(omd).max()
        assert np.abs(fea.matrix_sparse("m_matrix_data").toarray() - fea.m_matrix_dense()).max() \
            <= 1e-15 * np.abs(omd).max()
    else:
        assert fea.elements_permeability() == [float(g.elements[0].mu_total) for g in mesh.elements_groups]
    sysm_k = fea.matrix_sparse("k_matrix_data")
    np.testing.assert_array_equal(sysm_k.indices, ref["Ks_indices"])
    with pytest.raises(NotImplementedError):
        fea.matrix_sparse("no_such_data")
