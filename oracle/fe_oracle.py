"""CPU oracle for the finite_elements assembly-and-solve path.

TEST INFRASTRUCTURE ONLY.  Nothing in ``finite_elements_gb300`` imports this module:
it is the oracle that ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` compare the CUDA path against.

It restates, in numpy, what the reference computes (file:line of the reference
project ``finite_elements``), element by element and list by list, and then calls the
real scipy routines the reference calls:

* plane-elasticity triangle B, D and Ke = t*A*B^T D B   (elements.py:395-453, :466-511)
* plane-elasticity triangle mass Me                     (elements.py:513-536)
* linear tetrahedron B, isotropic 3D D, Ke = V B^T D B   (elements.py:719-827)
* linear tetrahedron mass Me = rho V / 20 * P12          (elements.py:829-858)
* magnetostatic triangle Ke = A/mu * (b_i b_j + c_i c_j) (elements.py:93-118)
* element -> node factors |detJ| * N_i(mid(p2, p3))     (elements.py:18-53, :156-191)
* ElementsLoad area split                               (loads.py:24-35)
* element/edge loads and conditions -> node lists       (analysis.py:201-239, :407-447)
* (node, dim) de-duplication, last value wins           (analysis.py:28-110)
* DOF numbering node*dim + (d-1)                        (core.py:89-108)
* COO triplets in group/element order                   (analysis.py:324-339, :714-735)
* Lagrange-multiplier rows n*dim + i                    (analysis.py:241-279, :509-543)
* scipy.sparse.csr_matrix of the triplets               (analysis.py:617-663)
* F vector                                              (analysis.py:665-708, :737-739)
* spsolve(K, F, permc_spec='NATURAL', use_umfpack=True) (analysis.py:798-830)
* magnet loads: contour edges, (M . t) L / 2 per end    (loads.py:129-147, analysis.py:556-577)
* continuity rows n + len(node_loads) + i, (1,1,-v,-v)  (analysis.py:175-199, conditions.py:196-241)
* dict-merged K / M as csc_matrix                       (analysis.py:345-405)

Two volmdlr quantities are restated from their definitions, because volmdlr is not
available: the unsigned triangle area |detJ|/2 and the barycentric shape-function
coefficients (a_i, b_i, c_i).  No reference test pins their values ("parity
unpinned" for those two); everything downstream of them is pinned by golden vectors
that ``tests/golden/make_golden.py`` produced by running the reference's own code.

The tetrahedron's volmdlr quantities are restated the same way: the unsigned volume
and the form-function rows (a_i, b_i, c_i, d_i) = 6V (coefficients of N_i), the
convention under which the reference's B = (1/(6V)) [b c d ...] is the gradient
matrix of the linear shape functions.  No reference test or fixture pins that
convention or any 3D value: the tetrahedron path is "parity unpinned"; its golden
vectors come from the reference's own 3D element code run on these restated
quantities.
"""
from __future__ import annotations

import warnings

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from finite_elements_gb300.problem import ELASTIC, ELASTIC3D, MAGNETIC, Problem

# ---------------------------------------------------------------- element level


def element_points(prob: Problem):
    """(E, 3, 2) vertex coordinates of every element, in connectivity order."""
    return prob.coords[prob.conn]


def triangle_area(p):
    """Unsigned area |detJ|/2 (volmdlr TriangularElement2D.area, restated)."""
    x1, y1 = p[:, 0, 0], p[:, 0, 1]
    x2, y2 = p[:, 1, 0], p[:, 1, 1]
    x3, y3 = p[:, 2, 0], p[:, 2, 1]
    return np.abs((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1)) / 2.0


def form_functions(p):
    """(E, 3, 3) rows (a_i, b_i, c_i): N_i = a_i + b_i x + c_i y, N_i(p_j) = delta_ij
    (volmdlr TriangularElement2D.form_functions, restated)."""
    x1, y1 = p[:, 0, 0], p[:, 0, 1]
    x2, y2 = p[:, 1, 0], p[:, 1, 1]
    x3, y3 = p[:, 2, 0], p[:, 2, 1]
    det = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1)
    ff = np.empty((p.shape[0], 3, 3))
    ff[:, 0, 0] = (x2 * y3 - x3 * y2) / det
    ff[:, 1, 0] = (x3 * y1 - x1 * y3) / det
    ff[:, 2, 0] = (x1 * y2 - x2 * y1) / det
    ff[:, 0, 1] = (y2 - y3) / det
    ff[:, 1, 1] = (y3 - y1) / det
    ff[:, 2, 1] = (y1 - y2) / det
    ff[:, 0, 2] = (x3 - x2) / det
    ff[:, 1, 2] = (x1 - x3) / det
    ff[:, 2, 2] = (x2 - x1) / det
    return ff


def b_matrix(p):
    """(E, 3, 6) strain-displacement matrix with the reference's signed detJ
    (elements.py:395-416)."""
    xs, ys = p[:, :, 0], p[:, :, 1]
    y23, y31, y12 = ys[:, 1] - ys[:, 2], ys[:, 2] - ys[:, 0], ys[:, 0] - ys[:, 1]
    x32, x13, x21 = xs[:, 2] - xs[:, 1], xs[:, 0] - xs[:, 2], xs[:, 1] - xs[:, 0]
    det = (xs[:, 0] - xs[:, 2]) * (ys[:, 1] - ys[:, 2]) - (ys[:, 0] - ys[:, 2]) * (xs[:, 1] - xs[:, 2])
    z = np.zeros_like(det)
    data = np.stack([y23, z, y31, z, y12, z,
                     z, x32, z, x13, z, x21,
                     x32, y23, x13, y31, x21, y12], axis=1).reshape(-1, 3, 6)
    return (1.0 / det)[:, None, None] * data


def d_matrix(E, nu, plane_strain, plane_stress):
    """(E, 3, 3) constitutive matrix; the flag checks and messages of
    elements.py:251-273 and the two formulas of elements.py:418-453."""
    if plane_strain and plane_stress:
        raise ValueError('just one of plane_strain or plane_stress can be True')
    if not plane_strain and not plane_stress:
        raise ValueError('one of plane_strain or plane_stress must be True')
    if plane_strain:
        a = (E * nu) / ((1 + nu) * (1 - 2 * nu))
    else:
        a = (E * nu) / (1 - nu ** 2)
    b = E / (2 * (1 + nu))
    c = a + 2 * b
    z = np.zeros_like(E)
    return np.stack([c, a, z, a, c, z, z, z, b], axis=1).reshape(-1, 3, 3)


def elastic_stiffness(prob: Problem):
    """(E, 36) row-major Ke = t * area * (B^T D) B (elements.py:466-511)."""
    p = element_points(prob)
    B = b_matrix(p)
    D = d_matrix(prob.E, prob.nu, prob.plane_strain, prob.plane_stress)
    ke = np.matmul(np.matmul(np.transpose(B, (0, 2, 1)), D), B)
    ke *= (prob.thickness * triangle_area(p))[:, None, None]
    return ke.reshape(-1, 36)


_MASS_PATTERN = np.array([2, 0, 1, 0, 1, 0,
                          0, 2, 0, 1, 0, 1,
                          1, 0, 2, 0, 1, 0,
                          0, 1, 0, 2, 0, 1,
                          1, 0, 1, 0, 2, 0,
                          0, 1, 0, 1, 0, 2], dtype=np.float64)


def elastic_mass(prob: Problem):
    """(E, 36) Me = rho * area * t / 12 * P (elements.py:513-536)."""
    p = element_points(prob)
    s = (prob.rho * triangle_area(p) * prob.thickness) / 12
    return s[:, None] * _MASS_PATTERN[None, :]


def magnetic_stiffness(prob: Problem):
    """(E, 9) row-major Ke_ij = 1/mu * (b_i b_j + c_i c_j) * area (elements.py:93-118)."""
    p = element_points(prob)
    ff = form_functions(p)
    b, c = ff[:, :, 1], ff[:, :, 2]
    g = b[:, :, None] * b[:, None, :] + c[:, :, None] * c[:, None, :]
    return ((1 / prob.mu)[:, None, None] * g * triangle_area(p)[:, None, None]).reshape(-1, 9)


def tet_volume(p):
    """Unsigned volume |det[p1-p0, p2-p0, p3-p0]| / 6 (volmdlr TetrahedralElement.volume,
    restated)."""
    a = p[:, 1] - p[:, 0]
    n = np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0])
    return np.abs(a[:, 0] * n[:, 0] + a[:, 1] * n[:, 1] + a[:, 2] * n[:, 2]) / 6.0


def tet_form_functions(p):
    """(E, 4, 4) rows (a_i, b_i, c_i, d_i) = 6V (coefficients of N_i): N_i = (a_i + b_i x +
    c_i y + d_i z) / (6V), N_i(p_j) = delta_ij, V the unsigned volume (volmdlr
    TetrahedralElement.form_functions, restated in the convention the reference's B of
    elements.py:719-748 divides by 6V)."""
    A = np.concatenate([np.ones(p.shape[:2] + (1,)), p], axis=2)       # rows [1, x_j, y_j, z_j]
    C = np.linalg.inv(A)                                                # column i: coefficients of N_i
    return (6.0 * tet_volume(p))[:, None, None] * np.transpose(C, (0, 2, 1))


def tet_b_matrix(p):
    """(E, 6, 12) B of elements.py:719-748: rows xx, yy, zz, xy, yz, zx, scaled by
    1 / (6 V)."""
    ff = tet_form_functions(p)
    b, c, d = ff[:, :, 1], ff[:, :, 2], ff[:, :, 3]
    z = np.zeros_like(b[:, 0])
    rows = [[], [], [], [], [], []]
    for i in range(4):
        rows[0] += [b[:, i], z, z]
        rows[1] += [z, c[:, i], z]
        rows[2] += [z, z, d[:, i]]
        rows[3] += [c[:, i], b[:, i], z]
        rows[4] += [z, d[:, i], c[:, i]]
        rows[5] += [d[:, i], z, b[:, i]]
    data = np.stack([np.stack(r, axis=1) for r in rows], axis=1)
    return (1 / (6 * tet_volume(p)))[:, None, None] * data


def d_matrix_3d(E, nu, plane_strain, plane_stress):
    """(E, 6, 6) isotropic D of elements.py:779-796 (both plane flags give it; the flag
    checks of elements.py:265-273 still apply)."""
    if plane_strain and plane_stress:
        raise ValueError('just one of plane_strain or plane_stress can be True')
    if not plane_strain and not plane_stress:
        raise ValueError('one of plane_strain or plane_stress must be True')
    ca = 1 - nu
    cb = (1 - 2 * nu) / 2
    z = np.zeros_like(E)
    data = np.stack([ca, nu, nu, z, z, z,
                     nu, ca, nu, z, z, z,
                     nu, nu, ca, z, z, z,
                     z, z, z, cb, z, z,
                     z, z, z, z, cb, z,
                     z, z, z, z, z, cb], axis=1).reshape(-1, 6, 6)
    coeff = E / ((1 + nu) * (1 - 2 * nu))
    return coeff[:, None, None] * data


def tet_stiffness(prob: Problem):
    """(E, 144) row-major Ke = V * ((B^T D) B) (elements.py:808-827)."""
    p = element_points(prob)
    B = tet_b_matrix(p)
    D = d_matrix_3d(prob.E, prob.nu, prob.plane_strain, prob.plane_stress)
    ke = tet_volume(p)[:, None, None] * np.matmul(np.matmul(np.transpose(B, (0, 2, 1)), D), B)
    return ke.reshape(-1, 144)


_TET_MASS_PATTERN = np.kron(np.ones((4, 4)) + np.eye(4), np.eye(3)).reshape(-1)


def tet_mass(prob: Problem):
    """(E, 144) Me = ((rho * V) / 20) * P12 (elements.py:829-858)."""
    s = (prob.rho * tet_volume(element_points(prob))) / 20
    return s[:, None] * _TET_MASS_PATTERN[None, :]


def element_stiffness(prob: Problem):
    if prob.kind == ELASTIC3D:
        return tet_stiffness(prob)
    return elastic_stiffness(prob) if prob.kind == ELASTIC else magnetic_stiffness(prob)


def element_node_factors(prob: Problem, elements=None):
    """(k, 3) |detJ| * (a_i + b_i (x2+x3)/2 + c_i (y2+y3)/2), written term by term as in
    elements.py:46-51 (it evaluates to (0, area, area))."""
    conn = prob.conn if elements is None else prob.conn[np.asarray(elements)]
    p = prob.coords[conn]
    x1, y1 = p[:, 0, 0], p[:, 0, 1]
    x2, y2 = p[:, 1, 0], p[:, 1, 1]
    x3, y3 = p[:, 2, 0], p[:, 2, 1]
    detj = np.abs((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1))
    ff = form_functions(p)
    out = np.empty((p.shape[0], 3))
    for i in range(3):
        a, b, c = ff[:, i, 0], ff[:, i, 1], ff[:, i, 2]
        out[:, i] = detj * (a + 0.5 * b * x2 + 0.5 * c * y2 + 0.5 * b * x3 + 0.5 * c * y3)
    return out


# ---------------------------------------------------------------- loads and conditions


def dedup_last_wins(keys, values):
    """Dict round trip of analysis.py:28-110: ``d[key] = value`` for every entry in
    order, then the items in insertion order.  Returns (unique keys in order of first
    occurrence, the LAST value seen for each)."""
    keys = np.asarray(keys, dtype=np.int64)
    values = np.asarray(values, dtype=np.float64)
    if keys.size == 0:
        return keys, values
    uniq, first = np.unique(keys, return_index=True)
    _, last_rev = np.unique(keys[::-1], return_index=True)
    last = keys.size - 1 - last_rev
    order = np.argsort(first, kind="stable")
    return uniq[order], values[last[order]]


def node_load_list(prob: Problem):
    """(dof keys, values) before de-duplication, in the order of
    source_c_matrix_loads (analysis.py:465-469): user NodeLoads, then element loads
    (analysis.py:407-429 with loads.py:24-35), then edge loads (analysis.py:431-447)."""
    d = prob.dim
    keys = [prob.node_load_node * d + (prob.node_load_dim - 1)]
    vals = [prob.node_load_value]
    if prob.kind == ELASTIC3D and prob.element_loads:
        raise AttributeError("'ElasticityTetrahedralElement3D' object has no attribute "
                             "'element_to_node_factors'")
    for s in prob.element_loads:
        conn = prob.conn[s.elements]
        area = triangle_area(prob.coords[conn])
        total_area = 0.0
        for a in area.tolist():          # sum(...) of loads.py:32, left to right
            total_area += a
        per_element = s.value * area / total_area
        fac = element_node_factors(prob, s.elements)
        keys.append((conn.astype(np.int64) * d + (s.dimension - 1)).reshape(-1))
        vals.append((per_element[:, None] * fac).reshape(-1))
    for (na, nb), dim, v in zip(prob.edge_load_nodes.tolist(), prob.edge_load_dim.tolist(),
                               prob.edge_load_value.tolist()):
        keys.append(np.array([na * d + dim - 1, nb * d + dim - 1]))
        vals.append(np.array([v * 0.5, v * 0.5]))
    return np.concatenate(keys).astype(np.int64), np.concatenate(vals)


def boundary_condition_list(prob: Problem):
    """(dof keys, values) before de-duplication, in the order of
    c_matrix_boundary_conditions (analysis.py:252-256): node conditions, element
    conditions (analysis.py:201-220), edge conditions (analysis.py:222-239)."""
    d = prob.dim
    keys = [prob.node_bc_node * d + (prob.node_bc_dim - 1)]
    vals = [prob.node_bc_value]
    if prob.kind == ELASTIC3D and prob.element_bc_element.size:
        raise AttributeError("'ElasticityTetrahedralElement3D' object has no attribute "
                             "'element_to_node_factors'")
    if prob.element_bc_element.size:
        fac = element_node_factors(prob, prob.element_bc_element)
        conn = prob.conn[prob.element_bc_element].astype(np.int64)
        keys.append((conn * d + (prob.element_bc_dim[:, None] - 1)).reshape(-1))
        vals.append((prob.element_bc_value[:, None] * fac).reshape(-1))
    if prob.edge_bc_nodes.size:
        keys.append((prob.edge_bc_nodes * d + (prob.edge_bc_dim[:, None] - 1)).reshape(-1))
        vals.append(np.repeat(prob.edge_bc_value * 0.5, 2))
    return np.concatenate(keys).astype(np.int64), np.concatenate(vals)


def boundary_conditions(prob: Problem):
    """De-duplicated (dof, value) of the multiplier rows, in multiplier order."""
    return dedup_last_wins(*boundary_condition_list(prob))


def node_loads(prob: Problem):
    return dedup_last_wins(*node_load_list(prob))


# ---------------------------------------------------------------- global system


def k_matrix_data(prob: Problem):
    """COO triplets of all element matrices (analysis.py:324-339, :714-735):
    row = repeat(L, len(L)), col = tile(L, len(L)) with L the element's DOFs
    (node-major, dimension-minor)."""
    d = prob.dim
    ke = element_stiffness(prob)
    nl = prob.npe * d
    L = (prob.conn.astype(np.int64)[:, :, None] * d + np.arange(d)[None, None, :]).reshape(-1, nl)
    row = np.repeat(L, nl, axis=1).reshape(-1)
    col = np.tile(L, (1, nl)).reshape(-1)
    return ke.reshape(-1), row, col


def m_matrix_data(prob: Problem):
    if not prob.elastic:
        raise NotImplementedError("mass matrices exist for elasticity elements only")
    d = prob.dim
    me = tet_mass(prob) if prob.kind == ELASTIC3D else elastic_mass(prob)
    nl = prob.npe * d
    L = (prob.conn.astype(np.int64)[:, :, None] * d + np.arange(d)[None, None, :]).reshape(-1, nl)
    return me.reshape(-1), np.repeat(L, nl, axis=1).reshape(-1), np.tile(L, (1, nl)).reshape(-1)


def continuity_matrix_data(prob: Problem):
    """c_matrix_continuity_conditions (analysis.py:175-199) as written: condition i at
    row len(nodes) + len(node_loads) + i (user NodeLoads only), columns the two node
    indices, data ContinuityCondition.c_matrix() = (1, 1, -value, -value)."""
    data, row, col = [], [], []
    base = prob.n_nodes + prob.node_load_node.size
    for i, (a, b, v) in enumerate(zip(prob.cont_node1.tolist(), prob.cont_node2.tolist(),
                                      prob.cont_value.tolist())):
        data += [1, 1, -v, -v]
        row += [base + i, a, base + i, b]
        col += [a, base + i, b, base + i]
    return np.array(data, np.float64), np.array(row, np.int64), np.array(col, np.int64)


def create_matrix(prob: Problem):
    """Augmented saddle-point matrix as scipy builds it (analysis.py:617-663): the
    triplets of k_matrix_data, c_matrix_continuity_conditions and
    c_matrix_boundary_conditions in that order."""
    data, row, col = k_matrix_data(prob)
    cd, cr, cc = continuity_matrix_data(prob)
    bc_dof, _ = boundary_conditions(prob)
    nd = prob.n_dof
    i = np.arange(bc_dof.size, dtype=np.int64)
    data = np.concatenate([data, cd, np.ones(2 * bc_dof.size)])
    row = np.concatenate([row, cr, np.stack([nd + i, bc_dof], axis=1).reshape(-1)])
    col = np.concatenate([col, cc, np.stack([bc_dof, nd + i], axis=1).reshape(-1)])
    return sp.csr_matrix((data, (row, col)))


def _interior_normal(a, b, c):
    tx, ty = b[0] - a[0], b[1] - a[1]
    length = np.sqrt(tx * tx + ty * ty)
    nx, ny = -ty / length, tx / length
    if nx * (c[0] - a[0]) + ny * (c[1] - a[1]) < 0:
        nx, ny = -nx, -ny
    return nx, ny


def magnet_source(prob: Problem):
    """(rows, values) of source_c_matrix_magnet_loads (analysis.py:556-577), in its order:
    per MagnetLoad the contour edges of contour_linear_elements (loads.py:129-147) --
    a dict of edges counted over the triangles' edges (p1,p2), (p2,p3), (p3,p1), kept
    when counted once and not both points non-contour -- each adding
    M . (-n_y, n_x) * length / 2 at its two points, n the edge's unit normal pointing
    into its triangle (volmdlr's LinearElement.interior_normal, restated)."""
    rows, vals = [], []
    for ml in prob.magnet_loads:
        count, info = {}, {}
        for e in ml.elements.tolist():
            t = prob.conn[e].tolist()
            for i in range(3):
                a, b, c = t[i], t[(i + 1) % 3], t[(i + 2) % 3]
                key = (min(a, b), max(a, b))
                if key not in count:
                    count[key] = 1
                    info[key] = (a, b, c)
                else:
                    count[key] += 1
        nc = set(ml.non_contour_nodes.tolist())
        mx, my = ml.magnetization
        for key, k in count.items():
            a, b, c = info[key]
            if k == 1 and (a not in nc or b not in nc):
                pa, pb, pc = prob.coords[a], prob.coords[b], prob.coords[c]
                nx, ny = _interior_normal(pa, pb, pc)
                length = np.sqrt((pb[0] - pa[0]) ** 2 + (pb[1] - pa[1]) ** 2)
                v = (mx * -ny + my * nx) * length / 2
                rows += [a, b]
                vals += [v, v]
    return np.array(rows, np.int64), np.array(vals, np.float64)


def create_source_matrix(prob: Problem):
    """Dense (n*dim + n_cont + n_bc, 1) right-hand side (analysis.py:665-708,
    :737-739): the de-duplicated loads, then += each magnet contribution in order,
    then the prescribed values at rows n*dim + i."""
    lk, lv = node_loads(prob)
    bc_dof, bc_val = boundary_conditions(prob)
    nd = prob.n_dof
    f = np.zeros((nd + prob.n_cont + bc_dof.size, 1))
    np.add.at(f[:, 0], lk, lv)
    for r, v in zip(*magnet_source(prob)):
        f[r, 0] += v
    f[nd:nd + bc_dof.size, 0] += bc_val
    return f


def solve(prob: Problem):
    """The reference's solve (analysis.py:816-828): spsolve with NATURAL column order
    (UMFPACK is not installed, so scipy uses SuperLU, as in a default install).
    Returns the list [u..., lambda...]."""
    k = create_matrix(prob)
    f = create_source_matrix(prob)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", sp.SparseEfficiencyWarning)
        x = spla.spsolve(k, f, permc_spec='NATURAL', use_umfpack=True)
    return list(x)


def _matrix_sparse(data, row, col):
    """Dict merge then csc_matrix (analysis.py:387-405); the dict sums duplicates
    in triplet order."""
    key = row * (max(int(col.max()), 0) + 1) + col if row.size else row
    order = np.argsort(key, kind="stable")
    ks = key[order]
    starts = np.flatnonzero(np.r_[True, ks[1:] != ks[:-1]]) if ks.size else ks
    vals = np.empty(starts.size)
    ds = data[order]
    ends = np.r_[starts[1:], ks.size]
    for j, (s, e) in enumerate(zip(starts.tolist(), ends.tolist())):
        acc = ds[s]
        for t in range(s + 1, e):
            acc = acc + ds[t]
        vals[j] = acc
    return sp.csc_matrix((vals, (row[order][starts], col[order][starts])))


def k_matrix_sparse(prob: Problem):
    return _matrix_sparse(*k_matrix_data(prob))


def m_matrix_sparse(prob: Problem):
    return _matrix_sparse(*m_matrix_data(prob))


# ---------------------------------------------------------------- large sizes


def reduced_system(prob: Problem):
    """Eliminated SPD system: K with the constrained DOFs removed and their values
    moved to the right-hand side.  Returns (A_ff, b_f, free dofs, bc dofs, bc values,
    full K (no multipliers), F loads)."""
    data, row, col = k_matrix_data(prob)
    nd = prob.n_dof
    K = sp.csr_matrix((data, (row, col)), shape=(nd, nd))
    lk, lv = node_loads(prob)
    F = np.zeros(nd)
    np.add.at(F, lk, lv)
    for r, v in zip(*magnet_source(prob)):
        F[r] += v
    bc_dof, bc_val = boundary_conditions(prob)
    mask = np.ones(nd, bool)
    mask[bc_dof] = False
    free = np.flatnonzero(mask)
    g = np.zeros(nd)
    g[bc_dof] = bc_val
    b = F - K @ g
    return K[free][:, free].tocsc(), b[free], free, bc_dof, bc_val, K, F


def solve_reduced(prob: Problem, method="direct", tol=1e-12, maxiter=200000):
    """Solution [u..., lambda...] from the eliminated system: SuperLU with COLAMD
    ("direct") or scipy CG with Jacobi ("cg").  Used where NATURAL spsolve on the
    saddle system does not fit in host memory; the multipliers come from
    lambda_k = (F - K u)[p_k], the first block row of the saddle system."""
    A, b, free, bc_dof, bc_val, K, F = reduced_system(prob)
    if method == "direct":
        uf = spla.spsolve(A, b, permc_spec='COLAMD')
    else:
        dinv = 1.0 / A.diagonal()
        M = spla.LinearOperator(A.shape, matvec=lambda v: dinv * v)
        uf, info = spla.cg(A, b, rtol=tol, atol=0.0, maxiter=maxiter, M=M)
    u = np.zeros(prob.n_dof)
    u[free] = uf
    u[bc_dof] = bc_val
    lam = (F - K @ u)[bc_dof]
    return np.concatenate([u, lam])


# ---------------------------------------------------------------- post-processing


def elastic_post(prob: Problem, u):
    """Per-element strain B q, stress (D B) q and energy 0.5 (q^T Ke) q
    (results.py:809-830, elements.py:275-292)."""
    d, nl = prob.dim, prob.npe * prob.dim
    q = np.asarray(u)[: prob.n_dof].reshape(-1, d)[prob.conn].reshape(-1, nl)
    p = element_points(prob)
    if prob.kind == ELASTIC3D:
        B = tet_b_matrix(p)
        D = d_matrix_3d(prob.E, prob.nu, prob.plane_strain, prob.plane_stress)
    else:
        B = b_matrix(p)
        D = d_matrix(prob.E, prob.nu, prob.plane_strain, prob.plane_stress)
    strain = np.einsum("eij,ej->ei", B, q)
    stress = np.einsum("eij,ej->ei", np.matmul(D, B), q)
    ke = element_stiffness(prob).reshape(-1, nl, nl)
    energy = 0.5 * np.einsum("ei,eij,ej->e", q, ke, q)
    return strain, stress, energy


def magnetic_field(prob: Problem, a):
    """Per-element (Bx, By) = (sum c_i A_i, -sum b_i A_i) (results.py:121-152)."""
    ff = form_functions(element_points(prob))
    A = np.asarray(a)[: prob.n_nodes][prob.conn]
    bx = (ff[:, :, 2] * A).sum(axis=1)
    by = -(ff[:, :, 1] * A).sum(axis=1)
    return np.stack([bx, by], axis=1)


def modal_analysis(prob: Problem, order, k):
    """The reference's modal_analysis (analysis.py:741-796) as written: 'largest' is
    eigsh(K, M=M, which='LM', k) on the matrices without conditions; 'smallest' is
    eigs(inv(K_dense) M, which='LM', k) and returns 1 / eigenvalues (complex).  K has
    no conditions here, so for a body that is free to move it is singular and the
    'smallest' branch inverts it anyway (scipy warns of an ill-conditioned matrix)."""
    import scipy.linalg
    K = k_matrix_sparse(prob)
    M = m_matrix_sparse(prob)
    if order == "largest":
        vals, vecs = spla.eigsh(A=K, M=M, which="LM", k=k)
        return vals, vecs.T
    if order == "smallest":
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            kinv = sp.csc_matrix(scipy.linalg.inv(K.toarray()))
        vals, vecs = spla.eigs(kinv @ M, which="LM", k=k)
        return 1 / vals, vecs.T
    raise ValueError("Order parameter should be either 'largest' or 'smallest'")


def generalized_eigenpairs(prob: Problem, k, which="smallest", sigma=-1.0):
    """The exact k smallest (shift-invert about sigma < 0) or largest eigenpairs of
    K v = lambda M v, by increasing eigenvalue: (values, vectors (k, n) of unit 2-norm)."""
    K = k_matrix_sparse(prob)
    M = m_matrix_sparse(prob)
    if which == "smallest":
        vals, vecs = spla.eigsh(K, k=k, M=M, sigma=sigma, which="LM")
    else:
        vals, vecs = spla.eigsh(K, k=k, M=M, which="LM")
    order = np.argsort(vals)
    vecs = vecs[:, order].T
    return vals[order], vecs / np.linalg.norm(vecs, axis=1, keepdims=True)
