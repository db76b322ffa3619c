"""The host smoothed-aggregation setup of libfe_gb300 (fe_amg_build_host, no device
call) against the CPU model oracle/amg_oracle.py on the benchmark family: the same
aggregates at every level, prolongators and Galerkin coarse operators within 1e-10,
the same number of levels, and the model's PCG converging with the library's
hierarchy as with its own."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from finite_elements_gb300 import _lib, meshgen
from oracle import amg_oracle as AMG
from oracle import fe_oracle as O


def to_block_csr(A, d):
    """Node-block CSR (ptr, col, vals) of a scipy matrix with d x d blocks."""
    n = A.shape[0] // d
    Ab = sp.bsr_matrix(A, blocksize=(d, d))
    Ab.sort_indices()
    return n, Ab.indptr.astype(np.int64), Ab.indices.astype(np.int32), np.ascontiguousarray(Ab.data.reshape(-1))


def from_block_csr(ptr, col, val, rd, cd, n_cols):
    n = ptr.size - 1
    return sp.bsr_matrix((val.reshape(-1, rd, cd), col, ptr), shape=(n * rd, n_cols * cd)).tocsr()


def build(A, B, d, theta=0.08, coarse=400):
    lib = _lib.load()
    n, ptr, col, val = to_block_csr(A, d)
    Bc = np.ascontiguousarray(B, np.float64)
    h = ctypes.c_void_p()
    _lib.check(lib.fe_amg_build_host(n, d, _lib.ptr(ptr), _lib.ptr(col), _lib.ptr(val), B.shape[1], _lib.ptr(Bc),
                                     theta, coarse, ctypes.byref(h)), "fe_amg_build_host")
    nl = ctypes.c_int32()
    lib.fe_amg_levels(h, ctypes.byref(nl))
    levels = []
    for l in range(nl.value + 1):
        nn, dd, na_, np_, nc, m = (ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64(),
                                   ctypes.c_int64(), ctypes.c_int32())
        lm = ctypes.c_double()
        lib.fe_amg_level_info(h, l, nn, dd, na_, np_, nc, m, ctypes.byref(lm))
        p = np.empty(nn.value + 1, np.int64)
        c = np.empty(max(na_.value, 1), np.int32)
        v = np.empty(max(na_.value, 1) * dd.value ** 2)
        lib.fe_amg_level_matrix(h, l, 0, _lib.ptr(p), _lib.ptr(c), _lib.ptr(v))
        Al = from_block_csr(p, c[:na_.value], v[:na_.value * dd.value ** 2], dd.value, dd.value, nn.value)
        lev = {"A": Al, "lmax": lm.value}
        if l < nl.value:
            pp = np.empty(nn.value + 1, np.int64)
            pc = np.empty(np_.value, np.int32)
            pv = np.empty(np_.value * dd.value * m.value)
            lib.fe_amg_level_matrix(h, l, 1, _lib.ptr(pp), _lib.ptr(pc), _lib.ptr(pv))
            lev["P"] = from_block_csr(pp, pc, pv, dd.value, m.value, nc.value)
            agg = np.empty(nn.value, np.int32)
            lib.fe_amg_level_aggregates(h, l, _lib.ptr(agg))
            lev["agg"] = agg
        levels.append(lev)
    lib.fe_amg_destroy(h)
    return levels


@pytest.mark.parametrize("nx,ny", [(30, 15), (80, 40)])
def test_hierarchy_matches_the_model(nx, ny):
    prob = meshgen.plane_strain_random(nx, ny, seed=1)
    A, b, free, *_ = O.reduced_system(prob)
    A = A.tocsr()
    B = AMG.rigid_modes_2d(prob.coords[free[0::2] // 2])
    ours = build(A, B, 2)
    model = AMG.SmoothedAggregation(A, B)
    assert len(ours) == len(model.levels) + 1
    Am = A
    d = 2
    Bm = B
    for l, (Aref, Minv, lm, P) in enumerate(model.levels):
        agg, na = AMG.aggregate(Aref, d)
        np.testing.assert_array_equal(ours[l]["agg"], agg)
        assert abs(ours[l]["lmax"] - lm) <= 1e-10 * lm
        assert abs(ours[l]["A"] - Aref).max() <= 1e-10 * abs(Aref).max()
        assert abs(ours[l]["P"] - P).max() <= 1e-10 * abs(P).max()
        d = 3
    Ac = model.levels[-1][3].T @ model.levels[-1][0] @ model.levels[-1][3]
    assert abs(ours[-1]["A"] - Ac).max() <= 1e-10 * abs(Ac).max()


def test_pcg_with_the_library_hierarchy():
    """The model's V-cycle on the library's operators converges as with its own."""
    prob = meshgen.plane_strain_random(60, 30, seed=2)
    A, b, free, *_ = O.reduced_system(prob)
    A = A.tocsr()
    B = AMG.rigid_modes_2d(prob.coords[free[0::2] // 2])
    model = AMG.SmoothedAggregation(A, B)
    _, it_model = AMG.pcg(A, b, model)
    ours = build(A, B, 2)
    # swap in the library's levels
    d = 2
    levels = []
    for lev in ours[:-1]:
        Minv = AMG.block_diag_inv(lev["A"], d)
        levels.append((lev["A"], Minv, lev["lmax"], lev["P"]))
        d = 3
    model.levels = levels
    model.smooth = [AMG.chebyshev(Al, Minv, lm, 30.0, model.k) for Al, Minv, lm, _ in levels]
    import scipy.sparse.linalg as spla
    Ac = sp.csc_matrix(ours[-1]["A"])
    model.lu = spla.splu(sp.csc_matrix(Ac + 1e-12 * abs(Ac.diagonal()).max() * sp.eye(Ac.shape[0])))
    x, it = AMG.pcg(A, b, model)
    assert abs(it - it_model) <= 1, (it, it_model)
    assert np.linalg.norm(A @ x - b) <= 1e-8 * np.linalg.norm(b)


def _check_against_model(A, B, d):
    ours = build(A, B, d)
    model = AMG.SmoothedAggregation(A, B, d=d)
    assert len(ours) == len(model.levels) + 1
    dd = d
    for l, (Aref, Minv, lm, P) in enumerate(model.levels):
        agg, na = AMG.aggregate(Aref, dd)
        np.testing.assert_array_equal(ours[l]["agg"], agg)
        assert abs(ours[l]["lmax"] - lm) <= 1e-10 * lm
        assert abs(ours[l]["P"] - P).max() <= 1e-10 * abs(P).max()
        dd = B.shape[1]
    Ac = model.levels[-1][3].T @ model.levels[-1][0] @ model.levels[-1][3]
    assert abs(ours[-1]["A"] - Ac).max() <= 1e-10 * abs(Ac).max()
    return model


def test_tetrahedra_with_six_rigid_modes():
    prob = meshgen.cantilever_3d(12, 4, 4, jitter=0.2, seed=3)
    A, b, free, *_ = O.reduced_system(prob)
    A = A.tocsr()
    B = AMG.rigid_modes_3d(prob.coords[free[0::3] // 3])
    model = _check_against_model(A, B, 3)
    x, it = AMG.pcg(A, b, model)
    assert np.linalg.norm(A @ x - b) <= 1e-8 * np.linalg.norm(b) and it <= 40, it


def test_magnetostatics_with_the_constant_mode():
    prob = meshgen.magnetostatic(60, 30, seed=1)
    A, b, free, *_ = O.reduced_system(prob)
    A = A.tocsr()
    B = np.ones((A.shape[0], 1))
    model = _check_against_model(A, B, 1)
    x, it = AMG.pcg(A, b, model)
    assert np.linalg.norm(A @ x - b) <= 1e-8 * np.linalg.norm(b) and it <= 40, it


def _library_handle(A, B, d):
    lib = _lib.load()
    n, ptr, col, val = to_block_csr(A, d)
    Bc = np.ascontiguousarray(B, np.float64)
    h = ctypes.c_void_p()
    _lib.check(lib.fe_amg_build_host(n, d, _lib.ptr(ptr), _lib.ptr(col), _lib.ptr(val), B.shape[1], _lib.ptr(Bc),
                                     0.08, 400, ctypes.byref(h)), "fe_amg_build_host")
    return lib, h


@pytest.mark.parametrize("case", ["plane_strain", "tet", "magnetic"])
def test_host_vcycle_matches_the_model(case):
    """fe_amg_vcycle_host (the row operations of the device cycle, run serially) gives
    the model's V-cycle on the same hierarchy, and PCG preconditioned by it converges
    in the model's iteration count."""
    if case == "plane_strain":
        prob = meshgen.plane_strain_random(60, 30, seed=4)
        d, modes = 2, lambda xy: AMG.rigid_modes_2d(xy)
    elif case == "tet":
        prob = meshgen.cantilever_3d(10, 4, 4, jitter=0.2, seed=5)
        d, modes = 3, lambda xy: AMG.rigid_modes_3d(xy)
    else:
        prob = meshgen.magnetostatic(50, 25, seed=2)
        d, modes = 1, None
    A, b, free, *_ = O.reduced_system(prob)
    A = A.tocsr()
    B = np.ones((A.shape[0], 1)) if modes is None else modes(prob.coords[free[0::d] // d])
    lib, h = _library_handle(A, B, d)
    ours = build(A, B, d)
    model = AMG.SmoothedAggregation(A, B, d=d)
    dd, levels = d, []
    for lev in ours[:-1]:
        levels.append((lev["A"], AMG.block_diag_inv(lev["A"], dd), lev["lmax"], lev["P"]))
        dd = B.shape[1]
    model.levels = levels
    model.smooth = [AMG.chebyshev(Al, Minv, lm, 30.0, model.k) for Al, Minv, lm, _ in levels]
    import scipy.sparse.linalg as spla
    Ac = sp.csc_matrix(ours[-1]["A"])
    model.lu = spla.splu(sp.csc_matrix(Ac + 1e-12 * abs(Ac.diagonal()).max() * sp.eye(Ac.shape[0])))
    r = np.random.default_rng(0).standard_normal(A.shape[0])
    x = np.empty_like(r)
    _lib.check(lib.fe_amg_vcycle_host(h, 3, _lib.ptr(r), _lib.ptr(x)), "fe_amg_vcycle_host")
    xm = model(r)
    assert np.linalg.norm(x - xm) <= 1e-9 * np.linalg.norm(xm)

    def M(v):
        v = np.ascontiguousarray(v)
        out = np.empty_like(v)
        lib.fe_amg_vcycle_host(h, 3, _lib.ptr(v), _lib.ptr(out))
        return out
    xs, it = AMG.pcg(A, b, M)
    _, it_model = AMG.pcg(A, b, model)
    assert abs(it - it_model) <= 1 and np.linalg.norm(A @ xs - b) <= 1e-8 * np.linalg.norm(b)
    lib.fe_amg_destroy(h)
