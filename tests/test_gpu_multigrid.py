"""Multigrid-preconditioned PCG (FP64 recurrence, FP32 smoothed-aggregation V-cycle)
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
        x, st = s.solve(precision="fp64", tol=1e-12, multigrid=True, accept_stagnation=True)
    finally:
        s.close()
    assert st.status == 0, st.as_dict()
    assert st.iterations <= 80, st.as_dict()
    assert np.linalg.norm(x - ref) <= 1e-9 * np.linalg.norm(ref), st.as_dict()


@pytest.mark.parametrize("name", ["plane_strain", "tet", "magnetic"])
def test_device_setup_matches_the_host_passes(gpu_lib, name):
    """fe_amg_build_device against fe_amg_build_parallel_host on the device's own level-0
    matrix: the same level-0 aggregates (integer passes on identical block norms), the
    same prolongator and coarse operator within 1e-10, and PCG with the host V-cycle on
    the device hierarchy converging."""
    import ctypes

    from finite_elements_gb300 import _lib
    from finite_elements_gb300.engine import GpuSystem
    from oracle import amg_oracle as AMG
    from test_amg_parallel_host import build, read_levels
    prob = _problems()[name]()
    s = GpuSystem(prob)
    lib = _lib.load()
    h = ctypes.c_void_p()
    try:
        _lib.check(lib.fe_amg_build_device(s.handle.h, 0.08, 400, ctypes.byref(h)), "fe_amg_build_device")
        dev = read_levels(lib, h)
        d = prob.dim
        A0 = dev[0]["A"]
        if d == 1:
            B = np.ones((A0.shape[0], 1))
        elif d == 2:
            B = AMG.rigid_modes_2d(prob.coords)
        else:
            B = AMG.rigid_modes_3d(prob.coords)
        B[s.bc_dof] = 0.0
        lib2, h2, host = build(A0, B, d)
        lib2.fe_amg_destroy(h2)
        np.testing.assert_array_equal(dev[0]["agg"], host[0]["agg"])
        assert abs(dev[0]["P"] - host[0]["P"]).max() <= 1e-10 * abs(host[0]["P"]).max()
        assert abs(dev[1]["A"] - host[1]["A"]).max() <= 1e-10 * abs(host[1]["A"]).max()
        b = np.random.default_rng(1).standard_normal(A0.shape[0])
        b[s.bc_dof] = 0.0

        def M(v):
            v = np.ascontiguousarray(v)
            out = np.empty_like(v)
            lib.fe_amg_vcycle_host(h, 3, _lib.ptr(v), _lib.ptr(out))
            return out
        x, it = AMG.pcg(A0, b, M)
        assert np.linalg.norm(A0 @ x - b) <= 1e-8 * np.linalg.norm(b) and it <= 60, it
    finally:
        if h.value:
            lib.fe_amg_destroy(h)
        s.close()


@pytest.mark.parametrize("name", ["plane_strain", "tet", "magnetic"])
def test_device_coarsest_inverse_is_the_inverse(gpu_lib, name):
    """With a coarsest size above the system's, the device hierarchy has no level and its
    coarsest inverse is that of the whole system (3782, 624 and 1891 DOFs: 119, 20 and
    60 block sweeps of 32 pivots, the last ones partial): the V-cycle is then x = A^-1 r
    for A with 1e-12 of its largest diagonal entry added to the diagonal (which moves
    the identity rows of the constrained DOFs), checked by its residual and symmetry."""
    import ctypes

    from finite_elements_gb300 import _lib
    from finite_elements_gb300.engine import GpuSystem
    from test_amg_parallel_host import read_levels
    prob = _problems()[name]()
    s = GpuSystem(prob)
    lib = _lib.load()
    h = ctypes.c_void_p()
    try:
        _lib.check(lib.fe_amg_build_device(s.handle.h, 0.08, 1 << 20, ctypes.byref(h)), "fe_amg_build_device")
        levels = read_levels(lib, h)
        assert len(levels) == 1
        import scipy.sparse as sp
        A = levels[0]["A"].tocsr()
        A = (A + 1e-12 * abs(A.diagonal()).max() * sp.eye(A.shape[0])).tocsr()
        rng = np.random.default_rng(2)
        r1, r2 = rng.standard_normal(A.shape[0]), rng.standard_normal(A.shape[0])

        def apply(v):
            v = np.ascontiguousarray(v)
            out = np.empty_like(v)
            _lib.check(lib.fe_amg_vcycle_host(h, 3, _lib.ptr(v), _lib.ptr(out)), "fe_amg_vcycle_host")
            return out
        x1, x2 = apply(r1), apply(r2)
        assert np.linalg.norm(A @ x1 - r1) <= 1e-9 * np.linalg.norm(r1)
        assert np.linalg.norm(A @ x2 - r2) <= 1e-9 * np.linalg.norm(r2)
        assert abs(r2 @ x1 - r1 @ x2) <= 1e-12 * abs(r1) @ abs(x2)
    finally:
        if h.value:
            lib.fe_amg_destroy(h)
        s.close()


def test_memory_pool_is_shared_and_trimmed(gpu_lib):
    """Two handles solve through the device's shared multigrid pool, which
    fe_trim_memory_pools empties between them; the solutions are bitwise equal."""
    from finite_elements_gb300 import _lib
    from finite_elements_gb300.engine import GpuSystem
    prob = _problems()["plane_strain"]()
    kw = dict(precision="mixed-cg64", tol=1e-10, multigrid=True, accept_stagnation=True)
    s1 = GpuSystem(prob)
    x1, st1 = s1.solve(**kw)
    s1.close()
    _lib.check(_lib.load().fe_trim_memory_pools(0), "fe_trim_memory_pools")
    s2 = GpuSystem(prob)
    x2, st2 = s2.solve(**kw)
    s2.close()
    assert st1.status == 0 and st2.status == 0
    np.testing.assert_array_equal(x1, x2)
