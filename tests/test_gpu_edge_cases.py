"""Edge cases of the assembly-and-solve path on the GPU, each against the oracle or
an exact answer: no loads (the solution is the prescribed field, zero multipliers),
displacement-driven problems (prescribed values only), a single element, every
precision on them, and calls made in the wrong order (statuses, no fault)."""
import numpy as np
import pytest

from finite_elements_gb300.problem import ELASTIC, MAGNETIC, Problem

pytestmark = pytest.mark.gpu

PRECISIONS = ["fp64", "mixed-cg64", "mixed"]


def strip(nx=6, ny=3, **kw):
    from finite_elements_gb300 import meshgen
    c, conn = meshgen.rect_grid(nx, ny, 2.0, 1.0)
    ne = len(conn)
    left = np.flatnonzero(np.abs(c[:, 0]) < 1e-12)
    right = np.flatnonzero(np.abs(c[:, 0] - 2.0) < 1e-12)
    return Problem(ELASTIC, c, conn, E=np.full(ne, 210e9), nu=np.full(ne, 0.3), thickness=np.full(ne, 1e-3),
                   rho=np.full(ne, 7800.0), plane_strain=False, plane_stress=True, **kw), left, right


@pytest.mark.parametrize("precision", PRECISIONS)
def test_no_loads_gives_the_prescribed_field(gpu_lib, precision):
    from finite_elements_gb300.engine import GpuSystem
    prob, left, _ = strip()
    prob.node_bc_node = np.repeat(left, 2)
    prob.node_bc_dim = np.tile([1, 2], left.size)
    prob.node_bc_value = np.zeros(2 * left.size)
    s = GpuSystem(prob)
    x, st = s.solve(precision=precision, tol=1e-10)
    assert st.status == 0
    assert np.all(x == 0.0)
    s.close()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_displacement_driven_strip_matches_oracle(gpu_lib, precision):
    """Left edge clamped, right edge pulled by a prescribed 1e-4 in x, no loads."""
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob, left, right = strip()
    prob.node_bc_node = np.concatenate([np.repeat(left, 2), right])
    prob.node_bc_dim = np.concatenate([np.tile([1, 2], left.size), np.ones(right.size, np.int64)])
    prob.node_bc_value = np.concatenate([np.zeros(2 * left.size), np.full(right.size, 1e-4)])
    ref = np.array(O.solve(prob))
    s = GpuSystem(prob)
    x, st = s.solve(precision=precision, tol=1e-12 if precision != "mixed" else 1e-9, accept_stagnation=True)
    assert st.status == 0, st.as_dict()
    n = prob.n_dof
    assert np.linalg.norm(x[:n] - ref[:n]) <= 1e-8 * np.linalg.norm(ref[:n])
    # the reactions (multipliers) balance: the sum over the pulled edge equals minus the clamped edge's
    lam = x[n:]
    assert abs(lam[-right.size:].sum() + lam[:2 * left.size][0::2].sum()) <= 1e-6 * np.abs(lam).max()
    s.close()


def test_single_element(gpu_lib):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    c = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    prob = Problem(ELASTIC, c, [[0, 1, 2]], E=[1e9], nu=[0.25], thickness=[1.0], rho=[1.0],
                   plane_strain=True, plane_stress=False,
                   node_load_node=[1], node_load_dim=[1], node_load_value=[100.0],
                   node_bc_node=[0, 0, 2], node_bc_dim=[1, 2, 1], node_bc_value=[0.0, 0.0, 0.0])
    ref = np.array(O.solve(prob))
    s = GpuSystem(prob)
    x, st = s.solve(precision="fp64", tol=1e-14, accept_stagnation=True)
    assert st.status == 0
    assert np.linalg.norm(x - ref) <= 1e-12 * np.linalg.norm(ref)
    s.close()


def test_single_magnetic_element(gpu_lib):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    c = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    prob = Problem(MAGNETIC, c, [[0, 1, 2]], mu=[4e-7 * np.pi],
                   node_load_node=[1], node_load_dim=[1], node_load_value=[2.0],
                   node_bc_node=[0], node_bc_dim=[1], node_bc_value=[0.0])
    ref = np.array(O.solve(prob))
    s = GpuSystem(prob)
    x, st = s.solve(precision="fp64", tol=1e-14, accept_stagnation=True)
    assert st.status == 0
    assert np.linalg.norm(x - ref) <= 1e-12 * np.linalg.norm(ref)
    s.close()


def test_calls_in_the_wrong_order_return_statuses(gpu_lib):
    """A handle that has a mesh but nothing assembled: solve, exports, modal and
    post-processing report FE_NOT_READY (or FE_BAD_INPUT), with a message."""
    import ctypes
    from finite_elements_gb300 import _lib
    prob, _, _ = strip()
    lib = _lib.load()
    h = _lib.Handle(_lib.FE_KIND_ELASTIC_TRI, prob.coords, prob.conn)
    o = _lib.SolveOpts()
    st = _lib.SolveStats()
    assert lib.fe_solve(h.h, o, None, st) == _lib.FE_NOT_READY
    a = np.zeros(prob.n_dof)
    assert lib.fe_modal(h.h, 0, 2, 0.0, 0, 0, _lib.ptr(a), _lib.ptr(a), _lib.ptr(a)) == _lib.FE_NOT_READY
    nr, nc, nz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    assert lib.fe_export_sizes(h.h, _lib.FE_MAT_K_AUGMENTED, nr, nc, nz) == _lib.FE_NOT_READY
    assert lib.fe_get_solution(h.h, _lib.ptr(a)) == _lib.FE_NOT_READY
    assert lib.fe_last_error()
    h.close()
