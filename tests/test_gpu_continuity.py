"""Continuity conditions and magnet loads on the GPU against the oracle (the
reference's create_matrix / create_source_matrix / spsolve restated).

Continuity conditions are solved by a projected FP64 PCG; the solution [u, lambda,
mu] must match spsolve on the reference's saddle-point system within 1e-10 relative,
and every condition must hold to 1e-12 of |u|.  Magnet loads are additive
right-hand-side entries: F within 1e-14 of the oracle's."""
import numpy as np
import pytest

from finite_elements_gb300 import meshgen
from finite_elements_gb300.problem import MAGNETIC, ElementLoadSet, MagnetLoadSet, Problem

pytestmark = pytest.mark.gpu


def periodic_problem(nx, ny, anti=False, seed=0):
    """Magnetostatics on an nx-by-ny grid: A = 0 on the bottom and top edges, the
    interior nodes of the left edge linked to those of the right edge (value 1, or -1
    with anti), a current load, and as many zero NodeLoads as Dirichlet conditions so
    that the reference's continuity rows follow its Dirichlet rows."""
    rng = np.random.default_rng(seed)
    coords, conn = meshgen.rect_grid(nx, ny, nx / ny, 1.0, jitter=0.2, rng=rng)
    ne = conn.shape[0]
    w = nx + 1
    bottom, top = list(range(w)), [ny * w + i for i in range(w)]
    left, right = [j * w for j in range(1, ny)], [j * w + nx for j in range(1, ny)]
    bc = bottom + top
    src = np.flatnonzero(np.arange(ne) % 9 == 4)
    return Problem(MAGNETIC, coords, conn, mu=np.full(ne, meshgen.MU0),
                   element_loads=[ElementLoadSet(src, 1e3, 1)],
                   node_load_node=np.full(len(bc), w + 1), node_load_dim=np.ones(len(bc), np.int64),
                   node_load_value=np.zeros(len(bc)),
                   node_bc_node=bc, node_bc_dim=np.ones(len(bc), np.int64), node_bc_value=np.zeros(len(bc)),
                   cont_node1=left, cont_node2=right, cont_value=np.full(len(left), -1.0 if anti else 1.0))


@pytest.mark.parametrize("anti", [False, True])
def test_periodic_matches_spsolve(gpu_lib, anti):
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob = periodic_problem(48, 24, anti)
    ref = np.array(O.solve(prob))
    s = GpuSystem(prob)
    x, st = s.solve(precision="fp64", tol=1e-13, accept_stagnation=True)
    assert st.status == 0, st.as_dict()
    assert x.shape == ref.shape
    assert np.linalg.norm(x - ref) <= 1e-10 * np.linalg.norm(ref), st.as_dict()
    u = x[: prob.n_dof]
    v = prob.cont_value
    assert np.abs(u[prob.cont_node1] - v * u[prob.cont_node2]).max() <= 1e-12 * np.abs(u).max()
    # create_matrix / create_source_matrix as the reference builds them
    K, R = s.create_matrix(), O.create_matrix(prob)
    np.testing.assert_array_equal(K.indices, R.indices)
    np.testing.assert_array_equal(K.indptr, R.indptr)
    assert np.abs(K.data - R.data).max() <= 1e-13 * np.abs(R.data).max()
    F, G = s.create_source_matrix(), O.create_source_matrix(prob)
    assert F.shape == G.shape and np.abs(F - G).max() <= 1e-14 * np.abs(G).max()
    s.close()


def test_chained_conditions(gpu_lib):
    """Trees longer than one link: node a = b, b = -c, c = d (values 1, -1, 0.5)."""
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    prob = periodic_problem(16, 8)
    w = 17
    a, b, c, d = 3 * w + 4, 3 * w + 9, 5 * w + 9, 6 * w + 2
    prob.cont_node1 = np.r_[prob.cont_node1, [a, b, d]]
    prob.cont_node2 = np.r_[prob.cont_node2, [b, c, c]]
    prob.cont_value = np.r_[prob.cont_value, [1.0, -1.0, 0.5]]
    prob.node_load_node = np.r_[prob.node_load_node, np.zeros(0, np.int64)]
    ref = np.array(O.solve(prob))
    s = GpuSystem(prob)
    x, st = s.solve(precision="fp64", tol=1e-13, accept_stagnation=True)
    assert st.status == 0
    assert np.linalg.norm(x - ref) <= 1e-10 * np.linalg.norm(ref)
    u = x[: prob.n_dof]
    assert abs(u[a] - u[b]) <= 1e-12 * np.abs(u).max() and abs(u[b] + u[c]) <= 1e-12 * np.abs(u).max()
    assert abs(u[d] - 0.5 * u[c]) <= 1e-12 * np.abs(u).max()
    s.close()


def test_cycles_and_dirichlet_overlap_are_refused(gpu_lib):
    from finite_elements_gb300 import _lib
    from finite_elements_gb300.engine import GpuSystem
    prob = periodic_problem(8, 4)
    prob.cont_node1 = np.r_[prob.cont_node1, prob.cont_node2[0]]
    prob.cont_node2 = np.r_[prob.cont_node2, prob.cont_node1[0]]
    prob.cont_value = np.r_[prob.cont_value, 1.0]
    with pytest.raises(_lib.FeError) as e:
        GpuSystem(prob)
    assert e.value.status == _lib.FE_BAD_INPUT
    prob = periodic_problem(8, 4)
    prob.cont_node1 = np.r_[prob.cont_node1, 0]          # node 0 carries A = 0
    prob.cont_node2 = np.r_[prob.cont_node2, 20]
    prob.cont_value = np.r_[prob.cont_value, 1.0]
    s = GpuSystem(prob)
    with pytest.raises(_lib.FeError) as e:
        s.solve(precision="fp64")
    assert e.value.status == _lib.FE_BAD_INPUT
    s.close()


def test_magnet_loads_match_oracle(gpu_lib):
    """A 120x60 magnetostatic grid with two magnets, one with a non-contour edge."""
    from finite_elements_gb300.engine import GpuSystem
    from oracle import fe_oracle as O
    nx, ny = 120, 60
    coords, conn = meshgen.rect_grid(nx, ny, 0.12, 0.06)
    ne = conn.shape[0]
    w = nx + 1
    boundary = sorted(set(list(range(w)) + [ny * w + i for i in range(w)] + [j * w for j in range(ny + 1)]
                          + [j * w + nx for j in range(ny + 1)]))
    block1 = [2 * (j * nx + i) + t for j in range(20, 30) for i in range(30, 50) for t in (0, 1)]
    block2 = [2 * (j * nx + i) + t for j in range(35, 40) for i in range(70, 72) for t in (0, 1)]
    mu = np.full(ne, meshgen.MU0)
    mu[block1] *= 1.05
    prob = Problem(MAGNETIC, coords, conn, mu=mu,
                   node_bc_node=boundary, node_bc_dim=np.ones(len(boundary), np.int64),
                   node_bc_value=np.zeros(len(boundary)),
                   magnet_loads=[MagnetLoadSet(np.array(block1), np.array([20 * w + 30, 20 * w + 31]), (9e5, 0.0)),
                                 MagnetLoadSet(np.array(block2), np.zeros(0, np.int64), (0.0, -4e5))])
    s = GpuSystem(prob)
    F, G = s.create_source_matrix(), O.create_source_matrix(prob)
    assert np.abs(F - G).max() <= 1e-14 * np.abs(G).max()
    x, st = s.solve(precision="fp64", tol=1e-12, accept_stagnation=True)
    ref = O.solve_reduced(prob)
    n = prob.n_dof
    assert np.linalg.norm(x[:n] - ref[:n]) <= 1e-9 * np.linalg.norm(ref[:n])
    s.close()
