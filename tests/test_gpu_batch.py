"""Batched solve of uneven instances (the persistent-kernel mixed-precision PCG)
against solving each one on its own and against the oracle's direct solve.

Tolerances: per instance ||u_batch - u_single|| <= 1e-8 ||u_single|| at tol 1e-10, the
single solve run to its FP64 floor (the FP64 true residual of the batch must meet the
tolerance: fe_batch_solve restarts an instance whose true residual missed it); against
the oracle 1e-9 at tol 1e-12.  Runs are deterministic: two solves of the same batch are
bitwise equal."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(n=12, seed=3):
    from finite_elements_gb300 import meshgen
    return meshgen.batch_c4(n, seed=seed, tri_min=200, tri_max=8000)


@pytest.mark.parametrize("degree", [1, 16])
def test_batch_matches_single_solves(gpu_lib, degree):
    from finite_elements_gb300.batch import BatchedSystem
    from finite_elements_gb300.engine import GpuSystem
    probs = _instances()
    b = BatchedSystem(probs)
    b.set_preconditioner(degree, 1e4)
    parts, st = b.solve(tol=1e-10)
    assert (st["status"] == 0).all(), st
    assert (st["relres"] <= 1e-10).all(), st["relres"]
    run = b.last_run()
    assert run["kernel_launches"] >= 1 and run["grid"] >= 152
    for k, p in enumerate(probs):
        s = GpuSystem(p)
        x, s1 = s.solve(precision="fp64", tol=1e-13, accept_stagnation=True)
        s.close()
        u = x[: p.n_dof]
        assert np.linalg.norm(parts[k] - u) <= 1e-8 * np.linalg.norm(u), k
    b.close()


def test_batch_chebyshev_cuts_iterations_and_replays_a_graph(gpu_lib):
    """Each instance's own Chebyshev interval: degree 16 needs several times fewer
    iterations than node-block Jacobi (3.2x to 4.3x on these small instances); the chunks
    replay from the captured graph."""
    from finite_elements_gb300.batch import BatchedSystem
    probs = _instances(8, seed=6)
    b = BatchedSystem(probs)
    b.set_preconditioner(1, 1e4)
    _, sj = b.solve(tol=1e-9)
    b.set_preconditioner(16, 1e4)
    _, sc = b.solve(tol=1e-9)
    assert (sj["status"] == 0).all() and (sc["status"] == 0).all()
    assert (sc["iterations"] * 2.5 <= sj["iterations"]).all(), (sc["iterations"], sj["iterations"])
    run = b.last_run()
    assert run["uses_graph"] and run["graph_launches"] >= 1, run
    b.close()


def test_batch_is_deterministic(gpu_lib):
    from finite_elements_gb300.batch import BatchedSystem
    b = BatchedSystem(_instances(10, seed=7))
    x1, s1 = b.solve(tol=1e-9)
    x2, s2 = b.solve(tol=1e-9)
    np.testing.assert_array_equal(s1["iterations"], s2["iterations"])
    for a, c in zip(x1, x2):
        np.testing.assert_array_equal(a, c)
    b.close()


def test_batch_against_oracle(gpu_lib):
    from finite_elements_gb300.batch import BatchedSystem
    from oracle import fe_oracle as O
    probs = _instances(4, seed=9)
    b = BatchedSystem(probs)
    parts, st = b.solve(tol=1e-12)
    assert (st["status"] == 0).all(), st
    for k, p in enumerate(probs[:2]):
        ref = np.array(O.solve(p))[: p.n_dof]
        assert np.linalg.norm(parts[k] - ref) <= 1e-9 * np.linalg.norm(ref)
    b.close()


def test_autotune_and_tiles(gpu_lib):
    from finite_elements_gb300.batch import BatchedSystem
    probs = _instances(6, seed=4)
    b = BatchedSystem(probs)
    tiles = b.autotune()
    assert tiles["blocks_per_sm"] >= 1 and tiles["slices_per_item"] in (1, 2, 4, 8)
    assert tiles["us_per_iteration"] > 0
    x1, st1 = b.solve(tol=1e-10)
    b.set_tiles(1, 1)
    x2, st2 = b.solve(tol=1e-10)
    assert b.last_run()["grid"] >= 152
    for a, c in zip(x1, x2):
        assert np.linalg.norm(a - c) <= 1e-8 * np.linalg.norm(c)
    b.close()


def test_batch_iteration_cap(gpu_lib):
    from finite_elements_gb300.batch import BatchedSystem
    b = BatchedSystem(_instances(5, seed=1))
    _, st = b.solve(tol=1e-12, max_iter=3)
    assert (st["status"] == 1).all() and (st["iterations"] <= 3).all()
    b.close()


def test_batch_bad_arguments(gpu_lib):
    from finite_elements_gb300 import _lib
    from finite_elements_gb300.batch import BatchedSystem
    b = BatchedSystem(_instances(2, seed=2))
    with pytest.raises(_lib.FeError):
        b.set_preconditioner(0, 1e4)
    with pytest.raises(_lib.FeError):
        b.set_tiles(1, 0)
    b.close()
