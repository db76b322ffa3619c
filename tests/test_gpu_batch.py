"""Batched solve of uneven instances against solving each one on its own (same
library, FP64, tight tolerance) and against the oracle's direct solve for a few.

Tolerance: per instance ||u_batch - u_single|| <= 1e-8 ||u_single|| at tol 1e-10 (true
residual within 3x the tolerance: the recurrence residual stops at tol, the FP64
true residual sits at or slightly above it)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(n=12, seed=3):
    from finite_elements_gb300 import meshgen
    return meshgen.batch_c4(n, seed=seed, tri_min=200, tri_max=8000)


def test_batch_matches_single_solves(gpu_lib):
    from finite_elements_gb300.batch import BatchedSystem
    from finite_elements_gb300.engine import GpuSystem
    probs = _instances()
    b = BatchedSystem(probs)
    parts, st = b.solve(tol=1e-10)
    assert (st["status"] == 0).all(), st
    assert (st["relres"] <= 3e-10).all(), st["relres"]
    for k, p in enumerate(probs):
        s = GpuSystem(p)
        x, s1 = s.solve(precision="fp64", tol=1e-13, accept_stagnation=True)
        s.close()
        u = x[: p.n_dof]
        assert np.linalg.norm(parts[k] - u) <= 1e-8 * np.linalg.norm(u), k
    b.close()


def test_batch_against_oracle(gpu_lib):
    from finite_elements_gb300.batch import BatchedSystem
    from oracle import fe_oracle as O
    probs = _instances(4, seed=9)
    b = BatchedSystem(probs)
    parts, st = b.solve(tol=1e-12)
    for k, p in enumerate(probs[:2]):
        ref = np.array(O.solve(p))[: p.n_dof]
        assert np.linalg.norm(parts[k] - ref) <= 1e-9 * np.linalg.norm(ref)
    b.close()


def test_autotune_and_tiles(gpu_lib):
    from finite_elements_gb300.batch import BatchedSystem
    probs = _instances(6, seed=4)
    b = BatchedSystem(probs)
    tiles = b.autotune()
    assert tiles["lanes"] in (1, 2, 4) and tiles["rows_per_chunk"] >= 256
    x1, st1 = b.solve(tol=1e-10)
    b.set_tiles(1, 256)
    x2, st2 = b.solve(tol=1e-10)
    for a, c in zip(x1, x2):
        assert np.linalg.norm(a - c) <= 1e-8 * np.linalg.norm(c)
    b.close()


def test_batch_iteration_cap(gpu_lib):
    from finite_elements_gb300.batch import BatchedSystem
    b = BatchedSystem(_instances(5, seed=1))
    _, st = b.solve(tol=1e-12, max_iter=3)
    assert (st["status"] == 1).all() and (st["iterations"] <= 3).all()
    b.close()
