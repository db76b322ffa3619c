"""The warm-start network's CPU oracle (torch autograd) against central finite
differences -- no GPU needed."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_oracle_gradient_matches_finite_differences():
    from finite_elements_gb300 import meshgen
    from oracle import gnn_oracle as G
    prob = meshgen.plane_strain_random(8, 4, seed=3)
    rng = np.random.default_rng(0)
    sizes = [16 * 64, 64] + [128 * 64, 64, 64 * 64] * 6 + [128, 2]
    p = np.concatenate([rng.uniform(-0.3, 0.3, s) for s in sizes])
    e = G.solution_energy(prob)
    L, g, u, f = G.loss_and_grad(prob, p, e)
    assert 0.0 <= L <= 1.0
    for idx in [3, 1100, 9000, 40000, 75100, 75329]:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (G.loss_and_grad(prob, pp, e)[0] - G.loss_and_grad(prob, pm, e)[0]) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-5 * max(1.0, abs(fd)), (idx, fd, g[idx])
