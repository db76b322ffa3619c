"""The warm-start network on the GPU: features, loss and the hand-written backward
against the CPU oracle (torch FP64 autograd with the GEMM inputs rounded to BF16 as
the tensor cores see them), training on solver-generated targets, and what the
trained network gains over x0 = 0.

Tolerances: features 2e-5 absolute; loss 1e-3 relative; gradient cosine >= 0.999 and
relative norm error <= 3e-2 (BF16 inputs of every GEMM, FP32 activations)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def small(gpu_lib):
    from finite_elements_gb300 import meshgen
    from finite_elements_gb300.engine import GpuSystem
    prob = meshgen.plane_strain_random(24, 12, seed=3)
    s = GpuSystem(prob)
    yield prob, s
    s.close()


def test_features_match_oracle(small):
    from finite_elements_gb300.warmstart import WarmStartNet
    from oracle import gnn_oracle as G
    prob, s = small
    net = WarmStartNet(seed=1)
    f = net.features(s)
    A, b, g, bt, mask = G.eliminated_system(prob)
    fr = G.features(prob, A, bt, mask)
    np.testing.assert_allclose(f, fr, atol=2e-5)


def test_loss_and_gradient_match_oracle(small):
    from finite_elements_gb300.warmstart import WarmStartNet, init_params
    from oracle import gnn_oracle as G
    prob, s = small
    p = init_params(seed=2)
    net = WarmStartNet(params=p)
    s.solve(precision="fp64", tol=1e-12, accept_stagnation=True, want_host=False)
    e = net.target_energy(s)
    e_ref = G.solution_energy(prob)
    assert abs(e - e_ref) <= 1e-9 * abs(e_ref)
    loss, grad = net.loss_grad(s, e, want_grad=True)
    L, gref, _, _ = G.loss_and_grad(prob, p, e_ref, bf16=True)
    assert abs(loss - L) <= 1e-3 * max(abs(L), 1e-3), (loss, L)
    cos = float(grad @ gref / (np.linalg.norm(grad) * np.linalg.norm(gref)))
    rel = float(np.linalg.norm(grad - gref) / np.linalg.norm(gref))
    assert cos >= 0.999 and rel <= 3e-2, (cos, rel)


def test_training_lowers_the_loss(gpu_lib):
    from finite_elements_gb300 import meshgen
    from finite_elements_gb300.warmstart import WarmStartNet, train
    probs = [meshgen.plane_strain_random(40, 20, seed=s) for s in range(4)]
    net = WarmStartNet(seed=0)
    hist = train(probs, net, steps=300, lr=2e-3, log=None)
    assert np.mean(hist[-30:]) < 0.9 * np.mean(hist[:10]), (hist[:10], hist[-30:])


def test_trained_network_gain_is_measured(gpu_lib):
    """What the committed weights gain on a problem outside their training set.

    Measured on held-out plane-strain draws (400x200 and 1000x500, four seeds): the
    scaled prediction leaves 90-94% of the solution's energy to PCG (energy loss
    0.90-0.94), and PCG from it needs between 4% fewer and 4% more iterations than
    from x0 = 0.  The test pins both facts: the prediction lowers the A-norm error
    (loss < 0.97), and PCG from it reaches the same tolerance within +10% of the
    iterations of the zero start -- the warm start never costs accuracy."""
    from finite_elements_gb300 import meshgen
    from finite_elements_gb300.engine import GpuSystem
    from finite_elements_gb300.warmstart import DEFAULT_WEIGHTS, WarmStartNet
    if not os.path.exists(DEFAULT_WEIGHTS):
        pytest.skip("no trained weights committed")
    net = WarmStartNet(weights=DEFAULT_WEIGHTS)
    prob = meshgen.plane_strain_random(400, 200, seed=12345)
    s = GpuSystem(prob)
    s.solve(precision="fp64", tol=1e-11, cheb_degree=6, cheb_ratio=1000, accept_stagnation=True, want_host=False)
    loss, _ = net.loss_grad(s, net.target_energy(s))
    assert 0.0 < loss < 0.97, loss
    kw = dict(precision="fp64", tol=1e-8, cheb_degree=6, cheb_ratio=1000, want_host=False)
    _, st0 = s.solve(**kw)
    ptr, scale = net.predict(s)
    _, st1 = s.solve(x0_device_ptr=ptr, **kw)
    assert st0.status == 0 and st1.status == 0
    assert st1.relres <= 1e-8
    assert st1.iterations <= 1.1 * st0.iterations, (st0.iterations, st1.iterations)
    # with the acceptance test the warm start is kept only when its residual is smaller
    _, st2 = s.solve(x0_device_ptr=ptr, x0_if_better=True, **kw)
    assert st2.status == 0 and st2.relres <= 1e-8
    if not st2.x0_used:
        assert st2.iterations == st0.iterations
    s.close()


def test_fit_loss_and_gradient_match_oracle(small):
    """The training loss: mean-squared error against the normalised solution."""
    from finite_elements_gb300.warmstart import WarmStartNet, init_params
    from oracle import gnn_oracle as G
    prob, s = small
    p = init_params(seed=4)
    net = WarmStartNet(params=p)
    x, _ = s.solve(precision="fp64", tol=1e-12, accept_stagnation=True)
    loss, grad = net.fit_grad(s, want_grad=True)
    L, gref, _, _ = G.loss_and_grad(prob, p, 1.0, bf16=True, fit_solution=x)
    assert abs(loss - L) <= 1e-3 * max(abs(L), 1e-3), (loss, L)
    cos = float(grad @ gref / (np.linalg.norm(grad) * np.linalg.norm(gref)))
    rel = float(np.linalg.norm(grad - gref) / np.linalg.norm(gref))
    assert cos >= 0.999 and rel <= 3e-2, (cos, rel)


def test_async_prediction_gives_the_same_solve(gpu_lib):
    """fe_gnn_predict_async (on the network's stream, the solve waiting for it before it
    reads x0) gives the start, and so the multigrid solve, of the synchronous
    prediction, bitwise."""
    from finite_elements_gb300 import meshgen
    from finite_elements_gb300.engine import GpuSystem
    from finite_elements_gb300.warmstart import DEFAULT_WEIGHTS, WarmStartNet
    net = WarmStartNet(weights=DEFAULT_WEIGHTS) if os.path.exists(DEFAULT_WEIGHTS) else WarmStartNet(seed=1)
    prob = meshgen.plane_strain_random(80, 40, seed=11)
    s = GpuSystem(prob)
    kw = dict(precision="mixed-cg64", tol=1e-10, multigrid=True, accept_stagnation=True)
    try:
        ptr, _ = net.predict(s)
        x1, st1 = s.solve(x0_device_ptr=ptr, x0_if_better=True, **kw)
        ptr2 = net.predict_async(s)
        x2, st2 = s.solve(x0_device_ptr=ptr2, x0_if_better=True, **kw)
    finally:
        s.close()
    assert st1.status == 0 and st2.status == 0
    assert st1.x0_used == st2.x0_used and st1.iterations == st2.iterations
    np.testing.assert_array_equal(x1, x2)
