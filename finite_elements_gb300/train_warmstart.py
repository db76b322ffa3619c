"""Train the warm-start network on solutions the library's own PCG produces, then
report what it gains on held-out problems.

    python -m finite_elements_gb300.train_warmstart [--n-train 300] [--steps 3000]
           [--out finite_elements_gb300/weights/warmstart_gnn.npz] [--eval-nx 2000]

Training problems (seeded): half plane-strain grids with per-element E = 10**U(9,12)
clamped on the left and loaded on the top edge (the distribution of the 4M-DOF
benchmark problem), half smooth Gaussian-random-field E fields with a random clamped
side and random loads on the opposite side; 20k-200k triangles each.  Held-out
evaluation: the benchmark's own 2000x1000 problem (seed 0, not in the training set)
and a 2000x1000 random-field draw.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import meshgen
from .engine import GpuSystem
from .warmstart import DEFAULT_WEIGHTS, WarmStartNet, init_params, save_weights, train


def training_problems(n, seed=1000):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        tri = float(np.exp(rng.uniform(np.log(2e4), np.log(2e5))))
        aspect = rng.uniform(1.5, 3.0)
        ny = max(8, int(round(np.sqrt(tri / (2 * aspect)))))
        nx = max(8, int(round(tri / (2 * ny))))
        s = int(rng.integers(1 << 30))
        if k % 2 == 0:
            out.append(meshgen.plane_strain_random(nx, ny, seed=s, lx=nx / ny, ly=1.0))
        else:
            out.append(meshgen.grf_elasticity(nx, ny, seed=s))
    return out


def evaluate(net, prob, label, solve_kw):
    s = GpuSystem(prob)
    s.solve(want_host=False, **solve_kw)                  # warm-up (graph capture, eigen estimate)
    _, st0 = s.solve(want_host=False, **solve_kw)
    t = time.perf_counter()
    ptr, scale = net.predict(s)
    x, st1 = s.solve(want_host=True, x0_device_ptr=ptr, **solve_kw)
    wall = time.perf_counter() - t
    s.close()
    r = {"problem": label, "dof": prob.n_dof, "iterations_x0_zero": st0.iterations,
         "iterations_x0_learned": st1.iterations, "solve_ms_x0_zero": st0.solve_ms,
         "solve_ms_x0_learned": st1.solve_ms, "predict_and_solve_wall_s": wall,
         "relres_learned": st1.relres, "status": [st0.status, st1.status]}
    print(json.dumps(r), flush=True)
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-train", type=int, default=300)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--eval-nx", type=int, default=2000)
    ap.add_argument("--init", default=None, help="start from these weights")
    a = ap.parse_args()
    t0 = time.perf_counter()
    probs = training_problems(a.n_train)
    net = WarmStartNet(weights=a.init) if a.init else WarmStartNet(params=init_params(a.seed))
    hist = train(probs, net, steps=a.steps, lr=a.lr, seed=a.seed)
    params = net.get_params()
    save_weights(a.out, params, meta={"loss_history": hist, "n_train": a.n_train, "steps": a.steps})
    print(f"trained in {time.perf_counter() - t0:.1f}s, final running loss "
          f"{np.mean(hist[-100:]):.4f}, saved {a.out}", flush=True)
    if a.eval_nx > 0:
        kw = dict(precision="mixed", tol=1e-8, cheb_degree=3)
        evaluate(net, meshgen.plane_strain_random(a.eval_nx, a.eval_nx // 2, seed=0), "benchmark problem", kw)
        evaluate(net, meshgen.grf_elasticity(a.eval_nx, a.eval_nx // 2, seed=777), "random-field draw", kw)


if __name__ == "__main__":
    main()
