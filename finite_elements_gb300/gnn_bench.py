"""Throughput of the warm-start network on one plane-strain mesh: inference (features,
six message-passing layers, decoder and smoothing, the scale) and one training step
(the same forward, the hand-written backward through the tcgen05 GEMMs, Adam), both
through the library's C ABI on the handle's stream, timed by wall clock around
synchronising calls after warm-up.

    python -m finite_elements_gb300.gnn_bench [--nx 2000 --ny 1000] [--reps 5]

Prints one JSON line: milliseconds per inference and per training step, and mesh nodes
per second for each.
"""
from __future__ import annotations

import argparse
import json
import time


def measure(nx, ny, reps=5, seed=0):
    """Times predict and loss_grad + adam_step on an nx x ny plane-strain grid."""
    from . import meshgen
    from .engine import GpuSystem
    from .warmstart import WarmStartNet

    prob = meshgen.plane_strain_random(nx, ny, seed=seed)
    s = GpuSystem(prob)
    net = WarmStartNet(seed=1)
    try:
        s.solve(precision="mixed-cg64", tol=1e-8, multigrid=True, want_host=False)
        energy = net.target_energy(s)
        for _ in range(2):
            net.predict(s)
            net.loss_grad(s, energy, want_grad=False)
        t0 = time.perf_counter()
        for _ in range(reps):
            net.predict(s)                    # ends with a read of two device sums
        t_pred = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            net.loss_grad(s, energy, want_grad=False)
            net.adam_step(1e-4)
        s.handle.call("fe_synchronize")
        t_train = (time.perf_counter() - t0) / reps
        return {"workload": f"{nx}x{ny} plane-strain grid ({prob.n_nodes:,} nodes, {prob.n_dof:,} DOF)",
                "predict_ms": 1e3 * t_pred, "train_step_ms": 1e3 * t_train,
                "predict_nodes_per_s": prob.n_nodes / t_pred, "train_nodes_per_s": prob.n_nodes / t_train,
                "gemms": "tcgen05.mma kind::f16 (BF16 in, FP32 accumulators in tensor memory): per layer the "
                         "N x 128 x 64 forward product, and in training the N x 64 x 128 data gradient and the "
                         "128 x 64 weight gradient over N rows"}
    finally:
        net.close()
        s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=2000)
    ap.add_argument("--ny", type=int, default=1000)
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args()
    print(json.dumps(measure(a.nx, a.ny, a.reps)))


if __name__ == "__main__":
    main()
