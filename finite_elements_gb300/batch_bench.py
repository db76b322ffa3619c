"""Batched solve of many uneven plane-stress instances against solving them one at a
time, both on the GPU with the library's mixed-precision PCG (FP64 recurrence, FP32
node-block Jacobi + Chebyshev preconditioner of the same degree) to the same relative
residual.

    python -m finite_elements_gb300.batch_bench [--n 512] [--seed 0] [--tol 1e-8]
    python -m torch.distributed.run --nproc-per-node N --master-addr 127.0.0.1 \
        -m finite_elements_gb300.batch_bench      # the instances sharded over N GPUs

Instances: triangle counts log-uniform in [2e3, 2e5], structured grids of aspect
ratio U(1, 8), E ~ U(50, 300) GPa, nu ~ U(0.2, 0.4), random right-edge loads.  Prints
one JSON line: DOF/s of the batch (device time of assembly + solve, and wall time
through the Python API) and of the one-at-a-time loop (wall time per instance: handle,
assembly, solve).
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import meshgen
from .batch import BatchedSystem, shard_instances
from .engine import GpuSystem


def run_sharded(a, probs_all, world):
    """One rank of N: the instances of its shard (shard_instances) batched on its own GPU;
    the ranks share only the barriers around the timed region and the reductions of the
    results.  Rank 0 prints the line: DOF/s = all instances' DOF over the slowest rank's
    device time (strong scaling: the total work is fixed)."""
    import ctypes

    import torch
    import torch.distributed as td

    from . import _lib
    if world > len(probs_all):
        # an empty shard would have no batch to build while the other ranks wait in the
        # barrier: refuse before any rank joins the group
        raise SystemExit(f"batch_bench: {world} ranks for {len(probs_all)} instances; use at most one rank "
                         "per instance")
    td.init_process_group("gloo")
    rank = td.get_rank()
    _lib.check(_lib.load().fe_set_device(int(os.environ.get("LOCAL_RANK", rank))), "fe_set_device")
    shard = shard_instances([p.n_dof for p in probs_all], world)[rank]
    probs = [probs_all[i] for i in shard]
    w = BatchedSystem(probs[:4])
    w.set_preconditioner(a.cheb, a.cheb_ratio)
    w.solve(tol=a.tol, want_x=False)
    w.close()
    b = BatchedSystem(probs)
    b.set_preconditioner(a.cheb, a.cheb_ratio)
    tiles = b.autotune()
    b.solve(tol=a.tol, want_x=False)                      # graph capture
    h = b.system.handle
    td.barrier()
    h.call("fe_event_record", 0)
    h.call("fe_assemble", 1 | 4 | 8)
    h.call("fe_event_record", 1)
    h.call("fe_synchronize")
    ms = ctypes.c_double()
    h.call("fe_event_elapsed_ms", 0, 1, ctypes.byref(ms))
    parts, st = b.solve(tol=a.tol, want_x=False)
    dev_s = (ms.value + st["solve_ms"]) / 1e3
    b.close()
    t = torch.tensor([dev_s, float(st["relres"].max()), float(st["iterations"].max())], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    c = torch.tensor([float(sum(p.n_dof for p in probs)), float((st["status"] == 0).sum()), float(len(probs))],
                     dtype=torch.float64)
    td.all_reduce(c, op=td.ReduceOp.SUM)
    if rank == 0:
        print(json.dumps({
            "workload": f"{len(probs_all)} plane-stress instances sharded over {world} GPUs (seed {a.seed})",
            "n_gpus": world, "scaling": "strong", "tol": a.tol,
            "instances": int(c[2]), "instances_converged": int(c[1]), "worst_relres": float(t[1]),
            "max_iterations": int(t[2]), "tiles_rank0": tiles,
            "slowest_rank_device_s": float(t[0]), "dof_per_s_device": float(c[0]) / float(t[0])}))
    td.destroy_process_group()


def measure(a, probs):
    """The batched solve of `probs` on this GPU against `a.single` of them (-1: all) solved
    one at a time; returns the result line as a dict."""
    dof = int(sum(p.n_dof for p in probs))
    tri = int(sum(p.n_elements for p in probs))
    # warm-up of the library (kernels, allocator) on a small batch
    w = BatchedSystem(probs[:4])
    w.set_preconditioner(a.cheb, a.cheb_ratio)
    w.solve(tol=a.tol, want_x=False)
    w.close()

    t0 = time.perf_counter()
    b = BatchedSystem(probs)
    b.set_preconditioner(a.cheb, a.cheb_ratio)
    t_setup = time.perf_counter() - t0
    tiles = b.autotune()
    b.solve(tol=a.tol, want_x=False)                      # graph capture
    # timed: assembly of the union on the device (pattern + elements + reduction + loads +
    # conditions + SELL copies), then the solve, which re-runs the per-instance
    # Chebyshev-interval probe for the new system
    import ctypes
    h = b.system.handle
    h.call("fe_event_record", 0)
    h.call("fe_assemble", 1 | 4 | 8)
    h.call("fe_event_record", 1)
    h.call("fe_synchronize")
    ms = ctypes.c_double()
    h.call("fe_event_elapsed_ms", 0, 1, ctypes.byref(ms))
    asm_ms = ms.value
    t1 = time.perf_counter()
    parts, st = b.solve(tol=a.tol, want_x=True)
    t_solve_wall = time.perf_counter() - t1
    run = b.last_run()
    ok = int((st["status"] == 0).sum())
    worst = float(st["relres"].max())
    b.close()

    n_single = len(probs) if a.single < 0 else min(a.single, len(probs))
    t2 = time.perf_counter()
    single_dev_ms = 0.0
    single_dof = 0
    for p in probs[:n_single]:
        s = GpuSystem(p)
        _, s1 = s.solve(precision="mixed-cg64", tol=a.tol, cheb_degree=a.cheb if a.cheb > 1 else 0,
                        cheb_ratio=a.cheb_ratio, want_host=True)
        single_dev_ms += s1.solve_ms + s1.assemble_ms
        single_dof += p.n_dof
        s.close()
    t_single = time.perf_counter() - t2
    batched_dev_s = (asm_ms + st["solve_ms"]) / 1e3
    out = {
        "workload": f"{a.n} plane-stress instances, {tri:,} triangles, {dof:,} DOF in total "
                    f"(2e3..2e5 triangles each, seed {a.seed})",
        "tol": a.tol, "instances_converged": ok, "worst_relres": worst,
        "tiles": tiles, "max_iterations": int(st["iterations"].max()), "persistent_kernel": run,
        "preconditioner": {"chebyshev_terms": a.cheb, "ratio": a.cheb_ratio},
        "batched": {"assemble_ms": asm_ms, "solve_ms": st["solve_ms"],
                    "dof_per_s_device": dof / batched_dev_s,
                    "solve_wall_s": t_solve_wall, "setup_wall_s": t_setup},
        "one_at_a_time": {"instances": n_single, "wall_s": t_single, "device_s": single_dev_ms / 1e3,
                          "dof_per_s_wall": single_dof / t_single,
                          "dof_per_s_device": single_dof / (single_dev_ms / 1e3)},
    }
    out["speedup_device"] = out["batched"]["dof_per_s_device"] / out["one_at_a_time"]["dof_per_s_device"]
    out["speedup_wall"] = out["batched"]["dof_per_s_device"] / out["one_at_a_time"]["dof_per_s_wall"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--single", type=int, default=-1, help="instances solved one at a time (-1: all)")
    ap.add_argument("--cheb", type=int, default=16, help="Chebyshev terms of the preconditioner (1: Jacobi)")
    ap.add_argument("--cheb-ratio", type=float, default=1e4)
    a = ap.parse_args()
    probs = meshgen.batch_c4(a.n, seed=a.seed)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        run_sharded(a, probs, world)
        return
    print(json.dumps(measure(a, probs)))


if __name__ == "__main__":
    main()
