#!/usr/bin/env python3
"""Benchmark of the assembly-and-solve path: seconds per solve to a 1e-8 relative
residual on the 4M-DOF plane-strain elasticity problem.

One step = one full solve of the reference's FiniteElementAnalysis.solve() kind:
pattern build, element kernels, segmented reduction, loads, Dirichlet elimination
and PCG, from inputs already resident in HBM (``value``), and the same through the
C ABI from host buffers, with the uploads of the mesh, materials, loads and
conditions and the download of [u, lambda] inside the timed region (``e2e``).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --workload tet      # secondary: 4M-DOF tetrahedral elasticity

Prints one JSON line (rank 0).  With N > 1 (torchrun) every rank solves its own
replica of the problem on its own GPU: the path has no data exchange between GPUs.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# DRAM bytes (read + write) per launch of the roofline kernel (the intermediate FP32
# Chebyshev step) from ncu captures of this workload, keyed by (grid, bytes of the
# L2-resident prefix): plain loads (profiles/cheb_step_fp32_plane_strain_4M.md) and the
# default 40 MB prefix (steady state of a run of steps,
# profiles/cheb_step_fp32_keep_plane_strain_4M.md); None for other workloads.
NCU_TRAFFIC = {(2000, 1000, 0): 278_710_784, (2000, 1000, 40_000_000): 265_900_000}
# The same for the multigrid roofline kernel (level 0's Chebyshev smoothing step of the
# V-cycle), the mean over its two timed launches, the first step from zero and the
# second, keyed by the grid (profiles/launches_multigrid_plane_strain_4M.md).
NCU_TRAFFIC_MG = {(2000, 1000): 266_744_832}

METRIC = "s/solve to 1e-8 rel. residual, 4M-DOF elasticity: mixed+learned vs plain PCG"
UNIT = "s/solve"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--nx", type=int, default=2000)
    ap.add_argument("--ny", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--cheb", type=int, default=96, help="Chebyshev degree of the mixed solve's preconditioner")
    ap.add_argument("--cheb-ratio", type=float, default=100000.0, help="Chebyshev interval lmax/lmin (mixed)")
    ap.add_argument("--plain-cheb", type=int, default=32, help="Chebyshev degree of the plain FP64 PCG")
    ap.add_argument("--plain-cheb-ratio", type=float, default=30000.0, help="Chebyshev interval (plain FP64)")
    ap.add_argument("--ir-cheb", type=int, default=16,
                    help="Chebyshev degree of the FP32-Krylov + iterative-refinement solve reported beside")
    ap.add_argument("--ir-cheb-ratio", type=float, default=3000.0)
    ap.add_argument("--no-learned", action="store_true", help="headline without the learned warm start")
    ap.add_argument("--quick", action="store_true",
                    help="headline steps only (no plain / oracle / e2e legs), for profiler runs")
    ap.add_argument("--quick-plain", action="store_true",
                    help="with --quick: time the plain FP64 PCG step instead of the headline")
    ap.add_argument("--quick-multigrid", action="store_true",
                    help="--quick with --solver multigrid")
    ap.add_argument("--profile", action="store_true",
                    help="with --quick: keep the live kernel and setup-phase timing on and report it")
    ap.add_argument("--solver", choices=("multigrid", "chebyshev"), default="multigrid",
                    help="preconditioner of the headline mixed-precision solve: the FP32 smoothed-aggregation "
                         "V-cycle (set up on the device every step) or node-block Jacobi + Chebyshev in FP32")
    ap.add_argument("--plain-steps", type=int, default=2, help="timed plain FP64 solves beside the headline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-n", type=int, default=512,
                    help="instances of the batched-solve leg (0: no batched leg)")
    ap.add_argument("--batch-single", type=int, default=64,
                    help="of them, solved one at a time for the comparison (-1: all)")
    ap.add_argument("--l2-keep", type=float, default=-1.0,
                    help="MB of the FP32 preconditioner matrix kept L2-resident across Chebyshev steps "
                         "(default: the library's 40 MB; 0 = plain loads)")
    ap.add_argument("--workload", choices=("plane_strain", "tet"), default="plane_strain",
                    help="tet: the secondary 3D line (solid cantilever of linear tetrahedra)")
    ap.add_argument("--tet-dims", type=int, nargs=3, default=(320, 64, 64),
                    help="cells of the tetrahedral cantilever (6 tetrahedra per cell)")
    ap.add_argument("--tet-cheb", type=int, default=24, help="Chebyshev degree of the 3D mixed solve")
    ap.add_argument("--tet-cheb-ratio", type=float, default=10000.0, help="its interval lmax/lmin")
    a = ap.parse_args()
    if a.quick_multigrid:
        a.quick, a.solver = True, "multigrid"
    return a


# ---------------------------------------------------------------- multi-process plumbing

class Dist:
    """Rank bookkeeping; with WORLD_SIZE > 1 a gloo group provides the barrier and the
    max over ranks (timing only: the solves exchange no data)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        for p in self.samples:
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for name, flag in zip(self.NAMES, p[3:7]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU baseline (oracle)

def cpu_direct_solve(prob):
    """The reference path on the host cores at the workload's full size, measured: the
    oracle's restatement of finite_elements' element and assembly code (vectorised over
    elements, so faster than the reference's per-element loop), Dirichlet elimination,
    and SuperLU -- the library of the reference's spsolve call (analysis.py:820-822) --
    on the eliminated SPD system, ordered by minimum degree on A^T + A.  The reference's
    own call (NATURAL order on the saddle system) does not fit in host memory at 4M DOF;
    this is the fastest direct method scipy offers for the same system.  SuperLU runs on
    one core.  Returns ([u, lambda], seconds, timings)."""
    from oracle import fe_oracle as O
    tm = {}
    t0 = time.perf_counter()
    x = O.solve_reduced(prob, "direct", timings=tm)
    return x, time.perf_counter() - t0, tm


CPU_METHOD = ("reduced-system direct: oracle assembly (COO, csr_matrix), Dirichlet elimination, SuperLU "
              "splu on the eliminated SPD system (MMD_AT_PLUS_A order, symmetric mode) -- not the "
              "reference's exact call, spsolve NATURAL on the saddle system, which does not fit in host "
              "memory at this size")


def cpu_info():
    try:
        model = [l.split(":", 1)[1].strip() for l in open("/proc/cpuinfo") if l.lower().startswith(("model name",))]
        model = model[0] if model else os.uname().machine
    except OSError:
        model = os.uname().machine
    return model, os.cpu_count()


# ---------------------------------------------------------------- our path

def run_ours(args, dist):
    import ctypes

    import numpy as np

    from finite_elements_gb300 import _lib, meshgen
    from finite_elements_gb300.engine import GpuSystem

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    if dist.world > 1:
        # one process per GPU: this rank's replica runs on its local device
        _lib.check(_lib.load().fe_set_device(dist.local_rank), "fe_set_device")
    prob = meshgen.plane_strain_random(args.nx, args.ny, seed=args.seed)
    s = GpuSystem(prob, assemble=True)           # inputs uploaded: resident in HBM from here
    h = s.handle
    if args.l2_keep >= 0:
        h.call("fe_set_l2_keep", int(args.l2_keep * 1e6))
    step_flags = _lib.FE_ASSEMBLE_PATTERN | _lib.FE_ASSEMBLE_K | _lib.FE_ASSEMBLE_F
    # headline: FP64 CG recurrence with an FP32 preconditioner -- the smoothed-aggregation
    # V-cycle, or node-block Jacobi + Chebyshev -- and the other one beside it, the
    # FP32-Krylov + iterative-refinement form and the plain FP64 PCG
    mg_mode = dict(precision="mixed-cg64", tol=args.tol, multigrid=True, want_host=False)
    cheb_mode = dict(precision="mixed-cg64", tol=args.tol, cheb_degree=args.cheb, cheb_ratio=args.cheb_ratio,
                     want_host=False)
    mode, other = (mg_mode, cheb_mode) if args.solver == "multigrid" else (cheb_mode, mg_mode)
    ir_mode = dict(precision="mixed", tol=args.tol, cheb_degree=args.ir_cheb, cheb_ratio=args.ir_cheb_ratio,
                   want_host=False)
    plain = dict(precision="fp64", tol=args.tol, cheb_degree=args.plain_cheb, cheb_ratio=args.plain_cheb_ratio,
                 want_host=False)
    net = None
    if not args.no_learned:
        from finite_elements_gb300.warmstart import DEFAULT_WEIGHTS, WarmStartNet
        if os.path.exists(DEFAULT_WEIGHTS):
            net = WarmStartNet(weights=DEFAULT_WEIGHTS)

    def device_step(opts, learned=False):
        h.call("fe_assemble", step_flags)
        if learned and net is not None:
            # the warm start is part of the step: predicted on the network's stream while
            # the solve sets up its hierarchy, the solve waiting for it before it reads x0
            ptr = net.predict_async(s)
            _, st = s.solve(x0_device_ptr=ptr, x0_if_better=True, **opts)
        else:
            _, st = s.solve(**opts)
        if st.status != _lib.FE_OK:
            raise RuntimeError(f"solve failed: {st.as_dict()}")
        return st

    def launches():
        c = ctypes.c_int64()
        h.call("fe_launch_count", ctypes.byref(c))
        return c.value

    def profile_read(precision):
        cm, cn, sm, sn = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64()
        h.call("fe_profile_read", precision, ctypes.byref(cm), ctypes.byref(cn), ctypes.byref(sm), ctypes.byref(sn))
        return {"cheb_us": 1e3 * cm.value / max(cn.value, 1), "cheb_n": cn.value,
                "spmv_us": 1e3 * sm.value / max(sn.value, 1), "spmv_n": sn.value}

    if args.quick and args.quick_plain:
        # profiler runs of the plain FP64 step: no event records, no other legs
        for _ in range(args.warmup):
            device_step(plain)
        h.call("fe_synchronize")
        h.call("fe_event_record", 0)
        pst = [device_step(plain) for _ in range(args.steps)]
        h.call("fe_event_record", 1)
        h.call("fe_synchronize")
        ms = ctypes.c_double()
        h.call("fe_event_elapsed_ms", 0, 1, ctypes.byref(ms))
        s.close()
        return {"metric": METRIC, "plain_s_per_solve": ms.value / 1e3 / args.steps, "quick": True,
                "iterations": pst[-1].iterations}

    # event records around the first iteration of every chunk of the captured PCG
    # loop time the kernels inside the measured solves (not in profiler runs)
    live_prof = 0 if (args.quick and not args.profile) else 1
    h.call("fe_profile_kernels", live_prof)
    for _ in range(args.warmup):
        device_step(mode, learned=True)

    # ---- headline: mixed precision, inputs resident in HBM
    clocks = ClockSampler(dist.local_rank)
    dist.barrier()
    h.call("fe_synchronize")
    h.call("fe_profile_kernels", live_prof)   # reset the kernel-time sums
    l0 = launches()
    clocks.start()
    h.call("fe_event_record", 0)
    stats = [device_step(mode, learned=True) for _ in range(args.steps)]
    h.call("fe_event_record", 1)
    h.call("fe_synchronize")
    clk = clocks.stop()
    n_launch = launches() - l0
    prof_mixed = profile_read(_lib.FE_PREC_MIXED_CG64)
    ms = ctypes.c_double()
    h.call("fe_event_elapsed_ms", 0, 1, ctypes.byref(ms))
    mg_prof = None
    if args.solver == "multigrid":
        v = [ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(),
             ctypes.c_int64()]
        h.call("fe_profile_read_multigrid", *[ctypes.byref(x) for x in v])
        ph = (ctypes.c_double * _lib.FE_MG_PHASES)()
        h.call("fe_profile_read_multigrid_phases", ph, _lib.FE_MG_PHASES)
        mg_prof = {"smooth_us": 1e3 * v[0].value / max(v[1].value, 1), "smooth_n": v[1].value,
                   "setup_ms": v[2].value / max(v[3].value, 1), "cycle_ms": v[4].value / max(v[5].value, 1),
                   "cycles": v[5].value,
                   "setup_phases_ms": {name: ph[k] / max(v[3].value, 1) for k, name in enumerate(_lib.MG_PHASE_NAMES)}}
    dist.barrier()
    t_total = dist.max(ms.value / 1e3)
    value = t_total / (args.steps * dist.world)
    x_mixed = np.empty(prob.n_dof + len(s.bc_dof))
    h.call("fe_get_solution", _lib.ptr(x_mixed))
    if args.quick:
        s.close()
        return {"metric": METRIC, "value": value, "unit": UNIT, "quick": True, "solver": args.solver,
                "iterations": stats[-1].iterations, "relres": stats[-1].relres, "solve_ms": stats[-1].solve_ms,
                "assemble_ms": stats[-1].assemble_ms, "learned_x0_used": stats[-1].x0_used,
                "gpu_launches": int(n_launch), "multigrid_profile": mg_prof if args.profile else None}

    # ---- mixed precision without the learned warm start, same step
    h.call("fe_synchronize")
    h.call("fe_event_record", 2)
    nstats = [device_step(mode) for _ in range(max(args.plain_steps, 1))]
    h.call("fe_event_record", 3)
    h.call("fe_synchronize")
    h.call("fe_event_elapsed_ms", 2, 3, ctypes.byref(ms))
    mixed_only_s = ms.value / 1e3 / max(args.plain_steps, 1)

    # ---- the other preconditioner of the mixed solve, same step (with the live timing
    # of the Chebyshev solve's kernels)
    device_step(other)
    h.call("fe_synchronize")
    h.call("fe_profile_kernels", 1)
    h.call("fe_event_record", 2)
    ostats = [device_step(other) for _ in range(max(args.plain_steps, 1))]
    h.call("fe_event_record", 3)
    h.call("fe_synchronize")
    h.call("fe_event_elapsed_ms", 2, 3, ctypes.byref(ms))
    other_s = ms.value / 1e3 / max(args.plain_steps, 1)
    if args.solver == "multigrid":
        prof_mixed = profile_read(_lib.FE_PREC_MIXED_CG64)
    h.call("fe_profile_kernels", 0)

    # ---- FP32 Krylov vectors and SpMV with FP64 iterative refinement, same step
    device_step(ir_mode)
    h.call("fe_synchronize")
    h.call("fe_event_record", 2)
    istats = [device_step(ir_mode) for _ in range(max(args.plain_steps, 1))]
    h.call("fe_event_record", 3)
    h.call("fe_synchronize")
    h.call("fe_event_elapsed_ms", 2, 3, ctypes.byref(ms))
    ir_s = ms.value / 1e3 / max(args.plain_steps, 1)

    # ---- plain FP64 PCG, same step
    device_step(plain)
    h.call("fe_synchronize")
    h.call("fe_profile_kernels", 1)
    h.call("fe_event_record", 2)
    pstats = [device_step(plain) for _ in range(args.plain_steps)]
    h.call("fe_event_record", 3)
    h.call("fe_synchronize")
    h.call("fe_event_elapsed_ms", 2, 3, ctypes.byref(ms))
    plain_s = ms.value / 1e3 / max(args.plain_steps, 1)
    prof_plain = profile_read(_lib.FE_PREC_FP64)
    h.call("fe_profile_kernels", 0)

    n = prob.n_dof
    err, err_ref = None, None
    if dist.world > 1 or args.no_cpu_baseline:
        # no CPU solve on this run: the error against the library's own FP64 PCG to 1e-11
        x_ref, _ = s.solve(precision="fp64", tol=1e-11, cheb_degree=args.plain_cheb,
                           cheb_ratio=args.plain_cheb_ratio, accept_stagnation=True)
        err = float(np.linalg.norm(x_mixed[:n] - x_ref[:n]) / np.linalg.norm(x_ref[:n]))
        err_ref = "the library's FP64 PCG to 1e-11 on the GPU (no CPU solve on this run)"

    # ---- roofline.  Algorithmic bytes per launch (2x2 node blocks, s = value size):
    # off-diagonal blocks (4 s value bytes + 4 column bytes each, 2 for the FP32 kernels'
    # 16-bit offsets) + per node: Chebyshev step --
    # FP64: diagonal block 4s and block-Jacobi inverse 4s; FP32: neither (the copy is
    # prescaled, in difference form; the ~0.1% of rows next to a Dirichlet condition
    # carry one more entry, not counted) -- and z_k, r (D^-1 r in FP32), z_{k-1} read
    # and z_{k+1} written (2s each); PCG SpMV -- diagonal 4s (FP32: A_rr to scale back),
    # p read and q written (2s each); + 4 bytes of slice offset per 32 rows.
    info = s.info()
    nnzb, n_nodes = info["n_blocks"], prob.n_nodes
    nb_off = nnzb - n_nodes
    slices = (n_nodes + 31) // 32 + 1

    col16 = s.sell_info()["col16"]

    def col_bytes(sz):
        return 2 if (sz == 4 and col16) else 4     # FP32 kernels read 16-bit column offsets

    def cheb_bytes(sz):
        diag_and_dinv = 8 * sz if sz == 8 else 0
        return nb_off * (4 * sz + col_bytes(sz)) + n_nodes * (diag_and_dinv + 4 * 2 * sz) + slices * 4

    def spmv_bytes(sz):
        return nb_off * (4 * sz + col_bytes(sz)) + n_nodes * (4 * sz + 2 * 2 * sz) + slices * 4

    def roof(bytes_, us):
        gbs = bytes_ / (us * 1e-6) / 1e9 if us > 0 else None
        return gbs, (gbs / hbm_peak if gbs else None)

    # the V-cycle's level-0 Chebyshev step: k_cheb_step on the prescaled FP32 SELL copy of
    # the eliminated K, as in the Chebyshev solve's steps, with D^-1 r, z_k read and z_k+1
    # written; the old iterate z_k-1 is read by the second of the two timed launches only
    # (the first one's is zero)
    def smooth_bytes():
        return cheb_bytes(4) - n_nodes * 2 * 4 / 2

    cheb_gbs, cheb_frac = roof(cheb_bytes(4), prof_mixed["cheb_us"])
    spmvmp_gbs, spmvmp_frac = roof(spmv_bytes(8), prof_mixed["spmv_us"])
    cheb64_gbs, cheb64_frac = roof(cheb_bytes(8), prof_plain["cheb_us"])
    spmv64_gbs, spmv64_frac = roof(spmv_bytes(8), prof_plain["spmv_us"])
    keep_bytes = 40_000_000 if args.l2_keep < 0 else int(args.l2_keep * 1e6)
    traffic = NCU_TRAFFIC.get((args.nx, args.ny, keep_bytes))
    cheb_line = {"bound": "hbm", "kernel": "k_cheb_step<2,float,double,2,0> (intermediate FP32 Chebyshev step of "
                                           f"the Chebyshev-preconditioned solve: {max(args.cheb - 2, 0)} of the "
                                           f"{args.cheb + 2} kernels of its iteration)",
                 "achieved": cheb_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": cheb_frac,
                 "peak_source": peak_src, "traffic": traffic,
                 "bytes_per_launch": cheb_bytes(4), "launch_us": prof_mixed["cheb_us"],
                 "launches_timed": prof_mixed["cheb_n"],
                 "timing": "CUDA events captured in the PCG graph around the run of intermediate Chebyshev steps "
                           "of the first iteration of each 16-iteration chunk, during the timed solves of that "
                           "solver; launch_us = that time / the launches it covers"}
    if mg_prof is not None:
        sm_gbs, sm_frac = roof(smooth_bytes(), mg_prof["smooth_us"])
        roofline = {"bound": "hbm",
                    "kernel": "k_cheb_step<2,float,float,0,*,1> (level-0 Chebyshev smoothing step of the FP32 "
                              "V-cycle on the prescaled FP32 SELL copy; 5 of the cycle's launches)",
                    "achieved": sm_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": sm_frac, "peak_source": peak_src,
                    "traffic": NCU_TRAFFIC_MG.get((args.nx, args.ny)), "bytes_per_launch": smooth_bytes(),
                    "launch_us": mg_prof["smooth_us"],
                    "launches_timed": mg_prof["smooth_n"],
                    "share_of_step": (mg_prof["smooth_us"] * 5 * 1e-6 * mg_prof["cycles"] / args.steps / value
                                      if value > 0 else None),
                    "timing": "CUDA events captured in the V-cycle graph around the two Chebyshev steps of level "
                              "0's pre-smoothing, read after every cycle of the timed solves; launch_us = that "
                              "time / 2 launches"}
        mg_section = {"setup_ms_per_solve": mg_prof["setup_ms"], "setup_phases_ms": mg_prof["setup_phases_ms"],
                      "cycle_ms": mg_prof["cycle_ms"],
                      "cycles_per_solve": mg_prof["cycles"] / max(args.steps, 1),
                      "level0_smoothing_us_per_launch": mg_prof["smooth_us"]}
    else:
        roofline, mg_section = cheb_line, None
    s.close()

    # ---- end to end through the C ABI, host buffers in and out
    h2d = (prob.coords.nbytes + prob.conn.nbytes + prob.E.nbytes + prob.nu.nbytes + prob.thickness.nbytes
           + prob.rho.nbytes + prob.node_load_node.size * 24 + prob.node_bc_node.size * 16)
    e2e_times = []
    e2e_opts = dict(mode, want_host=True)
    # the step's inputs in pinned host memory (page-locked once, outside the timed region)
    lib = _lib.load()
    pinned = [a for a in (prob.coords, prob.conn, prob.E, prob.nu, prob.thickness, prob.rho)
              if a is not None and a.nbytes > 0]
    for a in pinned:
        _lib.check(lib.fe_host_register(a.ctypes.data, a.nbytes), "fe_host_register")
    for k in range(args.steps + 1):
        dist.barrier()
        t0 = time.perf_counter()
        se = GpuSystem(prob, assemble=True)
        if net is not None:
            ptr = net.predict_async(se)
            x, st = se.solve(x0_device_ptr=ptr, x0_if_better=True, **e2e_opts)
        else:
            x, st = se.solve(**e2e_opts)
        dt = time.perf_counter() - t0
        d2h = x.nbytes
        se.close()
        if k > 0:      # the first one warms the allocator
            e2e_times.append(dt)
    for a in pinned:
        _lib.check(lib.fe_host_unregister(a.ctypes.data), "fe_host_unregister")
    e2e_value = dist.max(sum(e2e_times)) / (len(e2e_times) * dist.world)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total * 1e3 / args.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 CG recurrence (x, r, p, q, one SpMV per iteration) + f32 preconditioner"
                 + (" (V-cycle)" if args.solver == "multigrid" else " (Chebyshev)"),
        "data": f"synthetic, seeded (seed {args.seed})",
        "config": workload_config(args, prob.n_dof, dist.world),
        "solver": {
            "mode": ("mixed precision: FP64 CG recurrence on the FP64 copy of the eliminated system, "
                     "preconditioned by one FP32 smoothed-aggregation V-cycle per iteration (hierarchy set up on "
                     "the device every step, Chebyshev smoothing on node-block Jacobi (3 steps on level 0, 2 below), "
                     "dense coarsest solve)"
                     if args.solver == "multigrid" else
                     "mixed precision: FP64 CG recurrence on the FP64 SELL copy, node-block Jacobi + Chebyshev "
                     "preconditioner in FP32 on the prescaled FP32 copy")
                    + (" + learned warm start (predicted every step; kept when its FP64 residual beats the zero "
                       "start)" if net is not None else ""),
            "preconditioner": args.solver,
            "learned_warm_start": net is not None,
            "l2_keep_mb": 40.0 if args.l2_keep < 0 else args.l2_keep,
            "chebyshev": {"mixed": [args.cheb, args.cheb_ratio], "plain": [args.plain_cheb, args.plain_cheb_ratio],
                          "fp32_krylov_ir": [args.ir_cheb, args.ir_cheb_ratio]},
            "step": "pattern + element kernels + reduction + loads + elimination + "
                    + ("multigrid setup + " if args.solver == "multigrid" else "") + "PCG",
        },
        "iterations": stats[-1].iterations, "restarts": stats[-1].outer, "learned_x0_used": stats[-1].x0_used,
        "assemble_ms": stats[-1].assemble_ms, "solve_ms": stats[-1].solve_ms,
        "relres": stats[-1].relres, "err_vs_fp64": err, "err_vs_fp64_reference": err_ref,
        "plain_fp64": {"s_per_solve": plain_s, "iterations": pstats[-1].iterations if pstats else None,
                       "relres": pstats[-1].relres if pstats else None},
        "speedup_vs_plain": plain_s / value if value > 0 else None,
        "mixed_without_learned": {"s_per_solve": mixed_only_s, "iterations": nstats[-1].iterations},
        ("mixed_chebyshev" if args.solver == "multigrid" else "mixed_multigrid"): {
            "s_per_solve": other_s, "iterations": ostats[-1].iterations, "relres": ostats[-1].relres},
        "fp32_krylov_ir": {"s_per_solve": ir_s, "iterations": istats[-1].iterations,
                           "refinement_steps": istats[-1].outer},
        "roofline": roofline,
        "multigrid": mg_section,
        "kernels": {
            "mixed_cheb_step": cheb_line,
            "mixed_pcg_spmv": {"kernel": "k_pcg_spmv<2,double> (the Chebyshev-preconditioned solve's FP64 SpMV)",
                               "launch_us": prof_mixed["spmv_us"], "bytes_per_launch": spmv_bytes(8),
                               "achieved_gbs": spmvmp_gbs, "frac": spmvmp_frac,
                               "launches_timed": prof_mixed["spmv_n"]},
            "plain_pcg_spmv": {"kernel": "k_pcg_spmv<2,double>", "launch_us": prof_plain["spmv_us"],
                               "bytes_per_launch": spmv_bytes(8), "achieved_gbs": spmv64_gbs,
                               "frac": spmv64_frac, "launches_timed": prof_plain["spmv_n"],
                               "fp64_tflops": (8 * nnzb / (prof_plain["spmv_us"] * 1e-6) / 1e12
                                               if prof_plain["spmv_us"] > 0 else None)},
            "plain_cheb_step": {"kernel": "k_cheb_step<2,double,double,2,0>", "launch_us": prof_plain["cheb_us"],
                                "bytes_per_launch": cheb_bytes(8), "achieved_gbs": cheb64_gbs,
                                "frac": cheb64_frac, "launches_timed": prof_plain["cheb_n"]},
        },
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "inputs": "pinned host memory (fe_host_register)"},
        "gpu_launches": int(n_launch),
        "clocks": clk,
    }
    if dist.world == 1 and net is not None:
        # the learned part's own throughput on the same mesh: inference and one training
        # step (forward, backward through the tcgen05 GEMMs, Adam)
        from finite_elements_gb300 import gnn_bench
        out["learned_network"] = dict(gnn_bench.measure(args.nx, args.ny, reps=3, seed=args.seed),
                                      method=f"python -m finite_elements_gb300.gnn_bench --nx {args.nx} "
                                             f"--ny {args.ny} --reps 3")
    if dist.world == 1 and args.batch_n > 0:
        # hundreds of uneven instances in one batched system (persistent kernel, CUDA
        # graph, autotuned tiles) against the same instances solved one at a time
        from finite_elements_gb300 import batch_bench, meshgen as mg
        ba = argparse.Namespace(n=args.batch_n, seed=args.seed, tol=args.tol, single=args.batch_single, cheb=16,
                                cheb_ratio=1e4)
        out["batched"] = dict(batch_bench.measure(ba, mg.batch_c4(args.batch_n, seed=args.seed)),
                              method="python -m finite_elements_gb300.batch_bench --n "
                                     f"{args.batch_n} --single {args.batch_single} --seed {args.seed}")
    if dist.world == 1 and not args.no_cpu_baseline:
        # the CPU baseline at the full workload, measured, and the FP64 oracle solution the
        # mixed result's error is taken against
        x_cpu, dt, tm = cpu_direct_solve(prob)
        model, ncpu = cpu_info()
        out["cpu_baseline"] = {"value": dt, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"the full workload ({prob.n_dof:,} DOF), one solve: {CPU_METHOD}",
                               "assemble_s": tm["assemble_s"], "solve_s": tm["solve_s"],
                               "relres": tm["relres"], "host": f"{model}, {ncpu} cores"}
        out["err_vs_fp64"] = float(np.linalg.norm(x_mixed[:n] - x_cpu[:n]) / np.linalg.norm(x_cpu[:n]))
        out["err_vs_fp64_reference"] = "the CPU FP64 direct solve of the cpu_baseline leg (SuperLU)"
    return out


def run_tet(args):
    """Secondary measurement, not the headline: s/solve to args.tol of the solid
    cantilever of linear tetrahedra (scripts/Elasticity/beam3d_example_2.py set-up):
    the FP64 CG with the FP32 smoothed-aggregation V-cycle (six rigid-body modes;
    hierarchy set up on the device in every solve, its time included; `value`), the
    FP64 CG with the FP32 Chebyshev preconditioner, and plain FP64 PCG with the
    node-block Jacobi preconditioner.  Device time (CUDA events on the handle
    stream) of the solve, inputs resident; the matrices are far larger than L2."""
    import ctypes

    import numpy as np

    from finite_elements_gb300 import _lib, meshgen
    from finite_elements_gb300.engine import GpuSystem

    prob = meshgen.cantilever_3d(*args.tet_dims)
    s = GpuSystem(prob)
    runs = {"plain": dict(precision="fp64", cheb_degree=0),
            "chebyshev": dict(precision="mixed-cg64", cheb_degree=args.tet_cheb, cheb_ratio=args.tet_cheb_ratio),
            "multigrid": dict(precision="mixed-cg64", multigrid=True)}
    res = {}
    phases = None
    for name, kw in runs.items():
        ms, xs = [], None
        if name == "multigrid":
            s.handle.call("fe_profile_kernels", 1)   # setup phase times (and resets the sums)
        for k in range(args.warmup + args.steps):
            x, st = s.solve(tol=args.tol, **kw)
            if st.status != _lib.FE_OK:
                raise RuntimeError(f"{name} solve failed: {st.as_dict()}")
            if k >= args.warmup:
                ms.append(st.solve_ms)
            xs = x[: prob.n_dof]
        res[name] = {"s": statistics.mean(ms) / 1e3, "iterations": st.iterations, "relres": st.relres,
                     "assemble_ms": st.assemble_ms, "x": xs}
        if name == "multigrid":
            v = [ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(),
                 ctypes.c_int64()]
            s.handle.call("fe_profile_read_multigrid", *[ctypes.byref(x) for x in v])
            ph = (ctypes.c_double * _lib.FE_MG_PHASES)()
            s.handle.call("fe_profile_read_multigrid_phases", ph, _lib.FE_MG_PHASES)
            s.handle.call("fe_profile_kernels", 0)
            n_setup = max(v[3].value, 1)
            phases = {"setup_ms": v[2].value / n_setup, "cycle_ms": v[4].value / max(v[5].value, 1),
                      "setup_phases_ms": {nm: ph[k] / n_setup for k, nm in enumerate(_lib.MG_PHASE_NAMES)}}
    xp = np.linalg.norm(res["plain"]["x"])
    diff = float(np.linalg.norm(res["chebyshev"]["x"] - res["plain"]["x"]) / xp)
    diff_mg = float(np.linalg.norm(res["multigrid"]["x"] - res["plain"]["x"]) / xp)
    out = {"metric": f"s/solve to {args.tol:g} rel. residual, 3D tetrahedral elasticity: mixed precision "
                     "(multigrid) vs plain PCG",
           "value": res["multigrid"]["s"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": False, "dtype": "f64 recurrence, f32 preconditioner", "data": "synthetic",
           "config": {"workload": f"solid cantilever {args.tet_dims[0]}x{args.tet_dims[1]}x{args.tet_dims[2]} cells "
                                  f"x 6 tetrahedra ({prob.n_elements:,} elements, {prob.n_dof:,} DOF), "
                                  "x = 0 clamped, tip edge loaded in z", "l2": "inputs larger than L2",
                      "solver": "FP64 CG preconditioned by one FP32 smoothed-aggregation V-cycle (six rigid-body "
                                "modes, hierarchy set up on the device in every solve)"},
           "plain_s": res["plain"]["s"], "speedup_vs_plain": res["plain"]["s"] / res["multigrid"]["s"],
           "iterations": {k: res[k]["iterations"] for k in ("multigrid", "chebyshev", "plain")},
           "relres": {k: res[k]["relres"] for k in ("multigrid", "chebyshev", "plain")},
           "rel_diff_vs_plain": diff_mg, "assemble_ms": res["plain"]["assemble_ms"],
           "multigrid": phases or {},
           "chebyshev": {"s_per_solve": res["chebyshev"]["s"],
                         "speedup_vs_plain": res["plain"]["s"] / res["chebyshev"]["s"],
                         "degree_ratio": [args.tet_cheb, args.tet_cheb_ratio], "rel_diff_vs_plain": diff}}
    s.close()
    if not args.no_cpu_baseline:
        # the reference path on the host cores: the oracle's restatement (element loop, COO,
        # csr_matrix, NATURAL spsolve on the saddle system) on a bounded 3D sample
        from oracle import fe_oracle as O
        sample = meshgen.cantilever_3d(40, 8, 8)
        t0 = time.perf_counter()
        O.solve(sample)
        dt = time.perf_counter() - t0
        model, ncpu = cpu_info()
        out["cpu_baseline"] = {
            "value": dt, "unit": f"s/solve of the {sample.n_dof:,}-DOF sample (not scaled)", "cores": 1,
            "kind": "port",
            "sample": f"one solve of the tetrahedral cantilever 40x8x8 cells ({sample.n_dof:,} DOF) through "
                      "the oracle's restatement of the reference path (NATURAL spsolve on the saddle system); "
                      "a direct solve of the 3D workload itself does not fit the bench's time on the host",
            "host": f"{model}, {ncpu} cores"}
    return out


def workload_config(args, n_dof, world):
    """The configuration both arms name: the workload, its tolerance and placement."""
    return {"workload": f"plane strain {args.nx}x{args.ny} grid, {2 * args.nx * args.ny:,} triangles, "
                        f"{n_dof:,} DOF, E=10^U(9,12) per element, nu~U(0.2,0.45), left edge clamped, "
                        f"random top-edge traction, seed {args.seed}",
            "tol": args.tol,
            "l2": "inputs larger than L2 (BSR values alone 448 MB FP64 / 224 MB FP32)",
            "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"}


def run_reference(args, dist):
    """The reference's path on the host cores, measured on the full workload: one solve
    (assembly + elimination + SuperLU), however many steps were asked for -- a full solve
    takes minutes, so the --steps K --warmup W run would not end in the time allowed;
    the line says so in steps / steps_requested.  No sample is scaled."""
    from finite_elements_gb300 import meshgen
    prob = meshgen.plane_strain_random(args.nx, args.ny, seed=args.seed)
    x, dt, tm = cpu_direct_solve(prob)
    model, ncpu = cpu_info()
    base = {"value": dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"the full workload ({prob.n_dof:,} DOF), one solve: {CPU_METHOD}",
            "assemble_s": tm["assemble_s"], "solve_s": tm["solve_s"], "relres": tm["relres"],
            "host": f"{model}, {ncpu} cores"}
    return {"impl": "reference", "metric": METRIC, "value": dt, "unit": UNIT, "n_gpus": dist.world,
            "steps": 1, "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": False, "dtype": "f64", "data": f"synthetic, seeded "
            f"(seed {args.seed})", "config": workload_config(args, prob.n_dof, dist.world),
            "path": CPU_METHOD, "cpu_baseline": base,
            "e2e": {"value": dt, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse_args()
    dist = Dist()
    if args.workload == "tet":
        if dist.rank == 0:
            print(json.dumps(run_tet(args)))
        dist.close()
        return
    if args.impl == "reference":
        if dist.rank == 0:
            print(json.dumps(run_reference(args, dist)))
        dist.close()
        return
    out = run_ours(args, dist)
    if dist.rank == 0:
        print(json.dumps(out))
    dist.close()


if __name__ == "__main__":
    main()
