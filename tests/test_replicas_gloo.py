"""The N > 1 path of bench.py on CPU: one process per rank over gloo (world size 2,
127.0.0.1).  The single solve does not shard, so N GPUs run N independent replicas;
what the ranks share is the barrier around the timed region and the max over ranks
of the timings, both checked here, and the reference arm, which rank 0 alone runs
and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys, time
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
assert d.world == 2 and d.rank == int(os.environ["RANK"])
time.sleep(0.2 * d.rank)                 # rank 1 arrives later: the barrier waits for it
d.barrier()
t = time.perf_counter()
d.barrier()
m = d.max(float(d.rank + 1))             # max over ranks of a per-rank timing
out = {{"rank": d.rank, "max": m, "barrier_s": time.perf_counter() - t}}
open(os.path.join({tmp!r}, f"rank{{d.rank}}.json"), "w").write(json.dumps(out))
d.close()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_env(rank, port):
    env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    env.pop("CUDA_VISIBLE_DEVICES", None)
    return env


def test_two_ranks_share_barrier_and_max(tmp_path):
    pytest.importorskip("torch.distributed")
    port = free_port()
    script = RANK_SCRIPT.format(root=ROOT, tmp=str(tmp_path))
    procs = [subprocess.Popen([sys.executable, "-c", script], env=rank_env(r, port), cwd=ROOT)
             for r in range(2)]
    for p in procs:
        assert p.wait(timeout=120) == 0
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    assert [r["max"] for r in res] == [2.0, 2.0]


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    pytest.importorskip("torch.distributed")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-nx", "20"]
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0
    assert rec["cpu_baseline"]["kind"] == "port" and rec["e2e"]["h2d_bytes_per_step"] == 0
    # the sample's time carried to the 2000 x 1000 workload's DOF in proportion
    cb = rec["cpu_baseline"]
    assert cb["sample_dof"] == 2 * 21 * 11
    full = 2 * 2001 * 1001
    assert abs(rec["value"] - cb["sample_s"] * full / cb["sample_dof"]) <= 1e-9 * rec["value"]
    assert rec["e2e"]["value"] == rec["value"] == cb["value"]
