"""Sharding of the batched workload over ranks (one GPU each; the instances are
independent, so no data crosses between ranks): the split itself, and two gloo ranks
on CPU agreeing on it and covering every instance once.  The batched solves run on
the GPU (tests/test_gpu_batch.py)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from finite_elements_gb300 import meshgen
from finite_elements_gb300.batch import shard_instances
from test_replicas_gloo import ROOT, free_port, rank_env


def c4_dofs(n=512, seed=0):
    sizes, _ = meshgen.batch_instance_sizes(n, seed=seed)
    return [2 * (nx + 1) * (ny + 1) for nx, ny in sizes]


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_shards_cover_every_instance_once_and_balance(world):
    dofs = c4_dofs()
    shards = shard_instances(dofs, world)
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(dofs)))
    assert all(s == sorted(s) for s in shards)
    loads = [sum(dofs[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(dofs)
    assert shard_instances(dofs, world) == shards           # deterministic


def test_shard_edge_cases():
    assert shard_instances([], 3) == [[], [], []]
    assert shard_instances([5], 2) == [[0], []]
    assert shard_instances([4, 4, 4, 4], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard_instances([1], 0)


RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, {root!r})
import torch
import torch.distributed as td
from finite_elements_gb300 import meshgen
from finite_elements_gb300.batch import shard_instances
td.init_process_group("gloo")
rank, world = td.get_rank(), td.get_world_size()
sizes, _ = meshgen.batch_instance_sizes(512, seed=0)
dofs = [2 * (nx + 1) * (ny + 1) for nx, ny in sizes]
mine = shard_instances(dofs, world)[rank]
got = [None] * world
td.all_gather_object(got, mine)
c = torch.tensor([float(sum(dofs[i] for i in mine))], dtype=torch.float64)
td.all_reduce(c, op=td.ReduceOp.SUM)
open(os.path.join({tmp!r}, f"rank{{rank}}.json"), "w").write(json.dumps({{"all": got, "dof": c.item()}}))
td.destroy_process_group()
"""


def test_two_ranks_agree_on_the_shards(tmp_path):
    pytest.importorskip("torch.distributed")
    port = free_port()
    script = RANK_SCRIPT.format(root=ROOT, tmp=str(tmp_path))
    procs = [subprocess.Popen([sys.executable, "-c", script], env=rank_env(r, port), cwd=ROOT) for r in range(2)]
    for p in procs:
        assert p.wait(timeout=120) == 0
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    assert res[0]["all"] == res[1]["all"]
    flat = sorted(i for s in res[0]["all"] for i in s)
    assert flat == list(range(512))
    assert res[0]["dof"] == res[1]["dof"] == float(sum(c4_dofs()))
