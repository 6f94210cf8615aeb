"""Sharding of independent simulations over ranks (CPU; world size 2 over gloo)."""

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from etalon_gb300.shard import assignment, shard


def test_assignment_covers_every_item_once_and_balances():
    rng = np.random.default_rng(0)
    cells = [int(c) for c in rng.integers(256, 1537, 64) ** 2]
    for world in (1, 2, 3, 8):
        owner = assignment(cells, world)
        assert sorted(set(owner)) == list(range(min(world, len(cells))))
        load = np.bincount(owner, weights=cells, minlength=world)
        assert load.max() - load.min() <= max(cells)
        parts = [shard(list(range(64)), cells, r, world) for r in range(world)]
        assert sorted(sum(parts, [])) == list(range(64))


def test_assignment_rejects_empty_world():
    with pytest.raises(ValueError):
        assignment([1, 2], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


RANK_SCRIPT = """
import json, sys
import torch, torch.distributed as dist
from etalon_gb300.shard import shard
rank, world, cells = int(sys.argv[1]), int(sys.argv[2]), json.loads(sys.argv[3])
dist.init_process_group("gloo", rank=rank, world_size=world)
mine = shard(list(range(len(cells))), cells, rank, world)
got = [None] * world
dist.all_gather_object(got, mine)  # every rank derives the same split on its own
load = torch.tensor([float(sum(cells[k] for k in mine))])
dist.all_reduce(load, op=dist.ReduceOp.MAX)
print(json.dumps({"got": got, "max_load": float(load)}))
dist.barrier()
dist.destroy_process_group()
"""


def test_two_gloo_ranks_split_without_overlap():
    rng = np.random.default_rng(1)
    cells = [int(c) for c in rng.integers(512, 1025, 32) ** 2]
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()),
               PYTHONPATH=str(root) + os.pathsep + os.environ.get("PYTHONPATH", ""))  # fmt: skip
    procs = [subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, str(r), "2", json.dumps(cells)], env=env,
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for r in range(2)]  # fmt: skip
    outs = [p.communicate(timeout=180) for p in procs]
    for p, (_, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
    res = json.loads(outs[0][0].strip().splitlines()[-1])
    got, max_load = res["got"], res["max_load"]
    assert sorted(got[0] + got[1]) == list(range(32)) and not set(got[0]) & set(got[1])
    assert max_load <= sum(cells) / 2 + max(cells)
