"""Sharding of independent simulations over ranks (CPU; world size 2 over gloo)."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

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


def _worker(rank, world, port, cells, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard(list(range(len(cells))), cells, rank, world)
    got = [None] * world
    dist.all_gather_object(got, mine)  # every rank derives the same split on its own
    load = torch.tensor([float(sum(cells[k] for k in mine))])
    dist.all_reduce(load, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((got, float(load)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_split_without_overlap():
    rng = np.random.default_rng(1)
    cells = [int(c) for c in rng.integers(512, 1025, 32) ** 2]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, cells, q)) for r in range(2)]
    for p in procs:
        p.start()
    got, max_load = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert sorted(got[0] + got[1]) == list(range(32)) and not set(got[0]) & set(got[1])
    assert max_load <= sum(cells) / 2 + max(cells)
