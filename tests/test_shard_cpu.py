"""Sharding of the ensemble over ranks, and the bench's rank reductions,
on CPU with world size 2 over gloo (no GPU)."""

import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from ludwig_gb300 import shard  # noqa: E402


def uneven_box_extents(nbox=64, seed=20261203, edges=(32, 48, 64, 96)):
    rng = np.random.default_rng(seed)
    return [[int(rng.choice(edges)) for _ in range(3)] for _ in range(nbox)]


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_shards_partition_and_balance(world):
    boxes = uneven_box_extents()
    shards = shard.shard_boxes(boxes, world)
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(boxes)))
    loads = [sum(shard.box_sites(boxes[i]) for i in s) for s in shards]
    biggest = max(shard.box_sites(b) for b in boxes)
    # LPT: no rank carries more than the lightest plus one box
    assert max(loads) - min(loads) <= biggest
    assert shard.shard_boxes(boxes, world) == shards       # deterministic


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["RANK"] = str(rank)
    os.environ["WORLD_SIZE"] = str(world)
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, pg = bench.dist_setup()
    try:
        boxes = uneven_box_extents()
        mine = shard.shard_boxes(boxes, w)[r]
        stats = [shard.box_sites(boxes[i]) for i in mine]
        full = shard.gather_box_stats(pg, len(boxes), mine, stats)
        sites = bench.sum_over_ranks(pg, sum(stats))
        slowest = bench.max_over_ranks(pg, 10.0 + r)
        bench.barrier(pg)
        q.put((r, full, sites, slowest))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q))
             for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    boxes = uneven_box_extents()
    want = [shard.box_sites(b) for b in boxes]
    for r, full, sites, slowest in res:
        assert full == want                  # every box once, in order
        assert sites == sum(want)            # sum over ranks
        assert slowest == 11.0               # max over ranks
