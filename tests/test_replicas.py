"""Multi-GPU replica bookkeeping (csgrt/replicas.py) with two gloo ranks on the CPU: the
shards of a batch cover every view exactly once with balanced loads, the job time is the
slowest rank's, and the barrier and single-process paths work."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, costs, out_dir):
    sys.path.insert(0, str(ROOT / "cuda-csg-tree-raycasting_gb300"))
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch.distributed as tdist
    from csgrt import replicas
    dist = replicas.init("gloo")
    assert dist is not None and tdist.get_world_size() == world
    mine = replicas.shard(costs, rank, world)
    shards = [None] * world
    dist.all_gather_object(shards, mine)
    replicas.barrier(dist)
    slowest = replicas.max_over_ranks(dist, 10.0 + rank)
    with open(Path(out_dir) / f"rank{rank}.txt", "w") as f:
        f.write(repr((shards, slowest)))
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    costs = [float((7 * i) % 13 + 1) for i in range(37)]
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), costs, str(tmp_path)), nprocs=world, join=True)
    results = [eval((tmp_path / f"rank{r}.txt").read_text()) for r in range(world)]
    shards, slowest = results[0]
    assert all(r == results[0] for r in results)  # every rank saw the same shards and maximum
    assert slowest == 10.0 + world - 1
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(costs)))  # each view exactly once
    loads = [sum(costs[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(costs)  # greedy balance


def test_single_process_paths():
    sys.path.insert(0, str(ROOT / "cuda-csg-tree-raycasting_gb300"))
    from csgrt import replicas
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert replicas.dist_info() == (1, 0, 0)
    assert replicas.init("gloo") is None
    replicas.barrier(None)
    assert replicas.max_over_ranks(None, 3.5) == 3.5
    assert replicas.shard([1.0, 2.0, 3.0], 0, 1) == [0, 1, 2]
    assert replicas.throughput(1000, 4, 2.0) == pytest.approx(2.0e6)
