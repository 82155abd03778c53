"""Placement of batched scenes on ranks (host logic, no GPU): greedy
partition balance and a world_size-2 gloo run that gathers per-scene results
with no scene lost or duplicated."""
import os
import socket

import numpy as np
import pytest

from pbf_gb300 import scenes
from pbf_gb300.batch import gather_scene_results, imbalance, partition_scenes


def test_partition_covers_every_scene_once_and_balances():
    _, sc, _ = scenes.batch_scenes_spec()
    counts = [s["positions"].shape[0] for s in sc]
    for world in (1, 2, 4, 8):
        parts = partition_scenes(counts, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(counts)))
        # longest-first greedy: max load <= mean + largest scene
        loads = [sum(counts[i] for i in p) for p in parts]
        assert max(loads) <= sum(counts) / world + max(counts)
    assert imbalance(counts, partition_scenes(counts, 2)) < 1.02


def test_partition_is_deterministic():
    counts = [5, 5, 5, 5, 3, 3, 1]
    assert partition_scenes(counts, 3) == partition_scenes(list(counts), 3)
    assert partition_scenes(counts, 3) == [[0, 3], [1, 4, 6], [2, 5]]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, counts, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = partition_scenes(counts, world)[rank]
        # stand-in for a scene's metrics: a value only the owning rank computes
        local = {i: {"rank": rank, "value": float(np.sqrt(counts[i]) * (i + 1))} for i in mine}
        merged = gather_scene_results(local, dist)
        q.put((rank, merged))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo_gather_scene_results():
    import torch.multiprocessing as mp
    _, sc, _ = scenes.batch_scenes_spec(count=16, n_min=1000, n_max=20000, seed=5)
    counts = [s["positions"].shape[0] for s in sc]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, counts, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    parts = partition_scenes(counts, 2)
    for rank in (0, 1):
        merged = out[rank]
        assert sorted(merged) == list(range(16))
        for i, v in merged.items():
            assert v["rank"] == (0 if i in parts[0] else 1)
            assert v["value"] == pytest.approx(np.sqrt(counts[i]) * (i + 1))
