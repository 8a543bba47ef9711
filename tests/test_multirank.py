"""The multi-rank layer of the batched form on CPU (gloo, world size 2).

Scenes are independent, so ranks split them (partition_scenes) and exchange
nothing while stepping; the only collectives are the final gather of per-scene
statistics and the maximum of the ranks' times.  These run here with the gloo
backend on the host; no GPU is involved.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp

from tichi_sph_gb300 import workloads
from tichi_sph_gb300.partition import gather_scene_stats, max_over_ranks, partition_scenes


def _counts(n=256):
    return [sc["fluid"]["max_part_num"] for _, sc in workloads.batched_dambreaks(n)]


@pytest.mark.parametrize("ws", [1, 2, 3, 4, 8])
def test_partition_covers_every_scene_once_and_balances(ws):
    counts = _counts()
    parts = partition_scenes(counts, ws)
    assert len(parts) == ws
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(counts)))
    loads = [sum(counts[i] for i in p) for p in parts]
    assert max(loads) <= 1.01 * sum(loads) / ws + max(counts)  # greedy LPT bound
    assert max(loads) / (sum(loads) / ws) < 1.02
    assert partition_scenes(counts, ws) == parts  # deterministic


def test_partition_edge_cases():
    assert partition_scenes([], 2) == [[], []]
    assert partition_scenes([5], 3) == [[0], [], []]
    assert partition_scenes([3, 3, 3, 3], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        partition_scenes([1], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, n, queue):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        counts = [((7 * i) % 13 + 1) * 100 for i in range(n)]
        mine = partition_scenes(counts, ws)[rank]
        local = [{"scene": i, "div_iter": 2 + i % 3, "rank": rank} for i in mine]
        allst = gather_scene_stats(local, mine, n, dist)
        t = max_over_ranks(1.5 + rank, dist)
        queue.put((rank, allst, t))
    finally:
        dist.destroy_process_group()


def test_gather_and_max_over_ranks_gloo():
    ws, n = 2, 37
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, n, queue)) for r in range(ws)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(ws):
        rank, allst, t = queue.get(timeout=120)
        out[rank] = (allst, t)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    allst, t0 = out[0]
    assert out[1][0] is None  # only rank 0 receives the gather
    assert t0 == 2.5 and out[1][1] == 2.5
    assert [s["scene"] for s in allst] == list(range(n))
    counts = [((7 * i) % 13 + 1) * 100 for i in range(n)]
    parts = partition_scenes(counts, ws)
    for r in range(ws):
        for i in parts[r]:
            assert allst[i]["rank"] == r and allst[i]["div_iter"] == 2 + i % 3
