"""N>1 host logic on CPU: dataset sharding and the max-over-ranks timing,
with two gloo ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from gpu_inscy_gb300.replicas import combine, shard


def test_shard_covers_every_dataset_once():
    sizes = [50_000, 2_000, 7_000, 31_000, 2_500, 12_000, 9_999]
    for world in (1, 2, 3, 4):
        got = sorted(i for r in range(world) for i in shard(sizes, r, world))
        assert got == list(range(len(sizes)))
    a, b = shard(sizes, 0, 2), shard(sizes, 1, 2)
    la, lb = sum(sizes[i] for i in a), sum(sizes[i] for i in b)
    assert abs(la - lb) <= max(sizes)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank 0 processed 100 points in 10 ms, rank 1 processed 300 in 40 ms
    pts, ms = (100, 10.0) if rank == 0 else (300, 40.0)
    value, ms_max = combine(pts, ms)
    out[rank] = (value, ms_max)
    dist.destroy_process_group()


def test_combine_takes_slowest_rank_with_gloo():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        value, ms_max = out[r]
        assert ms_max == pytest.approx(40.0)
        assert value == pytest.approx(400 / 0.040)
