"""Replica partitioning and the max-over-ranks reduction, with 2 gloo ranks on the CPU."""
import os
import socket

import pytest

from redux_gb300.replicas import patch_range


def test_patch_range_partitions():
    for total in (1, 7, 225, 400):
        for world in (1, 2, 3, 8):
            got = [patch_range(total, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == total
            for (a, b), (c, d) in zip(got, got[1:]):
                assert b == c
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        patch_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from redux_gb300.replicas import max_over_ranks, patch_range
    a, b = patch_range(225, rank, world)
    local_ms = 100.0 + 10.0 * rank
    mx = max_over_ranks([local_ms, float(b - a)])
    q.put((rank, a, b, mx))
    dist.destroy_process_group()


def test_gloo_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert out[0][1:3] == (0, 113) and out[1][1:3] == (113, 225)
    assert out[0][3] == out[1][3] == [110.0, 113.0]
