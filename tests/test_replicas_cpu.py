"""CPU: the replica path with a world_size-2 gloo group (127.0.0.1)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from pycd_gb300 import replicas


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
    try:
        wall, steps = replicas.aggregate(1.5 + rank, 1000 * (rank + 1))
        out[rank] = (wall, steps, replicas.stream_offset(rank, 4096))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_aggregate_and_disjoint_streams():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        wall, steps, off = out[r]
        assert wall == 2.5 and steps == 3000.0
    assert out[0][2] == 0 and out[1][2] == 4096


def test_aggregate_without_group_is_identity():
    assert replicas.aggregate(2.0, 10) == (2.0, 10.0)
