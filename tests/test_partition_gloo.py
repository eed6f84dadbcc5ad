"""Multi-process host logic on CPU (gloo, world size 2): the batched work
list is split between replicas with no exchange; every sort lands on exactly
one rank and the bytes are balanced."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from spaghetty_gb300.batched import partition
        from spaghetty_gb300.workloads import batched_mix
        jobs = batched_mix(4096, seed=2024)
        mine = partition(jobs, rank, world)
        sizes = [None] * world
        dist.all_gather_object(sizes, mine)
        bytes_per = []
        for lst in sizes:
            b = 0
            for i in lst:
                n = 1
                for d in jobs[i]["dims"]:
                    n *= d
                b += n * (24 if jobs[i]["acc"] else 16)
            bytes_per.append(b)
        if rank == 0:
            q.put((sizes, bytes_per))
    finally:
        dist.destroy_process_group()


def test_partition_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    sizes, bytes_per = q.get()
    allidx = sorted(sizes[0] + sizes[1])
    assert allidx == list(range(4096))
    assert not set(sizes[0]) & set(sizes[1])
    assert abs(bytes_per[0] - bytes_per[1]) / max(bytes_per) < 0.05
