"""The multi-rank path of bench.py on CPU (gloo, world size 2, 127.0.0.1):
the job time is the maximum over ranks, every rank sees it, and under the
reference arm only rank 0 works (the others return without output)."""

import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, local = bench._dist()
    got = bench._reduce_max(1.5 + rank, torch.device("cpu"), w)
    dist.barrier()
    args = type("A", (), dict(steps=3, warmup=3, gpus=w))()
    ref = bench.run_reference(args) if rank != 0 else "rank0"
    dist.destroy_process_group()
    q.put((rank, w, r, got, ref))


def test_reduce_max_and_reference_arm_over_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[:3] for r in res] == [(0, 2, 0), (1, 2, 1)]
    assert all(r[3] == 2.5 for r in res)     # max over ranks on every rank
    assert res[1][4] is None                  # the reference arm: rank 1 does no work
