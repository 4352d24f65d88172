"""The N > 1 path of bench.py (replicas, no data-path collective) on CPU with
two gloo ranks: the whole-job value uses the slowest rank's time, every rank
agrees on it, and the reference arm does no work on ranks other than 0."""
import multiprocessing as mp
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = [100.0, 250.0][rank]
    v, t = bench.replica_value(dist, world, 5, 1_000_000, local_ms)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, v, t))


def test_replica_value_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, v, t in res:
        assert t == 250.0                                   # max over ranks
        assert abs(v - 2 * 5 * 1_000_000 / 0.25) < 1e-6     # whole-job vertices / job time


def test_reference_arm_other_ranks_idle():
    import argparse
    import bench
    args = argparse.Namespace(steps=2, warmup=1, impl="reference", gpus=2)
    assert bench.run_reference(args, 2, 1) == 0             # rank 1: no work, exit 0
