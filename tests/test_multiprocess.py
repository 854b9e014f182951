"""Multi-rank host logic of the benchmark (replicas: disjoint systems per rank, max-over-ranks timing),
run as world-size-2 gloo processes on the CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, _ = bench.dist_setup()
    seeds = list(bench.shard_seeds(r, 8))
    t = bench.max_over_ranks(1.0 + r, w)
    bench.barrier(w)
    gathered = [None] * w
    dist.all_gather_object(gathered, seeds)
    q.put((r, t, gathered))
    dist.destroy_process_group()


def test_replicas_shard_disjoint_and_time_is_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, gathered in out:
        assert t == 2.0
        assert len(set(gathered[0]) & set(gathered[1])) == 0
        assert len(gathered[0]) == len(gathered[1]) == 8
