"""The multi-GPU host path (independent replicas) on CPU with gloo, two
ranks: barrier, maximum of per-rank times, whole-job throughput."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "vulkan-compute-ray-tracing_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from rtgb import replicas
    w, r, local = replicas.init("gloo")
    assert (w, r, local) == (world, rank, rank)
    replicas.barrier(w)
    mine = 1.0 + rank * 0.5  # the slower rank sets the job time
    worst = replicas.max_over_ranks(mine, w)
    out.put((rank, worst, replicas.job_throughput(100.0, w, worst)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    import torch.multiprocessing as mp
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [1.5, 1.5]
    assert all(abs(r[2] - 200.0 / 1.5) < 1e-9 for r in res)


def test_single_process_is_world_one():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "vulkan-compute-ray-tracing_gb300"))
    from rtgb import replicas
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert replicas.init() == (1, 0, 0)
    assert replicas.max_over_ranks(3.0, 1) == 3.0
