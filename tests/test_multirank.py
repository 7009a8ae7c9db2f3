"""The N > 1 path of bench.py (replicas: one rig per rank, no collective on the data path) on two CPU ranks over
gloo: the step time every rank reports is the slowest rank's, and the whole-job value counts every rank's rigs."""
import os
import socket
import sys

import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, local, w = bench.dist_env()
    own = 10.0 + 5.0 * rank  # ms: rank 1 is the slow one
    slowest = bench.max_over_ranks(own, w, device="cpu")
    value = bench.replica_value(w, 4, 0.5, slowest / 1e3)
    q.put((r, local, w, slowest, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_over_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1] and all(g[2] == world for g in got)
    for r, local, w, slowest, value in got:
        assert local == r
        assert slowest == pytest.approx(15.0)                  # every rank sees the slowest rank's time
        assert value == pytest.approx(2 * 4 * 0.5 / 0.015)      # both ranks' rigs over that time


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_value(1, 2, 0.25, 0.5) == pytest.approx(1.0)
