"""The benchmark's multi-GPU form is replicas with no data-path collective:
each rank builds its own scene and the job's time is the slowest rank's.
That aggregation (bench.max_over_ranks) and the rank bookkeeping
(bench.rank_info), run as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), LOCAL_RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, local, w = bench.rank_info()
        assert (r, local, w) == (rank, rank, world)
        # each rank's own "step time"; every rank must see the largest
        got = bench.max_over_ranks(10.0 + 3.5 * rank, torch, "cpu", w)
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(out.get(timeout=10) for _ in range(world))
    assert res == [(0, 13.5), (1, 13.5)]


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(7.25, torch, "cpu", 1) == 7.25
