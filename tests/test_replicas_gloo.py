"""The benchmark's multi-rank path on CPU: two gloo ranks, as torchrun starts
them, join, pass the barrier and agree on the maximum timing over ranks; the
whole-job value counts every rank's evaluations against the slowest rank.
(The path runs independent replicas: no collective touches the data.)"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "PLK_BENCH_GLOO": "1"})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_setup(world)
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    dev_ms = 10.0 * (rank + 1)          # rank 1 is the slower replica
    max_ms = bench.reduce_max(w, dev_ms, "cpu")
    steps = 4
    value = w * steps / (max_ms / 1e3)
    out.put((rank, max_ms, value))
    dist.destroy_process_group()


def test_two_rank_replicas_take_the_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [20.0, 20.0]
    # 2 ranks x 4 evaluations over the slowest rank's 20 ms
    assert res[0][2] == pytest.approx(2 * 4 / 0.020)
