"""Replicas across ranks: bench.py's rank bookkeeping over gloo with two CPU
processes (the decode itself shards by frame, with no collective)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as tmp  # noqa: E402


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    w, r, local = bench._dist()
    bench._barrier(w)
    mx = bench._max_over_ranks(w, 10.0 + r)
    total = bench._sum_over_ranks(w, 300.0)
    out.put((r, w, local, mx, total, bench.workload_seed(r)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_gloo_bookkeeping():
    world, port = 2, _free_port()
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, local, mx, total, seed) in enumerate(res):
        assert (rank, w, local) == (r, 2, r)
        assert mx == 11.0            # max over ranks of 10 + rank
        assert total == 600.0        # frames summed over ranks
    assert res[0][5] != res[1][5]    # each replica decodes its own frames
