"""Replica timing across ranks on CPU (gloo, world size 2): the max-over-ranks
reduction and the whole-job throughput that rank 0 reports."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from hairfb import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 1 + r seconds for its 64 frames; one value the other way round
        got = replicas.max_over_ranks([1.0 + rank, 10.0 - rank], dist, "cpu")
        out.put((rank, got, replicas.job_throughput(64, world, got[0])))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world_2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, rate in res:
        assert got == [2.0, 10.0], (rank, got)
        assert rate == pytest.approx(2 * 64 / 2.0)


def test_single_process_is_identity():
    assert replicas.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
    assert replicas.job_throughput(10, 1, 2.0) == 5.0
