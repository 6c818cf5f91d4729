"""The multi-rank host logic of bench.py on CPU: two gloo ranks reduce their
step times to the slowest one (the value every rank then reports), and the
reference arm's non-zero ranks leave without work."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.reduce_max(10.0 + 5.0 * rank, world)
    finally:
        dist.destroy_process_group()


def test_reduce_max_two_gloo_ranks():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        ps = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
            assert p.exitcode == 0
        assert dict(out) == {0: 15.0, 1: 15.0}


def test_reduce_max_single_rank_is_identity():
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5


def test_reference_arm_nonzero_rank_exits_without_work(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class A:
        steps, warmup, gpus, body = 1, 0, 2, "mesh"

    def boom(*a, **k):
        raise AssertionError("rank 1 must not build the workload")
    monkeypatch.setattr(bench, "workload", boom)
    assert bench.run_reference(A()) == 0
