"""The host logic of bench.py on CPU: two gloo ranks reduce their step times
to the slowest one (the value every rank then reports), the reference arm's
non-zero ranks leave without work, and its rank 0 prints the arm's JSON
line."""
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
        steps, warmup, gpus, grid = 1, 0, 2, "320x160x128"

    def boom(*a, **k):
        raise AssertionError("rank 1 must not build the workload")
    monkeypatch.setattr(bench, "workload", boom)
    assert bench.run_reference(A()) == 0


def test_reference_arm_line_contract():
    """`bench.py --impl reference` on rank 0 prints one JSON line with the
    reference arm's contract: impl, the metric and unit of our arm, a value,
    at least three warm-up steps, a cpu_baseline describing the run and an
    e2e that moves no bytes between host and device."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1",
                        "--grid", "320x160x128"], cwd=root, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d["impl"] == "reference" and d["unit"] == "MLUPS" and d["metric"] == bench.METRIC
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] >= 3
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("320x160x128")


def test_both_arms_print_one_metric_string():
    """The two arms' lines carry the same metric string, the module's METRIC
    (MLUPS with the roofline share, the fp16-store against fp32 comparison),
    so that their values can be divided."""
    import inspect

    import bench
    assert bench.METRIC.startswith("MLUPS") and "FP16-store vs FP32" in bench.METRIC
    for fn in (bench.run_ours, bench.run_reference):
        src = inspect.getsource(fn)
        assert '"metric": METRIC' in src, fn.__name__
        assert '"metric": "' not in src, fn.__name__
