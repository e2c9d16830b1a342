"""Multi-process path of the benchmark on the CPU: world size 2 over gloo.

Runs on N GPUs are N independent replicas (one process per GPU); the only
cross-rank step is the timing reduction of ``dtmm_gb300.replicas``: the job's
time is the slowest rank's and its throughput counts every rank's units.
Checked here with two gloo ranks on 127.0.0.1 that report different times,
and, for the benchmark's reference arm, that a rank other than 0 returns
without work.
"""
import json
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from dtmm_gb300.replicas import job_throughput, job_time_ms

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
        job = job_time_ms(ms, dist, "cpu")
        value = job_throughput(1000.0, job, world)
        with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
            json.dump({"ms": ms, "job": job, "value": value}, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    if not torch.distributed.is_available():
        pytest.skip("torch.distributed not available")
    port = _free_port()
    mp.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(2)]
    assert [r["ms"] for r in res] == [10.0, 15.0]
    for r in res:
        assert r["job"] == 15.0  # max over ranks, on every rank
        assert r["value"] == pytest.approx(2 * 1000.0 / 0.015)


def test_single_process_is_its_own_job():
    from dtmm_gb300.replicas import job_throughput, job_time_ms

    assert job_time_ms(12.5) == 12.5
    assert job_throughput(500.0, 12.5, 1) == pytest.approx(40000.0)
    with pytest.raises(ValueError):
        job_throughput(1.0, 0.0, 1)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        warmup, steps, gpus = 0, 1, 2

    bench.run_reference(Args(), 1)  # rank 1: no work, no output
    assert capsys.readouterr().out == ""
