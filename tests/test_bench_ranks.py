"""The multi-GPU harness of bench.py, on CPU with gloo ranks.

The path does not shard (each rank is an independent replica of the
8192^3 GEMM, no collective on the data path), so what N > 1 adds is host
logic: every rank's timing is reduced to the slowest rank's, the reported
rate is the whole job's (weak scaling), and the reference arm runs on rank
0 only while the other ranks exit without work."""
import argparse
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 10.0 + 5.0 * rank          # rank 1 is the slow one
        out[rank] = bench.max_over_ranks(local_ms, world, torch.device("cpu"))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_time_and_the_rate_is_the_whole_job():
    world = 2
    with mp.Manager() as manager:
        out = manager.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        got = dict(out)
    assert got == {0: 15.0, 1: 15.0}
    # two replicas of 1 TFLOP each in the slowest rank's 15 ms
    assert bench.whole_job_rate(1e12, 0.015, world) == pytest.approx(2e12 / 0.015)
    # one rank: no collective, the value is the rank's own
    assert bench.max_over_ranks(7.0, 1, None) == 7.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(argparse.Namespace(steps=1, warmup=0, gpus=2))
    assert capsys.readouterr().out == ""


def test_headline_is_the_fastest_split_form_at_simt_error_or_better():
    ms = {"bf16x6": 3.9, "fp16x3": 2.5}
    assert bench.pick_headline(ms, {"bf16x6": 2.4e-7, "fp16x3": 3.6e-7}, 1.6e-6) == "fp16x3"
    # a faster form less accurate than SIMT does not count
    assert bench.pick_headline(ms, {"bf16x6": 2.4e-7, "fp16x3": 2.0e-6}, 1.6e-6) == "bf16x6"
    # none qualifies: the three-piece form is reported (and its error shows it)
    assert bench.pick_headline(ms, {"bf16x6": 2e-6, "fp16x3": 3e-6}, 1.6e-6) == "bf16x6"
    # every measure counts: accurate normwise but worse in its worst row
    simt = (1.6e-6, 2.0e-6, 1.5e-6)
    assert bench.pick_headline(ms, {"bf16x6": (2.4e-7, 3e-7, 2e-7),
                                    "fp16x3": (3.6e-7, 1.0, 3e-7)}, simt) == "bf16x6"
    assert bench.pick_headline(ms, {"bf16x6": (2.4e-7, 3e-7, 2e-7),
                                    "fp16x3": (3.6e-7, 5e-7, 3e-7)}, simt) == "fp16x3"
