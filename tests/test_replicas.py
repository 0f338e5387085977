"""The N > 1 path of bench.py on CPU: world size 2 over gloo.

The hot path does not shard (replicas only): every rank solves its own copy
and the job's time is the slowest rank's.  These tests run the rank logic --
rendezvous, the max-over-ranks reduction, the whole-job value -- in two
processes, without a GPU.
"""

from __future__ import annotations

import os
import pathlib
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, loc = bench.dist_env()
    ms = 100.0 + 25.0 * rank            # rank 1 is the slower replica
    job_ms = bench.job_time_max(ms, w)
    value = bench.whole_job_value(640_000 * 5000, 4, w, job_ms)
    dist.barrier()
    dist.destroy_process_group()
    out.put((r, w, loc, job_ms, value))


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in procs)
    assert [r[:3] for r in res] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, job_ms, value in res:
        assert job_ms == pytest.approx(125.0)
        # 2 replicas x 4 steps x 640,000 x 5000 updates in the slowest rank's 125 ms
        assert value == pytest.approx(2 * 4 * 640_000 * 5000 / 0.125)


def test_single_rank_is_unchanged():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.job_time_max(42.0, 1) == 42.0
    assert bench.whole_job_value(10.0, 3, 1, 1000.0) == pytest.approx(30.0)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit 0 without work."""
    import subprocess

    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
