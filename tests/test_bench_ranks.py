"""The bench's N>1 path on CPU: replicas on a world-size-2 gloo group.

bench.py runs one independent replica of the operator per rank (the path
does not shard across GPUs); the timed region is bracketed by barriers, the
time is the maximum over ranks and the value counts every rank's work.  These
tests run that aggregation with two gloo processes.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=ws)
    try:
        env = bench.dist_env()
        # rank r "took" 10 (r + 1) ms; every rank must see the slowest
        ms = bench.max_over_ranks(10.0 * (rank + 1), env[0], "cpu")
        val = bench.replica_value(1e9, ms, env[0])
        q.put((rank, env, ms, val))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_replica_value_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, env, ms, val in res:
        assert env == (2, rank, rank)
        assert ms == 20.0
        assert val == pytest.approx(2 * 1e9 / 0.020)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.replica_value(2e9, 4.0, 1) == pytest.approx(5e11)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Under torchrun the reference arm's other ranks exit without work."""
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference(None) is None
