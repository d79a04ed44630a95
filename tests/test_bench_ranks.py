"""The bench's multi-rank plumbing on CPU: world size 2 over gloo (one
replica per rank, no data-path collective; the ranks only agree on the
job's time), and the reference arm's rank-0-only behaviour."""
import argparse
import os
import socket

import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    w, r, local, dist = bench.dist_setup("gloo")
    try:
        # each rank's own time; every rank must end with the slowest one
        v = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        q.put((r, w, local, v))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(r, w, local) for r, w, local, _ in out] == [(0, 2, 0), (1, 2, 1)]
    assert [v for *_, v in out] == [2.5, 2.5]


def test_single_rank_needs_no_process_group(monkeypatch):
    for key in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(key, raising=False)
    w, r, local, dist = bench.dist_setup("gloo")
    assert (w, r, local, dist) == (1, 0, 0, None)
    assert bench.max_over_ranks(3.25, dist, "cpu") == 3.25


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun only rank 0 times the CPU implementation and prints;
    the other ranks exit without work."""
    monkeypatch.setenv("RANK", "1")
    args = argparse.Namespace(warmup=3, steps=1, gpus=2, mode="fp64", maxit=0, precond="")
    bench.run_reference(args, dict(bench.CONFIGS["c2"]))
    assert capsys.readouterr().out == ""
