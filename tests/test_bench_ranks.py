"""The benchmark's multi-process path, on the CPU with gloo.

The lattice path does not shard (one lattice per process), so `bench.py
--gpus N` runs N independent replicas: the ranks meet at barriers around the
timed region, the whole job's time is the slowest rank's and its projections
the sum over ranks, and only rank 0 prints. The reference arm runs on rank 0
alone; the other ranks exit at once. These are the reductions and rules the
N > 1 runs use, exercised here over two gloo ranks.
"""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(dist, torch)
        slowest = bench.max_over_ranks(1.5 + rank, dist, torch)
        total = bench.sum_over_ranks(10.0 * (rank + 1), dist, torch)
        bench.barrier(dist, torch)
        out.put((rank, slowest, total))
    finally:
        dist.destroy_process_group()


def test_replica_reductions_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # Every rank sees the slowest rank's time and the job's total work.
    assert results == [(0, 2.5, 30.0), (1, 2.5, 30.0)]


def test_single_process_reductions_are_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.0, None, None) == 3.0
    assert bench.sum_over_ranks(4.0, None, None) == 4.0
    bench.barrier(None, None)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    bench.run_reference(None)  # returns before touching its arguments
    assert capsys.readouterr().out == ""
