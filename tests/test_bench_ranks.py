"""The N > 1 bench path runs replicas: no data exchange, one all-reduce of the
step time (max) and of the binned pairs (sum).  Checked with two gloo ranks
on the CPU; rank 1 of the CPU reference arm exits without work."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    t, b = bench.aggregate_ranks(0.5 + rank, 1_000_000_007 * (rank + 1), ws, device="cpu")
    out.put((rank, t, b))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get() for _ in range(2))
    for rank, t, b in got:
        assert t == pytest.approx(1.5)          # the slowest rank's step time
        assert b == 1_000_000_007 * 3           # all ranks' binned pairs


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_ranks(0.25, 12345, 1) == (0.25, 12345)


def test_reference_arm_rank1_exits_without_work(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    bench.main()
    assert capsys.readouterr().out == ""
