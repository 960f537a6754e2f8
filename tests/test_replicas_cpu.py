"""The multi-GPU form is replicas only (one independent network per GPU, no data-path collective):
bench.py reports the slowest replica's time and the events of all replicas. Checked here with two
gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t, ev = bench.replica_totals(0.5 + rank, 1000 * (rank + 1), "cpu")
    q.put((rank, t, ev))
    dist.destroy_process_group()


def test_replica_totals_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, t, ev in got:
        assert t == 1.5  # the slowest replica
        assert ev == 3000.0  # all replicas' events


def test_replica_totals_single_process():
    import bench

    assert bench.replica_totals(0.25, 7) == (0.25, 7.0)


@pytest.mark.parametrize("rank", ["1"])
def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys, rank):
    """Under torchrun only rank 0 runs and prints the reference arm."""
    import sys

    import bench

    monkeypatch.setenv("RANK", rank)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    bench.main()
    assert capsys.readouterr().out == ""
