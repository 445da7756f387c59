"""Replica harness of bench.py on CPU: two gloo ranks (the multi-GPU path
runs independent replicas; the only cross-rank steps are the barrier and the
slowest-rank time)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        slowest = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        alone = bench.max_over_ranks(1.5 + rank, None)
        q.put((rank, slowest, alone))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_time_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5, 1.5), (1, 2.5, 2.5)]


def test_reference_arm_prints_on_rank_zero_only(capsys, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    args = type("A", (), dict(workload="serve", steps=1, warmup=0, gpus=2))()
    bench.run_reference(args)
    assert capsys.readouterr().out == ""
