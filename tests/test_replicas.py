"""The multi-GPU path is replicas (one domain per rank, no data exchange):
the bench's rank helpers on two gloo ranks on the CPU."""
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    bench.barrier(ws)
    slowest = bench.max_over_ranks(100.0 * (rank + 1), ws)    # ms of this rank's timed steps
    value = bench.replica_value(1_036_800, 500, 10, slowest, ws)
    q.put((rank, slowest, value))
    bench.barrier(ws)
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank_and_sum_the_cells():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expect = 2 * 1_036_800 * 500 * 10 / 0.2 / 1e9
    for rank, slowest, value in got:
        assert slowest == 200.0
        assert abs(value - expect) <= 1e-9 * expect


def test_reference_arm_only_rank_zero_works(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class A:
        config = "c1_4deg"
        subcycles = None
        steps = 1
        warmup = 0
        seed = 0
        gpus = 2
    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
