"""The N > 1 path of bench.py: independent replicas, step time = max over
ranks, throughput = all ranks' units / that time.  Two gloo ranks on the CPU."""
import os

import pytest


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from bench import replica_throughput

    ms, value = replica_throughput(10.0 + 5.0 * rank, 1000, world, "cpu")
    q.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas():
    import multiprocessing as mp
    import socket

    ctx = mp.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in got:
        assert ms == pytest.approx(15.0)
        assert value == pytest.approx(2 * 1000 / 15e-3)


def test_single_replica_without_process_group():
    from bench import replica_throughput

    ms, value = replica_throughput(20.0, 500, 1, "cpu")
    assert ms == 20.0 and value == pytest.approx(500 / 20e-3)
