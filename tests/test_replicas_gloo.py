"""Multi-GPU bench logic on the CPU: independent replicas, world_size 2 over
gloo (127.0.0.1).  Each rank reports its own elapsed time; the job's time is
the maximum over ranks and its throughput counts the cells of every rank."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    import bench
    td.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = [100.0, 250.0][rank]
    t_max, value = bench.replica_throughput(ms_local, cells=1000, steps=10, world=world, device="cpu")
    td.barrier()
    td.destroy_process_group()
    q.put((rank, t_max, value))


def test_replica_throughput_two_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_max, value in out:
        assert t_max == 250.0
        assert value == pytest.approx(1000 * 10 * 2 / 0.25)


def test_replica_throughput_single_rank():
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    import bench
    t, v = bench.replica_throughput(50.0, cells=100, steps=4, world=1)
    assert t == 50.0 and v == pytest.approx(100 * 4 / 0.05)
