"""The N>1 path of bench.py is replicas only: each rank applies its own copy
of the operator, and the job time is the max over ranks.  The reduction and
the whole-job value are exercised here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = [0.25, 0.75][rank]
    m = bench.allreduce_max(t, world, device="cpu")
    units = 1000
    q.put((rank, m, world * units / m))
    dist.destroy_process_group()


def test_two_rank_max_over_ranks_and_whole_job_value():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    for rank, m, value in out:
        assert m == 0.75
        assert abs(value - 2 * 1000 / 0.75) < 1e-9
