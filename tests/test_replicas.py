"""bench.py's N > 1 path: N independent replicas (the duct step does not
shard: every rank steps its own copy of the run), the whole-job value from the slowest
rank.  Two gloo ranks on the CPU stand in for two GPUs."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    value, ms_max = bench.replica_throughput(times[rank], 5, device="cpu")
    q.put((rank, value, ms_max))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_use_the_slowest_rank():
    times = [400.0, 500.0]   # ms for 5 steps on each rank
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = [q.get(timeout=120) for _ in procs]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    for _, value, ms_max in out:
        assert ms_max == 500.0
        assert value == pytest.approx(2 * 5 / 0.5)


def test_one_replica_without_a_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    value, ms_max = bench.replica_throughput(250.0, 5, device="cpu")
    assert ms_max == 250.0 and value == pytest.approx(20.0)
