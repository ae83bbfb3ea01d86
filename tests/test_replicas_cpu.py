"""The multi-GPU path is replicas only (one independent session per rank, no
collective on the data path). This checks the host-side aggregation of the
replica timings with two gloo ranks on CPU: max time over ranks, summed edges."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, edges, value = bench.aggregate(100.0 + 50.0 * rank, 1000 * (rank + 1))
    q.put((rank, ms, edges, value))
    tdist.barrier()
    tdist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, edges, value in out:
        assert ms == 150.0
        assert edges == 3000.0
        assert value == pytest.approx(3000.0 / 0.150)


def test_single_process_aggregation_is_identity():
    import bench
    ms, edges, value = bench.aggregate(200.0, 5000)
    assert (ms, edges) == (200.0, 5000) and value == pytest.approx(25000.0)
