"""Multi-process host logic of bench.py on CPU (gloo, world size 2): the
replicas' step times are combined by maximum, and the reference arm runs on
rank 0 only.  The GPU path is replicas only: no data-path collective."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank], dist, "cpu")
    # the reference arm: ranks other than 0 return at once, without work or output
    rc = bench.run_reference(None, [], rank, world) if rank != 0 else None
    out.put((rank, got, rc))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_times_take_the_maximum_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, got, rc in res:
        assert got == [2.0, 10.0]
        assert rc is None


def test_single_process_keeps_the_values():
    import bench
    assert bench.max_over_ranks([3.5, 1.25], None) == [3.5, 1.25]
