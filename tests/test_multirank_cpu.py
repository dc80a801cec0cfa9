"""The replica path of the benchmark on CPU: two gloo ranks, the job time is the max over
ranks (the slowest replica defines the wall time of the job)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [12.5, 30.0][rank]
    out = bench.reduce_max(ms, world)
    dist.barrier()
    q.put((rank, out))
    dist.destroy_process_group()


def test_reduce_max_over_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 30.0, 1: 30.0}
    assert all(p.exitcode == 0 for p in procs)


def test_reduce_max_single_rank_is_identity():
    import bench
    assert bench.reduce_max(7.25, 1) == 7.25
