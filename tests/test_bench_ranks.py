"""bench.py's multi-rank reduction (replicas, one request stream per rank):
times are the max over ranks, work counts the sum, on two gloo ranks."""
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


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    out = bench.reduce_ranks(world, [1.0 + rank, 10.0 - rank], [100.0 * (rank + 1)])
    q.put((rank, out))
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_ranks_gloo_two_ranks():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert res[r] == [2.0, 10.0, 300.0]


def test_request_stream_differs_per_rank_and_is_seeded():
    sys.path.insert(0, ROOT)
    import bench
    first = [bench.RequestStream(rank=0).next() for _ in range(2)]
    assert first[0] == first[1]                                  # seeded: same stream twice
    r0, r1 = bench.RequestStream(rank=0), bench.RequestStream(rank=1)
    assert [r0.next()["seed"] for _ in range(5)] != [r1.next()["seed"] for _ in range(5)]
    for r in (r0.next(), r1.next()):
        assert 256 <= r["capacity"] <= 32768 and 500 <= r["steps"] <= 20000


def test_single_rank_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_ranks(1, [1.5, 2.5], [7.0]) == [1.5, 2.5, 7.0]
