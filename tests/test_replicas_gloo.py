"""The replica path of bench.py on CPU: two gloo ranks (world size 2).

Serving requests and assembly replicas are independent per GPU ("replicas
only"); the one collective is the max over ranks of the step time, which
every rank must see, and the whole-job value is the sum over replicas.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    w, r, local = bench.dist_env()
    t = bench.max_over_ranks(1.0 + 0.5 * r, dist)  # rank 1 is the slow one
    q.put((r, w, local, t))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == 1.5 for o in out)  # every rank sees the slowest step time


def test_max_over_ranks_single():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(2.5, None) == 2.5
