"""bench.py's multi-rank path (one independent replica per rank, no data-path
collective): barrier and max-over-ranks timing with world_size 2 over gloo on CPU."""
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


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t_local = 1.0 + rank          # rank 1 is the slower replica
    bench._barrier(world)
    t = bench._max_over_ranks(t_local, world)
    value = bench.sypd(4, t) * world
    q.put((rank, t, value))
    dist.destroy_process_group()


def test_two_replicas_max_over_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res[0][1] == res[1][1] == 2.0          # both ranks report the slowest time
    sys.path.insert(0, ROOT)
    import bench
    assert res[0][2] == pytest.approx(2 * bench.sypd(4, 2.0))
