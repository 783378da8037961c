"""The N > 1 bench path on CPU: two gloo ranks shard the cases, meet at the barrier and
take the max of their times (bench.py's dist_init / barrier / reduce_max / shard)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    r, w, _ = bench.dist_init()
    lo, hi = bench.shard(3001, r, w)
    bench.barrier(w)
    t = bench.reduce_max(float(10 + r), w)
    q.put((r, lo, hi, t))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got[0][1:3] == (0, 1501) and got[1][1:3] == (1501, 3001)
    assert got[0][3] == got[1][3] == 11.0
